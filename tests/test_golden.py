"""The oracle (CPU) and the CUDA path (GPU) against the committed golden fixtures.

tests/golden/make_golden.py wrote the fixtures from seeded tiny scenes; each
stores its scene description, so inputs are rebuilt bit-identically on any
machine by the oracle's IEEE-only ray caster. The FP32 oracle uses only
correctly rounded binary32 operations, so it must reproduce the fixtures bit
for bit on x86 and Arm alike; the FP64 oracle uses the host libm (exp, pow),
so it is held to 1e-9 relative.
"""
import os

import numpy as np
import pytest

from oracle import binding as O
from stratusgfx_gb300 import abi, stage
from stratusgfx_gb300 import scene as S

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
sys_path_helper = os.path.join(HERE, "make_golden.py")

import importlib.util  # noqa: E402

_spec = importlib.util.spec_from_file_location("make_golden", sys_path_helper)
make_golden = importlib.util.module_from_spec(_spec)
_spec.loader.exec_module(make_golden)


def load_case(name):
    d = dict(np.load(os.path.join(HERE, name + ".npz")))
    scene = S.scene_from_arrays({k[len("scene_"):]: v for k, v in d.items() if k.startswith("scene_")})
    w, _, overrides = make_golden.CASES[name]
    return w, scene, overrides, d


@pytest.mark.parametrize("name", sorted(make_golden.CASES))
def test_oracle_reproduces_golden_fixture(name):
    w, scene, overrides, d = load_case(name)
    out = make_golden.run_case(w, scene, overrides)
    for k, v in out.items():
        ref = d[k]
        if k.startswith("f32_"):
            same = (v == ref) | (np.isnan(v) & np.isnan(ref))
            assert same.all(), f"{name}:{k} differs in {(~same).sum()} values"
        else:
            np.testing.assert_allclose(v, ref, rtol=1e-9, atol=1e-12, err_msg=f"{name}:{k}")


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(make_golden.CASES))
def test_cuda_path_reproduces_golden_fixture(name):
    torch = pytest.importorskip("torch")
    from helpers import upload_cubes, upload_gbuffer
    w, scene, overrides, d = load_case(name)
    hs = O.HostScene(scene, w)
    cfg = stage.workload_config(w, **overrides)
    g = [upload_gbuffer(x) for x in hs.gbuffers]
    csm_t = [torch.from_numpy(x).cuda() for x in hs.csm_depth]
    cube_t, cubes = upload_cubes(hs.cube_storage, w.cube_format, scene.layers_per_atlas)
    st = stage.GiStage(cfg)
    st.set_lights(torch.from_numpy(scene.vpls).cuda(), torch.from_numpy(scene.entries).cuda(),
                  torch.from_numpy(scene.points).cuda() if len(scene.points) else None)
    out = torch.empty((w.height, w.width, 4), dtype=torch.float16, device="cuda")
    for k in (1, 2):
        st.set_shadow_maps(stage.csm_struct(scene, k, csm_t[k].data_ptr(), w.csm_resolution), cubes)
        st.render_frame(g[k], g[k - 1], hs.camera(k), out, make_golden.TIME + 16.0 * k, make_golden.FPS)
        torch.cuda.synchronize()
        got = out.cpu().numpy().astype(np.float32)[..., :3]
        ref = d[f"f32_k{k}_combined"][..., :3]
        same = (got == ref) | (np.isnan(got) & np.isnan(ref))
        assert same.all(), f"{name} frame {k}: {(~same).sum()} HDR values differ"
        vis = st.read_debug(abi.SGI_DEBUG_VISIBLE_INDEX, np.int32)
        cnt = int(d[f"f32_k{k}_visible_index"][0])
        assert np.array_equal(vis[:1 + cnt], d[f"f32_k{k}_visible_index"][:1 + cnt])
    st.close()
