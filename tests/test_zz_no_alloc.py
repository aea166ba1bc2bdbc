"""sgi_cull_vpls_noalloc: the VPL visibility cull with no context and no allocation.

Its results are compared with the oracle's cull (a CPU restatement of
viscull_vpls.cs) and with the context entry point sgi_cull_vpls on the same
scene, for two calls in a row on caller-owned buffers (the second call reuses
the library's fixed flag array after the first). The work is integer and byte
copying, so the tolerance is exact equality. A separate process checks that the
calls leave the device's free memory unchanged.
"""
import ctypes as C
import os
import subprocess
import sys

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from oracle import binding as O  # noqa: E402
from stratusgfx_gb300 import abi, stage  # noqa: E402
from stratusgfx_gb300 import scene as S  # noqa: E402

MAX_VPLS = 16384   # SGI_NOALLOC_CULL_MAX_VPLS


def _p(t):
    return C.c_void_p(None if t is None else t.data_ptr())


def scene(num_vpls=300, seed=41):
    w = S.Workload("room12_96x64_vpl%d" % num_vpls, 96, 64, 12, num_vpls, 0, 512, 16, abi.SGI_CUBE_F32, 4, 3, 1)
    ds = stage.DeviceScene(S.workload_scene(w, seed), w)
    ds.vpls[::3, 1] = -1.0   # every third VPL below the floor: shadowed by the CSM
    return w, ds


def context_cull(w, ds, max_visible):
    st = stage.GiStage(stage.workload_config(w, max_visible=max_visible))
    st.set_lights(ds.vpls, ds.entries, ds.points)
    st.set_shadow_maps(ds.csms[1], ds.cubes)
    st.cull_vpls()
    torch.cuda.synchronize()
    idx = st.read_debug(abi.SGI_DEBUG_VISIBLE_INDEX, np.int32)
    cv = st.read_debug(abi.SGI_DEBUG_COMPACT_VPLS, np.float32).reshape(-1, 16)
    ce = st.read_debug(abi.SGI_DEBUG_COMPACT_ENTRIES, np.int32).reshape(-1, 2)
    st.close()
    return idx, cv, ce


def noalloc_cull(lib, ds, n, max_visible):
    cv = torch.full((max_visible, 16), -7.0, dtype=torch.float32, device="cuda")
    ce = torch.full((max_visible, 2), -7, dtype=torch.int32, device="cuda")
    idx = torch.full((1 + max_visible,), -7, dtype=torch.int32, device="cuda")
    st = lib.sgi_cull_vpls_noalloc(_p(ds.vpls), _p(ds.entries), n, C.byref(ds.csms[1]), max_visible, _p(cv), _p(ce),
                                   _p(idx), None)
    torch.cuda.synchronize()
    return st, idx.cpu().numpy(), cv.cpu().numpy(), ce.cpu().numpy()


@pytest.mark.parametrize("max_visible", [300, 61])
def test_noalloc_cull_matches_context_cull_twice(max_visible):
    lib = abi.load()
    w, ds = scene()
    n = ds.vpls.shape[0]
    ref_idx, ref_cv, ref_ce = context_cull(w, ds, max_visible)
    cnt = int(ref_idx[0])
    assert 0 < cnt <= max_visible
    # the oracle's cull on the same VPLs and CSM
    host_depth = ds.csm_depth[1].cpu().numpy()
    host_csm = stage.csm_struct(ds.scene, 1, host_depth.ctypes.data, w.csm_resolution)
    host_vpls = ds.vpls.cpu().numpy()
    oracle_idx = O.vis_cull(32, host_vpls, host_csm, max_visible)
    assert int(oracle_idx[0]) == cnt
    assert np.array_equal(oracle_idx[1:1 + cnt], ref_idx[1:1 + cnt])
    assert np.array_equal(ref_cv[:cnt].view(np.uint32), host_vpls[oracle_idx[1:1 + cnt]].view(np.uint32))
    for _ in range(2):
        st, idx, cv, ce = noalloc_cull(lib, ds, n, max_visible)
        assert st == abi.SGI_OK
        assert idx[0] == cnt
        assert np.array_equal(idx[1:1 + cnt], ref_idx[1:1 + cnt])
        assert np.array_equal(cv[:cnt].view(np.uint32), ref_cv[:cnt].view(np.uint32))
        assert np.array_equal(ce[:cnt], ref_ce[:cnt])
        assert np.all(idx[1 + cnt:] == -7)       # nothing written past the count


def test_noalloc_cull_limits_and_arguments():
    lib = abi.load()
    w, ds = scene(num_vpls=40)
    # more VPLs than the fixed flag array holds: rejected, nothing launched
    big = torch.zeros((MAX_VPLS + 1, 16), dtype=torch.float32, device="cuda")
    big_e = torch.zeros((MAX_VPLS + 1, 2), dtype=torch.int32, device="cuda")
    out = torch.full((64, 16), -7.0, device="cuda")
    out_e = torch.full((64, 2), -7, dtype=torch.int32, device="cuda")
    idx = torch.full((65,), -7, dtype=torch.int32, device="cuda")
    st = lib.sgi_cull_vpls_noalloc(_p(big), _p(big_e), MAX_VPLS + 1, C.byref(ds.csms[1]), 64, _p(out), _p(out_e),
                                   _p(idx), None)
    assert st == abi.SGI_ERR_CAP
    torch.cuda.synchronize()
    assert int(idx[0].item()) == -7
    # bad arguments
    assert lib.sgi_cull_vpls_noalloc(_p(ds.vpls), _p(ds.entries), 40, None, 64, _p(out), _p(out_e), _p(idx),
                                     None) == abi.SGI_ERR_ARG
    assert lib.sgi_cull_vpls_noalloc(_p(ds.vpls), _p(ds.entries), 40, C.byref(ds.csms[1]), 0, _p(out), _p(out_e),
                                     _p(idx), None) == abi.SGI_ERR_ARG
    assert lib.sgi_cull_vpls_noalloc(C.c_void_p(ds.vpls.data_ptr() + 4), _p(ds.entries), 39, C.byref(ds.csms[1]), 64,
                                     _p(out), _p(out_e), _p(idx), None) == abi.SGI_ERR_ARG
    # no VPLs: the count is written as zero
    st = lib.sgi_cull_vpls_noalloc(None, None, 0, C.byref(ds.csms[1]), 64, _p(out), _p(out_e), _p(idx), None)
    assert st == abi.SGI_OK
    torch.cuda.synchronize()
    assert int(idx[0].item()) == 0


def test_noalloc_cull_at_the_flag_array_limit():
    """16384 VPLs (the whole flag array): 40 distinct VPLs repeated, so VPL i is
    visible exactly when VPL i % 40 is."""
    lib = abi.load()
    w, ds = scene(num_vpls=40)
    _, small_idx, _, _ = noalloc_cull(lib, ds, 40, 40)
    vis40 = np.zeros(40, bool)
    vis40[small_idx[1:1 + small_idx[0]]] = True
    reps = (MAX_VPLS + 39) // 40
    ds.vpls = ds.vpls.repeat(reps, 1)[:MAX_VPLS].contiguous()
    ds.entries = ds.entries.repeat(reps, 1)[:MAX_VPLS].contiguous()
    st, idx, cv, _ = noalloc_cull(lib, ds, MAX_VPLS, MAX_VPLS)
    assert st == abi.SGI_OK
    expect = np.nonzero(vis40[np.arange(MAX_VPLS) % 40])[0]
    assert idx[0] == len(expect)
    assert np.array_equal(idx[1:1 + len(expect)], expect)
    assert np.array_equal(cv[:len(expect)].view(np.uint32), ds.vpls.cpu().numpy()[expect].view(np.uint32))


MEMORY_PROBE = r"""
import ctypes as C, sys
import torch
sys.path.insert(0, sys.argv[1])
from stratusgfx_gb300 import abi, stage
from stratusgfx_gb300 import scene as S
lib = abi.load()
w = S.Workload("room12_96x64_vpl300", 96, 64, 12, 300, 0, 512, 16, abi.SGI_CUBE_F32, 4, 3, 1)
ds = stage.DeviceScene(S.workload_scene(w, 41), w)
# warm the library: a context cull loads the cull kernels' module and runs them once
st = stage.GiStage(stage.workload_config(w))
st.set_lights(ds.vpls, ds.entries, ds.points)
st.set_shadow_maps(ds.csms[1], ds.cubes)
st.cull_vpls()
torch.cuda.synchronize()
st.close()
cv = torch.empty((300, 16), dtype=torch.float32, device="cuda")
ce = torch.empty((300, 2), dtype=torch.int32, device="cuda")
idx = torch.empty((301,), dtype=torch.int32, device="cuda")
p = lambda t: C.c_void_p(t.data_ptr())
torch.cuda.synchronize()
free0 = torch.cuda.mem_get_info()[0]
for _ in range(2):   # the first call of this process on the device, then a second one
    assert lib.sgi_cull_vpls_noalloc(p(ds.vpls), p(ds.entries), 300, C.byref(ds.csms[1]), 300, p(cv), p(ce),
                                     p(idx), None) == abi.SGI_OK
torch.cuda.synchronize()
free1 = torch.cuda.mem_get_info()[0]
assert int(idx[0].item()) > 0
print("free", free0, free1)
sys.exit(0 if free0 == free1 else 3)
"""


def test_noalloc_cull_leaves_device_memory_unchanged():
    """In a fresh process, after the library's cull kernels have run once through a context: the first
    and a second sgi_cull_vpls_noalloc call leave cudaMemGetInfo's free memory exactly as it was."""
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    res = subprocess.run([sys.executable, "-c", MEMORY_PROBE, root], stdout=subprocess.PIPE,
                         stderr=subprocess.STDOUT, text=True, timeout=600)
    assert res.returncode == 0, res.stdout[-2000:]
