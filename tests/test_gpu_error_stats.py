"""sgi_gi_error_stats: the FP64 error statistics behind the reported PSNRs, on the
device, against the same statistics in numpy float64 (and twice: the reduction
order is fixed, so the results are identical)."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from stratusgfx_gb300 import stage  # noqa: E402


def test_error_stats_match_numpy_float64():
    H, W = 257, 391   # not a multiple of any block shape
    rng = np.random.default_rng(5)
    g = stage.GBufferTensors(H, W, "cuda")
    alb = rng.integers(0, 256, (H, W, 4), dtype=np.uint8)
    g.albedo.copy_(torch.from_numpy(alb))
    hdr = rng.uniform(0, 4, (H, W, 4)).astype(np.float16)
    direct = rng.uniform(0, 2, (H, W, 4)).astype(np.float16)
    target = rng.uniform(0, 3, (H, W, 4)).astype(np.float32)
    h_t, d_t, t_t = (torch.from_numpy(a).cuda() for a in (hdr, direct, target))
    got = stage.gi_error_stats(g, h_t, d_t, t_t)
    again = stage.gi_error_stats(g, h_t, d_t, t_t)
    assert got == again

    w = (np.maximum(alb[..., :3].astype(np.float64) / 255.0, 0.01) + 1e-5).astype(np.float16).astype(np.float64)
    r_gi = w * target[..., :3].astype(np.float64)
    d = direct[..., :3].astype(np.float64)
    r = d + r_gi
    o = hdr[..., :3].astype(np.float64)
    ef, eg = o - r, (o - d) - r_gi
    assert got["values"] == 3 * H * W
    assert got["sse_frame"] == pytest.approx(float((ef ** 2).sum()), rel=1e-12)
    assert got["sse_gi"] == pytest.approx(float((eg ** 2).sum()), rel=1e-12)
    assert got["peak_frame"] == float(np.abs(r).max())
    assert got["peak_gi"] == float(np.abs(r_gi).max())
    assert got["max_abs_frame"] == float(np.abs(ef).max())
    assert got["max_abs_gi"] == float(np.abs(eg).max())
    psnr = 10 * np.log10(np.abs(r).max() ** 2 / (ef ** 2).mean())
    assert got["psnr_frame"] == pytest.approx(psnr, abs=1e-9)
