"""3x3 convolution layers of the learned denoiser on the tcgen05 tensor cores.

Every layer shape of the U-Net (and the transposed shapes its input gradients
use) runs through ``sgi_nn_conv3x3`` on both engines (tcgen05.mma with TMEM
accumulators, and warp-level mma.sync) and is compared with a plain PyTorch fp32
convolution of the same BF16 inputs. Inputs and outputs are strided channel
views inside wider buffers (as in the network's concatenation buffers), and the
widths are not multiples of the 128-pixel tile.

Tolerance: both engines accumulate in FP32 and round the result to BF16
(relative 2^-8), in different summation orders, so
|got - ref| <= 1e-2 |ref| + 2e-3 max|ref| per element.
"""
import ctypes as C

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from stratusgfx_gb300 import abi  # noqa: E402

# (cin, cout, mode): mode 0 = bias + ReLU, 1 = bias only (head), 2 = neither (input gradients)
SHAPES = [(16, 32, 0), (32, 32, 0), (32, 64, 0), (64, 64, 0), (64, 128, 0), (128, 128, 0), (192, 64, 0), (96, 32, 0),
          (32, 32, 1), (32, 32, 2), (64, 32, 2), (64, 64, 2), (128, 64, 2), (128, 128, 2), (64, 192, 2), (32, 96, 2)]


def reference(x, w, bias, mode):
    """fp32 conv of BF16 tensors: x [B,H,W,cin], w [cout,9,cin]."""
    cout, _, cin = w.shape
    xf = x.float().permute(0, 3, 1, 2)
    wf = w.float().reshape(cout, 3, 3, cin).permute(0, 3, 1, 2)
    y = torch.nn.functional.conv2d(xf, wf, padding=1)
    if mode != 2:
        y = y + bias.view(1, -1, 1, 1)
    if mode == 0:
        y = torch.relu(y)
    return y.permute(0, 2, 3, 1)


def run(lib, path, cin, cout, mode, xbuf, x_off, w, bias, B, H, W, err):
    """Runs one layer reading channels [x_off, x_off + cin) of xbuf and writing
    channels [8, 8 + cout) of a zeroed buffer with 8 spare channels either side."""
    ys = cout + 16
    ybuf = torch.zeros((B, H, W, ys), dtype=torch.bfloat16, device="cuda")
    st = lib.sgi_nn_conv3x3(path, cin, cout, mode, C.c_void_p(xbuf.data_ptr() + 2 * x_off), xbuf.shape[3],
                            C.c_void_p(w.data_ptr()), C.c_void_p(bias.data_ptr()), C.c_void_p(ybuf.data_ptr() + 16),
                            ys, B, H, W, C.c_void_p(err.data_ptr()), None)
    assert st == abi.SGI_OK, st
    torch.cuda.synchronize()
    assert not ybuf[..., :8].any() and not ybuf[..., 8 + cout:].any(), "wrote outside its channels"
    return ybuf[..., 8:8 + cout].float()


@pytest.mark.parametrize("cin,cout,mode", SHAPES)
@pytest.mark.parametrize("B,H,W", [(2, 5, 200), (1, 1, 3)])
def test_conv_layer_matches_fp32(cin, cout, mode, B, H, W):
    lib = abi.load()
    g = torch.Generator(device="cpu").manual_seed(cin * 1000 + cout * 10 + mode)
    xbuf = torch.randn((B, H, W, cin + 16), generator=g).to("cuda", torch.bfloat16)
    w = (torch.randn((cout, 9, cin), generator=g) * (2.0 / (9 * cin)) ** 0.5).to("cuda", torch.bfloat16)
    bias = (torch.randn(cout, generator=g) * 0.1).cuda()
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    ref = reference(xbuf[..., 8:8 + cin], w, bias, mode)
    tol = 1e-2 * ref.abs() + 2e-3 * ref.abs().max() + 1e-6
    outs = {}
    for path in (abi.SGI_NN_CONV_TCGEN05, abi.SGI_NN_CONV_WARP_MMA):
        got = run(lib, path, cin, cout, mode, xbuf, 8, w, bias, B, H, W, err)
        bad = (got - ref).abs() > tol
        assert not bad.any(), (path, int(bad.sum()), float((got - ref).abs().max()))
        outs[path] = got
    assert int(err.item()) == 0
    d = (outs[abi.SGI_NN_CONV_TCGEN05] - outs[abi.SGI_NN_CONV_WARP_MMA]).abs()
    assert float(d.max()) <= float(2e-2 * ref.abs().max()) + 1e-6


def test_conv_layer_larger_frame():
    """A 384 x 64 frame: 3 tiles per row, every row boundary and image edge."""
    lib = abi.load()
    B, H, W, cin, cout = 1, 64, 384, 96, 32
    g = torch.Generator(device="cpu").manual_seed(11)
    xbuf = torch.randn((B, H, W, cin + 16), generator=g).to("cuda", torch.bfloat16)
    w = (torch.randn((cout, 9, cin), generator=g) * 0.05).to("cuda", torch.bfloat16)
    bias = (torch.randn(cout, generator=g) * 0.1).cuda()
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    ref = reference(xbuf[..., 8:8 + cin], w, bias, 0)
    got = run(lib, abi.SGI_NN_CONV_TCGEN05, cin, cout, 0, xbuf, 8, w, bias, B, H, W, err)
    assert int(err.item()) == 0
    assert not ((got - ref).abs() > 1e-2 * ref.abs() + 2e-3 * ref.abs().max()).any()


def test_conv_rejects_bad_layout():
    lib = abi.load()
    x = torch.zeros((1, 4, 4, 40), dtype=torch.bfloat16, device="cuda")
    w = torch.zeros((32, 9, 32), dtype=torch.bfloat16, device="cuda")
    b = torch.zeros(32, device="cuda")
    y = torch.zeros((1, 4, 4, 32), dtype=torch.bfloat16, device="cuda")
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    args = lambda xp, xs, path, e: (path, 32, 32, 0, C.c_void_p(xp), xs, C.c_void_p(w.data_ptr()),  # noqa: E731
                                    C.c_void_p(b.data_ptr()), C.c_void_p(y.data_ptr()), 32, 1, 4, 4, e, None)
    ok = C.c_void_p(err.data_ptr())
    assert lib.sgi_nn_conv3x3(*args(x.data_ptr() + 2, 40, abi.SGI_NN_CONV_TCGEN05, ok)) == abi.SGI_ERR_ARG
    assert lib.sgi_nn_conv3x3(*args(x.data_ptr(), 36, abi.SGI_NN_CONV_TCGEN05, ok)) == abi.SGI_ERR_ARG
    assert lib.sgi_nn_conv3x3(*args(x.data_ptr(), 40, abi.SGI_NN_CONV_TCGEN05, None)) == abi.SGI_ERR_ARG
    assert lib.sgi_nn_conv3x3(*args(x.data_ptr(), 40, 7, ok)) == abi.SGI_ERR_ARG
    assert lib.sgi_nn_conv3x3(*(args(x.data_ptr(), 40, abi.SGI_NN_CONV_TCGEN05, ok)[:1] + (48,) +
                               args(x.data_ptr(), 40, abi.SGI_NN_CONV_TCGEN05, ok)[2:])) == abi.SGI_ERR_ARG
    torch.cuda.synchronize()
    assert int(err.item()) == 0
    np.testing.assert_array_equal(y.float().cpu().numpy(), 0.0)
