"""Host-side VPL preparation of the C ABI (sgi_prepare_vpls) against the
restatement of the reference's UpdatePointLights_ / InitVplFrameData_: frustum
test, distance order with ties in input order, the cap, and the packed
records, on seeded scenes (bit-exact)."""
import ctypes as C
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

from oracle.host_prep import prepare_vpls  # noqa: E402
from stratusgfx_gb300 import abi  # noqa: E402


def frustum_planes(fov_deg, aspect, near, far, eye, yaw):
    """Inward view-frustum planes (a, b, c, d) of a camera at `eye` looking along yaw."""
    f = np.array([np.cos(yaw), 0.0, np.sin(yaw)])
    r = np.array([-np.sin(yaw), 0.0, np.cos(yaw)])
    u = np.cross(r, f)
    t = np.tan(np.radians(fov_deg) / 2)
    planes = []
    for n in (f, -f):
        planes.append(n)
    for s in (1, -1):
        planes.append(f * t * aspect + s * r)     # left / right: normal points inside
        planes.append(f * t + s * u)              # bottom / top
    out = []
    for k, n in enumerate([f, -f] + planes[2:]):
        n = n / np.linalg.norm(n)
        if k == 0:
            d = -np.dot(n, eye + near * f)
        elif k == 1:
            d = -np.dot(n, eye + far * f)
        else:
            d = -np.dot(n, eye)
        out.append([n[0], n[1], n[2], d])
    return np.array(out, np.float32)


def run(pos, radii, far, inten, planes, cam, cap):
    lib = abi.load()
    n = len(radii)
    out = np.zeros((max(cap, 1), 16), np.float32)
    src = np.zeros(max(cap, 1), np.int32)
    cnt = C.c_int32()
    p = lambda a: a.ctypes.data_as(C.c_void_p)   # noqa: E731
    assert lib.sgi_prepare_vpls(p(pos), p(radii), p(far), p(inten), n, p(planes), p(cam), cap, p(out), p(src),
                                C.byref(cnt)) == abi.SGI_OK
    return out[:cnt.value], src[:cnt.value]


@pytest.mark.parametrize("seed,n,cap", [(1, 500, 10000), (2, 3000, 700), (3, 64, 10)])
def test_matches_the_reference_preparation(seed, n, cap):
    rng = np.random.default_rng(seed)
    pos = rng.uniform(-20, 20, (n, 3)).astype(np.float32)
    if n > 100:   # duplicated positions: equal distances must keep the input order
        pos[50:60] = pos[40:50]
    radii = rng.uniform(0.5, 8, n).astype(np.float32)
    far = (radii * 1.5).astype(np.float32)
    inten = rng.uniform(1, 50, n).astype(np.float32)
    cam = np.array([1.0, 2.0, -3.0], np.float32)
    planes = frustum_planes(70.0, 16 / 9, 0.1, 25.0, cam.astype(np.float64), 0.3 * seed)
    got, src = run(pos, radii, far, inten, planes, cam, cap)
    want, wsrc = prepare_vpls(pos, radii, far, inten, planes, cam, cap)
    assert 0 < len(got) <= cap
    assert np.array_equal(src, wsrc)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


def test_empty_and_bad_arguments():
    lib = abi.load()
    cnt = C.c_int32(5)
    planes = np.zeros((6, 4), np.float32)
    cam = np.zeros(3, np.float32)
    p = lambda a: a.ctypes.data_as(C.c_void_p)   # noqa: E731
    assert lib.sgi_prepare_vpls(None, None, None, None, 0, p(planes), p(cam), 0, None, None, C.byref(cnt)) == abi.SGI_OK
    assert cnt.value == 0
    assert lib.sgi_prepare_vpls(None, None, None, None, 3, p(planes), p(cam), 4, None, None, C.byref(cnt)) == \
        abi.SGI_ERR_ARG


def test_plane_products_are_added_in_pairs():
    """A sphere on a plane boundary where the two addition orders disagree: the
    products are -2, 0, -2^-23 and -2^-23. Added left to right they give -2 (the
    last two additions round back to -2), added in pairs as glm's vec4 dot does,
    (-2 + 0) + (-2^-23 - 2^-23) = -2 - 2^-22, which is below -radius = -2: the
    reference culls this VPL."""
    tiny = np.float32(2.0 ** -23)
    planes = np.zeros((6, 4), np.float32)
    planes[:, 3] = 1.0e6                       # five planes far away on the inner side
    planes[0] = [1.0, 0.0, 1.0, -tiny]
    pos = np.array([[-2.0, 0.0, -tiny], [-1.0, 0.0, 0.0]], np.float32)
    radii = np.array([2.0, 2.0], np.float32)
    far = np.ones(2, np.float32)
    inten = np.ones(2, np.float32)
    cam = np.zeros(3, np.float32)
    seq = np.float32(np.float32(np.float32(-2.0) + np.float32(0.0)) + -tiny) + -tiny
    assert seq == np.float32(-2.0)             # the left-to-right sum would keep it
    got, src = run(pos, radii, far, inten, planes, cam, 8)
    want, wsrc = prepare_vpls(pos, radii, far, inten, planes, cam, 8)
    assert list(src) == [1] and list(wsrc) == [1]
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


@pytest.mark.parametrize("what", ["position", "radius", "camera", "plane"])
def test_non_finite_input_is_rejected(what):
    lib = abi.load()
    pos = np.zeros((3, 3), np.float32)
    radii = np.ones(3, np.float32)
    far = np.ones(3, np.float32)
    inten = np.ones(3, np.float32)
    planes = np.zeros((6, 4), np.float32)
    planes[:, 3] = 1.0
    cam = np.zeros(3, np.float32)
    {"position": pos, "radius": radii, "camera": cam, "plane": planes}[what].flat[1] = np.nan
    out = np.zeros((3, 16), np.float32)
    cnt = C.c_int32(0)
    p = lambda a: a.ctypes.data_as(C.c_void_p)   # noqa: E731
    assert lib.sgi_prepare_vpls(p(pos), p(radii), p(far), p(inten), 3, p(planes), p(cam), 3, p(out), None,
                                C.byref(cnt)) == abi.SGI_ERR_ARG
    assert cnt.value == 0
