"""The cascade set-up of the directional light's CSM (scene.fit_cascades), the
restatement of RendererFrontend::UpdateCascadeData_ (StratusRendererFrontend.cpp:558-807):
split distances, containment of each frustum slice in its cascade, texel
snapping of the cascade centres, and the blend planes the shaders read."""
import math

import numpy as np
import pytest

from stratusgfx_gb300 import scene as S

FOVY, ASPECT, ZFAR, RES = 60.0, 16.0 / 9.0, 30.0, 2048


def camera_world(eye, target):
    return np.linalg.inv(S.look_at(np.asarray(eye, float), np.asarray(target, float), (0.0, 1.0, 0.0)))


def unpack(cm):
    """column-major (16,) -> 4x4"""
    return np.asarray(cm, np.float64).reshape(4, 4).T


def slice_corners(cam_world, a, b):
    t = math.tan(math.radians(FOVY) / 2.0)
    pts = []
    for d in (a, b):
        for sx in (1, -1):
            for sy in (1, -1):
                pts.append([sx * d * ASPECT * t, sy * d * t, -d, 1.0])
    return (cam_world @ np.array(pts).T).T


@pytest.fixture(scope="module")
def setup():
    L = np.array([0.3, 0.8, 0.2])
    L /= np.linalg.norm(L)
    cw = camera_world([2.0, 2.0, 3.0], [9.0, 0.5, 5.0])
    return L, cw, S.fit_cascades(cw, L, FOVY, ASPECT, ZFAR, RES)


def test_split_distances_are_the_reference_mix_of_log_and_uniform():
    # lambda 0.5 between znear * ratio^p and znear + range * p, floored (:614-625): znear 1, zfar 30
    ends = [math.floor(0.5 * 30.0 ** p + 0.5 * (1.0 + 29.0 * p)) for p in (0.25, 0.5, 0.75, 1.0)]
    assert ends == [5, 10, 17, 30]


def test_each_frustum_slice_lies_inside_its_cascade(setup):
    L, cw, f = setup
    ends = [5.0, 10.0, 17.0, 30.0]
    begins = [0.0] + [e - 4.0 for e in ends[:-1]]
    for i in range(4):
        pv = unpack(f.cascade_proj_view[i])
        c = (pv @ slice_corners(cw, begins[i], ends[i]).T).T
        ndc = c[:, :3] / c[:, 3:4]
        # the snapped centre moves the box by less than a texel on each side
        assert np.all(np.abs(ndc[:, :2]) <= 1.0 + 2.0 / RES + 1e-4), (i, ndc)
        assert ndc[:, 2].min() >= -1e-4 and ndc[:, 2].max() <= 1.0 + 1e-4
        # and the inverse matrices invert
        assert np.allclose(unpack(f.inv_cascade_proj_view[i]) @ pv, np.eye(4), atol=1e-4)


def test_cascade_centres_are_snapped_to_texels(setup):
    L, cw, f = setup
    for i in range(4):
        pv = unpack(f.cascade_proj_view[i])
        dk = 2.0 / pv[0, 0]                       # ortho scale 2 / dk
        T = dk / RES
        sk = -pv[:2, 3] * dk / 2.0                # translation column = ortho * (-sk)
        q = sk / T
        assert np.allclose(q, np.round(q), atol=1e-3), (i, q)


def test_moving_the_camera_along_the_light_keeps_the_snapped_grid():
    """A translation of the camera keeps every cascade centre on the texel grid of that cascade (so a
    static scene's shadow texels do not swim)."""
    L = np.array([0.3, 0.8, 0.2])
    L /= np.linalg.norm(L)
    for dx in (0.0, 0.013, 0.377):
        cw = camera_world([2.0 + dx, 2.0, 3.0], [9.0 + dx, 0.5, 5.0])
        f = S.fit_cascades(cw, L, FOVY, ASPECT, ZFAR, RES)
        for i in range(4):
            pv = unpack(f.cascade_proj_view[i])
            dk = 2.0 / pv[0, 0]
            q = (-pv[:2, 3] * dk / 2.0) / (dk / RES)
            assert np.allclose(q, np.round(q), atol=1e-3)


def test_blend_planes_measure_the_overlap_of_consecutive_cascades(setup):
    """cascadePlanes[i-1] . (p, 1) is 0 where cascade i begins and 1 where cascade i-1 ends, along the view
    direction (:760-790), so pbr.glsl's blend weights run 0 -> 1 across the 4-unit overlap."""
    L, cw, f = setup
    ends = [5.0, 10.0, 17.0, 30.0]
    fwd = -cw[:3, 2]
    eye = cw[:3, 3]
    for i in range(1, 4):
        plane = np.asarray(f.cascade_planes[i - 1], np.float64)
        ak = ends[i - 1] - 4.0
        for d, want in ((ak, 0.0), (ends[i - 1], 1.0)):
            p = eye + fwd * d
            assert abs(plane[:3] @ p + plane[3] - want) < 1e-4
