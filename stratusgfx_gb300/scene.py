"""Seeded synthetic scenes for the GI/lighting stage.

StratusGFX renders real meshes (its demo assets are external downloads); the
stage's inputs are only G-buffer textures, light records and shadow maps. The
workloads here are seeded rooms of axis-aligned boxes:

* a 10 x 10 x 10 m room, open at the top so the sun reaches inside, with N
  boxes of size U[0.3, 2.5] m placed on the floor or stacked; materials have
  albedo U[0.05, 0.95]^3, roughness U[0.05, 1], metallic Bernoulli(0.2);
* a directional light with elevation U[30, 75] degrees, and the four
  cascades of its shadow map fitted to the camera frustum exactly as
  RendererFrontend::UpdateCascadeData_ does (StratusRendererFrontend.cpp:558-807);
* VPLs at the first hits of stratified sun rays through the room opening,
  1 cm off the surface, coloured by the surface albedo (vpl_light_color.cs:41-75
  colours a VPL with the diffuse cube sampled towards the sun);
* a camera path of seeded small moves (GL conventions of glm::perspective
  and glm::lookAt).

Everything here is float64 host math, converted to float32 once.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

ROOM = 10.0
WALL = 0.5


def perspective(fovy_rad: float, aspect: float, znear: float, zfar: float) -> np.ndarray:
    """glm::perspective (right-handed, NDC z in [-1, 1]); row-major math form."""
    f = 1.0 / math.tan(fovy_rad / 2.0)
    m = np.zeros((4, 4))
    m[0, 0] = f / aspect
    m[1, 1] = f
    m[2, 2] = (zfar + znear) / (znear - zfar)
    m[2, 3] = 2.0 * zfar * znear / (znear - zfar)
    m[3, 2] = -1.0
    return m


def look_at(eye, center, up) -> np.ndarray:
    """glm::lookAt (right-handed)."""
    eye, center, up = (np.asarray(v, dtype=np.float64) for v in (eye, center, up))
    f = center - eye
    f /= np.linalg.norm(f)
    s = np.cross(f, up)
    s /= np.linalg.norm(s)
    u = np.cross(s, f)
    m = np.eye(4)
    m[0, :3], m[1, :3], m[2, :3] = s, u, -f
    m[0, 3], m[1, 3], m[2, 3] = -s @ eye, -u @ eye, f @ eye
    return m


def colmajor(m: np.ndarray) -> np.ndarray:
    """Row-major math matrix -> 16 float32 in glm (column-major) order."""
    return np.ascontiguousarray(np.asarray(m, dtype=np.float64).T.reshape(16).astype(np.float32))


@dataclass
class CameraFrame:
    proj_view: np.ndarray         # (16,) float32 column-major
    inv_proj_view: np.ndarray
    prev_proj_view: np.ndarray
    position: np.ndarray          # (4,) float32
    world: np.ndarray             # 4x4 float64 camera world transform


@dataclass
class CsmFrame:
    cascade_proj_view: np.ndarray     # (4, 16) float32
    inv_cascade_proj_view: np.ndarray  # (4, 16) float32
    cascade_planes: np.ndarray        # (3, 4) float32
    znear: float
    zfar: float


@dataclass
class Scene:
    seed: int
    width: int
    height: int
    boxes: np.ndarray                 # (nb, 16) float32, sgi_box records
    light_direction: np.ndarray       # (4,) float32 towards the light
    light_color: np.ndarray           # (4,) float32 luminance
    vpls: np.ndarray                  # (N, 16) float32, sgi_vpl records
    entries: np.ndarray               # (N, 2) int32, sgi_atlas_entry records
    points: np.ndarray                # (M, 12) float32, sgi_point_light records
    cameras: list = field(default_factory=list)   # CameraFrame per rendered frame (+1 history seed at [0])
    csms: list = field(default_factory=list)      # CsmFrame per camera
    fovy_deg: float = 60.0
    znear: float = 0.1
    zfar: float = 30.0
    layers_per_atlas: int = 320


def _box_record(lo, hi, albedo, roughness, metallic, reflectance, ident) -> np.ndarray:
    r = np.zeros(16, dtype=np.float32)
    r[0:3], r[4:7] = lo, hi
    r[8:11] = albedo
    r[11] = 0.0
    r[12], r[13], r[14], r[15] = roughness, metallic, reflectance, ident
    return r


def make_boxes(rng: np.random.Generator, num_boxes: int) -> np.ndarray:
    recs = []
    ident = 1

    def material():
        return (rng.uniform(0.05, 0.95, 3), rng.uniform(0.05, 1.0), float(rng.random() < 0.2))

    # floor and four walls (slabs outside the [0, ROOM]^3 interior); no ceiling
    slabs = [
        ((-WALL, -WALL, -WALL), (ROOM + WALL, 0.0, ROOM + WALL)),
        ((-WALL, -WALL, -WALL), (0.0, ROOM, ROOM + WALL)),
        ((ROOM, -WALL, -WALL), (ROOM + WALL, ROOM, ROOM + WALL)),
        ((-WALL, -WALL, -WALL), (ROOM + WALL, ROOM, 0.0)),
        ((-WALL, -WALL, ROOM), (ROOM + WALL, ROOM, ROOM + WALL)),
    ]
    for lo, hi in slabs:
        a, r, m = material()
        recs.append(_box_record(lo, hi, a, r, 0.0, 0.5, ident))
        ident += 1
    placed = []
    for _ in range(num_boxes):
        size = rng.uniform(0.3, 2.5, 3)
        a, r, m = material()
        if placed and rng.random() < 0.3:
            base = placed[rng.integers(len(placed))]
            cx = rng.uniform(base[0][0], base[1][0])
            cz = rng.uniform(base[0][2], base[1][2])
            lo = np.array([cx - size[0] / 2, base[1][1], cz - size[2] / 2])
        else:
            lo = np.array([rng.uniform(0.0, ROOM - size[0]), 0.0, rng.uniform(0.0, ROOM - size[2])])
        lo[0] = min(max(lo[0], 0.0), ROOM - size[0])
        lo[2] = min(max(lo[2], 0.0), ROOM - size[2])
        hi = lo + size
        placed.append((lo, hi))
        recs.append(_box_record(lo, hi, a, r, m, 0.5, ident))
        ident += 1
    return np.stack(recs)


def ray_boxes(boxes: np.ndarray, o: np.ndarray, d: np.ndarray):
    """First hit (t > 0) of rays o + t d against all boxes, float64. Returns t, box index, normal."""
    o = np.asarray(o, dtype=np.float64)
    d = np.asarray(d, dtype=np.float64)
    lo = boxes[:, 0:3].astype(np.float64)[None]
    hi = boxes[:, 4:7].astype(np.float64)[None]
    with np.errstate(divide="ignore", invalid="ignore"):
        inv = 1.0 / d[:, None, :]
        t1 = (lo - o[:, None, :]) * inv
        t2 = (hi - o[:, None, :]) * inv
    tmin = np.where(np.isnan(t1), -np.inf, np.minimum(t1, t2))
    tmax = np.where(np.isnan(t1), np.inf, np.maximum(t1, t2))
    tnear = tmin.max(axis=2)
    tfar = tmax.min(axis=2)
    axis = tmin.argmax(axis=2)
    hit = (tnear <= tfar) & (tnear > 1e-9)
    tn = np.where(hit, tnear, np.inf)
    bi = tn.argmin(axis=1)
    t = tn[np.arange(len(o)), bi]
    ax = axis[np.arange(len(o)), bi]
    n = np.zeros((len(o), 3))
    n[np.arange(len(o)), ax] = -np.sign(d[np.arange(len(o)), ax])
    return t, bi, n


def inside_any(boxes: np.ndarray, p: np.ndarray, margin: float = 0.3) -> bool:
    lo = boxes[:, 0:3] - margin
    hi = boxes[:, 4:7] + margin
    return bool(np.any(np.all((p >= lo) & (p <= hi), axis=1)))


def light_basis(L: np.ndarray):
    """World and view transforms of the light camera (GetDirection() == L)."""
    view = look_at(np.zeros(3), L, (0.0, 1.0, 0.0))
    return view.T.copy(), view   # world (rotation) = view^T


def fit_cascades(cam_world: np.ndarray, light_dir: np.ndarray, fovy_deg: float, aspect: float, zfar: float,
                 resolution: int, num_cascades: int = 4) -> CsmFrame:
    """RendererFrontend::UpdateCascadeData_, StratusRendererFrontend.cpp:558-807."""
    light_world, light_view = light_basis(light_dir)
    transpose_light_world = light_world.T
    Lm = light_view @ cam_world
    proj_plane_dist = math.tan(math.radians(fovy_deg) / 2.0)
    znear = 1.0
    lam = 0.5
    clip_range = zfar - znear
    ratio = zfar / znear
    ends = []
    for i in range(num_cascades):
        p = (i + 1) / float(num_cascades)
        log = znear * ratio ** p
        uni = znear + clip_range * p
        ends.append(math.floor(lam * log + (1.0 - lam) * uni))
    begins = [0.0] + [e - 4.0 for e in ends[:-1]]
    pvs, invs, planes = [], [], []
    for i in range(num_cascades):
        ak, bk = begins[i], ends[i]
        xn, xf = ak * aspect * proj_plane_dist, bk * aspect * proj_plane_dist
        yn, yf = ak * proj_plane_dist, bk * proj_plane_dist
        corners = np.array([[xn, yn, -ak, 1], [-xn, yn, -ak, 1], [xn, -yn, -ak, 1], [-xn, -yn, -ak, 1],
                            [xf, yf, -bk, 1], [-xf, yf, -bk, 1], [xf, -yf, -bk, 1], [-xf, -yf, -bk, 1]], dtype=np.float64)
        max_len = 0.0
        for a in range(len(corners) - 1):
            for b in range(1, len(corners)):
                max_len = max(max_len, float(np.linalg.norm(corners[a] - corners[b])))
        dk = math.ceil(max_len)
        T = dk / resolution
        ls = (Lm @ corners.T).T[:, :3]
        mn, mx = ls.min(axis=0), ls.max(axis=0)
        sk = np.array([math.floor((mx[0] + mn[0]) / (2.0 * T)) * T, math.floor((mx[1] + mn[1]) / (2.0 * T)) * T, mn[2]])
        cview = np.eye(4)
        cview[:3, :3] = transpose_light_world[:3, :3]
        cview[:3, 3] = -sk
        ortho = np.diag([2.0 / dk, 2.0 / dk, 1.0 / (mx[2] - mn[2]), 1.0])
        pv = ortho @ cview
        pvs.append(pv)
        invs.append(np.linalg.inv(pv))
        if i > 0:
            n = -cam_world[:3, 2]
            c = cam_world[:3, 3]
            fk = np.array([n[0], n[1], n[2], float(-n @ c) - ak]) * (1.0 / (ends[i - 1] - ak))
            planes.append(fk)
    return CsmFrame(cascade_proj_view=np.stack([colmajor(m) for m in pvs]),
                    inv_cascade_proj_view=np.stack([colmajor(m) for m in invs]),
                    cascade_planes=np.stack(planes).astype(np.float32), znear=znear, zfar=zfar)


def make_scene(seed: int, width: int, height: int, num_boxes: int, num_vpls: int, num_frames: int,
               vpl_radius: float = 8.0, num_points: int = 0, csm_resolution: int = 1024,
               vpl_color_scale: float = 50.0, fovy_deg: float = 60.0, camera_seed: int | None = None) -> Scene:
    """Seeded room + lights + camera path. cameras[0] seeds the history; frames 1..num_frames are rendered.
    The room and its lights depend on `seed` only; with camera_seed the camera path comes from its own
    generator (another view of the same room)."""
    rng = np.random.default_rng(seed)
    boxes = make_boxes(rng, num_boxes)
    el = math.radians(rng.uniform(30.0, 75.0))
    az = rng.uniform(0.0, 2.0 * math.pi)
    L = np.array([math.cos(el) * math.cos(az), math.sin(el), math.cos(el) * math.sin(az)])
    sun = np.array([1.0, 0.95, 0.9]) * 4.0   # InfiniteLight intensity_ = 4 (StratusLight.h:37)

    # VPLs: stratified sun rays through the opening at y = ROOM
    g = max(1, int(math.ceil(math.sqrt(num_vpls))))
    ij = np.array([(i, j) for j in range(g) for i in range(g)][:num_vpls], dtype=np.float64)
    jit = rng.random((num_vpls, 2))
    top = np.stack([(ij[:, 0] + jit[:, 0]) / g * ROOM, np.full(num_vpls, ROOM - 1e-3),
                    (ij[:, 1] + jit[:, 1]) / g * ROOM], axis=1)
    d = np.tile(-L, (num_vpls, 1))
    t, bi, n = ray_boxes(boxes, top, d)
    t = np.where(np.isfinite(t), t, 0.0)
    hitp = top + d * t[:, None]
    pos = hitp + 0.01 * n
    albedo = boxes[bi, 8:11].astype(np.float64)
    col = albedo * sun * vpl_color_scale
    cosl = np.clip((n * L).sum(axis=1), 1e-3, None)
    mag = np.minimum(0.01 / cosl, vpl_radius)
    spec = pos - 1.1 * mag[:, None] * L
    vpls = np.zeros((num_vpls, 16), dtype=np.float32)
    vpls[:, 0:3], vpls[:, 3] = pos, 1.0
    vpls[:, 4:7], vpls[:, 7] = col, 1.0
    vpls[:, 8:11], vpls[:, 11] = spec, 1.0
    vpls[:, 12], vpls[:, 13], vpls[:, 14] = vpl_radius, vpl_radius, 1.0
    layers = 320
    entries = np.stack([np.arange(num_vpls) // layers, np.arange(num_vpls) % layers], axis=1).astype(np.int32)

    points = np.zeros((num_points, 12), dtype=np.float32)
    for k in range(num_points):
        points[k, 0:3] = rng.uniform([1.0, 2.0, 1.0], [9.0, 6.0, 9.0])
        points[k, 3] = 1.0
        points[k, 4:7] = rng.uniform(0.5, 1.0, 3) * 50.0
        points[k, 7] = 1.0
        points[k, 8], points[k, 9] = 15.0, 15.0

    # camera path: eye near one wall, looking across the room and slightly down
    if camera_seed is not None:
        rng = np.random.default_rng(camera_seed)
    aspect = width / height
    proj = perspective(math.radians(fovy_deg), aspect, 0.1, 30.0)
    for _ in range(100):
        eye = np.array([rng.uniform(1.0, 3.0), rng.uniform(1.5, 2.5), rng.uniform(1.0, 9.0)])
        if not inside_any(boxes, eye):
            break
    target = np.array([ROOM - 1.0, rng.uniform(0.0, 1.0), rng.uniform(3.0, 7.0)])
    step = rng.normal(size=3) * np.array([0.04, 0.01, 0.04])
    tstep = rng.normal(size=3) * 0.03
    cams, csms = [], []
    prev_pv = None
    for k in range(num_frames + 1):
        e = eye + step * k
        view = look_at(e, target + tstep * k, (0.0, 1.0, 0.0))
        pv = proj @ view
        world = np.linalg.inv(view)
        cams.append(CameraFrame(proj_view=colmajor(pv), inv_proj_view=colmajor(np.linalg.inv(pv)),
                                prev_proj_view=colmajor(prev_pv if prev_pv is not None else pv),
                                position=np.array([e[0], e[1], e[2], 1.0], dtype=np.float32), world=world))
        csms.append(fit_cascades(world, L, fovy_deg, aspect, 30.0, csm_resolution))
        prev_pv = pv
    return Scene(seed=seed, width=width, height=height, boxes=boxes,
                 light_direction=np.array([L[0], L[1], L[2], 0.0], dtype=np.float32),
                 light_color=np.array([sun[0], sun[1], sun[2], 1.0], dtype=np.float32),
                 vpls=vpls, entries=entries, points=points, cameras=cams, csms=csms, fovy_deg=fovy_deg)


# Workloads (sizes of the configurations the stage is measured and checked on)
@dataclass(frozen=True)
class Workload:
    name: str
    width: int
    height: int
    num_boxes: int
    num_vpls: int
    num_points: int
    csm_resolution: int
    cube_size: int
    cube_format: int
    samples: int
    denoise_passes: int
    frames: int
    tile_size: int = 16
    max_per_tile: int = 64
    vpl_radius: float = 8.0


# plain method, 320x180, 12 boxes, 64 VPLs with 6x64^2 FP32 cubes, 4x1024^2 CSM,
# K = 8, 5 denoise passes, 2 frames
SMALL = Workload("room12_320x180_vpl64_k8", 320, 180, 12, 64, 0, 1024, 64, 0, 8, 5, 2)
# plain method, 1920x1080, 40 boxes, 4 point lights, 4x2048^2 CSM, 2048 VPLs with
# 6x128^2 FP16 cubes, <= 64 VPLs per 16x16 tile, K = 8, 8 frames
HD = Workload("room40_1920x1080_vpl2048_k8", 1920, 1080, 40, 2048, 4, 2048, 128, 1, 8, 5, 8)
# 3840x2160, the same room generator, 4096 VPLs with 6x128^2 FP16 cubes, K = 4, 4-frame path
# (the neural comparison at 4K: plain a-trous vs the BF16 and FP8 U-Net)
UHD = Workload("room40_3840x2160_vpl4096_k4", 3840, 2160, 40, 4096, 4, 2048, 128, 1, 4, 5, 4)


def workload_scene(w: Workload, seed: int) -> Scene:
    return make_scene(seed, w.width, w.height, w.num_boxes, w.num_vpls, w.frames, vpl_radius=w.vpl_radius,
                      num_points=w.num_points, csm_resolution=w.csm_resolution)


def scene_arrays(s: Scene) -> dict:
    """Flat arrays of a Scene (for fixtures: host math never needs to be recomputed)."""
    d = dict(seed=np.int64(s.seed), width=np.int64(s.width), height=np.int64(s.height), boxes=s.boxes,
             light_direction=s.light_direction, light_color=s.light_color, vpls=s.vpls, entries=s.entries,
             points=s.points, fovy_deg=np.float64(s.fovy_deg))
    d["cam_proj_view"] = np.stack([c.proj_view for c in s.cameras])
    d["cam_inv_proj_view"] = np.stack([c.inv_proj_view for c in s.cameras])
    d["cam_prev_proj_view"] = np.stack([c.prev_proj_view for c in s.cameras])
    d["cam_position"] = np.stack([c.position for c in s.cameras])
    d["csm_proj_view"] = np.stack([c.cascade_proj_view for c in s.csms])
    d["csm_inv_proj_view"] = np.stack([c.inv_cascade_proj_view for c in s.csms])
    d["csm_planes"] = np.stack([c.cascade_planes for c in s.csms])
    d["csm_znear_zfar"] = np.array([[c.znear, c.zfar] for c in s.csms])
    return d


def scene_from_arrays(d) -> Scene:
    cams = [CameraFrame(proj_view=d["cam_proj_view"][k], inv_proj_view=d["cam_inv_proj_view"][k],
                        prev_proj_view=d["cam_prev_proj_view"][k], position=d["cam_position"][k], world=np.eye(4))
            for k in range(d["cam_proj_view"].shape[0])]
    csms = [CsmFrame(cascade_proj_view=d["csm_proj_view"][k], inv_cascade_proj_view=d["csm_inv_proj_view"][k],
                     cascade_planes=d["csm_planes"][k], znear=float(d["csm_znear_zfar"][k][0]),
                     zfar=float(d["csm_znear_zfar"][k][1])) for k in range(d["csm_proj_view"].shape[0])]
    return Scene(seed=int(d["seed"]), width=int(d["width"]), height=int(d["height"]), boxes=d["boxes"],
                 light_direction=d["light_direction"], light_color=d["light_color"], vpls=d["vpls"],
                 entries=d["entries"], points=d["points"], cameras=cams, csms=csms, fovy_deg=float(d["fovy_deg"]))
