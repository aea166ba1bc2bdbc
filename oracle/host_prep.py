"""Oracle (test infrastructure): the host-side VPL preparation of StratusGFX,
restated in numpy binary32 so that the C ABI's sgi_prepare_vpls can be
checked against it.

- UpdatePointLights_, VPL branch (Source/Engine/StratusRendererBackend.cpp:1357-1389):
  distance = glm::distance(camera, light) taken as a double key; a VPL is kept
  when IsSphereInFrustum (Source/Engine/StratusMath.h:401-412) holds, i.e. no
  plane gives dot(plane, vec4(center, 1)) < -radius, where glm's vec4 dot adds
  the products in pairs, (x + y) + (z + w) (glm/detail/func_geometric.inl:64-70)
  and its vec3 dot left to right, (x + y) + z (:54-60); keys go into a
  std::multiset ordered by distance (equal keys after the earlier ones), and
  the first MAX_TOTAL_VPLS_BEFORE_CULLING are taken.
- InitVplFrameData_ (:1281-1292): position (x, y, z, 1), far plane, radius,
  intensity; colour and specular position zero.
"""
from __future__ import annotations

import numpy as np

f32 = np.float32


def prepare_vpls(pos, radii, far, inten, planes, cam, cap):
    """Returns (records [k, 16] float32 as sgi_vpl, source indices [k])."""
    pos = np.asarray(pos, f32).reshape(-1, 3)
    planes = np.asarray(planes, f32).reshape(6, 4)
    cam = np.asarray(cam, f32)
    keys = []
    for i in range(pos.shape[0]):
        c = pos[i]
        inside = True
        for g in planes:
            d = f32(f32(f32(g[0] * c[0]) + f32(g[1] * c[1])) + f32(f32(g[2] * c[2]) + f32(g[3] * f32(1.0))))
            if d < -f32(radii[i]):
                inside = False
                break
        if not inside:
            continue
        dx, dy, dz = f32(c[0] - cam[0]), f32(c[1] - cam[1]), f32(c[2] - cam[2])
        s = f32(f32(f32(dx * dx) + f32(dy * dy)) + f32(dz * dz))
        keys.append((float(np.sqrt(s)), i))
    keys.sort(key=lambda t: t[0])          # stable: equal distances keep the input order
    keys = keys[:cap]
    rec = np.zeros((len(keys), 16), f32)
    src = np.array([i for _, i in keys], np.int32)
    for k, (_, i) in enumerate(keys):
        rec[k, 0:3] = pos[i]
        rec[k, 3] = 1.0
        rec[k, 12] = radii[i]
        rec[k, 13] = far[i]
        rec[k, 14] = inten[i]
    return rec, src
