// sgi_host.cpp - C ABI of include/sgi_host.h: the frame's VPL buffer on the host.
//
// Host sources are compiled with -ffp-contract=off, so the distances and plane
// tests round operation by operation as the header states, on any host.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <vector>

#include "../../include/sgi_host.h"

namespace {

// glm::dot of two vec4 forms the four products and adds them pairwise,
// (x + y) + (z + w) (glm/detail/func_geometric.inl:64-70, compute_dot<tvec4>).
bool sphere_in_frustum(const float* c, float radius, const float* planes) {
    for (int i = 0; i < 6; ++i) {
        const float* g = planes + 4 * i;
        const float distance = (g[0] * c[0] + g[1] * c[1]) + (g[2] * c[2] + g[3] * 1.0f);
        if (distance < -radius) return false;
    }
    return true;
}

bool all_finite(const float* v, size_t n) {
    for (size_t i = 0; i < n; ++i)
        if (!std::isfinite(v[i])) return false;
    return true;
}

// glm::distance of two vec3: sqrt((x + y) + z) of the squared differences.
float distance_to(const float* p, const float* cam) {
    const float dx = p[0] - cam[0], dy = p[1] - cam[1], dz = p[2] - cam[2];
    return std::sqrt(dx * dx + dy * dy + dz * dz);
}

}  // namespace

extern "C" sgi_status sgi_prepare_vpls(const float* positions, const float* radii, const float* far_planes,
                                       const float* intensities, int32_t n, const float* planes,
                                       const float* camera, int32_t cap, sgi_vpl* out, int32_t* source,
                                       int32_t* count) {
    if (n < 0 || cap < 0 || !count || !planes || !camera) return SGI_ERR_ARG;
    if (n > 0 && (!positions || !radii || !far_planes || !intensities)) return SGI_ERR_ARG;
    if (cap > 0 && !out) return SGI_ERR_ARG;
    *count = 0;
    // A NaN distance would break the strict weak order the sort needs, and a NaN
    // plane or radius makes the frustum test meaningless: such input is rejected.
    if (!all_finite(planes, 24) || !all_finite(camera, 3)) return SGI_ERR_ARG;
    if (n > 0 && (!all_finite(positions, 3 * (size_t)n) || !all_finite(radii, (size_t)n))) return SGI_ERR_ARG;
    struct Key {
        double distance;
        int32_t index;
    };
    std::vector<Key> keys;
    try {
        keys.reserve((size_t)n);
    } catch (...) {
        return SGI_ERR_OOM;
    }
    for (int32_t i = 0; i < n; ++i) {
        const float* p = positions + 3 * (size_t)i;
        if (!sphere_in_frustum(p, radii[i], planes)) continue;
        keys.push_back(Key{(double)distance_to(p, camera), i});
    }
    // the multiset's order: by distance, equal distances in insertion order
    std::stable_sort(keys.begin(), keys.end(), [](const Key& a, const Key& b) { return a.distance < b.distance; });
    const int32_t kept = (int32_t)std::min<size_t>(keys.size(), (size_t)cap);
    for (int32_t k = 0; k < kept; ++k) {
        const int32_t i = keys[k].index;
        sgi_vpl v;
        std::memset(&v, 0, sizeof(v));
        v.position[0] = positions[3 * (size_t)i];
        v.position[1] = positions[3 * (size_t)i + 1];
        v.position[2] = positions[3 * (size_t)i + 2];
        v.position[3] = 1.0f;
        v.radius = radii[i];
        v.far_plane = far_planes[i];
        v.intensity = intensities[i];
        out[k] = v;
        if (source) source[k] = i;
    }
    *count = kept;
    return SGI_OK;
}
