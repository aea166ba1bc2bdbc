// sgi_shade_common.cuh - device helpers shared by the culling kernels
// (sgi_kernels.cu) and the shading kernels (sgi_shade.cu): texel packing,
// bilinear sampling, the CSM lookup of calculateInfiniteShadowValue
// (pbr.glsl:158-227) and the VPL cube-map shadow tests (pbr.glsl:81-136).
// Every function is __forceinline__ device code. Texel choices, bilinear
// weights, the CSM compare and the cube-map shadow compares are written with
// the correctly rounded x* operations of sgi_math.cuh, so they are identical in
// the exact and the tolerance build of the shading kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "sgi_internal.h"
#include "sgi_math.cuh"

namespace sgi {
// ------------------------------------------------------------------ texels --
SGI_D uint2 ld_u2(const uint2* p, size_t i) { return __ldg(p + i); }
SGI_D void unpack_h4(uint2 t, float& a, float& b, float& c, float& d) {
    a = h2f((uint16_t)(t.x & 0xffffu)); b = h2f((uint16_t)(t.x >> 16));
    c = h2f((uint16_t)(t.y & 0xffffu)); d = h2f((uint16_t)(t.y >> 16));
}
SGI_D uint2 pack_h4(float a, float b, float c, float d) {
    return make_uint2((uint32_t)f2h(a) | ((uint32_t)f2h(b) << 16), (uint32_t)f2h(c) | ((uint32_t)f2h(d) << 16));
}

// The texels and weights of one bilinear sample: several channels sampled at
// the same uv share them (each channel then evaluates exactly the sum that
// bilinear() below forms).
struct Bilinear {
    size_t o00, o10, o01, o11;
    float w00, w10, w01, w11;
};
SGI_D Bilinear bilinear_at(int W, int H, float s, float t) {
    const float u = xsub(xmul(s, float(W)), 0.5f), v = xsub(xmul(t, float(H)), 0.5f);
    const float fu = floorf(u), fv = floorf(v);
    const float a = xsub(u, fu), b = xsub(v, fv);
    const int i0 = tex_index(fu, W), i1 = tex_index(xadd(fu, 1.0f), W);
    const size_t r0 = (size_t)tex_index(fv, H) * W, r1 = (size_t)tex_index(xadd(fv, 1.0f), H) * W;
    Bilinear q;
    q.o00 = r0 + i0; q.o10 = r0 + i1; q.o01 = r1 + i0; q.o11 = r1 + i1;
    q.w00 = xmul(xsub(1.0f, a), xsub(1.0f, b)); q.w10 = xmul(a, xsub(1.0f, b));
    q.w01 = xmul(xsub(1.0f, a), b); q.w11 = xmul(a, b);
    return q;
}
SGI_D float bilinear_sum(const Bilinear& q, float f00, float f10, float f01, float f11) {
    return __fmaf_rn(f11, q.w11, __fmaf_rn(f01, q.w01, __fmaf_rn(f10, q.w10, xmul(f00, q.w00))));
}

// Bilinear sample (LINEAR, CLAMP_TO_EDGE) at uv of a scalar image.
template <class F> SGI_D float bilinear(F fetch, int W, int H, float s, float t) {
    const Bilinear q = bilinear_at(W, H, s, t);
    const int i0 = (int)(q.o00 % W), i1 = (int)(q.o10 % W), j0 = (int)(q.o00 / W), j1 = (int)(q.o01 / W);
    return bilinear_sum(q, fetch(i0, j0), fetch(i1, j0), fetch(i0, j1), fetch(i1, j1));
}

// ------------------------------------------------------------------- CSM --
// texture(sampler2DArrayShadow) with LINEAR + LEQUAL: bilinear weights over
// the four 0/1 compare results.
SGI_D float csm_pcf(const float* __restrict__ base, int R, float s, float t, float ref) {
    const Bilinear q = bilinear_at(R, R, s, t);
    const float c00 = ref <= __ldg(base + q.o00) ? 1.0f : 0.0f;
    const float c10 = ref <= __ldg(base + q.o10) ? 1.0f : 0.0f;
    const float c01 = ref <= __ldg(base + q.o01) ? 1.0f : 0.0f;
    const float c11 = ref <= __ldg(base + q.o11) ? 1.0f : 0.0f;
    return bilinear_sum(q, c00, c10, c01, c11);
}

// The 3x3 filtered samples of one cascade (pbr.glsl:206-215): the sum over
// yi (outer), xi (inner) in -1..1 of csm_pcf at (s + xi wh, t + yi wh), added
// in that order. The samples share their coordinates per axis (u depends on
// xi only, v on yi only), so the texel columns, rows and fractions are formed
// once per axis value. Where the columns of the three xi form the run
// c - 1 .. c + 2 (and the rows likewise) -- away from the map's edges, where
// the clamp repeats a texel -- the 16 texels of that window are read and
// compared once; otherwise each sample reads its own four. Either way every
// sample's weights and compare results are those csm_pcf forms.
SGI_D float csm_pcf9(const float* __restrict__ base, int R, float s, float t, float wh, float ref) {
    float a[3], b[3];
    int c0[3], c1[3];
    size_t r0[3], r1[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float o = xmul(float(k - 1), wh);
        const float u = xsub(xmul(xadd(s, o), float(R)), 0.5f), v = xsub(xmul(xadd(t, o), float(R)), 0.5f);
        const float fu = floorf(u), fv = floorf(v);
        a[k] = xsub(u, fu);
        b[k] = xsub(v, fv);
        c0[k] = tex_index_clamped(fu, R);
        c1[k] = tex_index_clamped(xadd(fu, 1.0f), R);
        r0[k] = (size_t)tex_index_clamped(fv, R) * R;
        r1[k] = (size_t)tex_index_clamped(xadd(fv, 1.0f), R) * R;
    }
    const bool run = c0[0] + 1 == c0[1] && c0[1] + 1 == c0[2] && c1[0] == c0[0] + 1 && c1[2] == c0[2] + 1 &&
                     r0[0] + R == r0[1] && r0[1] + R == r0[2] && r1[0] == r0[0] + R && r1[2] == r0[2] + R;
    float light = 0.0f;
    if (run) {
        float cmp[4][4];   // [row r0[0] + i R][column c0[0] + j]
        bool any = false;
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                cmp[i][j] = ref <= __ldg(base + r0[0] + (size_t)i * R + c0[0] + j) ? 1.0f : 0.0f;
                any = any || cmp[i][j] != 0.0f;
            }
        // every compare 0 (the window is in shadow): each sample is fma(0, w, ... 0 * w00) = +0 for the
        // weights in [0, 1], and so is their sum, which the loop below would form
        if (!any) return 0.0f;
#pragma unroll
        for (int yi = 0; yi < 3; ++yi)
#pragma unroll
            for (int xi = 0; xi < 3; ++xi) {
                const float w00 = xmul(xsub(1.0f, a[xi]), xsub(1.0f, b[yi])), w10 = xmul(a[xi], xsub(1.0f, b[yi]));
                const float w01 = xmul(xsub(1.0f, a[xi]), b[yi]), w11 = xmul(a[xi], b[yi]);
                const float f = __fmaf_rn(cmp[yi + 1][xi + 1], w11,
                                          __fmaf_rn(cmp[yi + 1][xi], w01, __fmaf_rn(cmp[yi][xi + 1], w10,
                                                                                    xmul(cmp[yi][xi], w00))));
                light = xadd(light, f);
            }
    } else {
#pragma unroll
        for (int yi = 0; yi < 3; ++yi)
#pragma unroll
            for (int xi = 0; xi < 3; ++xi) {
                const float w00 = xmul(xsub(1.0f, a[xi]), xsub(1.0f, b[yi])), w10 = xmul(a[xi], xsub(1.0f, b[yi]));
                const float w01 = xmul(xsub(1.0f, a[xi]), b[yi]), w11 = xmul(a[xi], b[yi]);
                const float d00 = ref <= __ldg(base + r0[yi] + c0[xi]) ? 1.0f : 0.0f;
                const float d10 = ref <= __ldg(base + r0[yi] + c1[xi]) ? 1.0f : 0.0f;
                const float d01 = ref <= __ldg(base + r1[yi] + c0[xi]) ? 1.0f : 0.0f;
                const float d11 = ref <= __ldg(base + r1[yi] + c1[xi]) ? 1.0f : 0.0f;
                light = xadd(light, __fmaf_rn(d11, w11, __fmaf_rn(d01, w01, __fmaf_rn(d10, w10, xmul(d00, w00)))));
            }
    }
    return light;
}

// calculateInfiniteShadowValue, pbr.glsl:158-227: lit fraction.
SGI_D float infinite_shadow(const sgi_csm& csm, V3 fragPos, V3 normal, bool useDepthBias) {
    V3 blends = v3(dot4(csm.cascade_planes[0], fragPos), dot4(csm.cascade_planes[1], fragPos),
                   dot4(csm.cascade_planes[2], fragPos));
    float bias = xdiv(csm.depth_bias, xsub(csm.zfar, csm.znear));
    if (!useDepthBias) bias = 0.0f;
    V3 L = v3(csm.light_direction[0], csm.light_direction[1], csm.light_direction[2]);
    V3 position = xadd3(fragPos, xmul3(xmul3(normal, xsub(1.0f, saturate(xdot(normal, L)))), 1.0f));
    bool beyond2 = blends.y >= 0.0f;
    bool beyond3 = blends.z >= 0.0f;
    int index1 = beyond2 ? 2 : 0;
    int index2 = beyond3 ? 3 : 1;
    V4 c1 = mat4_mul(csm.cascade_proj_view[index1], position.x, position.y, position.z, 1.0f);
    V4 c2 = mat4_mul(csm.cascade_proj_view[index2], position.x, position.y, position.z, 1.0f);
    V3 cc1 = xadd3(xmul3(xdiv3(v3(c1.x, c1.y, c1.z), c1.w), 0.5f), v3s(0.5f));
    V3 cc2 = xadd3(xmul3(xdiv3(v3(c2.x, c2.y, c2.z), c2.w), 0.5f), v3s(0.5f));
    float depth1 = cc1.z;
    float depth2 = beyond3 ? saturate(cc2.z) : cc2.z;
    float weight = beyond2 ? xsub(saturate(blends.y), saturate(blends.z)) : xsub(1.0f, saturate(blends.x));
    const int R = csm.resolution;
    float wh = xdiv(1.0f, float(R));
    const float* b1 = csm.depth + (size_t)index1 * R * R;
    const float* b2 = csm.depth + (size_t)index2 * R * R;
    float ref1 = xsub(depth1, bias), ref2 = xsub(depth2, bias);
    const float light1 = csm_pcf9(b1, R, cc1.x, cc1.y, wh, ref1);
    const float light2 = csm_pcf9(b2, R, cc2.x, cc2.y, wh, ref2);
    const float samples = 9.0f;   // the nine samples counted one by one: exact
    return xmul(xmixf(light2, light1, weight), xdiv(1.0f, samples));
}

// ------------------------------------------------------------- cube maps --
// Nearest texel of a cube face_size n in direction d: returns its offset within the layer stack.
SGI_D size_t cube_texel(int layer, int n, V3 d) {
    float ax = gabs(d.x), ay = gabs(d.y), az = gabs(d.z);
    int face; float sc, tc, ma;
    if (ax >= ay && ax >= az) {
        ma = ax;
        if (d.x >= 0.0f) { face = 0; sc = -d.z; tc = -d.y; } else { face = 1; sc = d.z; tc = -d.y; }
    } else if (ay >= az) {
        ma = ay;
        if (d.y >= 0.0f) { face = 2; sc = d.x; tc = d.z; } else { face = 3; sc = d.x; tc = -d.z; }
    } else {
        ma = az;
        if (d.z >= 0.0f) { face = 4; sc = d.x; tc = -d.y; } else { face = 5; sc = -d.x; tc = -d.y; }
    }
    float s = xmul(0.5f, xadd(xdiv(sc, ma), 1.0f));
    float t = xmul(0.5f, xadd(xdiv(tc, ma), 1.0f));
    int i = nearest_index(s, n), j = nearest_index(t, n);
    return (((size_t)layer * 6 + face) * n + j) * n + i;
}

// Offset of texel (i, j) of face `face` of cube `layer`, face size n:
// ((layer * 6 + face) * n + j) * n + i = layer * 6n^2 + ((face * n + j) * n + i).
// The second term is below 6n^2 < 2^31 (n <= SGI_MAX_CUBE_FACE, checked when the
// atlas is set), so it is formed in 32-bit arithmetic and added to the 64-bit
// layer offset: the same value with one wide multiply-add.
SGI_D size_t cube_offset(int layer, int face, int n, int j, int i) {
    const uint32_t in_cube = (uint32_t)((face * n + j) * n + i);
    return (size_t)(uint32_t)layer * (size_t)(6u * (uint32_t)n * (uint32_t)n) + in_cube;
}

SGI_D float cube_fetch(const sgi_cube_atlas& at, sgi_atlas_entry e, V3 d) {
    if (e.index < 0 || e.index >= at.num_atlases || e.layer < 0 || e.layer >= at.layers_per_atlas) return 1.0f;
    float ax = gabs(d.x), ay = gabs(d.y), az = gabs(d.z);
    int face; float sc, tc, ma;
    if (ax >= ay && ax >= az) {
        ma = ax;
        if (d.x >= 0.0f) { face = 0; sc = -d.z; tc = -d.y; } else { face = 1; sc = d.z; tc = -d.y; }
    } else if (ay >= az) {
        ma = ay;
        if (d.y >= 0.0f) { face = 2; sc = d.x; tc = d.z; } else { face = 3; sc = d.x; tc = -d.z; }
    } else {
        ma = az;
        if (d.z >= 0.0f) { face = 4; sc = d.x; tc = -d.y; } else { face = 5; sc = -d.x; tc = -d.y; }
    }
    float s = xmul(0.5f, xadd(xdiv(sc, ma), 1.0f));
    float t = xmul(0.5f, xadd(xdiv(tc, ma), 1.0f));
    const int n = at.face_size;
    int i = nearest_index(s, n), j = nearest_index(t, n);
    const size_t off = cube_offset(e.layer, face, n, j, i);   // 0 <= e.layer < layers_per_atlas
    const void* base = at.atlas[e.index];
    if (at.format == SGI_CUBE_F16) return h2f(__ldg((const unsigned short*)base + off));
    if (at.format == SGI_CUBE_F32) return __ldg((const float*)base + off);
    return unorm16(__ldg((const unsigned short*)base + off));   // = b / 65535, correctly rounded
}

// calculateShadowValue1Sample, pbr.glsl:116-136 (1 = occluded), given the
// direction fragPos - lightPos and its length
SGI_D float shadow_1sample_dir(const sgi_cube_atlas& at, sgi_atlas_entry e, float farPlane, V3 fragDir,
                               float currentDepth, float lightNormalDot, float minBias) {
    float bias = xmul(currentDepth, gmax(minBias, xmul(saturate(lightNormalDot), 0.03f)));
    float depth = cube_fetch(at, e, fragDir);
    depth = xmul(depth, farPlane);
    return xsub(currentDepth, bias) > depth ? 1.0f : 0.0f;
}
SGI_D float shadow_1sample(const sgi_cube_atlas& at, sgi_atlas_entry e, float farPlane, V3 fragPos, V3 lightPos,
                           float lightNormalDot, float minBias) {
    V3 fragDir = xsub3(fragPos, lightPos);
    float currentDepth = xlength(fragDir);
    float bias = xmul(currentDepth, gmax(minBias, xmul(saturate(lightNormalDot), 0.03f)));
    float depth = cube_fetch(at, e, fragDir);
    depth = xmul(depth, farPlane);
    return xsub(currentDepth, bias) > depth ? 1.0f : 0.0f;
}

// calculateShadowValue8Samples, pbr.glsl:81-113 (fraction occluded): eight taps at
// the direction offset by (+-0.3, +-0.3, +-0.3), x outermost.
SGI_D float shadow_8samples(const sgi_cube_atlas& at, sgi_atlas_entry e, float farPlane, V3 fragPos, V3 lightPos,
                            float lightNormalDot, float minBias) {
    V3 fragDir = xsub3(fragPos, lightPos);
    float currentDepth = xlength(fragDir);
    float bias = xmul(currentDepth, gmax(minBias, xmul(saturate(lightNormalDot), 0.03f)));
    float shadow = 0.0f;
    const float offs[2] = {-0.3f, 0.3f};
#pragma unroll
    for (int x = 0; x < 2; ++x)
#pragma unroll
        for (int y = 0; y < 2; ++y)
#pragma unroll
            for (int z = 0; z < 2; ++z) {
                float depth = cube_fetch(at, e, xadd3(fragDir, v3(offs[x], offs[y], offs[z])));
                depth = xmul(depth, farPlane);
                if (xsub(currentDepth, bias) > depth) shadow = xadd(shadow, 1.0f);
            }
    return xdiv(shadow, 8.0f);
}

}  // namespace sgi
