// sgi_selftest.cu - bitwise self-check of the packed (two-lane) shading math.
//
// The a-trous passes evaluate two taps per instruction with the packed
// functions of sgi_math.cuh (expf_ieee2, pow128x2, atrous_weight2); their
// contract is that each lane returns the scalar function's result bit for
// bit. sgi_lane_selftest evaluates the packed operations and functions both
// ways on operands drawn from a hash of the thread index (realistic ranges,
// rounding ties, subnormal and special values) and counts the threads whose
// results differ in any bit.
// Compiled with -fmad=false like the kernels it checks.
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/sgi.h"
#include "sgi_math.cuh"

namespace sgi {
namespace {

constexpr int kChecks = SGI_LANE_CHECKS;
constexpr int kRecord = 16;   // floats recorded for the first mismatch of each check

SGI_D uint32_t mix32(uint32_t x) {
    x ^= x >> 16; x *= 0x7feb352dU; x ^= x >> 15; x *= 0x846ca68bU; x ^= x >> 16;
    return x;
}

struct Draw {
    uint32_t state;
    SGI_D float unit() { state = mix32(state + 0x9e3779b9U); return float(state >> 8) * (1.0f / 16777216.0f); }
    SGI_D float range(float lo, float hi) { return lo + (hi - lo) * unit(); }
    SGI_D V3 box(float lo, float hi) { return v3(range(lo, hi), range(lo, hi), range(lo, hi)); }
    SGI_D V3 dir() { return normalize(box(-1.0f, 1.0f) + v3s(1e-3f)); }
    // any finite binary32, subnormals and signed zeros included
    SGI_D float bits() {
        state = mix32(state + 0x9e3779b9U);
        uint32_t b = state;
        if (((b >> 23) & 0xffu) == 0xffu) b &= ~(1u << 30);
        return __uint_as_float(b);
    }
};

SGI_D bool same(float a, float b) { return __float_as_uint(a) == __float_as_uint(b); }

struct Recorder {
    unsigned* counts;
    float* first;
    SGI_D void check(int k, const float* got, const float* want, int m, const float* in, int nin) {
        bool ok = true;
        for (int i = 0; i < m; ++i) ok = ok && same(got[i], want[i]);
        if (ok) return;
        if (atomicAdd(counts + k, 1u) == 0u) {
            float* r = first + k * kRecord;
            int j = 0;
            for (int i = 0; i < m && j < kRecord; ++i) { r[j++] = got[i]; }
            for (int i = 0; i < m && j < kRecord; ++i) { r[j++] = want[i]; }
            for (int i = 0; i < nin && j < kRecord; ++i) { r[j++] = in[i]; }
        }
    }
};

SGI_D void put2(float* g, float2 v) { g[0] = v.x; g[1] = v.y; }

__global__ void lane_selftest_kernel(int n, unsigned* counts, float* first) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    Recorder rec{counts, first};
    Draw d{mix32((uint32_t)t * 2654435761U)};
    float g[4], w[4];
    // 0-2: packed add, multiply and multiply-add on arbitrary finite operands
    // with normal results
    {
        const float a0 = d.bits(), a1 = d.bits(), b0 = d.bits(), b1 = d.bits(), c0 = d.bits(), c1 = d.bits();
        const float in[6] = {a0, a1, b0, b1, c0, c1};
        auto normal = [](float v) { return fabsf(v) >= 0x1p-126f && fabsf(v) <= 3.4028234e38f; };
        w[0] = a0 + b0; w[1] = a1 + b1;
        if (normal(a0) && normal(a1) && normal(b0) && normal(b1) && normal(w[0]) && normal(w[1])) {
            put2(g, add2(make_float2(a0, a1), make_float2(b0, b1)));
            rec.check(0, g, w, 2, in, 4);
        }
        w[0] = a0 * b0; w[1] = a1 * b1;
        if (normal(a0) && normal(a1) && normal(b0) && normal(b1) && normal(w[0]) && normal(w[1])) {
            put2(g, mul2(make_float2(a0, a1), make_float2(b0, b1)));
            rec.check(1, g, w, 2, in, 4);
        }
        w[0] = __fmaf_rn(a0, b0, c0); w[1] = __fmaf_rn(a1, b1, c1);
        if (normal(a0) && normal(a1) && normal(b0) && normal(b1) && normal(c0) && normal(c1) &&
            normal(a0 * b0) && normal(a1 * b1) && normal(w[0]) && normal(w[1])) {
            put2(g, fma2(make_float2(a0, a1), make_float2(b0, b1), make_float2(c0, c1)));
            rec.check(2, g, w, 2, in, 6);
        }
    }
    // 3-5: exact rounding ties (odd 13- and 12-bit significands; an odd 24-bit
    // integer plus or minus one half)
    {
        const uint32_t h = mix32((uint32_t)t ^ 0xa5a5a5a5U);
        const float a0 = float((h & 0xfffu) | 0x1001u) * 0x1p-12f, b0 = float(((h >> 12) & 0x7ffu) | 0x801u) * 0x1p-11f;
        const float a1 = -a0, b1 = b0 * 2.0f;
        const float in[4] = {a0, b0, a1, b1};
        put2(g, mul2(make_float2(a0, a1), make_float2(b0, b1)));
        w[0] = a0 * b0; w[1] = a1 * b1;
        rec.check(3, g, w, 2, in, 4);
        const float big0 = float(((h >> 8) & 0x7fffffu) | 0x800001u), big1 = -float((h & 0x7fffffu) | 0x800001u);
        const float in2[2] = {big0, big1};
        put2(g, add2(make_float2(big0, big1), make_float2(0.5f, -0.5f)));
        w[0] = big0 + 0.5f; w[1] = big1 + -0.5f;
        rec.check(4, g, w, 2, in2, 2);
        put2(g, fma2(make_float2(a0, a1), make_float2(b0, b1), make_float2(1.0f, -3.0f)));
        w[0] = __fmaf_rn(a0, b0, 1.0f); w[1] = __fmaf_rn(a1, b1, -3.0f);
        rec.check(5, g, w, 2, in, 4);
    }
    // 10-11: packed multiply-add with a subnormal multiplicand (a tiny filter
    // weight) onto zero and onto normal sums
    {
        const float f0 = d.unit() * 0x1p-126f, f1 = __uint_as_float(mix32((uint32_t)t) & 0x7fffffu);
        const float a0 = d.range(0.0f, 64.0f), a1 = __half2float(__float2half_rn(d.range(0.0f, 2.0f)));
        const float in[4] = {f0, f1, a0, a1};
        put2(g, fma2(make_float2(f0, f1), make_float2(a0, a1), make_float2(0.0f, 0.0f)));
        w[0] = __fmaf_rn(f0, a0, 0.0f); w[1] = __fmaf_rn(f1, a1, 0.0f);
        rec.check(10, g, w, 2, in, 4);
        const float c0 = d.range(0.0f, 1e-30f), c1 = d.range(0.0f, 4.0f);
        put2(g, fma2(make_float2(f0, f1), make_float2(a0, a1), make_float2(c0, c1)));
        w[0] = __fmaf_rn(f0, a0, c0); w[1] = __fmaf_rn(f1, a1, c1);
        rec.check(11, g, w, 2, in, 4);
    }
    // 6: exp over its whole range: normal, tiny, underflowing and special arguments,
    // and arguments around the bound below which the range reduction is skipped
    // (packed, and the scalar expf_exact_near0 and expf_exact_mid, against the full scalar path)
    {
        float x[2];
        for (int l = 0; l < 2; ++l) {
            const int c = (int)(d.unit() * 8.0f);
            x[l] = c == 0 ? -d.range(80.0f, 110.0f) : c == 1 ? d.range(80.0f, 90.0f) : c == 2 ? d.bits() * 1e-30f
                 : c == 3 ? (d.unit() < 0.5f ? 0.0f : -0.0f) : c == 4 ? -d.range(86.0f, 88.0f)
                 : c == 5 ? d.range(-0.4f, 0.4f) : -d.range(0.0f, 8.0f);
        }
        put2(g, expf_ieee2(make_float2(x[0], x[1])));
        w[0] = expf_exact(x[0]); w[1] = expf_exact(x[1]);
        rec.check(6, g, w, 2, x, 2);
        g[0] = expf_exact_near0(x[0]); g[1] = expf_exact_near0(x[1]);
        rec.check(6, g, w, 2, x, 2);
        g[0] = expf_exact_mid(x[0]); g[1] = expf_exact_mid(x[1]);
        rec.check(6, g, w, 2, x, 2);
    }
    // 7: x^128 for x in [0, 1.001], small values included
    {
        float x[2];
        for (int l = 0; l < 2; ++l) {
            const int c = (int)(d.unit() * 4.0f);
            x[l] = c == 0 ? d.range(0.0f, 0.6f) : c == 1 ? d.range(0.45f, 0.55f) : c == 2 ? d.unit() * 1e-20f
                                                                                     : d.range(0.0f, 1.001f);
        }
        put2(g, pow128x2(make_float2(x[0], x[1])));
        w[0] = pow128(x[0]); w[1] = pow128(x[1]);
        rec.check(7, g, w, 2, x, 2);
    }
    // 8-9: a pair of a-trous tap weights, and their accumulation into the four
    // channel sums, against the scalar tap loop
    {
        const V3 cn = d.dir();
        const float cd = d.range(0.0f, 120.0f);
        float4 q[2];
        for (int l = 0; l < 2; ++l) {
            const int c = (int)(d.unit() * 4.0f);
            const V3 n = c == 0 ? d.dir() : normalize(cn + d.box(-0.4f, 0.4f) * (c == 1 ? 1.0f : 0.1f));
            const float z = c == 3 ? cd + d.range(-100.0f, 100.0f) : cd + d.range(-2.0f, 2.0f);
            q[l] = make_float4(n.x, n.y, n.z, z);
        }
        const float2 f = atrous_weight2(f2s(cn.x), f2s(cn.y), f2s(cn.z), -cd, q[0], q[1]);
        w[0] = atrous_weight(cn, cd, q[0]); w[1] = atrous_weight(cn, cd, q[1]);
        put2(g, f);
        // on a mismatch: the packed and scalar dot, x^128 and exp of both lanes
        const float2 dz = add2(make_float2(q[0].w, q[1].w), f2s(-cd));
        const float2 wz = expf_ieee2(make_float2(dz.x < 0.0f ? dz.x : -dz.x, dz.y < 0.0f ? dz.y : -dz.y));
        const float2 dn = fma2(f2s(cn.z), make_float2(q[0].z, q[1].z),
                                     fma2(f2s(cn.y), make_float2(q[0].y, q[1].y),
                                                mul2(f2s(cn.x), make_float2(q[0].x, q[1].x))));
        const float2 wn = pow128x2(make_float2(gmax(0.0f, dn.x), gmax(0.0f, dn.y)));
        const float sdn0 = dot(cn, v3(q[0].x, q[0].y, q[0].z)), sdn1 = dot(cn, v3(q[1].x, q[1].y, q[1].z));
        const float in[12] = {dn.x, sdn0, dn.y, sdn1, wn.x, pow128(gmax(0.0f, sdn0)), wn.y, pow128(gmax(0.0f, sdn1)),
                              wz.x, expf_ieee(-gabs(cd - q[0].w)), wz.y, expf_ieee(-gabs(cd - q[1].w))};
        rec.check(8, g, w, 2, in, 12);
        // texels: FP16 values (non-negative), sums as after some earlier taps
        float tex[2][4], acc[4];
        for (int k = 0; k < 4; ++k) {
            acc[k] = d.unit() < 0.25f ? 0.0f : __half2float(__float2half_rn(d.range(0.0f, 4.0f)));
            for (int l = 0; l < 2; ++l) {
                const float u = d.unit();
                tex[l][k] = __half2float(__float2half_rn(u < 0.2f ? 0.0f : u < 0.4f ? u * 1e-6f : u * 30.0f));
            }
        }
        float2 a01 = make_float2(acc[0], acc[1]), a23 = make_float2(acc[2], acc[3]);
        for (int l = 0; l < 2; ++l) {
            a01 = fma2(f2s(l == 0 ? f.x : f.y), make_float2(tex[l][0], tex[l][1]), a01);
            a23 = fma2(f2s(l == 0 ? f.x : f.y), make_float2(tex[l][2], tex[l][3]), a23);
        }
        const float sw0 = w[0], sw1 = w[1];
        for (int k = 0; k < 4; ++k) w[k] = __fmaf_rn(sw1, tex[1][k], __fmaf_rn(sw0, tex[0][k], acc[k]));
        g[0] = a01.x; g[1] = a01.y; g[2] = a23.x; g[3] = a23.y;
        rec.check(9, g, w, 4, in, 8);
    }
}

}  // namespace
}  // namespace sgi

extern "C" sgi_status sgi_lane_selftest(int32_t n, uint32_t* counts, float* first) {
    if (n < 1 || !counts) return SGI_ERR_ARG;
    unsigned* dc = nullptr;
    float* df = nullptr;
    const size_t nf = (size_t)sgi::kChecks * sgi::kRecord;
    if (cudaMalloc(&dc, sgi::kChecks * sizeof(unsigned)) != cudaSuccess) return SGI_ERR_OOM;
    if (cudaMalloc(&df, nf * sizeof(float)) != cudaSuccess) {
        cudaFree(dc);
        return SGI_ERR_OOM;
    }
    cudaError_t e = cudaMemset(dc, 0, sgi::kChecks * sizeof(unsigned));
    if (e == cudaSuccess) e = cudaMemset(df, 0, nf * sizeof(float));
    if (e == cudaSuccess) {
        sgi::lane_selftest_kernel<<<(n + 255) / 256, 256>>>(n, dc, df);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(counts, dc, sgi::kChecks * sizeof(unsigned), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && first) e = cudaMemcpy(first, df, nf * sizeof(float), cudaMemcpyDeviceToHost);
    cudaFree(dc);
    cudaFree(df);
    return e == cudaSuccess ? SGI_OK : SGI_ERR_CUDA;
}
