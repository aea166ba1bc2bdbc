// sgi_math.cuh - device-side shading math of the GI/lighting stage.
//
// The exact build of the kernels is compiled with -fmad=false, -prec-div=true
// and -prec-sqrt=true: each +, -, *, / and sqrtf below is one correctly rounded
// binary32 operation, and multiply-adds are fused only where __fmaf_rn is
// written, evaluated in the order the expression tree gives. That makes the
// results reproducible on any IEEE-754 machine, which is how the per-pixel
// results are checked bit for bit against a CPU restatement of the StratusGFX
// shaders. No CUDA math-library transcendental is called there: exp is
// computed by Cody-Waite range reduction plus a degree-7 Taylor polynomial, and
// pow only appears with the integer exponents 5 and 128.
//
// The tolerance build of the shading kernels (SGI_FAST_MATH = 1, compiled with
// contraction and approximate division and square root) evaluates the same
// expressions faster, except for everything a branch decision or a texel
// choice depends on: those are written with the x* functions below
// (__fadd_rn, __fmul_rn, __fdiv_rn, __fsqrt_rn, __fmaf_rn), which no compiler
// flag contracts or approximates, so both builds take the same branches, read
// the same texels and keep the same per-tile lists; only continuous values
// differ between them.
//
// Implementation-defined GLSL arithmetic, fixed here: dot products, matrix
// rows, polynomial steps and weighted sums are fused multiply-add chains;
// a vector divided by a scalar is multiplied by the scalar's correctly
// rounded reciprocal; normalize(v) = v * (1 / sqrt(dot(v, v))).
//
// GLSL built-in semantics used throughout (GLSL 4.60 spec wording):
//   min(x, y) = y < x ? y : x,  max(x, y) = x < y ? y : x,
//   clamp(x, a, b) = min(max(x, a), b),  mix(x, y, a) = fma(y, a, x*(1-a)).
#pragma once

#include <cuda_fp16.h>
#include <stdint.h>

namespace sgi {

#define SGI_D __device__ __forceinline__

constexpr float kPi = 3.14159265359f;          // common.glsl:3
constexpr float kEps = 0.00001f;               // PREVENT_DIV_BY_ZERO, common.glsl:4
constexpr float kHalfMax = 65504.0f;           // HALF_FLOAT_MAX, common.glsl:6
constexpr float kFloatMax = 3.402823466e+38f;  // FLOAT_MAX, common.glsl:7

// the global nanosecond timer (bounded waits)
SGI_D long long global_ns() {
    long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

SGI_D float gmin(float x, float y) { return y < x ? y : x; }
SGI_D float gmax(float x, float y) { return x < y ? y : x; }
SGI_D float gclamp(float x, float lo, float hi) { return gmin(gmax(x, lo), hi); }
SGI_D float saturate(float x) { return gclamp(x, 0.0f, 1.0f); }
SGI_D float fma_rn(float a, float b, float c) { return __fmaf_rn(a, b, c); }
SGI_D float mixf(float x, float y, float a) { return __fmaf_rn(y, a, x * (1.0f - a)); }
SGI_D float gabs(float x) { return x < 0.0f ? -x : x; }

#ifndef SGI_FAST_MATH
#define SGI_FAST_MATH 0
#endif

// Correctly rounded binary32 operations in every build (see the header comment).
SGI_D float xadd(float a, float b) { return __fadd_rn(a, b); }
SGI_D float xsub(float a, float b) { return __fsub_rn(a, b); }
SGI_D float xmul(float a, float b) { return __fmul_rn(a, b); }
SGI_D float xdiv(float a, float b) { return __fdiv_rn(a, b); }
SGI_D float xsqrt(float a) { return __fsqrt_rn(a); }
SGI_D float xmixf(float x, float y, float a) { return __fmaf_rn(y, a, xmul(x, xsub(1.0f, a))); }

// expf_ieee's Taylor polynomial of the reduced argument r, in Horner form.
SGI_D float exp_poly(float r) {
    float p = __fmaf_rn(r, 1.0f / 5040.0f, 1.0f / 720.0f);
    p = __fmaf_rn(p, r, 1.0f / 120.0f);
    p = __fmaf_rn(p, r, 1.0f / 24.0f);
    p = __fmaf_rn(p, r, 1.0f / 6.0f);
    p = __fmaf_rn(p, r, 0.5f);
    p = __fmaf_rn(p, r, 1.0f);
    return __fmaf_rn(p, r, 1.0f);
}
// |x| < kExpNoReduce: x * log2(e) + 0.5 rounds into (0, 1), so k = 0, the
// reduction returns r = x - 0 - 0 = x (signed zeros included) and the scaling
// multiplies by 2^0 = 1: the result is exp_poly(x) alone. The bound is below
// ln(2) / 2 = 0.3466 with room for the roundings of the product and the sum.
constexpr float kExpNoReduce = 0.34f;

// expf_ieee's arithmetic (below) with every operation explicitly rounded: the
// same value in every build.
SGI_D float expf_exact(float x) {
    if (x != x) return x;
    if (x > 88.72283935546875f) return __int_as_float(0x7f800000);
    if (x < -103.97283935546875f) return 0.0f;
    float kf = floorf(xadd(xmul(x, 1.44269502162933349609375f), 0.5f));
    int k = (int)kf;
    float r = xsub(xsub(x, xmul(kf, 0.693145751953125f)), xmul(kf, 1.428606765330187045037746429443359375e-06f));
    float p = exp_poly(r);
    if (k > 127) { p = xmul(p, 1.7014118346046923e+38f); k -= 127; }
    if (k < -126) { p = xmul(p, 1.1754943508222875e-38f); k += 126; }
    return xmul(p, __int_as_float((k + 127) << 23));
}

// expf_exact for |x| <= 87 with one test: there k lies in [-125, 126], so none of
// the full path's range and scaling tests applies and 2^k and the result are
// normal; NaN and larger arguments take the full path. The same value.
SGI_D float expf_exact_mid(float x) {
    if (!(fabsf(x) <= 87.0f)) return expf_exact(x);
    const float kf = floorf(xadd(xmul(x, 1.44269502162933349609375f), 0.5f));
    const int k = (int)kf;
    const float r =
        xsub(xsub(x, xmul(kf, 0.693145751953125f)), xmul(kf, 1.428606765330187045037746429443359375e-06f));
    return xmul(exp_poly(r), __int_as_float((k + 127) << 23));
}

// exp(x): Cody & Waite (1980) reduction x = k*ln2 + r with ln2 split into a
// 15-bit head (exact products for |k| < 512) and a tail, exp(r) by its Taylor
// series to r^7 in Horner form, then exact scaling by 2^k. In the tolerance
// build of the shading kernels (SGI_FAST_MATH) it is the hardware exponential.
// expf_exact for arguments that are mostly near 0 (depth weights): below
// kExpNoReduce the polynomial alone, the same value.
SGI_D float expf_exact_near0(float x) { return fabsf(x) < kExpNoReduce ? exp_poly(x) : expf_exact(x); }
#if SGI_FAST_MATH
SGI_D float expf_ieee(float x) { return __expf(x); }
SGI_D float expf_ieee_near0(float x) { return __expf(x); }
#else
SGI_D float expf_ieee(float x) { return expf_exact(x); }
SGI_D float expf_ieee_near0(float x) { return expf_exact_near0(x); }
#endif
SGI_D float pow5(float x) { float x2 = x * x; float x4 = x2 * x2; return x4 * x; }
SGI_D float pow128(float x) {
    float y = x * x; y = y * y; y = y * y; y = y * y; y = y * y; y = y * y; y = y * y; return y;
}

// Two lanes of the same functions on the packed FP32 pipe (sm_100+). Each
// packed component rounds like the scalar operation it stands for, with one
// exception the lane self-check in sgi_selftest.cu found: a packed multiply
// whose result feeds a packed add can be contracted into a packed fused
// multiply-add despite -fmad=false and an explicit .rn (the scalar operations
// are not). So no packed add below takes a packed product as an operand; a
// product that is then added is formed per lane.
SGI_D float2 f2s(float s) { return make_float2(s, s); }
SGI_D unsigned long long pk2(float2 a) {
    unsigned long long r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a.x), "f"(a.y));
    return r;
}
SGI_D float2 upk2(unsigned long long r) {
    float2 a;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(a.x), "=f"(a.y) : "l"(r));
    return a;
}
SGI_D float2 add2(float2 a, float2 b) {
    unsigned long long d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(pk2(a)), "l"(pk2(b)));
    return upk2(d);
}
SGI_D float2 mul2(float2 a, float2 b) {
    unsigned long long d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(pk2(a)), "l"(pk2(b)));
    return upk2(d);
}
SGI_D float2 fma2(float2 a, float2 b, float2 c) {
    unsigned long long d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(pk2(a)), "l"(pk2(b)), "l"(pk2(c)));
    return upk2(d);
}
// x in [-87, 88] with |x| >= 2^-100, or 0: the reduced argument, the
// polynomial, 2^k and the result are all normal numbers (or exact), and
// expf_ieee's extra scaling steps do not apply; other lanes (underflow,
// overflow, tiny and special arguments) take the scalar code.
SGI_D bool exp_packable(float x) {
    const float a = fabsf(x);
    return a == 0.0f || (a >= 0x1p-100f && x >= -87.0f && x <= 88.0f);
}
// expf_ieee's range reduction, per lane (its products feed sums).
SGI_D float exp_reduce(float x, float& kf) {
    kf = floorf(x * 1.44269502162933349609375f + 0.5f);
    return (x - kf * 0.693145751953125f) - kf * 1.428606765330187045037746429443359375e-06f;
}
// exp_poly in both lanes.
SGI_D float2 exp_poly2(float2 r) {
    float2 p = fma2(r, f2s(1.0f / 5040.0f), f2s(1.0f / 720.0f));
    p = fma2(p, r, f2s(1.0f / 120.0f));
    p = fma2(p, r, f2s(1.0f / 24.0f));
    p = fma2(p, r, f2s(1.0f / 6.0f));
    p = fma2(p, r, f2s(0.5f));
    p = fma2(p, r, f2s(1.0f));
    return fma2(p, r, f2s(1.0f));
}
SGI_D float2 expf_ieee2(float2 x) {
#if SGI_FAST_MATH
    return make_float2(__expf(x.x), __expf(x.y));
#endif
    // k = 0 in both lanes: the polynomial alone. Each lane equals exp_poly even for tiny or
    // subnormal arguments: every Horner step then rounds to its constant and the result is 1,
    // whether or not the packed operations flush the argument.
    if (fabsf(x.x) < kExpNoReduce && fabsf(x.y) < kExpNoReduce) return exp_poly2(x);
    if (!(exp_packable(x.x) && exp_packable(x.y))) return make_float2(expf_ieee(x.x), expf_ieee(x.y));
    float2 kf;
    const float2 r = make_float2(exp_reduce(x.x, kf.x), exp_reduce(x.y, kf.y));
    const float2 p = exp_poly2(r);
    const int k0 = (int)kf.x, k1 = (int)kf.y;   // in [-126, 127]
    return mul2(p, make_float2(__int_as_float((k0 + 127) << 23), __int_as_float((k1 + 127) << 23)));
}
// x^128 by seven squarings, the first six packed and the last one per lane:
// for 0 <= x <= 1 the squares decrease, so if x^64 >= 2^-126 every packed
// square was a normal number, and otherwise x^64 < 2^-126 in both forms and
// the last square is 0 in both (for x >= 1 the squares grow).
SGI_D float2 pow128x2(float2 x) {
    float2 y = mul2(x, x);
#pragma unroll
    for (int i = 0; i < 5; ++i) y = mul2(y, y);
    return make_float2(y.x * y.x, y.y * y.y);
}

// ---------------------------------------------------------------- vectors --
struct V3 { float x, y, z; };
SGI_D V3 v3(float x, float y, float z) { return V3{x, y, z}; }
SGI_D V3 v3s(float s) { return V3{s, s, s}; }
SGI_D V3 operator+(V3 a, V3 b) { return V3{a.x + b.x, a.y + b.y, a.z + b.z}; }
SGI_D V3 operator-(V3 a, V3 b) { return V3{a.x - b.x, a.y - b.y, a.z - b.z}; }
SGI_D V3 operator*(V3 a, V3 b) { return V3{a.x * b.x, a.y * b.y, a.z * b.z}; }
SGI_D V3 operator/(V3 a, V3 b) { return V3{a.x / b.x, a.y / b.y, a.z / b.z}; }
SGI_D V3 operator*(V3 a, float s) { return V3{a.x * s, a.y * s, a.z * s}; }
SGI_D V3 operator*(float s, V3 a) { return V3{s * a.x, s * a.y, s * a.z}; }
SGI_D V3 operator/(V3 a, float s) { const float r = 1.0f / s; return V3{a.x * r, a.y * r, a.z * r}; }
SGI_D V3 operator+(V3 a, float s) { return V3{a.x + s, a.y + s, a.z + s}; }
SGI_D V3 operator-(V3 a, float s) { return V3{a.x - s, a.y - s, a.z - s}; }
SGI_D V3 operator-(float s, V3 a) { return V3{s - a.x, s - a.y, s - a.z}; }
SGI_D V3 operator/(float s, V3 a) { return V3{s / a.x, s / a.y, s / a.z}; }
SGI_D float dot(V3 a, V3 b) { return __fmaf_rn(a.z, b.z, __fmaf_rn(a.y, b.y, a.x * b.x)); }
SGI_D float length(V3 a) { return sqrtf(dot(a, a)); }
#if SGI_FAST_MATH
SGI_D V3 normalize(V3 a) { const float r = rsqrtf(dot(a, a)); return a * r; }
#else
SGI_D V3 normalize(V3 a) { const float r = 1.0f / sqrtf(dot(a, a)); return a * r; }
#endif
SGI_D V3 vmin(V3 a, float s) { return V3{gmin(a.x, s), gmin(a.y, s), gmin(a.z, s)}; }
SGI_D V3 vmix(V3 x, V3 y, float a) {
    const float b = 1.0f - a;
    return V3{__fmaf_rn(y.x, a, x.x * b), __fmaf_rn(y.y, a, x.y * b), __fmaf_rn(y.z, a, x.z * b)};
}
// the decision-side vector operations (correctly rounded in every build)
SGI_D V3 xadd3(V3 a, V3 b) { return V3{xadd(a.x, b.x), xadd(a.y, b.y), xadd(a.z, b.z)}; }
SGI_D V3 xsub3(V3 a, V3 b) { return V3{xsub(a.x, b.x), xsub(a.y, b.y), xsub(a.z, b.z)}; }
SGI_D V3 xmul3(V3 a, float s) { return V3{xmul(a.x, s), xmul(a.y, s), xmul(a.z, s)}; }
SGI_D V3 xdiv3(V3 a, float s) { const float r = xdiv(1.0f, s); return xmul3(a, r); }
SGI_D float xdot(V3 a, V3 b) { return __fmaf_rn(a.z, b.z, __fmaf_rn(a.y, b.y, xmul(a.x, b.x))); }
SGI_D float xlength(V3 a) { return xsqrt(xdot(a, a)); }
SGI_D V3 xnormalize(V3 a) { const float r = xdiv(1.0f, xsqrt(xdot(a, a))); return xmul3(a, r); }

struct V4 { float x, y, z, w; };
// column-major mat4 times (x, y, z, w), column-wise accumulation
// (exact in every build: positions feed the culls' and the shadow tests' decisions)
SGI_D V4 mat4_mul(const float* m, float x, float y, float z, float w) {
    V4 r;
    r.x = __fmaf_rn(m[12], w, __fmaf_rn(m[8], z, __fmaf_rn(m[4], y, xmul(m[0], x))));
    r.y = __fmaf_rn(m[13], w, __fmaf_rn(m[9], z, __fmaf_rn(m[5], y, xmul(m[1], x))));
    r.z = __fmaf_rn(m[14], w, __fmaf_rn(m[10], z, __fmaf_rn(m[6], y, xmul(m[2], x))));
    r.w = __fmaf_rn(m[15], w, __fmaf_rn(m[11], z, __fmaf_rn(m[7], y, xmul(m[3], x))));
    return r;
}
SGI_D float dot4(const float* pl, V3 p) {
    return __fmaf_rn(pl[3], 1.0f, __fmaf_rn(pl[2], p.z, __fmaf_rn(pl[1], p.y, xmul(pl[0], p.x))));
}

// worldPositionFromDepth, common.glsl:143-155 (exact in every build)
SGI_D V3 world_from_depth(float u, float v, float depth, const float* inv_pv) {
    float z = xsub(xmul(depth, 2.0f), 1.0f);
    V4 w = mat4_mul(inv_pv, xsub(xmul(u, 2.0f), 1.0f), xsub(xmul(v, 2.0f), 1.0f), z, 1.0f);
    return xdiv3(V3{w.x, w.y, w.z}, w.w);
}

// Edge-stopping weight of one a-trous tap q for the centre (cn, cd)
// (filterInput, vpl_pbr_gi_denoise.fs:142-190, sigmaZ = 1):
// pow(max(0, cn . nq), 128) * exp(-|cd - zq|).
SGI_D float atrous_weight(V3 cn, float cd, float4 gq) {
    const float wz = expf_ieee_near0(-gabs(cd - gq.w));
    const float wn = pow128(gmax(0.0f, dot(cn, v3(gq.x, gq.y, gq.z))));
    return wn * wz;
}
// The weights of two taps at once, each lane equal to atrous_weight. The
// depth term uses zq - cd (ncd = -cd): |zq - cd| and |cd - zq| are the same
// value. The final product is taken per lane (it may be subnormal).
SGI_D float2 atrous_weight2(float2 cx, float2 cy, float2 cz, float ncd, float4 g0, float4 g1) {
    const float2 dz = add2(make_float2(g0.w, g1.w), f2s(ncd));
    const float2 wz = expf_ieee2(make_float2(dz.x < 0.0f ? dz.x : -dz.x, dz.y < 0.0f ? dz.y : -dz.y));
    const float2 dn = fma2(cz, make_float2(g0.z, g1.z), fma2(cy, make_float2(g0.y, g1.y), mul2(cx, make_float2(g0.x, g1.x))));
    const float2 wn = pow128x2(make_float2(gmax(0.0f, dn.x), gmax(0.0f, dn.y)));
    return make_float2(wn.x * wz.x, wn.y * wz.y);
}

// hash / floatConstruct / random(vec3), common.glsl:183-214
SGI_D uint32_t ghash(uint32_t x) {
    x += (x << 10u); x ^= (x >> 6u); x += (x << 3u); x ^= (x >> 11u); x += (x << 15u);
    return x;
}
SGI_D float random3(float sx, float sy, float sz) {
    uint32_t h = ghash(__float_as_uint(sx) ^ ghash(__float_as_uint(sy)) ^ ghash(__float_as_uint(sz)));
    return __uint_as_float((h & 0x007FFFFFu) | 0x3F800000u) - 1.0f;
}

// b / 255 for a UNORM8 byte b: the product with the rounded reciprocal plus one
// fused correction step returns the correctly rounded quotient for every one
// of the 256 bytes (checked exhaustively in exact rational arithmetic), so it
// equals the IEEE division without the division's instruction sequence.
SGI_D float unorm8(uint32_t t, int ch) {
    const float b = float((t >> (8 * ch)) & 0xffu);
    const float r = 1.0f / 255.0f;
    const float q = xmul(b, r);
    return __fmaf_rn(__fmaf_rn(-q, 255.0f, b), r, q);
}
// b / 65535 for a UNORM16 value b (a unorm16 depth cube texel): the same
// reciprocal step returns the correctly rounded quotient for every one of the
// 65536 values (checked exhaustively in exact rational arithmetic).
SGI_D float unorm16(uint32_t b) {
    const float x = float(b & 0xffffu);
    const float r = 1.0f / 65535.0f;
    const float q = xmul(x, r);
    return __fmaf_rn(__fmaf_rn(-q, 65535.0f, x), r, q);
}
SGI_D V3 decode_normal(uint32_t t) {   // normalize(rgb * 2 - 1), common.glsl:216-220 (exact in every build)
    V3 c = v3(unorm8(t, 0), unorm8(t, 1), unorm8(t, 2));
    return xnormalize(V3{xsub(xmul(c.x, 2.0f), 1.0f), xsub(xmul(c.y, 2.0f), 1.0f), xsub(xmul(c.z, 2.0f), 1.0f)});
}
SGI_D float h2f(uint16_t h) { return __half2float(__ushort_as_half(h)); }
SGI_D uint16_t f2h(float f) { return __half_as_ushort(__float2half_rn(f)); }

// clamped texel index of a floor'ed coordinate (NaN -> 0)
SGI_D int tex_index(float f, int n) {
    if (f >= float(n - 1)) return n - 1;
    if (f >= 0.0f) return (int)f;
    return 0;
}
// tex_index as a clamp of the coordinate (n - 1 at or above n - 1, (int) f in
// between, 0 below 0; fmaxf returns 0 for a NaN f): the same index, the form
// the CSM filter's twelve indices per cascade run faster with
SGI_D int tex_index_clamped(float f, int n) { return (int)fminf(fmaxf(f, 0.0f), float(n - 1)); }
SGI_D int nearest_index(float s, int n) { return tex_index(floorf(xmul(s, float(n))), n); }

// ------------------------------------------------------- shading library --
struct ShadeParams {
    float min_roughness;
    int perceptual;
    float fog_density;
    float fog_color[3];
    float point_ambient;
};

// applyFog, fog.glsl:38-42
SGI_D V3 apply_fog(V3 color, float dist, float intensity, const ShadeParams& sp) {
    float f = expf_ieee(-sp.fog_density * dist);
    V3 fc = v3(sp.fog_color[0], sp.fog_color[1], sp.fog_color[2]) * intensity;
    return color * f + fc * (1.0f - f);
}
// NDF_GGX, pbr2.glsl:51-55
SGI_D float ndf_ggx(float NdotH, float r) {
    float r2 = r * r;
    float f = (NdotH * r2 - NdotH) * NdotH + 1.0f;
    return r2 / gmax(kPi * f * f, kEps);
}
// Visibility_G_SmithGGX, pbr2.glsl:59-64
SGI_D float vis_smith_ggx(float NdotV, float NdotL, float r) {
    float a2 = r * r;
    float ggxv = NdotL * sqrtf((NdotV - a2 * NdotV) * NdotV + a2);
    float ggxl = NdotV * sqrtf((NdotL - a2 * NdotL) * NdotL + a2);
    return 0.5f / gmax(ggxv + ggxl, kEps);
}
// Fr_Fresnel_Schlick, pbr2.glsl:73-76
SGI_D V3 fr_fresnel(float u, V3 f0) { float f = pow5(1.0f - u); return v3s(f) + f0 * (1.0f - f); }
// Fd_Fresnel_Schlick, pbr2.glsl:85-88
SGI_D float fd_fresnel(float u, float f0, float f90) { float f = pow5(1.0f - u); return f0 + (f90 - f0) * f; }
// Fd_Burley, pbr2.glsl:91-96
SGI_D float fd_burley(float NdotV, float NdotL, float LdotH, float r) {
    float f90 = 0.5f + 2.0f * r * LdotH * LdotH;
    float ls = fd_fresnel(NdotL, 1.0f, f90);
    float vs = fd_fresnel(NdotV, 1.0f, f90);
    return ls * vs * (1.0f / kPi);
}
// singleScatteringBRDF_Specular, pbr2.glsl:102-115
SGI_D V3 spec_brdf(float NdotV, float NdotL, float NdotH, float LdotH, float r, V3 f0) {
    float ndf = ndf_ggx(NdotH, r);
    V3 fres = fr_fresnel(LdotH, f0);
    float vis = vis_smith_ggx(NdotV, NdotL, r);
    return (ndf * vis) * fres;
}
// The view-side factors of spec_brdf, which depend only on the pixel: N.V,
// a^2 and the square root of Visibility_G_SmithGGX's view term. spec_brdf_v
// then evaluates the remaining operations of spec_brdf in their order, so a
// pixel's lights or samples share the factors with the same results.
struct SpecView {
    float NdotV, a2, sqrtV;
};
SGI_D SpecView spec_view(V3 N, V3 V, float r) {
    SpecView s;
    s.NdotV = saturate(dot(N, V));
    s.a2 = r * r;
    s.sqrtV = sqrtf((s.NdotV - s.a2 * s.NdotV) * s.NdotV + s.a2);
    return s;
}
SGI_D V3 spec_brdf_v(const SpecView& sv, float NdotL, float NdotH, float LdotH, V3 f0) {
    float f = (NdotH * sv.a2 - NdotH) * NdotH + 1.0f;
    float ndf = sv.a2 / gmax(kPi * f * f, kEps);
    V3 fres = fr_fresnel(LdotH, f0);
    float ggxv = NdotL * sv.sqrtV;
    float ggxl = sv.NdotV * sqrtf((NdotL - sv.a2 * NdotL) * NdotL + sv.a2);
    float vis = 0.5f / gmax(ggxv + ggxl, kEps);
    return (ndf * vis) * fres;
}
// RemapRoughness, pbr2.glsl:139-144
SGI_D float remap_roughness(float r, const ShadeParams& sp) {
    if (sp.perceptual) r = r * r;
    return gmax(gmax(0.0f, sp.min_roughness), r);
}
// BRDF_Base, pbr2.glsl:146-168
SGI_D void brdf_base(V3 baseColor, V3 baseRefl, float roughness, float metallic, V3 diffDivisor, V3 specMult,
                     const ShadeParams& sp, float& remapped, V3& diffuseColor, V3& f0) {
    remapped = remap_roughness(roughness, sp);
    diffuseColor = (1.0f - metallic) * baseColor;
    diffuseColor = diffuseColor / (diffDivisor + kEps);
    f0 = 0.16f * baseRefl * baseRefl * (1.0f - metallic) + baseColor * metallic;
    f0 = f0 * specMult;
}
// BRDF_DotProducts, pbr2.glsl:170-188
SGI_D void brdf_dots(V3 V, V3 lightDir, V3 N, float& NdotV, float& NdotL, float& NdotH, float& LdotH) {
    V3 L = normalize(lightDir);
    V3 H = normalize(V + L);
    NdotV = saturate(dot(N, V));
    NdotL = saturate(dot(N, L));
    NdotH = saturate(dot(N, H));
    LdotH = saturate(dot(L, H));
}
// BRDF_Burley, pbr2.glsl:194-250
SGI_D V3 brdf_burley(V3 lightDir, V3 V, V3 N, V3 baseColor, V3 baseRefl, float roughness, float metallic,
                     V3 diffDivisor, V3 specMult, const ShadeParams& sp) {
    float rr; V3 dc, f0;
    brdf_base(baseColor, baseRefl, roughness, metallic, diffDivisor, specMult, sp, rr, dc, f0);
    float NdotV, NdotL, NdotH, LdotH;
    brdf_dots(V, lightDir, N, NdotV, NdotL, NdotH, LdotH);
    V3 Fr = spec_brdf(NdotV, NdotL, NdotH, LdotH, rr, f0);
    V3 Fd = dc * fd_burley(NdotV, NdotL, LdotH, rr);
    return (Fd + Fr) * NdotL;
}
// calculateLighting_Burley, pbr2.glsl:454-478
SGI_D V3 lighting_burley(V3 lightColor, V3 lightDir, V3 V, V3 N, V3 baseColor, float viewDist, float fogIntensity,
                         float roughness, float metallic, float ao, float shadowFactor, V3 baseRefl, float atten,
                         float ambientIntensity, const ShadeParams& sp) {
    V3 brdf = brdf_burley(lightDir, V, N, baseColor, baseRefl, roughness, metallic, v3s(1.0f), v3s(1.0f), sp);
    V3 ambient = brdf * ao * lightColor * ambientIntensity;
    V3 finalB = brdf * lightColor;
    return atten * (ambient + shadowFactor * apply_fog(finalB, viewDist, fogIntensity, sp));
}
// lighting_burley split like vpl_pixel / vpl_lighting2_sample: the part that
// depends only on the pixel (BRDF_Base with unit divisors, the fog factor of
// the view distance and the view-side specular factors) once per pixel, the
// rest per light; the operations and their order per light are those of
// lighting_burley. N and V are the pixel's normal and view direction.
struct BurleyPixel {
    V3 dc, f0;
    float rr, fogF;
    SpecView sv;
};
SGI_D BurleyPixel burley_pixel(V3 baseColor, V3 baseRefl, float roughness, float metallic, float viewDist, V3 N,
                               V3 V, const ShadeParams& sp) {
    BurleyPixel b;
    brdf_base(baseColor, baseRefl, roughness, metallic, v3s(1.0f), v3s(1.0f), sp, b.rr, b.dc, b.f0);
    b.fogF = expf_ieee(-sp.fog_density * viewDist);
    b.sv = spec_view(N, V, b.rr);
    return b;
}
SGI_D V3 lighting_burley_px(const BurleyPixel& b, V3 lightColor, V3 lightDir, V3 V, V3 N, float fogIntensity,
                            float ao, float shadowFactor, float atten, float ambientIntensity, const ShadeParams& sp) {
    float NdotV, NdotL, NdotH, LdotH;
    brdf_dots(V, lightDir, N, NdotV, NdotL, NdotH, LdotH);   // NdotV is b.sv.NdotV
    V3 Fr = spec_brdf_v(b.sv, NdotL, NdotH, LdotH, b.f0);
    V3 Fd = b.dc * fd_burley(NdotV, NdotL, LdotH, b.rr);
    V3 brdf = (Fd + Fr) * NdotL;
    V3 ambient = brdf * ao * lightColor * ambientIntensity;
    V3 finalB = brdf * lightColor;
    V3 fc = v3(sp.fog_color[0], sp.fog_color[1], sp.fog_color[2]) * fogIntensity;
    return atten * (ambient + shadowFactor * (finalB * b.fogF + fc * (1.0f - b.fogF)));
}
// lighting_burley_px for a light direction whose length len is already known
// (the light's distance, computed for the range test): normalize(lightDir) is
// lightDir * (1 / len), and in the exact build len is the square root that
// normalize would take, so the result is the same.
SGI_D V3 lighting_burley_pxl(const BurleyPixel& b, V3 lightColor, V3 lightDir, float len, V3 V, V3 N,
                             float fogIntensity, float ao, float shadowFactor, float atten, float ambientIntensity,
                             const ShadeParams& sp) {
    const V3 L = lightDir * (1.0f / len);
    const V3 H = normalize(V + L);
    const float NdotV = b.sv.NdotV, NdotL = saturate(dot(N, L));
    const float NdotH = saturate(dot(N, H)), LdotH = saturate(dot(L, H));
    V3 Fr = spec_brdf_v(b.sv, NdotL, NdotH, LdotH, b.f0);
    V3 Fd = b.dc * fd_burley(NdotV, NdotL, LdotH, b.rr);
    V3 brdf = (Fd + Fr) * NdotL;
    V3 ambient = brdf * ao * lightColor * ambientIntensity;
    V3 finalB = brdf * lightColor;
    V3 fc = v3(sp.fog_color[0], sp.fog_color[1], sp.fog_color[2]) * fogIntensity;
    return atten * (ambient + shadowFactor * (finalB * b.fogF + fc * (1.0f - b.fogF)));
}
// quadraticAttenuation, pbr.glsl:255-258, with |lightDir| given
SGI_D float quadratic_atten_len(float d) { return 1.0f / (1.0f + d * d); }
// quadraticAttenuation, pbr.glsl:255-258
SGI_D float quadratic_atten(V3 lightDir) { float d = length(lightDir); return 1.0f / (1.0f + d * d); }
// vplDiffuseAttenuation / vplSpecularAttenuation, pbr.glsl:260-271, with d = |lightDir|
SGI_D float vpl_atten_len(float d, float radius) {
    float ratio = gmin(d / radius, 1.0f);
#if SGI_FAST_MATH
    float minDist = mixf(10.0f, 1.0f, expf_ieee(-3.0f * ratio)) * radius;
#else
    float minDist = mixf(10.0f, 1.0f, expf_exact_mid(-3.0f * ratio)) * radius;   // -3 <= x <= 0 or NaN
#endif
    return 1.0f / (minDist + 1.0f * d * d);
}
SGI_D float vpl_atten(V3 lightDir, float radius) {
    float d = length(lightDir);
    float ratio = gmin(d / radius, 1.0f);
    float minDist = mixf(10.0f, 1.0f, expf_ieee(-3.0f * ratio)) * radius;
    return 1.0f / (minDist + 1.0f * d * d);
}
// The per-pixel part of vpl_lighting2: everything that does not depend on the
// VPL (BRDF_Base's remapped roughness, diffuse colour and F0, and the fog
// factor of the view distance), computed once per pixel instead of once per
// sample; vpl_lighting2_sample then evaluates exactly the remaining operations.
struct VplPixel {
    V3 fragPos, N, V, dc, f0, fogAdd;
    float rr, fogF, ao;
    SpecView sv;
};
SGI_D VplPixel vpl_pixel(V3 fragPos, V3 baseColor, V3 N, V3 V, float viewDist, float roughness, float metallic,
                         float ao, V3 baseRefl, const ShadeParams& sp) {
    VplPixel q;
    q.fragPos = fragPos; q.N = N; q.V = V; q.ao = ao;
    const V3 specMult = 1.0f / (baseColor + kEps);
    brdf_base(baseColor, baseRefl, roughness, metallic, baseColor, specMult, sp, q.rr, q.dc, q.f0);
    q.sv = spec_view(N, V, q.rr);
    // applyFog(color, viewDist, 0) = color * f + fc * (1 - f), fc = fogColor * 0
    q.fogF = expf_ieee(-sp.fog_density * viewDist);
    const V3 fc = v3(sp.fog_color[0], sp.fog_color[1], sp.fog_color[2]) * 0.0f;
    q.fogAdd = fc * (1.0f - q.fogF);
    return q;
}
// diffLen: |diffPos - fragPos| when the caller has it (the gather's distance to
// the VPL, the same square root in the exact build), else negative
SGI_D V3 vpl_lighting2_sample(const VplPixel& q, V3 specPos, V3 diffPos, V3 lightColor, float radius,
                              float diffLen = -1.0f) {
    V3 specDir = specPos - q.fragPos;
    V3 diffDir = diffPos - q.fragPos;
    const float specLen = length(specDir);
    if (!(diffLen >= 0.0f)) diffLen = length(diffDir);
    float specAtten = vpl_atten_len(specLen, radius);
    float diffAtten = vpl_atten_len(diffLen, radius);
    float NdotL, NdotH, LdotH;
    {   // brdf_dots(q.V, specDir, ...) with normalize(specDir) = specDir * (1 / |specDir|)
        const V3 L = specDir * (1.0f / specLen);
        const V3 H = normalize(q.V + L);
        NdotL = saturate(dot(q.N, L));
        NdotH = saturate(dot(q.N, H));
        LdotH = saturate(dot(L, H));
    }
    V3 Fr = spec_brdf_v(q.sv, NdotL, NdotH, LdotH, q.f0) * NdotL;
    NdotL = saturate(dot(q.N, diffDir * (1.0f / diffLen)));   // brdf_dots(q.V, diffDir, ...): only N.L is used
    V3 Fd = (q.dc * (1.0f / kPi)) * NdotL;
    V3 bs = specAtten * Fr;
    V3 bd = diffAtten * Fd;
    V3 brdf = bs + bd;
    V3 ambient = brdf * q.ao * lightColor * 0.0f;
    V3 finalB = brdf * lightColor;
    // the shader scales the fogged term by 1.0 - 0.0, which is exactly 1
    return ambient + (finalB * q.fogF + q.fogAdd);
}
// calculateVirtualPointLighting2 (shadowFactor argument 0, fog intensity 0,
// ambient intensity 0) -> calculateLighting_Lambert_SeparateDiffuseSpecular ->
// BRDF_Lambert_SeparateDiffuseSpecular; pbr2.glsl:613-657, :541-574, :382-452:
// the two parts above in sequence.
SGI_D V3 vpl_lighting2(V3 fragPos, V3 baseColor, V3 N, V3 V, V3 specPos, V3 diffPos, V3 lightColor, float viewDist,
                       float radius, float roughness, float metallic, float ao, V3 baseRefl, const ShadeParams& sp) {
    return vpl_lighting2_sample(vpl_pixel(fragPos, baseColor, N, V, viewDist, roughness, metallic, ao, baseRefl, sp),
                                specPos, diffPos, lightColor, radius);
}

}  // namespace sgi
