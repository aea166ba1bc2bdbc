// oracle/glsl.hpp - TEST INFRASTRUCTURE ONLY (the CPU oracle).
//
// A C++ restatement of the GLSL built-ins and shading library that the
// StratusGFX GI/lighting shaders use, templated on the scalar type:
//   T = float  : the parity oracle. Every operation is one correctly rounded
//                IEEE-754 binary32 +, -, *, /, sqrt or explicit fused
//                multiply-add, in a fixed order (the file is compiled with
//                -ffp-contract=off, so the compiler adds no fusion of its
//                own), so a CUDA kernel that evaluates the same expression
//                trees produces bit-identical results.
//   T = double : the accuracy oracle (std::exp / std::pow, no FP16 storage).
//
// Parity is UNPINNED by the reference: StratusGFX has no golden vectors or
// shader tests, and its GLSL runs only inside an OpenGL 4.6 driver, which
// does not exist on these machines. This file is pinned only by the shader
// source lines it cites (paths relative to the StratusGFX project root).
//
// Built-ins whose GLSL precision is implementation-defined get one fixed
// definition here (the CUDA kernels use the same one). GLSL allows a
// multiply-add to be fused and vector divisions to be evaluated through a
// reciprocal, so the definitions below fuse explicitly (fma = one rounding)
// in the places a GPU compiler would, and nowhere else:
//   min(x,y) = y < x ? y : x ; max(x,y) = x < y ? y : x   (GLSL spec wording)
//   dot(a,b) = fma(az, bz, fma(ay, by, ax*bx))
//   mat4*vec4: per row fma(m3, w, fma(m2, z, fma(m1, y, m0*x)))
//   vec / s  = vec * (1/s)  (one correctly rounded reciprocal)
//   normalize(v) = v * (1/sqrt(dot(v,v)))
//   mix(x,y,a) = fma(y, a, x*(1-a))
//   exp(x)   : Cody-Waite range reduction (ln2 split hi/lo) + degree-7 Taylor
//              polynomial in fused Horner form + exact power-of-two scaling.
//   pow(x,5) = (x*x)*(x*x)*x ; pow(x,128) = seven squarings (integer exponents
//              are the only ones the path uses).
// Scalar a / b stays a correctly rounded division.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>

namespace oracle {

// ---------------------------------------------------------------- scalars --
template <class T> inline T gfma(T a, T b, T c) { return std::fma(a, b, c); }
template <class T> inline T gmin(T x, T y) { return y < x ? y : x; }
template <class T> inline T gmax(T x, T y) { return x < y ? y : x; }
template <class T> inline T gclamp(T x, T lo, T hi) { return gmin(gmax(x, lo), hi); }
template <class T> inline T saturate(T x) { return gclamp(x, T(0), T(1)); }   // common.glsl:99-101
template <class T> inline T mix(T x, T y, T a) { return gfma(y, a, x * (T(1) - a)); }
template <class T> inline T gabs(T x) { return x < T(0) ? -x : x; }
template <class T> inline T gfloor(T x) { return std::floor(x); }

// exp for binary32 (see header comment). Returns exactly 1 for +-0.
inline float exp_f32(float x) {
    if (x != x) return x;
    if (x > 88.72283935546875f) return INFINITY;
    if (x < -103.97283935546875f) return 0.0f;
    float kf = std::floor(x * 1.44269502162933349609375f + 0.5f);
    int k = (int)kf;
    float r = (x - kf * 0.693145751953125f) - kf * 1.428606765330187045037746429443359375e-06f;
    float p = std::fma(r, 1.0f / 5040.0f, 1.0f / 720.0f);
    p = std::fma(p, r, 1.0f / 120.0f);
    p = std::fma(p, r, 1.0f / 24.0f);
    p = std::fma(p, r, 1.0f / 6.0f);
    p = std::fma(p, r, 0.5f);
    p = std::fma(p, r, 1.0f);
    p = std::fma(p, r, 1.0f);
    if (k > 127) { p = p * 1.7014118346046923e+38f; k -= 127; }      // 2^127
    if (k < -126) { p = p * 1.1754943508222875e-38f; k += 126; }      // 2^-126
    uint32_t bits = (uint32_t)(k + 127) << 23;
    float s; std::memcpy(&s, &bits, 4);
    return p * s;
}

inline float pow5_f32(float x) { float x2 = x * x; float x4 = x2 * x2; return x4 * x; }
inline float pow128_f32(float x) {
    float y = x * x; y = y * y; y = y * y; y = y * y; y = y * y; y = y * y; y = y * y; return y;
}

// float -> IEEE binary16 bits, round to nearest even (the rounding of an
// RGBA16F render target in this build).
inline uint16_t f32_to_f16(float f) {
    uint32_t x; std::memcpy(&x, &f, 4);
    uint32_t sign = (x >> 16) & 0x8000u;
    uint32_t ax = x & 0x7fffffffu;
    if (ax >= 0x7f800000u) return (uint16_t)(sign | 0x7c00u | (ax > 0x7f800000u ? 0x200u : 0u));
    if (ax >= 0x477ff000u) return (uint16_t)(sign | 0x7c00u);
    if (ax >= 0x38800000u) {
        uint32_t mant = ax & 0x7fffffu;
        uint32_t e = (ax >> 23) - 127u + 15u;
        uint32_t h = (e << 10) | (mant >> 13);
        uint32_t rem = mant & 0x1fffu;
        if (rem > 0x1000u || (rem == 0x1000u && (h & 1u))) h++;
        return (uint16_t)(sign | h);
    }
    if (ax < 0x33000000u) return (uint16_t)sign;
    uint32_t full = (ax & 0x7fffffu) | 0x800000u;
    int e = (int)(ax >> 23) - 127;          // -25 .. -15
    int shift = -(e + 1);                   // 14 .. 24
    uint32_t q = full >> shift;
    uint32_t rem = full & ((1u << shift) - 1u);
    uint32_t halfway = 1u << (shift - 1);
    if (rem > halfway || (rem == halfway && (q & 1u))) q++;
    return (uint16_t)(sign | q);
}

inline float f16_to_f32(uint16_t h) {
    uint32_t sign = (uint32_t)(h & 0x8000u) << 16;
    uint32_t e = (h >> 10) & 0x1fu;
    uint32_t m = h & 0x3ffu;
    uint32_t bits;
    if (e == 0) {
        if (m == 0) { bits = sign; }
        else {  // subnormal: value = m * 2^-24, exact in binary32
            float v = (float)m * 5.9604644775390625e-08f;
            std::memcpy(&bits, &v, 4);
            bits |= sign;
        }
    } else if (e == 31) {
        bits = sign | 0x7f800000u | (m << 13);
    } else {
        bits = sign | ((e - 15u + 127u) << 23) | (m << 13);
    }
    float f; std::memcpy(&f, &bits, 4);
    return f;
}

// Precision policy: the transcendental built-ins and the FP16 storage rounding.
template <class T> struct Prec;
template <> struct Prec<float> {
    static float exp(float x) { return exp_f32(x); }
    static float pow5(float x) { return pow5_f32(x); }
    static float pow128(float x) { return pow128_f32(x); }
    static float sqrt(float x) { return std::sqrt(x); }
    // value after a store into a 16-bit float texture
    static float store16(float x) { return f16_to_f32(f32_to_f16(x)); }
};
template <> struct Prec<double> {
    static double exp(double x) { return std::exp(x); }
    static double pow5(double x) { return std::pow(x, 5.0); }
    static double pow128(double x) { return std::pow(x, 128.0); }
    static double sqrt(double x) { return std::sqrt(x); }
    static double store16(double x) { return x; }
};

// ---------------------------------------------------------------- vectors --
template <class T> struct V3 {
    T x, y, z;
    V3() : x(0), y(0), z(0) {}
    V3(T a, T b, T c) : x(a), y(b), z(c) {}
    explicit V3(T a) : x(a), y(a), z(a) {}
};
template <class T> inline V3<T> operator+(V3<T> a, V3<T> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class T> inline V3<T> operator-(V3<T> a, V3<T> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class T> inline V3<T> operator*(V3<T> a, V3<T> b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
template <class T> inline V3<T> operator/(V3<T> a, V3<T> b) { return {a.x / b.x, a.y / b.y, a.z / b.z}; }
template <class T> inline V3<T> operator*(V3<T> a, T s) { return {a.x * s, a.y * s, a.z * s}; }
template <class T> inline V3<T> operator*(T s, V3<T> a) { return {s * a.x, s * a.y, s * a.z}; }
template <class T> inline V3<T> operator/(V3<T> a, T s) { T r = T(1) / s; return {a.x * r, a.y * r, a.z * r}; }
template <class T> inline V3<T> operator+(V3<T> a, T s) { return {a.x + s, a.y + s, a.z + s}; }
template <class T> inline V3<T> operator-(V3<T> a, T s) { return {a.x - s, a.y - s, a.z - s}; }
template <class T> inline V3<T> operator-(T s, V3<T> a) { return {s - a.x, s - a.y, s - a.z}; }
template <class T> inline V3<T> operator/(T s, V3<T> a) { return {s / a.x, s / a.y, s / a.z}; }
template <class T> inline T dot(V3<T> a, V3<T> b) { return gfma(a.z, b.z, gfma(a.y, b.y, a.x * b.x)); }
template <class T> inline T length(V3<T> a) { return Prec<T>::sqrt(dot(a, a)); }
template <class T> inline V3<T> normalize(V3<T> a) { T r = T(1) / Prec<T>::sqrt(dot(a, a)); return a * r; }
template <class T> inline V3<T> vmin(V3<T> a, T s) { return {gmin(a.x, s), gmin(a.y, s), gmin(a.z, s)}; }
template <class T> inline V3<T> vmix(V3<T> x, V3<T> y, T a) {
    T b = T(1) - a;
    return {gfma(y.x, a, x.x * b), gfma(y.y, a, x.y * b), gfma(y.z, a, x.z * b)};
}

// column-major mat4 (glm layout) times (x,y,z,w): column-wise accumulation
template <class T> struct V4 { T x, y, z, w; };
template <class T> inline V4<T> mat4_mul(const float* m, T x, T y, T z, T w) {
    V4<T> r;
    r.x = gfma(T(m[12]), w, gfma(T(m[8]), z, gfma(T(m[4]), y, T(m[0]) * x)));
    r.y = gfma(T(m[13]), w, gfma(T(m[9]), z, gfma(T(m[5]), y, T(m[1]) * x)));
    r.z = gfma(T(m[14]), w, gfma(T(m[10]), z, gfma(T(m[6]), y, T(m[2]) * x)));
    r.w = gfma(T(m[15]), w, gfma(T(m[11]), z, gfma(T(m[7]), y, T(m[3]) * x)));
    return r;
}
template <class T> inline T dot4(const float* plane, V3<T> p) {   // dot(plane, vec4(p, 1.0))
    return gfma(T(plane[3]), T(1), gfma(T(plane[2]), p.z, gfma(T(plane[1]), p.y, T(plane[0]) * p.x)));
}

// ---------------------------------------------------------- common.glsl --
template <class T> struct C {
    static constexpr double PI_D = 3.14159265359;           // common.glsl:3
    static T PI() { return T(PI_D); }
    static T EPS() { return T(0.00001); }                    // PREVENT_DIV_BY_ZERO, common.glsl:4
    static T HALF_MAX() { return T(65504.0); }               // HALF_FLOAT_MAX, common.glsl:6
};

// worldPositionFromDepth, common.glsl:143-155
template <class T> inline V3<T> world_from_depth(T u, T v, T depth, const float* inv_pv) {
    T z = depth * T(2) - T(1);
    V4<T> w = mat4_mul<T>(inv_pv, u * T(2) - T(1), v * T(2) - T(1), z, T(1));
    return V3<T>(w.x, w.y, w.z) / w.w;
}

// hash / floatConstruct / random, common.glsl:183-214 (always integer/binary32)
inline uint32_t ghash(uint32_t x) {
    x += (x << 10u); x ^= (x >> 6u); x += (x << 3u); x ^= (x >> 11u); x += (x << 15u);
    return x;
}
inline uint32_t fbits(float f) { uint32_t u; std::memcpy(&u, &f, 4); return u; }
inline float random3(float sx, float sy, float sz) {
    uint32_t h = ghash(fbits(sx) ^ ghash(fbits(sy)) ^ ghash(fbits(sz)));
    uint32_t m = (h & 0x007FFFFFu) | 0x3F800000u;
    float f; std::memcpy(&f, &m, 4);
    return f - 1.0f;
}

// unorm8 channel -> float (c / 255)
template <class T> inline T unorm8(uint32_t texel, int ch) { return T((texel >> (8 * ch)) & 0xffu) / T(255); }

// normalize(rgb * 2 - 1) of an RGB8 normal texel, common.glsl:216-220
template <class T> inline V3<T> decode_normal(uint32_t texel) {
    V3<T> c(unorm8<T>(texel, 0), unorm8<T>(texel, 1), unorm8<T>(texel, 2));
    return normalize(c * T(2) - V3<T>(T(1)));
}

// ---------------------------------------------------------------- fog.glsl --
struct FogParams { float density; float color[3]; };
// applyFog, fog.glsl:38-42
template <class T> inline V3<T> apply_fog(V3<T> color, T dist, T intensity, const FogParams& fog) {
    T f = Prec<T>::exp(-T(fog.density) * dist);
    V3<T> fc = V3<T>(T(fog.color[0]), T(fog.color[1]), T(fog.color[2])) * intensity;
    return color * f + fc * (T(1) - f);
}

// ---------------------------------------------------------------- pbr2.glsl --
struct BrdfParams { float min_roughness; int perceptual; };

// NDF_GGX, pbr2.glsl:51-55
template <class T> inline T ndf_ggx(T NdotH, T r) {
    T r2 = r * r;
    T f = (NdotH * r2 - NdotH) * NdotH + T(1);
    return r2 / gmax(C<T>::PI() * f * f, C<T>::EPS());
}
// Visibility_G_SmithGGX, pbr2.glsl:59-64
template <class T> inline T vis_smith_ggx(T NdotV, T NdotL, T r) {
    T a2 = r * r;
    T ggxv = NdotL * Prec<T>::sqrt((NdotV - a2 * NdotV) * NdotV + a2);
    T ggxl = NdotV * Prec<T>::sqrt((NdotL - a2 * NdotL) * NdotL + a2);
    return T(0.5) / gmax(ggxv + ggxl, C<T>::EPS());
}
// Fr_Fresnel_Schlick, pbr2.glsl:73-76
template <class T> inline V3<T> fr_fresnel(T u, V3<T> f0) {
    T f = Prec<T>::pow5(T(1) - u);
    return V3<T>(f) + f0 * (T(1) - f);
}
// Fd_Fresnel_Schlick, pbr2.glsl:85-88
template <class T> inline T fd_fresnel(T u, T f0, T f90) {
    T f = Prec<T>::pow5(T(1) - u);
    return f0 + (f90 - f0) * f;
}
// Fd_Burley, pbr2.glsl:91-96
template <class T> inline T fd_burley(T NdotV, T NdotL, T LdotH, T r) {
    T f90 = T(0.5) + T(2) * r * LdotH * LdotH;
    T ls = fd_fresnel(NdotL, T(1), f90);
    T vs = fd_fresnel(NdotV, T(1), f90);
    return ls * vs * (T(1) / C<T>::PI());
}
// singleScatteringBRDF_Specular, pbr2.glsl:102-115
template <class T> inline V3<T> spec_brdf(T NdotV, T NdotL, T NdotH, T LdotH, T r, V3<T> f0) {
    T ndf = ndf_ggx(NdotH, r);
    V3<T> fres = fr_fresnel(LdotH, f0);
    T vis = vis_smith_ggx(NdotV, NdotL, r);
    return (ndf * vis) * fres;
}
// RemapRoughness, pbr2.glsl:139-144
template <class T> inline T remap_roughness(T r, const BrdfParams& bp) {
    if (bp.perceptual) r = r * r;
    return gmax(gmax(T(0), T(bp.min_roughness)), r);
}
// BRDF_Base, pbr2.glsl:146-168
template <class T> inline void brdf_base(V3<T> baseColor, V3<T> baseRefl, T roughness, T metallic,
                                         V3<T> diffDivisor, V3<T> specMult, const BrdfParams& bp,
                                         T& remapped, V3<T>& diffuseColor, V3<T>& f0) {
    remapped = remap_roughness(roughness, bp);
    diffuseColor = (T(1) - metallic) * baseColor;
    diffuseColor = diffuseColor / (diffDivisor + C<T>::EPS());
    f0 = T(0.16) * baseRefl * baseRefl * (T(1) - metallic) + baseColor * metallic;
    f0 = f0 * specMult;
}
// BRDF_DotProducts, pbr2.glsl:170-188
template <class T> inline void brdf_dots(V3<T> V, V3<T> lightDir, V3<T> N, T& NdotV, T& NdotL, T& NdotH, T& LdotH) {
    V3<T> L = normalize(lightDir);
    V3<T> H = normalize(V + L);
    NdotV = saturate(dot(N, V));
    NdotL = saturate(dot(N, L));
    NdotH = saturate(dot(N, H));
    LdotH = saturate(dot(L, H));
}
// BRDF_Burley, pbr2.glsl:194-250
template <class T> inline V3<T> brdf_burley(V3<T> lightDir, V3<T> V, V3<T> N, V3<T> baseColor, V3<T> baseRefl,
                                            T roughness, T metallic, V3<T> diffDivisor, V3<T> specMult,
                                            const BrdfParams& bp) {
    T rr; V3<T> dc, f0;
    brdf_base(baseColor, baseRefl, roughness, metallic, diffDivisor, specMult, bp, rr, dc, f0);
    T NdotV, NdotL, NdotH, LdotH;
    brdf_dots(V, lightDir, N, NdotV, NdotL, NdotH, LdotH);
    V3<T> Fr = spec_brdf(NdotV, NdotL, NdotH, LdotH, rr, f0);
    V3<T> Fd = dc * fd_burley(NdotV, NdotL, LdotH, rr);
    return (Fd + Fr) * NdotL;
}
// BRDF_Lambert_SeparateDiffuseSpecular, pbr2.glsl:382-452
template <class T> inline void brdf_lambert_sep(V3<T> specDir, V3<T> diffDir, V3<T> V, V3<T> N, V3<T> baseColor,
                                                V3<T> baseRefl, T roughness, T metallic, V3<T> diffDivisor,
                                                V3<T> specMult, const BrdfParams& bp, V3<T>& spec, V3<T>& diff) {
    T rr; V3<T> dc, f0;
    brdf_base(baseColor, baseRefl, roughness, metallic, diffDivisor, specMult, bp, rr, dc, f0);
    T NdotV, NdotL, NdotH, LdotH;
    brdf_dots(V, specDir, N, NdotV, NdotL, NdotH, LdotH);
    V3<T> Fr = spec_brdf(NdotV, NdotL, NdotH, LdotH, rr, f0) * NdotL;
    brdf_dots(V, diffDir, N, NdotV, NdotL, NdotH, LdotH);
    V3<T> Fd = (dc * (T(1) / C<T>::PI())) * NdotL;   // Fd_Lambert = 1/PI, pbr2.glsl:98-100
    spec = Fr;
    diff = Fd;
}
// calculateLighting_Burley, pbr2.glsl:454-478
template <class T> inline V3<T> lighting_burley(V3<T> lightColor, V3<T> lightDir, V3<T> V, V3<T> N, V3<T> baseColor,
                                                T viewDist, T fogIntensity, T roughness, T metallic, T ao,
                                                T shadowFactor, V3<T> baseRefl, T atten, T ambientIntensity,
                                                V3<T> diffDivisor, V3<T> specMult, const BrdfParams& bp,
                                                const FogParams& fog) {
    V3<T> brdf = brdf_burley(lightDir, V, N, baseColor, baseRefl, roughness, metallic, diffDivisor, specMult, bp);
    V3<T> ambient = brdf * ao * lightColor * ambientIntensity;
    V3<T> finalB = brdf * lightColor;
    return atten * (ambient + shadowFactor * apply_fog(finalB, viewDist, fogIntensity, fog));
}
// calculateLighting_Lambert_SeparateDiffuseSpecular, pbr2.glsl:541-574
template <class T> inline V3<T> lighting_lambert_sep(V3<T> lightColor, V3<T> specDir, V3<T> diffDir, V3<T> V, V3<T> N,
                                                     V3<T> baseColor, T viewDist, T fogIntensity, T roughness,
                                                     T metallic, T ao, T shadowFactor, V3<T> baseRefl,
                                                     T specAtten, T diffAtten, T ambientIntensity,
                                                     V3<T> diffDivisor, V3<T> specMult, const BrdfParams& bp,
                                                     const FogParams& fog) {
    V3<T> bs, bd;
    brdf_lambert_sep(specDir, diffDir, V, N, baseColor, baseRefl, roughness, metallic, diffDivisor, specMult, bp, bs, bd);
    bs = specAtten * bs;
    bd = diffAtten * bd;
    V3<T> brdf = bs + bd;
    V3<T> ambient = brdf * ao * lightColor * ambientIntensity;
    V3<T> finalB = brdf * lightColor;
    return ambient + shadowFactor * apply_fog(finalB, viewDist, fogIntensity, fog);
}
// quadraticAttenuation, pbr.glsl:255-258
template <class T> inline T quadratic_atten(V3<T> lightDir) {
    T d = length(lightDir);
    return T(1) / (T(1) + d * d);
}
// vplDiffuseAttenuation, pbr.glsl:260-267 (vplSpecularAttenuation :269-271 is the same)
template <class T> inline T vpl_atten(V3<T> lightDir, T radius) {
    T d = length(lightDir);
    T ratio = gmin(d / radius, T(1));
    T minDist = mix(T(10), T(1), Prec<T>::exp(T(-3) * ratio)) * radius;
    return T(1) / (minDist + T(1) * d * d);
}
// calculatePointLighting2, pbr2.glsl:593-611
template <class T> inline V3<T> point_lighting2(V3<T> fragPos, V3<T> baseColor, V3<T> N, V3<T> V, V3<T> lightPos,
                                                V3<T> lightColor, T viewDist, T roughness, T metallic, T ao,
                                                T shadowFactor, V3<T> baseRefl, T pointAmbient,
                                                const BrdfParams& bp, const FogParams& fog) {
    V3<T> lightDir = lightPos - fragPos;
    return lighting_burley(lightColor, lightDir, V, N, baseColor, viewDist, length(lightColor) / T(12), roughness,
                           metallic, ao, T(1) - shadowFactor, baseRefl, quadratic_atten(lightDir), pointAmbient,
                           V3<T>(T(1)), V3<T>(T(1)), bp, fog);
}
// calculateDirectionalLighting, pbr2.glsl:576-591
template <class T> inline V3<T> directional_lighting(V3<T> lightColor, V3<T> lightDir, V3<T> V, V3<T> N,
                                                     V3<T> baseColor, T viewDist, T roughness, T metallic, T ao,
                                                     T shadowFactor, V3<T> baseRefl, T ambientIntensity,
                                                     const BrdfParams& bp, const FogParams& fog) {
    return lighting_burley(lightColor, lightDir, V, N, baseColor, viewDist, T(0), roughness, metallic, ao,
                           T(1) - shadowFactor, baseRefl, T(1), ambientIntensity, V3<T>(T(1)), V3<T>(T(1)), bp, fog);
}
// calculateVirtualPointLighting2, pbr2.glsl:613-657
template <class T> inline V3<T> vpl_lighting2(V3<T> fragPos, V3<T> baseColor, V3<T> N, V3<T> V, V3<T> specPos,
                                              V3<T> diffPos, V3<T> lightColor, T viewDist, T radius, T roughness,
                                              T metallic, T ao, T shadowFactor, V3<T> baseRefl,
                                              const BrdfParams& bp, const FogParams& fog) {
    V3<T> specDir = specPos - fragPos;
    V3<T> diffDir = diffPos - fragPos;
    T adjusted = T(1) - shadowFactor;
    return lighting_lambert_sep(lightColor, specDir, diffDir, V, N, baseColor, viewDist, T(0), roughness, metallic,
                                ao, adjusted, baseRefl, vpl_atten(specDir, radius), vpl_atten(diffDir, radius), T(0),
                                baseColor, T(1) / (baseColor + C<T>::EPS()), bp, fog);
}

}  // namespace oracle
