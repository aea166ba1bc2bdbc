// oracle/counted.hpp - TEST INFRASTRUCTURE ONLY (the CPU oracle).
//
// Two instrumented scalar types for the templated passes: Counted (below) and
// Tracked (further down, the decision margins of the tolerance tests).
//
// Counted: a binary32 scalar that tallies the algorithmic floating-point work
// of the restated passes. The passes are templates on their scalar type; with
// T = Counted they take the same branches and produce the same values as the
// FP32 instantiation, and every operation on the way is counted once per call,
// per thread (OpenMP), into a tally the C entry points read and reset.
//
// What counts (one "FLOP" each unless stated):
//   +, -, *, /, sqrt, floor            1
//   fused multiply-add                 2
//   exp                                1 (one special-function operation)
//   pow(x, 5), pow(x, 128)             the 3 / 7 multiplications of their definition
// Comparisons, min/max/clamp selections and abs count separately as "cmps";
// negation, conversions, FP16 storage rounding and the integer RNG path
// (hash of the seed bits) are not counted. This is the algorithm's work as the
// reference shaders state it, not the instructions a GPU executes for it.
#pragma once

#include <omp.h>

#include <cmath>
#include <cstdint>
#include <type_traits>

#include "glsl.hpp"

namespace oracle {

struct alignas(64) OpTally {
    uint64_t flops = 0, cmps = 0;
};
constexpr int kMaxTallyThreads = 512;
inline OpTally* tallies() {
    static OpTally t[kMaxTallyThreads];
    return t;
}
inline OpTally& tally() { return tallies()[omp_get_thread_num() % kMaxTallyThreads]; }
inline void tally_reset() {
    for (int i = 0; i < kMaxTallyThreads; ++i) tallies()[i] = OpTally{};
}
inline void tally_read(uint64_t* flops, uint64_t* cmps) {
    uint64_t f = 0, c = 0;
    for (int i = 0; i < kMaxTallyThreads; ++i) { f += tallies()[i].flops; c += tallies()[i].cmps; }
    *flops = f;
    *cmps = c;
}
inline void count_flops(uint64_t n) { tally().flops += n; }
inline void count_cmp() { tally().cmps += 1; }

struct Counted {
    float v;
    Counted() = default;
    template <class A, class = std::enable_if_t<std::is_arithmetic<A>::value>>
    Counted(A a) : v((float)a) {}
    explicit operator float() const { return v; }
    explicit operator double() const { return v; }
    explicit operator int() const { return (int)v; }
    Counted& operator+=(Counted o) { count_flops(1); v = v + o.v; return *this; }
    Counted& operator-=(Counted o) { count_flops(1); v = v - o.v; return *this; }
    Counted& operator*=(Counted o) { count_flops(1); v = v * o.v; return *this; }
    Counted& operator/=(Counted o) { count_flops(1); v = v / o.v; return *this; }
};
static_assert(sizeof(Counted) == sizeof(float), "Counted buffers alias float buffers");

inline Counted mk(float f) { Counted c; c.v = f; return c; }
inline Counted operator+(Counted a, Counted b) { count_flops(1); return mk(a.v + b.v); }
inline Counted operator-(Counted a, Counted b) { count_flops(1); return mk(a.v - b.v); }
inline Counted operator*(Counted a, Counted b) { count_flops(1); return mk(a.v * b.v); }
inline Counted operator/(Counted a, Counted b) { count_flops(1); return mk(a.v / b.v); }
inline Counted operator-(Counted a) { return mk(-a.v); }
inline bool operator<(Counted a, Counted b) { count_cmp(); return a.v < b.v; }
inline bool operator>(Counted a, Counted b) { count_cmp(); return a.v > b.v; }
inline bool operator<=(Counted a, Counted b) { count_cmp(); return a.v <= b.v; }
inline bool operator>=(Counted a, Counted b) { count_cmp(); return a.v >= b.v; }
inline bool operator==(Counted a, Counted b) { count_cmp(); return a.v == b.v; }
inline bool operator!=(Counted a, Counted b) { count_cmp(); return a.v != b.v; }

inline Counted gfma(Counted a, Counted b, Counted c) { count_flops(2); return mk(std::fma(a.v, b.v, c.v)); }
inline Counted gfloor(Counted a) { count_flops(1); return mk(std::floor(a.v)); }

template <> struct Prec<Counted> {
    static Counted exp(Counted x) { count_flops(1); return mk(exp_f32(x.v)); }
    static Counted pow5(Counted x) { Counted x2 = x * x; Counted x4 = x2 * x2; return x4 * x; }
    static Counted pow128(Counted x) {
        Counted y = x * x; y = y * y; y = y * y; y = y * y; y = y * y; y = y * y; y = y * y; return y;
    }
    static Counted sqrt(Counted x) { count_flops(1); return mk(std::sqrt(x.v)); }
    static Counted store16(Counted x) { return mk(f16_to_f32(f32_to_f16(x.v))); }
};

// ---------------------------------------------------------------------------
// Tracked: a binary64 scalar that records, per pixel, how close the pass's
// branch decisions come to going the other way, in two kinds:
//   0  comparisons that pick a branch or a discontinuous value (a < b, ...):
//      the relative margin |a - b| / max(|a|, |b|);
//   1  nearest-texel choices: the distance of the texel coordinate to the next
//      texel boundary relative to the coordinate's magnitude.
// The continuous selections min, max, clamp, saturate and abs record nothing.
// A pass evaluated in another arithmetic (the CUDA kernels' tolerance mode) can
// only take another branch at a pixel whose smallest margin of some kind is
// within that arithmetic's error; those pixels form the decision-margin mask of
// the tolerance tests.
namespace margin_detail {
inline double* current() {
    static thread_local double m[2] = {1e300, 1e300};
    return m;
}
inline double*& output() {
    static double* out = nullptr;
    return out;
}
}  // namespace margin_detail

inline void record_margin(int kind, double m) {
    double& c = margin_detail::current()[kind];
    if (m < c) c = m;
}
inline void set_margin_output(double* out) { margin_detail::output() = out; }

struct Tracked {
    double v;
    Tracked() = default;
    template <class A, class = std::enable_if_t<std::is_arithmetic<A>::value>>
    Tracked(A a) : v((double)a) {}
    explicit operator float() const { return (float)v; }
    explicit operator double() const { return v; }
    explicit operator int() const { return (int)v; }
    Tracked& operator+=(Tracked o) { v += o.v; return *this; }
    Tracked& operator-=(Tracked o) { v -= o.v; return *this; }
    Tracked& operator*=(Tracked o) { v *= o.v; return *this; }
    Tracked& operator/=(Tracked o) { v /= o.v; return *this; }
};
inline Tracked mt(double d) { Tracked t; t.v = d; return t; }
inline void record_cmp(double a, double b) {
    const double s = std::fmax(std::fabs(a), std::fabs(b));
    record_margin(0, s > 0.0 ? std::fabs(a - b) / s : 1e300);
}
inline Tracked operator+(Tracked a, Tracked b) { return mt(a.v + b.v); }
inline Tracked operator-(Tracked a, Tracked b) { return mt(a.v - b.v); }
inline Tracked operator*(Tracked a, Tracked b) { return mt(a.v * b.v); }
inline Tracked operator/(Tracked a, Tracked b) { return mt(a.v / b.v); }
inline Tracked operator-(Tracked a) { return mt(-a.v); }
inline bool operator<(Tracked a, Tracked b) { record_cmp(a.v, b.v); return a.v < b.v; }
inline bool operator>(Tracked a, Tracked b) { record_cmp(a.v, b.v); return a.v > b.v; }
inline bool operator<=(Tracked a, Tracked b) { record_cmp(a.v, b.v); return a.v <= b.v; }
inline bool operator>=(Tracked a, Tracked b) { record_cmp(a.v, b.v); return a.v >= b.v; }
inline bool operator==(Tracked a, Tracked b) { return a.v == b.v; }
inline bool operator!=(Tracked a, Tracked b) { return a.v != b.v; }

inline Tracked gfma(Tracked a, Tracked b, Tracked c) { return mt(std::fma(a.v, b.v, c.v)); }
inline Tracked gfloor(Tracked a) { return mt(std::floor(a.v)); }
inline Tracked gmin(Tracked x, Tracked y) { return y.v < x.v ? y : x; }
inline Tracked gmax(Tracked x, Tracked y) { return x.v < y.v ? y : x; }
inline Tracked gclamp(Tracked x, Tracked lo, Tracked hi) { return gmin(gmax(x, lo), hi); }
inline Tracked saturate(Tracked x) { return gclamp(x, mt(0.0), mt(1.0)); }
inline Tracked gabs(Tracked x) { return x.v < 0.0 ? -x : x; }

template <> struct Prec<Tracked> {
    static Tracked exp(Tracked x) { return mt(std::exp(x.v)); }
    static Tracked pow5(Tracked x) { return mt(std::pow(x.v, 5.0)); }
    static Tracked pow128(Tracked x) { return mt(std::pow(x.v, 128.0)); }
    static Tracked sqrt(Tracked x) { return mt(std::sqrt(x.v)); }
    static Tracked store16(Tracked x) { return x; }
};

// per-pixel bracket of the pass loops: the margin starts unbounded, and the
// smallest one the pixel's evaluation recorded is written to the output buffer
template <class T> inline void margin_begin() {}
template <class T> inline void margin_end(size_t) {}
template <> inline void margin_begin<Tracked>() { margin_detail::current()[0] = margin_detail::current()[1] = 1e300; }
template <> inline void margin_end<Tracked>(size_t i) {
    if (margin_detail::output()) {
        margin_detail::output()[2 * i] = margin_detail::current()[0];
        margin_detail::output()[2 * i + 1] = margin_detail::current()[1];
    }
}

}  // namespace oracle
