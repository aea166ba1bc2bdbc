// sgi_nn_tc.cu - 3x3 convolutions of the learned denoiser on the 5th-generation
// tensor cores: a persistent, warp-specialised implicit GEMM with TMA loads,
// an mbarrier ring and double-buffered TMEM accumulators.
//
// Tile: R consecutive rows x 128 consecutive pixels of one image, all COUT
// output channels. Output row r of the tile is one tcgen05.mma accumulator
// D_r[m][n] (M = 128 pixels, N = COUT) = sum over 16-channel chunks, taps t and
// channels k of A_{r,t}[m][k] * B_t[n][k], where A_{r,t}[m][k] is input pixel
// (y0 + r + ky - 1, x0 + m + kx - 1), channel k (zero outside the image) and
// B_t[n][k] = w[n][t][k].
//
// Shared memory holds STAGES chunk buffers of KC input channels (KC = 16 or 32),
// each filled by two TMA loads with the 32- or 64-byte swizzle (a pixel's KC
// channels are one swizzle row of 2 KC bytes):
//   halo: box {KC channels, 130 pixels, R + 2 rows, 1} of the NHWC input view at
//       (c0, x0 - 1, y0 - 1, b) -> [row][pixel][KC], zero-filled outside the
//       image. A_{r,t} starts at pixel (r + ky, kx) of it: a K-major operand
//       whose 8-row groups are 8 * 2 KC bytes apart (SBO); each 16-channel MMA
//       step advances the start by 32 bytes. The tensor core applies the swizzle
//       to absolute shared-memory addresses, as TMA does, so the start may sit at
//       any pixel row (descriptor base offset 0).
//   weights: box {KC channels, COUT, 9 taps} of w [COUT][9][CIN] -> [tap][n][KC];
//       B_t starts at tap * COUT * 2 KC bytes.
// Both buffers start on 1024-byte boundaries.
// Roles (192 threads): warp 0 lane 0 issues the TMA loads of each chunk after
// the MMAs of the chunk that used the buffer have completed (empty barrier,
// tcgen05.commit); warp 1 lane 0 issues the 9 * R MMAs of each chunk when its
// loads have landed (full barrier, complete_tx) and commits the finished tile
// to a TMEM buffer (two buffers, so the epilogue of one tile overlaps the MMAs
// of the next); warps 2..5 read the accumulators with tcgen05.ld (warp w owns
// TMEM lanes 32 (w % 4) ...), add the bias, apply the ReLU and store BF16 —
// optionally also the 2x2 mean (the next level's input), so no pooling pass
// runs. (Writing the decoder's 2x upsampled copy from the epilogue as well was
// slower than the separate upsampling kernel: four scattered 16-byte stores per
// channel group.)
// Every wait is bounded by the global timer: a role that gives up records an
// error in *err and raises a shared abort flag that ends the other roles' waits.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_fp8.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>
#include <stdint.h>

#include <mutex>

#include "sgi_nn_apply.cuh"
#include "sgi_nn_internal.h"

namespace sgi {
namespace nn {

typedef __nv_bfloat16 bf16;

constexpr int kTcM = 128;                    // pixels per tile row (MMA M)
constexpr int kHaloPix = kTcM + 2;           // 130
constexpr int kThreads = 192;
constexpr unsigned long long kWaitNs = 200ull * 1000ull * 1000ull;   // default bound on every wait
constexpr int kSmemBudget = 220 * 1024;

__host__ __device__ constexpr int round_up(int v, int m) { return (v + m - 1) / m * m; }
__host__ __device__ constexpr int pow2_cols(int c) {
    return c <= 32 ? 32 : c <= 64 ? 64 : c <= 128 ? 128 : c <= 256 ? 256 : 512;
}

// F8: FP8 E4M3 operands (one byte per channel, 32 channels per MMA step) instead
// of BF16 (two bytes, 16 channels); either way an MMA step reads 32 bytes of a row.
template <int CIN, int COUT, bool F8 = false> struct TcShape {
    static constexpr int ROWB = (COUT <= 64 && CIN % (F8 ? 64 : 32) == 0) ? 64 : 32;   // bytes per pixel row
    static constexpr int KC = F8 ? ROWB : ROWB / 2;                       // input channels per stage
    static constexpr int NCH = (CIN + KC - 1) / KC;                       // stages per tile (the last zero-padded)
    static constexpr uint32_t LAYOUT = ROWB == 64 ? 4u : 6u;             // descriptor: 64B / 32B swizzle
    static constexpr int R = COUT == 32 ? 4 : (COUT <= 128 ? 2 : 1);     // output rows per tile
    static constexpr int HALO_ROWS = R + 2;
    static constexpr int HALO = HALO_ROWS * kHaloPix * ROWB;
    static constexpr int W_OFF = round_up(HALO, 1024);
    static constexpr int WBYTES = 9 * COUT * ROWB;
    static constexpr int STAGE = round_up(W_OFF + WBYTES, 1024);
    static constexpr int STAGES = kSmemBudget / STAGE < 6 ? kSmemBudget / STAGE : 6;
    static constexpr int TMEM_COLS = pow2_cols(2 * R * COUT);          // two accumulator buffers
    static constexpr int BUF_COLS = TMEM_COLS / 2;
    static constexpr uint32_t TX_BYTES = HALO + WBYTES;
    static constexpr size_t SMEM = (size_t)STAGES * STAGE + 1024 /* alignment slack */ + 256 /* barriers */ +
                                   3 * COUT * 4 /* bias, weight scales, output scales */;
    static_assert(STAGES >= 2, "stage ring");
    static_assert(R * COUT <= BUF_COLS, "accumulators");
};

__device__ __forceinline__ uint32_t s_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// sm_100 shared-memory matrix descriptor: no swizzle, descriptor version 1.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// Instruction descriptor, FP32 D, both operands K-major, M x N: kind::f16 with BF16
// A and B, or kind::f8f6f4 with E4M3 A and B (format code 0).
__host__ __device__ constexpr uint32_t instr_desc(int M, int N, bool f8) {
    return (1u << 4) | (f8 ? 0u : (1u << 7) | (1u << 10)) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// One MMA from descriptor low words a, b (shared high word hi): D (+)= A * B^T.
template <bool F8>
__device__ __forceinline__ void umma(uint32_t d, uint32_t a, uint32_t b, uint32_t hi, uint32_t idesc, uint32_t accum) {
    if constexpr (F8) {
        asm volatile(
            "{\n .reg .pred p;\n .reg .b64 ad, bd;\n setp.ne.b32 p, %5, 0;\n"
            " mov.b64 ad, {%1, %3};\n mov.b64 bd, {%2, %3};\n"
            " tcgen05.mma.cta_group::1.kind::f8f6f4 [%0], ad, bd, %4, p;\n}\n" ::"r"(d),
            "r"(a), "r"(b), "r"(hi), "r"(idesc), "r"(accum)
            : "memory");
    } else {
        asm volatile(
            "{\n .reg .pred p;\n .reg .b64 ad, bd;\n setp.ne.b32 p, %5, 0;\n"
            " mov.b64 ad, {%1, %3};\n mov.b64 bd, {%2, %3};\n"
            " tcgen05.mma.cta_group::1.kind::f16 [%0], ad, bd, %4, p;\n}\n" ::"r"(d),
            "r"(a), "r"(b), "r"(hi), "r"(idesc), "r"(accum)
            : "memory");
    }
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ bool mbar_test(uint32_t bar, uint32_t parity) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    return done != 0;
}

// try_wait that may suspend the thread for up to `hint_ns` (instead of the system's
// default limit) while the phase is incomplete: a waiting warp then takes no issue slots.
__device__ __forceinline__ bool mbar_test_sleep(uint32_t bar, uint32_t parity, uint32_t hint_ns) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(bar), "r"(parity), "r"(hint_ns)
        : "memory");
    return done != 0;
}

// Bounded wait for the phase of `parity`; false on timeout or when another role aborted.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, volatile int* abort_flag,
                                          unsigned long long limit_ns) {
    if (mbar_test(bar, parity)) return true;
    const unsigned long long deadline = global_ns() + limit_ns;
    while (true) {
        if (mbar_test_sleep(bar, parity, 20000u)) return true;
        if (*abort_flag) return false;
        if (global_ns() > deadline) return false;
    }
}

__device__ __forceinline__ void give_up(volatile int* abort_flag, int* err) {
    *abort_flag = 1;
    atomicExch(err, 1);
}

__device__ __forceinline__ void tma_load_4d(uint32_t dst, const CUtensorMap* map, int c0, int c1, int c2, int c3,
                                            uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
        "[%6];\n" ::"r"(dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(bar)
        : "memory");
}

__device__ __forceinline__ void tma_load_3d(uint32_t dst, const CUtensorMap* map, int c0, int c1, int c2,
                                            uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];\n" ::"r"(
            dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(bar)
        : "memory");
}

__device__ __forceinline__ void tma_load_5d(uint32_t dst, const CUtensorMap* map, int c0, int c1, int c2, int c3,
                                            int c4, uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.5d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5, "
        "%6}], [%7];\n" ::"r"(dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(c4), "r"(bar)
        : "memory");
}

__device__ __forceinline__ void mma_commit(uint32_t bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(bar)
                 : "memory");
}

__device__ __forceinline__ void bf8_unpack(const uint4& v, float* f) {
    const __nv_bfloat162* h = reinterpret_cast<const __nv_bfloat162*>(&v);
#pragma unroll
    for (int j = 0; j < 4; ++j) { const float2 t = __bfloat1622float2(h[j]); f[2 * j] = t.x; f[2 * j + 1] = t.y; }
}

__device__ __forceinline__ uint4 shfl_down_u4(uint4 v, int d) {
    v.x = __shfl_down_sync(0xffffffffu, v.x, d);
    v.y = __shfl_down_sync(0xffffffffu, v.y, d);
    v.z = __shfl_down_sync(0xffffffffu, v.z, d);
    v.w = __shfl_down_sync(0xffffffffu, v.w, d);
    return v;
}

// 16 consecutive 32-bit TMEM columns of this warp's 32 lanes (one per thread).
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t* v) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15}, [%16];\n"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
          "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
        : "r"(taddr));
}

// 32 consecutive 32-bit TMEM columns of this warp's 32 lanes (one per thread).
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t* v) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];\n"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
          "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]),
          "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]),
          "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
        : "r"(taddr));
}

// Epilogue of NC (16 or 32) output channels n0 .. n0 + NC - 1 of one pixel: f holds
// the FP32 accumulators; they are scaled (F8: by the weights' per-channel scale),
// biased, passed through the ReLU (mode 0) and packed into NC / 16 vectors of 16
// FP8 channels (OUT8, multiplied by the next layer's per-channel inverse scale) or
// NC / 8 vectors of 8 BF16 channels.
template <int NC, int MODE, bool F8, bool OUT8>
__device__ __forceinline__ void epilogue_n(float* f, int n0, const float* bias_s, const float* ws_s,
                                           const float* oinv_s, uint4* out) {
#pragma unroll
    for (int j = 0; j < NC; ++j) {
        float x = f[j];
        if (F8) x *= ws_s[n0 + j];
        if (MODE != 2) x += bias_s[n0 + j];
        if (MODE == 0) x = fmaxf(x, 0.0f);
        f[j] = x;
    }
    if constexpr (OUT8) {
#pragma unroll
        for (int v = 0; v < NC / 16; ++v) {
            uint32_t w[4];
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int c = 16 * v + 4 * j;
                const __nv_fp8x2_storage_t lo = __nv_cvt_float2_to_fp8x2(
                    make_float2(f[c] * oinv_s[n0 + c], f[c + 1] * oinv_s[n0 + c + 1]), __NV_SATFINITE, __NV_E4M3);
                const __nv_fp8x2_storage_t hi = __nv_cvt_float2_to_fp8x2(
                    make_float2(f[c + 2] * oinv_s[n0 + c + 2], f[c + 3] * oinv_s[n0 + c + 3]), __NV_SATFINITE,
                    __NV_E4M3);
                w[j] = (uint32_t)lo | ((uint32_t)hi << 16);
            }
            out[v] = make_uint4(w[0], w[1], w[2], w[3]);
        }
    } else {
#pragma unroll
        for (int v = 0; v < NC / 8; ++v) {
            uint4 o;
            __nv_bfloat162* oh = reinterpret_cast<__nv_bfloat162*>(&o);
#pragma unroll
            for (int j = 0; j < 4; ++j) oh[j] = __floats2bfloat162_rn(f[8 * v + 2 * j], f[8 * v + 2 * j + 1]);
            out[v] = o;
        }
    }
}

// FP8 E4M3 x 16 -> float
__device__ __forceinline__ void fp8x16_unpack(const uint4& v, float* f) {
    const uint32_t w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
    for (int j = 0; j < 4; ++j) {
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const __half2_raw r = __nv_cvt_fp8x2_to_halfraw2((__nv_fp8x2_storage_t)(w[j] >> (16 * h)), __NV_E4M3);
            __half2 hh;
            hh = *reinterpret_cast<const __half2*>(&r);
            const float2 t = __half22float2(hh);
            f[4 * j + 2 * h] = t.x;
            f[4 * j + 2 * h + 1] = t.y;
        }
    }
}

// 2x2 mean of four packed vectors, summed in the order given, re-packed in the same format
// (an FP8 mean keeps the per-channel scale of its inputs).
template <bool OUT8>
__device__ __forceinline__ uint4 mean4(const uint4& a, const uint4& b, const uint4& c, const uint4& d) {
    if constexpr (OUT8) {
        float a0[16], a1[16], a2[16], a3[16];
        fp8x16_unpack(a, a0);
        fp8x16_unpack(b, a1);
        fp8x16_unpack(c, a2);
        fp8x16_unpack(d, a3);
        uint32_t w[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            float m[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const int k = 4 * j + i;
                m[i] = 0.25f * (((a0[k] + a1[k]) + a2[k]) + a3[k]);
            }
            const __nv_fp8x2_storage_t lo = __nv_cvt_float2_to_fp8x2(make_float2(m[0], m[1]), __NV_SATFINITE, __NV_E4M3);
            const __nv_fp8x2_storage_t hi = __nv_cvt_float2_to_fp8x2(make_float2(m[2], m[3]), __NV_SATFINITE, __NV_E4M3);
            w[j] = (uint32_t)lo | ((uint32_t)hi << 16);
        }
        return make_uint4(w[0], w[1], w[2], w[3]);
    } else {
        float a0[8], a1[8], a2[8], a3[8], pv[8];
        bf8_unpack(a, a0);
        bf8_unpack(b, a1);
        bf8_unpack(c, a2);
        bf8_unpack(d, a3);
#pragma unroll
        for (int j = 0; j < 8; ++j) pv[j] = 0.25f * (((a0[j] + a1[j]) + a2[j]) + a3[j]);
        uint4 po;
        __nv_bfloat162* ph2 = reinterpret_cast<__nv_bfloat162*>(&po);
#pragma unroll
        for (int j = 0; j < 4; ++j) ph2[j] = __floats2bfloat162_rn(pv[2 * j], pv[2 * j + 1]);
        return po;
    }
}

struct TcTiles {
    int tiles_x, tiles_y, total;
};

template <int CIN, int COUT, int MODE, bool F8, bool OUT8>
__global__ void __launch_bounds__(kThreads, 1)
    conv3x3_tc_kernel(const __grid_constant__ CUtensorMap map_x, const __grid_constant__ CUtensorMap map_w,
                      ConvArgs a, TcTiles tl, int* err) {
    using S = TcShape<CIN, COUT, F8>;
    constexpr int R = S::R, KC = S::KC, NCH = S::NCH;
    constexpr int NV = OUT8 ? 2 : 4;   // output vectors per 32 channels
    static_assert(CIN % 16 == 0 && COUT % 16 == 0 && COUT >= 16 && COUT <= 256, "shape");
    extern __shared__ unsigned char smem_raw[];
    unsigned char* smem =
        reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
    unsigned char* ctrl = smem + (size_t)S::STAGES * S::STAGE;
    uint64_t* full = reinterpret_cast<uint64_t*>(ctrl);            // [STAGES]
    uint64_t* empty = full + S::STAGES;                            // [STAGES]
    uint64_t* tfull = empty + S::STAGES;                           // [2]
    uint64_t* tempty = tfull + 2;                                  // [2]
    uint64_t* drain = tempty + 2;                                  // [1]
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(drain + 1);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);
    float* bias_s = reinterpret_cast<float*>(ctrl + 256);            // [COUT]
    float* ws_s = bias_s + COUT;                                     // [COUT] weight scales (F8)
    float* oinv_s = ws_s + COUT;                                     // [COUT] output inverse scales (OUT8)

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(s_addr(tmem_slot)),
                     "r"(S::TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
    }
    if (tid == 0) {
        for (int s = 0; s < S::STAGES; ++s) {
            mbar_init(s_addr(full + s), 1);
            mbar_init(s_addr(empty + s), 1);
        }
        for (int b = 0; b < 2; ++b) {
            mbar_init(s_addr(tfull + b), 1);
            mbar_init(s_addr(tempty + b), 4);   // one arrival per epilogue warp
        }
        mbar_init(s_addr(drain), 1);
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
        asm volatile("prefetch.tensormap [%0];\n" ::"l"(reinterpret_cast<uint64_t>(&map_x)) : "memory");
        asm volatile("prefetch.tensormap [%0];\n" ::"l"(reinterpret_cast<uint64_t>(&map_w)) : "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    pdl_wait();   // every global access below follows the previous kernel's completion
    pdl_trigger();
    const unsigned long long wait_ns = a.wait_ns ? a.wait_ns : kWaitNs;
    const uint32_t tmem = *tmem_slot;
    const uint32_t smem_base = s_addr(smem);

    if (warp == 0) {
        // ------------------------------------------------ TMA producer
        if (lane == 0 && !a.skip_producer) {
            int s = 0;
            uint32_t ph = 0;
            bool ok = true;
            for (int t = blockIdx.x; t < tl.total && ok; t += gridDim.x) {
                const int tx = t % tl.tiles_x, rest = t / tl.tiles_x;
                const int ty = rest % tl.tiles_y, b = rest / tl.tiles_y;
                const int x0 = tx * kTcM, y0 = ty * R;
                for (int ch = 0; ch < NCH; ++ch) {
                    if (!mbar_wait(s_addr(empty + s), ph ^ 1u, abort_flag, wait_ns)) { ok = false; break; }
                    const uint32_t bar = s_addr(full + s);
                    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(bar),
                                 "r"(S::TX_BYTES)
                                 : "memory");
                    const uint32_t st = smem_base + s * S::STAGE;
                    tma_load_4d(st, &map_x, ch * KC, x0 - 1, y0 - 1, b, bar);
                    tma_load_3d(st + S::W_OFF, &map_w, ch * KC, 0, 0, bar);
                    if (++s == S::STAGES) { s = 0; ph ^= 1u; }
                }
            }
            if (!ok) give_up(abort_flag, err);
        }
    } else if (warp == 1) {
        // ------------------------------------------------ MMA issuer
        if (lane == 0) {
            constexpr uint32_t IDESC = instr_desc(kTcM, COUT, F8);
            // Descriptors are split into a 32-bit low word (start address >> 4, leading
            // byte offset field 1) and a constant high word (stride byte offset =
            // 8 rows, version 1, swizzle mode). Every MMA of a chunk adds a
            // compile-time offset to the low word of the stage's base descriptor.
            constexpr uint32_t HI = (uint32_t)((8 * S::ROWB) >> 4) | (1u << 14) | (S::LAYOUT << 29);
            int s = 0, acc = 0;
            uint32_t ph = 0, aph = 0;
            bool ok = true, issued = false;
            for (int t = blockIdx.x; t < tl.total && ok; t += gridDim.x) {
                if (!mbar_wait(s_addr(tempty + acc), aph ^ 1u, abort_flag, wait_ns)) { ok = false; break; }
                asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
                const uint32_t d0 = tmem + (uint32_t)(acc * S::BUF_COLS);
                for (int ch = 0; ch < NCH; ++ch) {
                    if (!mbar_wait(s_addr(full + s), ph, abort_flag, wait_ns)) { ok = false; break; }
                    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
                    const uint32_t st = smem_base + s * S::STAGE;
                    const uint32_t a_lo = ((st >> 4) & 0x3FFFu) | (1u << 16);
                    const uint32_t b_lo = (((st + S::W_OFF) >> 4) & 0x3FFFu) | (1u << 16);
                    const uint32_t first = ch > 0 ? 1u : 0u;
#pragma unroll
                    for (int r = 0; r < R; ++r) {
#pragma unroll
                        for (int tap = 0; tap < 9; ++tap) {
#pragma unroll
                            for (int ks = 0; ks < S::ROWB / 32; ++ks) {
                                const int ky = tap / 3, kx = tap % 3;
                                const uint32_t a =
                                    a_lo + (uint32_t)((((r + ky) * kHaloPix + kx) * S::ROWB + ks * 32) >> 4);
                                const uint32_t b = b_lo + (uint32_t)((tap * COUT * S::ROWB + ks * 32) >> 4);
                                const uint32_t accum = (tap > 0 || ks > 0) ? 1u : first;
                                umma<F8>(d0 + (uint32_t)(r * COUT), a, b, HI, IDESC, accum);
                            }
                        }
                    }
                    issued = true;
                    mma_commit(s_addr(empty + s));   // frees the stage when these MMAs are done
                    if (++s == S::STAGES) { s = 0; ph ^= 1u; }
                }
                if (!ok) break;
                mma_commit(s_addr(tfull + acc));     // the tile's accumulators are complete
                if (++acc == 2) { acc = 0; aph ^= 1u; }
            }
            if (!ok) {
                give_up(abort_flag, err);
                if (issued) {
                    // let the MMAs already issued finish before the TMEM is released
                    mma_commit(s_addr(drain));
                    const unsigned long long deadline = global_ns() + wait_ns;
                    while (!mbar_test(s_addr(drain), 0) && global_ns() < deadline) {
                    }
                }
            }
        }
    } else {
        // ------------------------------------------------ epilogue (warps 2..5)
        const int q = warp & 3;   // TMEM lane quarter of this warp
        const int et = tid - 64;  // 0..127
        for (int c = et; c < COUT; c += 128) {
            if (MODE != 2) bias_s[c] = a.bias[c];
            if (F8) ws_s[c] = a.wscale[c];
            if (OUT8) oinv_s[c] = a.oinv[c];
        }
        asm volatile("bar.sync 1, 128;\n" ::: "memory");   // epilogue warps only
        // the fused 2x2 mean pairs rows (r, r + 1) of one thread and pixels of lanes (2j, 2j + 1)
        constexpr bool CAN_POOL = (R % 2 == 0) && COUT <= 64;
        const bool pooling = CAN_POOL && a.pool.p != nullptr;
        uint4 held[CAN_POOL ? COUT / 32 * NV : 1];
        int acc = 0;
        uint32_t aph = 0;
        for (int t = blockIdx.x; t < tl.total; t += gridDim.x) {
            // one lane polls the barrier (polling from every lane competes with the MMA
            // operand reads in shared memory); the warp then leaves or proceeds together,
            // as tcgen05.ld below is a warp-wide (.sync.aligned) instruction
            int ready = 0;
            if (lane == 0) ready = mbar_wait(s_addr(tfull + acc), aph, abort_flag, wait_ns) ? 1 : 0;
            ready = __shfl_sync(0xffffffffu, ready, 0);
            if (!ready) {
                if (lane == 0) give_up(abort_flag, err);
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
            const int tx = t % tl.tiles_x, rest = t / tl.tiles_x;
            const int ty = rest % tl.tiles_y, b = rest / tl.tiles_y;
            const int px = tx * kTcM + q * 32 + lane;
#pragma unroll 1
            for (int r = 0; r < R; ++r) {
                const int gy = ty * R + r;
                const bool valid = px < a.W && gy < a.H;
                const size_t pix = valid ? (size_t)gy * a.W + px : 0;
                bf16* yp = a.y.p + a.y.at(b, pix, 0);
#pragma unroll
                for (int n0 = 0; n0 < COUT; n0 += 32) {
                    uint32_t v[32];
                    tmem_ld32(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(acc * S::BUF_COLS + r * COUT + n0), v);
                    asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
                    float f[32];
#pragma unroll
                    for (int j = 0; j < 32; ++j) f[j] = __uint_as_float(v[j]);
                    uint4 o[NV];
                    epilogue_n<32, MODE, F8, OUT8>(f, n0, bias_s, ws_s, oinv_s, o);
#pragma unroll
                    for (int g = 0; g < NV; ++g) {
                        const int k = n0 / (OUT8 ? 16 : 8) + g;   // 16-byte vector of the pixel
                        if (valid) *reinterpret_cast<uint4*>(yp + (size_t)k * (size_t)a.y.grp) = o[g];
                        if (CAN_POOL && pooling) {
                            if ((r & 1) == 0) {
                                held[CAN_POOL ? k : 0] = o[g];
                            } else {
                                // mean of (r - 1, px), (r - 1, px + 1), (r, px), (r, px + 1), summed in that order
                                const uint4 nh = shfl_down_u4(held[CAN_POOL ? k : 0], 1), nc = shfl_down_u4(o[g], 1);
                                if (valid && (lane & 1) == 0)
                                    *reinterpret_cast<uint4*>(
                                        a.pool.p + a.pool.at(b, (size_t)(gy / 2) * (a.W / 2) + px / 2, k)) =
                                        mean4<OUT8>(held[CAN_POOL ? k : 0], nh, o[g], nc);
                            }
                        }
                    }
                }
            }
            asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
            __syncwarp();
            if (lane == 0)
                asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(s_addr(tempty + acc)) : "memory");
            if (++acc == 2) { acc = 0; aph ^= 1u; }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    if (warp == 1)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(S::TMEM_COLS)
                     : "memory");
}

// ---------------------------------- 32 output channels: row streaming, taps accumulated in TMEM
//
// With COUT = 32 an MMA of N = 32 costs about as much as one of N = 96 (both are
// bounded by reading the 128-row A operand from shared memory), so the three
// vertical taps share one MMA. A CTA walks strips of 128 pixels x 16 rows from
// the top. Output row j of a strip (image row y0 + j) owns the 32 TMEM columns
// C(j) = 32 (15 - j). Halo row i (image row y0 - 1 + i) feeds row i - ky with
// vertical tap ky, i.e. columns C(i) + 32 ky, so one MMA with B = taps
// (0..2, kx) stacked along N = 96 and D at column C(i) adds halo row i into
// rows i, i - 1 and i - 2:
//   D[m][C(i) + 32 ky + n] += sum over kx, k of X[i][x0 - 1 + m + kx][k] * W[n][ky][kx][k].
// At the strip's top and bottom only the taps that land on rows 0 .. nrows - 1
// are issued (N = 32 or 64, with B and D advanced by 32 ky_lo). Row j is complete
// after halo row j + 2: the epilogue reads its 32 columns, writes zeros back (the
// MMAs only accumulate, so every row slot starts at zero) and hands the slot to
// the next strip's row j. Each halo row is loaded once, two rows per TMA box (the
// copy engine streams narrow pixel rows faster in larger boxes); the weights of all
// taps and input channels (at most 55 KB, [chunk][kx][ky][n][KC]) stay in shared
// memory. FP8 with 96 input channels takes one 128-byte chunk per pixel (three
// 32-channel K steps, the fourth slice of the row is zero fill and skipped).
// COUT_ = 32 or 64 output channels (row slots of COUT_ TMEM columns, N = 3 COUT_).
// ROWS_ x COUT_ = 512: one CTA per SM holds all TMEM columns; = 256: two CTAs per
// SM (at most 110 KB of shared memory each), two independent pipelines per SM for
// the price of more halo rows per strip (10 / 8 instead of 18 / 16 for COUT_ = 32).
template <int CIN, bool F8 = false, int ROWS_ = 16, int COUT_ = 32> struct RsShape {
    static constexpr int COUT = COUT_, NX = 3 * COUT_;
    static constexpr int EB = F8 ? 1 : 2;                           // bytes per channel
    static constexpr int ROWB = (F8 && CIN == 96) ? 128 : CIN % (F8 ? 64 : 32) == 0 ? 64 : 32;
    static constexpr int KC = ROWB / EB;
    static constexpr uint32_t LAYOUT = ROWB == 128 ? 2u : ROWB == 64 ? 4u : 6u;   // 128B / 64B / 32B swizzle
    static constexpr int NCH = (CIN + KC - 1) / KC;
    static constexpr int KS = ROWB / 32;                            // 32-byte K steps of a full chunk
    static constexpr int KS_LAST = ((CIN - (NCH - 1) * KC) * EB + 31) / 32;   // of the last chunk
    static constexpr int ROWS = ROWS_;                              // output rows per strip = TMEM row slots
    static constexpr int HPS = 2;                                   // halo rows per stage (one TMA box)
    static constexpr int HROW = kHaloPix * ROWB;                    // bytes of one halo row of one chunk
    static constexpr uint32_t STAGE_TX = HPS * HROW;
    static constexpr int STAGE = round_up(HPS * HROW, 1024);
    static constexpr int WCH = 9 * COUT * ROWB;                     // weights of one chunk
    static constexpr int WBYTES = NCH * WCH;
    static constexpr int ST_OFF = round_up(WBYTES, 1024);
    static constexpr int TMEM_COLS = ROWS * COUT;
    static constexpr int CTAS = 512 / TMEM_COLS;                     // CTAs per SM
    static constexpr int BUDGET = CTAS == 1 ? kSmemBudget : 110 * 1024;
    static constexpr int STAGES = (BUDGET - ST_OFF) / STAGE < 16 ? (BUDGET - ST_OFF) / STAGE : 16;
    static constexpr int CTRL = 640;                                // barriers, TMEM address, abort flag
    // one CTA per SM (all 512 TMEM columns): at least 120 KB, so that no second CTA waits for TMEM
    static constexpr size_t SMEM_USED = (size_t)ST_OFF + (size_t)STAGES * STAGE + 1024 + CTRL + 2 * COUT * 4;
    static constexpr size_t SMEM = (CTAS == 2 || SMEM_USED > 120 * 1024) ? SMEM_USED : 120 * 1024;
    static constexpr bool FITS = STAGES >= 2 * NCH && SMEM_USED <= (size_t)(CTAS == 1 ? 227 * 1024 : 113 * 1024);
    static_assert(WCH % 1024 == 0, "shape");
    static_assert((TMEM_COLS == 256 || TMEM_COLS == 512) && ROWS % HPS == 0, "tmem");
    static_assert((2 * STAGES + ROWS + 2) * 8 + 8 <= CTRL, "control block");
};

constexpr int kRsThreads = 320;   // producer, MMA issuer, 8 epilogue warps

__device__ __forceinline__ void tmem_st16_zero(uint32_t taddr) {
    asm volatile(
        "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, "
        "%1};\n" ::"r"(taddr),
        "r"(0u)
        : "memory");
}

// 16 FP32 accumulators -> y = act(acc * sc + bb) in FP32 (packed FMAs).
template <int MODE>
__device__ __forceinline__ void act16(const uint32_t* v, const float* sc, const float* bb, float* f) {
#pragma unroll
    for (int p = 0; p < 8; ++p) {
        unsigned long long x, s, c, d;
        asm("mov.b64 %0, {%1, %2};" : "=l"(x) : "r"(v[2 * p]), "r"(v[2 * p + 1]));
        asm("mov.b64 %0, {%1, %2};" : "=l"(s) : "f"(sc[2 * p]), "f"(sc[2 * p + 1]));
        asm("mov.b64 %0, {%1, %2};" : "=l"(c) : "f"(bb[2 * p]), "f"(bb[2 * p + 1]));
        asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(x), "l"(s), "l"(c));
        float lo, hi;
        asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(d));
        f[2 * p] = MODE == 0 ? fmaxf(lo, 0.0f) : lo;
        f[2 * p + 1] = MODE == 0 ? fmaxf(hi, 0.0f) : hi;
    }
}

// 16 floats -> 16 E4M3 channels (one 16-byte vector, OUT8) or 16 BF16 channels (two).
template <bool OUT8>
__device__ __forceinline__ void pack16(const float* f, uint4* out) {
    uint32_t w[8];
#pragma unroll
    for (int p = 0; p < 8; ++p) {
        if constexpr (OUT8) {
            uint16_t r;
            asm("cvt.rn.satfinite.e4m3x2.f32 %0, %1, %2;" : "=h"(r) : "f"(f[2 * p + 1]), "f"(f[2 * p]));
            w[p] = r;
        } else {
            asm("cvt.rn.bf16x2.f32 %0, %1, %2;" : "=r"(w[p]) : "f"(f[2 * p + 1]), "f"(f[2 * p]));
        }
    }
    if constexpr (OUT8) {
        out[0] = make_uint4(w[0] | (w[1] << 16), w[2] | (w[3] << 16), w[4] | (w[5] << 16), w[6] | (w[7] << 16));
    } else {
        out[0] = make_uint4(w[0], w[1], w[2], w[3]);
        out[1] = make_uint4(w[4], w[5], w[6], w[7]);
    }
}

// 16 FP32 accumulators -> y = act(acc * sc + bb) (packed FMAs), as 16 E4M3 channels
// (one 16-byte vector, OUT8) or 16 BF16 channels (two vectors). ReLU (mode 0) is
// applied by the conversion.
template <int MODE, bool OUT8>
__device__ __forceinline__ void epilogue16(const uint32_t* v, const float* sc, const float* bb, uint4* out) {
    uint32_t w[8];
#pragma unroll
    for (int p = 0; p < 8; ++p) {
        unsigned long long x, s, c, d;
        asm("mov.b64 %0, {%1, %2};" : "=l"(x) : "r"(v[2 * p]), "r"(v[2 * p + 1]));
        asm("mov.b64 %0, {%1, %2};" : "=l"(s) : "f"(sc[2 * p]), "f"(sc[2 * p + 1]));
        asm("mov.b64 %0, {%1, %2};" : "=l"(c) : "f"(bb[2 * p]), "f"(bb[2 * p + 1]));
        asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(x), "l"(s), "l"(c));
        float lo, hi;
        asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(d));
        if constexpr (OUT8) {
            uint16_t r;
            if constexpr (MODE == 0)
                asm("cvt.rn.satfinite.relu.e4m3x2.f32 %0, %1, %2;" : "=h"(r) : "f"(hi), "f"(lo));
            else
                asm("cvt.rn.satfinite.e4m3x2.f32 %0, %1, %2;" : "=h"(r) : "f"(hi), "f"(lo));
            w[p] = r;
        } else {
            if constexpr (MODE == 0)
                asm("cvt.rn.relu.bf16x2.f32 %0, %1, %2;" : "=r"(w[p]) : "f"(hi), "f"(lo));
            else
                asm("cvt.rn.bf16x2.f32 %0, %1, %2;" : "=r"(w[p]) : "f"(hi), "f"(lo));
        }
    }
    if constexpr (OUT8) {
        out[0] = make_uint4(w[0] | (w[1] << 16), w[2] | (w[3] << 16), w[4] | (w[5] << 16), w[6] | (w[7] << 16));
    } else {
        out[0] = make_uint4(w[0], w[1], w[2], w[3]);
        out[1] = make_uint4(w[4], w[5], w[6], w[7]);
    }
}

// Two CTAs per SM (256 TMEM columns each) where that shape fits (at least two
// halo-row pairs of stages), else one; 0 when neither fits (the 9-tap kernel runs).
template <int CIN, bool F8, int COUT> constexpr int rs_rows() {
    return RsShape<CIN, F8, 256 / COUT, COUT>::FITS ? 256 / COUT : RsShape<CIN, F8, 512 / COUT, COUT>::FITS ? 512 / COUT : 0;
}

template <int CIN, bool F8, int COUT> constexpr int rs_rows_any() {
    if constexpr (COUT == 32 || COUT == 64) return rs_rows<CIN, F8, COUT>();
    else return 0;
}

// The head's epilogue with the kernel apply (mode 3): the pixel's 32 logits
// as the plain head stores them (accumulator + bias, rounded to BF16), then the
// kernel apply and composite of kpcn_apply_kernel (sgi_nn_apply.cuh) with the
// 5x5 neighbours of the noisy estimate read from global memory (clamped; a
// warp's 32 consecutive pixels share them in L1). Exchanging one load per lane
// and row by shuffles instead measured the same.
__device__ __forceinline__ void head_apply_px(const ConvArgs& a, const uint32_t* v, const float* sc, const float* bb,
                                              int y, int x) {
    float lf[32];
    act16<1>(v, sc, bb, lf);
    act16<1>(v + 16, sc + 16, bb + 16, lf + 16);
#pragma unroll
    for (int j = 0; j < 32; ++j) lf[j] = __bfloat162float(__float2bfloat16_rn(lf[j]));
    const int W = a.W, H = a.H;
    const size_t i = (size_t)y * W + x;
    const ConvArgs::ApplyFuse& f = a.fuse;
    const float4 pv = f.prev[i];
    const float pr[3] = {pv.x, pv.y, pv.z};
    float l[25], sp[3], alpha, o[3];
    kpcn_apply_px(lf,
                  [&](int k) {
                      const int yy = min(max(y + k / 5 - 2, 0), H - 1), xx = min(max(x + k % 5 - 2, 0), W - 1);
                      return rgba16_to_f4(__ldg(f.noisy + (size_t)yy * W + xx));
                  },
                  pr, l, sp, alpha, o);
    composite_px(o[0], o[1], o[2], f.screen, f.albedo, f.hdr, f.gi_out, f.hist_out, i);
}

template <int CIN, int MODE, bool F8, bool OUT8, int ROWS_, int COUT_>
__global__ void __launch_bounds__(kRsThreads, 512 / (ROWS_ * COUT_))
    conv3x3_rs_kernel(const __grid_constant__ CUtensorMap map_x, const __grid_constant__ CUtensorMap map_w,
                      ConvArgs a, TcTiles tl, int* err) {
    using S = RsShape<CIN, F8, ROWS_, COUT_>;
    constexpr int COUT = COUT_, NX = S::NX, NCH = S::NCH, KC = S::KC, ROWS = S::ROWS, NP = ROWS / 2;
    constexpr int CPT = COUT / 2;             // output channels of each epilogue group
    extern __shared__ unsigned char smem_raw[];
    unsigned char* smem =
        reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
    unsigned char* ctrl = smem + (size_t)S::ST_OFF + (size_t)S::STAGES * S::STAGE;
    uint64_t* full = reinterpret_cast<uint64_t*>(ctrl);            // [STAGES]
    uint64_t* empty = full + S::STAGES;                            // [STAGES]
    uint64_t* pairfull = empty + S::STAGES;                        // [NP] rows 2p, 2p + 1 accumulated
    uint64_t* pairfree = pairfull + NP;                            // [NP] rows 2p, 2p + 1 read and zeroed
    uint64_t* wbar = pairfree + NP;                                // [1]
    uint64_t* drain = wbar + 1;                                    // [1]
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(drain + 1);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);
    float* sc_s = reinterpret_cast<float*>(ctrl + S::CTRL);         // [COUT] accumulator scales
    float* bb_s = sc_s + COUT;                                       // [COUT] biases (scaled)

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(s_addr(tmem_slot)),
                     "r"(S::TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
    }
    if (tid == 0) {
        for (int s = 0; s < S::STAGES; ++s) {
            mbar_init(s_addr(full + s), 1);
            mbar_init(s_addr(empty + s), 1);
        }
        for (int p = 0; p < NP; ++p) {
            mbar_init(s_addr(pairfull + p), 1);
            mbar_init(s_addr(pairfree + p), 8);   // one arrival per epilogue warp
        }
        mbar_init(s_addr(wbar), 1);
        mbar_init(s_addr(drain), 1);
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
        asm volatile("prefetch.tensormap [%0];\n" ::"l"(reinterpret_cast<uint64_t>(&map_x)) : "memory");
        asm volatile("prefetch.tensormap [%0];\n" ::"l"(reinterpret_cast<uint64_t>(&map_w)) : "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    pdl_wait();   // every global access below follows the previous kernel's completion
    pdl_trigger();
    const unsigned long long wait_ns = a.wait_ns ? a.wait_ns : kWaitNs;
    const uint32_t tmem = *tmem_slot;
    const uint32_t smem_base = s_addr(smem);
    const uint32_t stage_base = smem_base + S::ST_OFF;

    if (warp == 0) {
        // ------------------------------------------------ TMA producer
        if (lane == 0 && !a.skip_producer) {
            // resident weights: one box {KC, COUT n, 3 ky, 3 kx} per chunk
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(s_addr(wbar)),
                         "r"((uint32_t)S::WBYTES)
                         : "memory");
            for (int ch = 0; ch < NCH; ++ch)
                tma_load_4d(smem_base + ch * S::WCH, &map_w, ch * KC, 0, 0, 0, s_addr(wbar));
            int s = 0;
            uint32_t ph = 0;
            bool ok = true;
            for (int t = blockIdx.x; t < tl.total && ok; t += gridDim.x) {
                const int sx = t % tl.tiles_x, rest = t / tl.tiles_x;
                const int sy = rest % tl.tiles_y, b = rest / tl.tiles_y;
                const int x0 = sx * kTcM, yb = sy * ROWS;
                const int nrows = min(ROWS, a.H - yb);
                for (int i = 0; i < nrows + 2 && ok; i += 2) {
                    for (int ch = 0; ch < NCH; ++ch) {
                        if (!mbar_wait(s_addr(empty + s), ph ^ 1u, abort_flag, wait_ns)) { ok = false; break; }
                        const uint32_t bar = s_addr(full + s);
                        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(bar),
                                     "r"(S::STAGE_TX)
                                     : "memory");
                        // halo rows i, i + 1 (a row past the strip's last is loaded and not used)
                        tma_load_4d(stage_base + s * S::STAGE, &map_x, ch * KC, x0 - 1, yb - 1 + i, b, bar);
                        if (++s == S::STAGES) { s = 0; ph ^= 1u; }
                    }
                }
            }
            if (!ok) give_up(abort_flag, err);
        }
    } else if (warp == 1) {
        // ------------------------------------------------ MMA issuer
        // Halo rows go in pairs (one stage per chunk). Pair k first touches output
        // rows 2k, 2k + 1, whose columns must have been zeroed (pairfree[k]); the
        // output pairs whose last tap it adds are committed to pairfull.
        if (lane == 0) {
            constexpr uint32_t IDESC0 = instr_desc(kTcM, 0, F8);   // N added per MMA
            constexpr uint32_t HI = (uint32_t)((8 * S::ROWB) >> 4) | (1u << 14) | (S::LAYOUT << 29);
            int s = 0;
            uint32_t ph = 0;
            uint32_t pf_ph = 0;   // bit p: parity of the next phase of pairfree[p]
            bool ok = mbar_wait(s_addr(wbar), 0, abort_flag, wait_ns), issued = false;
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
            const uint32_t w_lo = ((smem_base >> 4) & 0x3FFFu) | (1u << 16);
            for (int t = blockIdx.x; t < tl.total && ok; t += gridDim.x) {
                const int sy = (t / tl.tiles_x) % tl.tiles_y;
                const int nrows = min(ROWS, a.H - sy * ROWS);
                const int nh = nrows + 2;
                int next_p = 0;   // next output pair to commit
                for (int i0 = 0; i0 < nh && ok; i0 += 2) {
                    for (int ch = 0; ch < NCH; ++ch) {
                        const int sc = (s + ch) % S::STAGES;
                        const uint32_t pc = ph ^ (uint32_t)((s + ch) / S::STAGES);
                        if (!mbar_wait(s_addr(full + sc), pc, abort_flag, wait_ns)) { ok = false; break; }
                    }
                    const int k = i0 >> 1;
                    if (ok && 2 * k < nrows) {   // rows 2k, 2k + 1 start here: wait until they are zero
                        ok = mbar_wait(s_addr(pairfree + k), (pf_ph >> k) & 1u, abort_flag, wait_ns);
                        pf_ph ^= 1u << k;
                    }
                    if (!ok) break;
                    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
                    for (int r = 0; r < 2; ++r) {
                        const int i = i0 + r;
                        if (i >= nh) break;
                        // taps of halo row i that land on rows 0 .. nrows - 1
                        const int ky_lo = max(0, i - nrows + 1), ky_hi = min(2, i);
                        const uint32_t d = tmem + (uint32_t)(COUT * (ROWS - 1 - i + ky_lo));
                        const uint32_t idesc = IDESC0 | ((uint32_t)((COUT / 8) * (ky_hi - ky_lo + 1)) << 17);
                        const uint32_t b_ky = (uint32_t)((COUT * ky_lo * S::ROWB) >> 4);
                        for (int ch = 0; ch < NCH; ++ch) {
                            const int sc = (s + ch) % S::STAGES;
                            const uint32_t a_lo =
                                (((stage_base + sc * S::STAGE + r * S::HROW) >> 4) & 0x3FFFu) | (1u << 16);
                            const uint32_t b_lo = w_lo + (uint32_t)((ch * S::WCH) >> 4) + b_ky;
                            const int kss = ch == NCH - 1 ? S::KS_LAST : S::KS;
#pragma unroll
                            for (int kx = 0; kx < 3; ++kx) {
#pragma unroll
                                for (int ks = 0; ks < S::KS; ++ks) {
                                    if (ks >= kss) break;
                                    const uint32_t av = a_lo + (uint32_t)((kx * S::ROWB + ks * 32) >> 4);
                                    const uint32_t bv = b_lo + (uint32_t)((kx * NX * S::ROWB + ks * 32) >> 4);
                                    umma<F8>(d, av, bv, HI, idesc, 1u);
                                }
                            }
                        }
                        issued = true;
                    }
                    // output pair p is complete once halo row (its last row) + 2 is in
                    const int last = min(i0 + 1, nh - 1);
                    while (2 * next_p < nrows && min(2 * next_p + 1, nrows - 1) + 2 <= last) {
                        mma_commit(s_addr(pairfull + next_p));
                        ++next_p;
                    }
                    for (int ch = 0; ch < NCH; ++ch) {
                        mma_commit(s_addr(empty + s));
                        if (++s == S::STAGES) { s = 0; ph ^= 1u; }
                    }
                }
            }
            if (!ok) {
                give_up(abort_flag, err);
                if (issued) {
                    mma_commit(s_addr(drain));
                    const unsigned long long deadline = global_ns() + wait_ns;
                    while (!mbar_test(s_addr(drain), 0) && global_ns() < deadline) {
                    }
                }
            }
        }
    } else {
        // ------------------------------------------------ epilogue (warps 2..9)
        // Two groups of four warps (one per TMEM lane quarter) split the COUT output
        // channels (CPT each, in 16-channel pieces); every thread owns one pixel of a
        // row and handles the rows in pairs (the 2x2 mean of a pooled output needs both).
        const int q = warp & 3;
        const int grp = (warp - 2) >> 2;
        const int c0 = CPT * grp;               // first output channel of this group
        constexpr int NVG = OUT8 ? 1 : 2;       // 16-byte output vectors per 16 channels
        const int et = tid - 64;
        for (int c = et; c < COUT; c += 256) {
            // y = act((acc * wscale + bias) * oinv) = act(acc * (wscale * oinv) + bias * oinv), oinv > 0
            float sc = F8 ? a.wscale[c] : 1.0f, bb = MODE != 2 ? a.bias[c] : 0.0f;
            if (OUT8) {
                const float o = a.oinv[c];
                sc *= o;
                bb *= o;
            }
            sc_s[c] = sc;
            bb_s[c] = bb;
        }
        const uint32_t lane_base = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)c0;
        // every row slot starts at zero: the MMAs only accumulate
#pragma unroll
        for (int j = 0; j < ROWS; ++j)
#pragma unroll
            for (int u = 0; u < CPT / 16; ++u) tmem_st16_zero(lane_base + (uint32_t)(COUT * j + 16 * u));
        asm volatile("tcgen05.wait::st.sync.aligned;\n" ::: "memory");
        asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
        __syncwarp();
        if (lane == 0)
            for (int p = 0; p < NP; ++p)
                asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(s_addr(pairfree + p)) : "memory");
        asm volatile("bar.sync 1, 256;\n" ::: "memory");
        float sc_r[16], bb_r[16];               // the piece's scales and biases (kept when CPT = 16)
#pragma unroll
        for (int j = 0; j < 16; ++j) {
            sc_r[j] = sc_s[c0 + j];
            bb_r[j] = bb_s[c0 + j];
        }
        const bool pooling = a.pool.p != nullptr;
        uint32_t pf_ph = 0;   // bit p: parity of the next phase of pairfull[p]
        bool ok = true;
        for (int t = blockIdx.x; t < tl.total && ok; t += gridDim.x) {
            const int sx = t % tl.tiles_x, rest = t / tl.tiles_x;
            const int sy = rest % tl.tiles_y, b = rest / tl.tiles_y;
            const int yb = sy * ROWS;
            const int nrows = min(ROWS, a.H - yb);
            const int px = sx * kTcM + q * 32 + lane;
            const bool valid = px < a.W;
            for (int p = 0; 2 * p < nrows; ++p) {
                int ready = 0;
                if (lane == 0) ready = mbar_wait(s_addr(pairfull + p), (pf_ph >> p) & 1u, abort_flag, wait_ns) ? 1 : 0;
                ready = __shfl_sync(0xffffffffu, ready, 0);
                pf_ph ^= 1u << p;
                if (!ready) {
                    if (lane == 0) give_up(abort_flag, err);
                    ok = false;
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
                const bool two = 2 * p + 1 < nrows;
                const int y = yb + 2 * p;   // even: strips start on multiples of 4
                bf16* yp0 = a.y.p + a.y.at(b, valid ? (size_t)y * a.W + px : 0, 0);
                bf16* yp1 = a.y.p + a.y.at(b, valid && two ? (size_t)(y + 1) * a.W + px : 0, 0);
                if constexpr (MODE == 3) {
                    // the head with the kernel apply: group g takes row 2p + g with all 32 logits
                    const int r = 2 * p + grp;
                    const uint32_t ta = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(COUT * (ROWS - 1 - r));
                    uint32_t v[32];
                    tmem_ld16(ta, v);
                    tmem_ld16(ta + 16, v + 16);
                    asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
                    tmem_st16_zero(ta);
                    tmem_st16_zero(ta + 16);
                    if (r < nrows && valid) head_apply_px(a, v, sc_s, bb_s, yb + r, px);
                } else {
#pragma unroll
                for (int u = 0; u < CPT / 16; ++u) {
                    const int cb = c0 + 16 * u;   // first channel of this piece
                    if (CPT > 16) {
#pragma unroll
                        for (int j = 0; j < 16; ++j) {
                            sc_r[j] = sc_s[cb + j];
                            bb_r[j] = bb_s[cb + j];
                        }
                    }
                    const uint32_t ta0 = lane_base + (uint32_t)(COUT * (ROWS - 1 - 2 * p) + 16 * u);   // row 2p
                    const uint32_t ta1 = ta0 - (uint32_t)COUT;                                         // row 2p + 1
                    uint32_t v0[16], v1[16];
                    tmem_ld16(ta0, v0);
                    tmem_ld16(ta1, v1);
                    asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
                    tmem_st16_zero(ta0);
                    tmem_st16_zero(ta1);
                    uint4 o0[NVG], o1[NVG], om[NVG];
                    if (pooling) {
                        // the 2x2 mean of the activations in FP32 (H is even when pooling, so the pair is whole)
                        float f0[16], f1[16];
                        act16<MODE>(v0, sc_r, bb_r, f0);
                        act16<MODE>(v1, sc_r, bb_r, f1);
                        pack16<OUT8>(f0, o0);
                        pack16<OUT8>(f1, o1);
#pragma unroll
                        for (int j = 0; j < 16; ++j) {
                            const float m = f0[j] + f1[j];
                            f0[j] = (m + __shfl_down_sync(0xffffffffu, m, 1)) * 0.25f;
                        }
                        pack16<OUT8>(f0, om);
                    } else {
                        epilogue16<MODE, OUT8>(v0, sc_r, bb_r, o0);
                        epilogue16<MODE, OUT8>(v1, sc_r, bb_r, o1);
                    }
#pragma unroll
                    for (int g = 0; g < NVG; ++g) {
                        const int k = cb / (OUT8 ? 16 : 8) + g;   // 16-byte vector of the pixel
                        if (valid) *reinterpret_cast<uint4*>(yp0 + (size_t)k * (size_t)a.y.grp) = o0[g];
                        if (valid && two) *reinterpret_cast<uint4*>(yp1 + (size_t)k * (size_t)a.y.grp) = o1[g];
                        if (pooling && valid && (lane & 1) == 0)
                            *reinterpret_cast<uint4*>(a.pool.p +
                                                      a.pool.at(b, (size_t)(y / 2) * (a.W / 2) + px / 2, k)) = om[g];
                    }
                }
                }
                asm volatile("tcgen05.wait::st.sync.aligned;\n" ::: "memory");
                asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
                __syncwarp();
                if (lane == 0)
                    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(s_addr(pairfree + p)) : "memory");
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    if (warp == 1)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(S::TMEM_COLS)
                     : "memory");
}

// ---------------------------------------------------------------- host side

static PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    });
    return fn;
}

static int sm_count() {
    int dev = 0, n = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
    return n;
}

template <int CIN, int COUT, int MODE, bool F8, bool OUT8>
static cudaError_t run_tc(const ConvArgs& a, int* err, cudaStream_t s) {
    using S = TcShape<CIN, COUT, F8>;
    constexpr cuuint64_t EB = F8 ? 1 : 2;   // bytes per element
    const CUtensorMapDataType dt = F8 ? CU_TENSOR_MAP_DATA_TYPE_UINT8 : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16;
    if (a.pool.p && (!view_ok(a.pool) || S::R % 2 != 0 || COUT > 64 || (a.H | a.W) & 1)) return cudaErrorInvalidValue;
    auto encode = encode_fn();
    if (!encode) return cudaErrorNotSupported;
    const CUtensorMapSwizzle swz = S::ROWB == 64 ? CU_TENSOR_MAP_SWIZZLE_64B : CU_TENSOR_MAP_SWIZZLE_32B;
    CUtensorMap mx, mw;
    const cuuint32_t one[4] = {1, 1, 1, 1};
    // NHWC input view: {CIN channels, W, H, B}, box {KC, 130, R + 2, 1} (channels past CIN read as zero)
    const cuuint64_t xdim[4] = {(cuuint64_t)CIN, (cuuint64_t)a.W, (cuuint64_t)a.H, (cuuint64_t)a.B};
    const cuuint64_t xstr[3] = {(cuuint64_t)a.x.pix * 2, (cuuint64_t)a.x.pix * a.W * 2, (cuuint64_t)a.x.img * 2};
    const cuuint32_t xbox[4] = {(cuuint32_t)S::KC, (cuuint32_t)kHaloPix, (cuuint32_t)S::HALO_ROWS, 1};
    if (encode(&mx, dt, 4, (void*)a.x.p, xdim, xstr, xbox, one, CU_TENSOR_MAP_INTERLEAVE_NONE, swz,
               CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
        return cudaErrorInvalidValue;
    // weights [COUT][9][CIN] viewed as {CIN channels, COUT, 9 taps}, box {KC, COUT, 9}
    const cuuint64_t wdim[3] = {(cuuint64_t)CIN, (cuuint64_t)COUT, 9};
    const cuuint64_t wstr[2] = {(cuuint64_t)9 * CIN * EB, (cuuint64_t)CIN * EB};
    const cuuint32_t wbox[3] = {(cuuint32_t)S::KC, (cuuint32_t)COUT, 9};
    if (encode(&mw, dt, 3, (void*)a.w, wdim, wstr, wbox, one,
               CU_TENSOR_MAP_INTERLEAVE_NONE, swz, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
        return cudaErrorInvalidValue;
    TcTiles tl;
    tl.tiles_x = (a.W + kTcM - 1) / kTcM;
    tl.tiles_y = (a.H + S::R - 1) / S::R;
    const long long total = (long long)tl.tiles_x * tl.tiles_y * a.B;
    if (total > 0x7fffffffLL) return cudaErrorInvalidValue;
    tl.total = (int)total;
    const int sms = sm_count();
    if (sms <= 0) return cudaErrorInvalidDevice;
    auto kern = conv3x3_tc_kernel<CIN, COUT, MODE, F8, OUT8>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)S::SMEM);
    if (e != cudaSuccess) return e;
    const int grid = tl.total < sms ? tl.total : sms;
    return launch_pdl(kern, dim3(grid), dim3(kThreads), S::SMEM, s, mx, mw, a, tl, err);
}

template <int CIN, int COUT, int MODE, bool F8, bool OUT8>
static cudaError_t run_rs(const ConvArgs& a, int* err, cudaStream_t s) {
    constexpr int ROWS_ = rs_rows<CIN, F8, COUT>();
    static_assert(ROWS_ > 0, "row-streaming shape does not fit");
    using S = RsShape<CIN, F8, ROWS_, COUT>;
    constexpr cuuint64_t EB = F8 ? 1 : 2;   // bytes per element
    const CUtensorMapDataType dt = F8 ? CU_TENSOR_MAP_DATA_TYPE_UINT8 : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16;
    if (a.pool.p && (!view_ok(a.pool) || (a.H | a.W) & 1)) return cudaErrorInvalidValue;
    auto encode = encode_fn();
    if (!encode) return cudaErrorNotSupported;
    const CUtensorMapSwizzle swz = S::ROWB == 128 ? CU_TENSOR_MAP_SWIZZLE_128B
                                   : S::ROWB == 64 ? CU_TENSOR_MAP_SWIZZLE_64B : CU_TENSOR_MAP_SWIZZLE_32B;
    CUtensorMap mx, mw;
    const cuuint32_t one[4] = {1, 1, 1, 1};
    // NHWC input view: {CIN channels, W, H, B}, box {KC, 130, 2 rows, 1} (channels past CIN read as zero)
    const cuuint64_t xdim[4] = {(cuuint64_t)CIN, (cuuint64_t)a.W, (cuuint64_t)a.H, (cuuint64_t)a.B};
    const cuuint64_t xstr[3] = {(cuuint64_t)a.x.pix * 2, (cuuint64_t)a.x.pix * a.W * 2, (cuuint64_t)a.x.img * 2};
    const cuuint32_t xbox[4] = {(cuuint32_t)S::KC, (cuuint32_t)kHaloPix, (cuuint32_t)S::HPS, 1};
    if (encode(&mx, dt, 4, (void*)a.x.p, xdim, xstr, xbox, one, CU_TENSOR_MAP_INTERLEAVE_NONE, swz,
               CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
        return cudaErrorInvalidValue;
    // weights [COUT][ky][kx][CIN] viewed as {CIN channels, COUT n, 3 ky, 3 kx}, box {KC, COUT, 3, 3} -> [kx][ky][n][KC]
    const cuuint64_t wdim[4] = {(cuuint64_t)CIN, (cuuint64_t)COUT, 3, 3};
    const cuuint64_t wstr[3] = {(cuuint64_t)9 * CIN * EB, (cuuint64_t)3 * CIN * EB, (cuuint64_t)CIN * EB};
    const cuuint32_t wbox[4] = {(cuuint32_t)S::KC, (cuuint32_t)COUT, 3, 3};
    if (encode(&mw, dt, 4, (void*)a.w, wdim, wstr, wbox, one,
               CU_TENSOR_MAP_INTERLEAVE_NONE, swz, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
        return cudaErrorInvalidValue;
    TcTiles tl;
    tl.tiles_x = (a.W + kTcM - 1) / kTcM;
    tl.tiles_y = (a.H + S::ROWS - 1) / S::ROWS;
    const long long total = (long long)tl.tiles_x * tl.tiles_y * a.B;
    if (total > 0x7fffffffLL) return cudaErrorInvalidValue;
    tl.total = (int)total;
    const int sms = sm_count();
    if (sms <= 0) return cudaErrorInvalidDevice;
    auto kern = conv3x3_rs_kernel<CIN, MODE, F8, OUT8, ROWS_, COUT>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)S::SMEM);
    if (e != cudaSuccess) return e;
    const int grid = tl.total < sms * S::CTAS ? tl.total : sms * S::CTAS;
    return launch_pdl(kern, dim3(grid), dim3(kRsThreads), S::SMEM, s, mx, mw, a, tl, err);
}

// 32- and 64-channel outputs take the row-streaming kernel where its resident
// weights fit in shared memory, the others the 9-tap kernel.
template <int CIN, int COUT, bool F8, bool OUT8>
static cudaError_t run_shape(int mode, const ConvArgs& a, int* err, cudaStream_t s) {
    if constexpr (rs_rows_any<CIN, F8, COUT>() > 0) {
        if (mode == 0) return run_rs<CIN, COUT, 0, F8, OUT8>(a, err, s);
        if (mode == 1) return run_rs<CIN, COUT, 1, F8, OUT8>(a, err, s);
        return run_rs<CIN, COUT, 2, F8, OUT8>(a, err, s);
    } else {
        if (mode == 0) return run_tc<CIN, COUT, 0, F8, OUT8>(a, err, s);
        if (mode == 1) return run_tc<CIN, COUT, 1, F8, OUT8>(a, err, s);
        return run_tc<CIN, COUT, 2, F8, OUT8>(a, err, s);
    }
}

cudaError_t conv3x3_tc(int cin, int cout, int mode, const ConvArgs& a, int* err, cudaStream_t s) {
    // TMA: 16-byte aligned base addresses and strides; the input's channels contiguous (NHWC view)
    if (!err || !view_ok(a.x) || !view_ok(a.y) || a.x.grp != 8 || (((uintptr_t)a.w) & 15) || a.B < 1 || a.H < 1 ||
        a.W < 1)
        return cudaErrorInvalidValue;
#define SGI_TC_CASE(CI, CO)                                                  \
    if (cin == CI && cout == CO) return run_shape<CI, CO, false, false>(mode, a, err, s);
    SGI_TC_CASE(16, 32)
    SGI_TC_CASE(32, 32)
    SGI_TC_CASE(32, 64)
    SGI_TC_CASE(64, 64)
    SGI_TC_CASE(64, 128)
    SGI_TC_CASE(128, 128)
    SGI_TC_CASE(192, 64)
    SGI_TC_CASE(96, 32)
    SGI_TC_CASE(64, 32)
    SGI_TC_CASE(128, 64)
    SGI_TC_CASE(64, 192)
    SGI_TC_CASE(32, 96)
#undef SGI_TC_CASE
    return cudaErrorInvalidValue;
}

cudaError_t conv3x3_head_apply(const ConvArgs& a, int* err, cudaStream_t s) {
    const ConvArgs::ApplyFuse& f = a.fuse;
    if (!err || !view_ok(a.x) || a.x.grp != 8 || (((uintptr_t)a.w) & 15) || !a.bias || a.B != 1 || a.H < 1 ||
        a.W < 1 || !f.noisy || !f.prev || !f.screen || !f.albedo || !f.hdr || !f.gi_out || !f.hist_out)
        return cudaErrorInvalidValue;
    return run_rs<32, 32, 3, false, false>(a, err, s);
}

cudaError_t conv3x3_tc_fp8(int cin, int cout, int mode, bool in8, bool out8, const ConvArgs& a, int* err,
                           cudaStream_t s) {
    // FP8 tensors use BF16-unit views (two channels per unit): 16-byte vectors hold 16 channels
    if (!err || !view_ok(a.x) || !view_ok(a.y) || a.x.grp != 8 || (((uintptr_t)a.w) & 15) || (in8 && !a.wscale) ||
        a.B < 1 || a.H < 1 || a.W < 1 || (out8 && !a.oinv) || (mode != 2 && !a.bias) || (!in8 && !out8))
        return cudaErrorInvalidValue;
    // BF16 operands with an E4M3 output: the first layer, whose input features keep BF16
    if (!in8) {
        if (cin == 16 && cout == 32) return run_shape<16, 32, false, true>(mode, a, err, s);
        return cudaErrorInvalidValue;
    }
#define SGI_TC8_CASE(CI, CO)                                                         \
    if (cin == CI && cout == CO)                                                     \
        return out8 ? run_shape<CI, CO, true, true>(mode, a, err, s) : run_shape<CI, CO, true, false>(mode, a, err, s);
    SGI_TC8_CASE(16, 32)
    SGI_TC8_CASE(32, 32)
    SGI_TC8_CASE(32, 64)
    SGI_TC8_CASE(64, 64)
    SGI_TC8_CASE(64, 128)
    SGI_TC8_CASE(128, 128)
    SGI_TC8_CASE(192, 64)
    SGI_TC8_CASE(96, 32)
#undef SGI_TC8_CASE
    return cudaErrorInvalidValue;
}

// ------------------------------------------------------- weight gradients
//
// dw[co][t][ci] = sum over pixels p of dz[p][co] * x[p + off(t)][ci], a GEMM
// with the pixels as its reduction dimension. One tcgen05.mma accumulator per
// tap: D_t[m][n] (M = 128 rows for the output channels, zero past COUT; N = CC
// input channels of the CTA's group) += A[m][k] * B_t[n][k] over 16-pixel K
// steps, both operands K-major with the 64-byte swizzle (a row is 32 pixels of
// one channel, 64 bytes). The operands are transposes of the NHWC tensors, so
// the producers build them: a stage is 32 pixels of one image row (pixels past
// the row end are zero); each producer thread loads 8 pixels x 8 channels
// (eight 16-byte loads, zero outside the image for the shifted taps),
// transposes them in registers and stores 8 channel rows of 16 bytes at the
// swizzled chunk (the tensor core reads the swizzle from absolute addresses;
// each operand block starts on a 512-byte boundary). Roles (288 threads):
// warps 0..7 produce the stages (4-stage ring) and afterwards read the
// accumulators; warp 8 issues the MMAs and commits each stage back.
//
// A CTA owns one group of CC input channels and one contiguous slice of the
// image-row segments; it writes its sums to part[slice][co][t][ci], and a
// second kernel adds the slices in a fixed order to dw. The bias gradient
// (the per-channel sums of dz) comes from the producers of the A operand, which
// load every dz value of the slice anyway: part[slice][COUT * 9 * CIN + co],
// added by the same kernel into the bias that follows the weights. No atomics:
// the gradients are the same on every run.
constexpr int kWgSeg = 32;          // pixels per stage (one 64-byte K-major row)
constexpr int kWgStages = 4;
constexpr int kWgThreads = 288;
constexpr int kWgMaxSlices = 152;

template <int CC> struct WgShape {
    static constexpr int A_BYTES = 128 * 64;
    static constexpr int B_BYTES = 9 * CC * 64;
    static constexpr int STAGE = round_up(A_BYTES + B_BYTES, 1024);
    static constexpr int TMEM_COLS = pow2_cols(9 * CC);
    // CTAs that together would ask for more than the 512 TMEM columns of an SM do not share one
    static constexpr int SMEM_NEED = kWgStages * STAGE + 1024 /* alignment */ + 256 /* barriers */;
    static constexpr int SMEM = TMEM_COLS > 256 && SMEM_NEED < 120 * 1024 ? 120 * 1024 : SMEM_NEED;
};

__device__ __forceinline__ uint32_t perm(uint32_t a, uint32_t b, uint32_t sel) { return __byte_perm(a, b, sel); }

// r[i] = 8 channels of pixel i (16 bytes) -> o[c] = channel c of the 8 pixels
__device__ __forceinline__ void transpose8x8(const uint4* r, uint4* o) {
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const uint32_t w0 = (&r[0].x)[j], w1 = (&r[1].x)[j], w2 = (&r[2].x)[j], w3 = (&r[3].x)[j];
        const uint32_t w4 = (&r[4].x)[j], w5 = (&r[5].x)[j], w6 = (&r[6].x)[j], w7 = (&r[7].x)[j];
        o[2 * j] = make_uint4(perm(w0, w1, 0x5410), perm(w2, w3, 0x5410), perm(w4, w5, 0x5410), perm(w6, w7, 0x5410));
        o[2 * j + 1] =
            make_uint4(perm(w0, w1, 0x7632), perm(w2, w3, 0x7632), perm(w4, w5, 0x7632), perm(w6, w7, 0x7632));
    }
}

// row `row` (64 bytes, 32 pixels) of a K-major 64-byte-swizzled operand block, 16-byte chunk `chunk`
__device__ __forceinline__ uint4* sw64(unsigned char* block, int row, int chunk) {
    return reinterpret_cast<uint4*>(block + row * 64 + ((chunk ^ ((row >> 1) & 3)) << 4));
}

template <int CC>
__global__ void __launch_bounds__(kWgThreads, 1) wgrad_tc_kernel(WgradArgs a, int slices, int segs_per_row) {
    using S = WgShape<CC>;
    extern __shared__ unsigned char smem_raw[];
    unsigned char* smem =
        reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
    unsigned char* ctrl = smem + (size_t)kWgStages * S::STAGE;
    uint64_t* full = reinterpret_cast<uint64_t*>(ctrl);     // [stages], one arrival per producer warp
    uint64_t* empty = full + kWgStages;                      // [stages], tcgen05.commit
    uint64_t* done = empty + kWgStages;                      // accumulators complete
    uint64_t* drain = done + 1;
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(drain + 1);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int group = blockIdx.x % (a.cin / CC), slice = blockIdx.x / (a.cin / CC);
    const int ci0 = group * CC;
    const long long nseg = (long long)a.B * a.H * segs_per_row;
    const long long seg0 = nseg * slice / slices, seg1 = nseg * (slice + 1) / slices;
    const int nst = (int)(seg1 - seg0);
    const unsigned long long wait_ns = a.wait_ns ? a.wait_ns : kWaitNs;

    if (warp == 8) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(s_addr(tmem_slot)),
                     "r"(S::TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
    }
    if (tid == 0) {
        for (int s = 0; s < kWgStages; ++s) {
            mbar_init(s_addr(full + s), 8);
            mbar_init(s_addr(empty + s), 1);
        }
        mbar_init(s_addr(done), 1);
        mbar_init(s_addr(drain), 1);
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    // rows COUT..127 of every stage's A block stay zero
    for (int s = 0; s < kWgStages; ++s)
        for (int i = a.cout * 4 + tid; i < 128 * 4; i += kWgThreads)
            reinterpret_cast<uint4*>(smem + (size_t)s * S::STAGE)[i] = make_uint4(0u, 0u, 0u, 0u);
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    const uint32_t tmem = *tmem_slot;
    const uint32_t smem_base = s_addr(smem);

    if (warp < 8) {
        // ------------------------------------------------ producers
        // item it < 9 * CC / 2: B block of tap it / (CC / 2), channels ((it / 4) % (CC / 8)) * 8, pixels (it % 4) * 8;
        // then A: output channels ((it - nb) / 4) * 8, pixels (it % 4) * 8
        constexpr int NB = 9 * (CC / 8) * 4;
        const int na = a.cout / 2;
        const int it = tid;
        int s = 0;
        uint32_t ph = 0;
        bool ok = true;
        float bsum[8] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};   // A items: this thread's pixels of dz
        for (int st = 0; st < nst && !a.skip_producer; ++st) {
            int free_ = 0;
            if (lane == 0) free_ = mbar_wait(s_addr(empty + s), ph ^ 1u, abort_flag, wait_ns) ? 1 : 0;
            free_ = __shfl_sync(0xffffffffu, free_, 0);
            if (!free_) { ok = false; break; }
            const long long sg = seg0 + st;
            const int xs = (int)(sg % segs_per_row) * kWgSeg;
            const long long rowi = sg / segs_per_row;
            const int y = (int)(rowi % a.H), b = (int)(rowi / a.H);
            unsigned char* stage = smem + (size_t)s * S::STAGE;
            if (it < NB + na) {
                uint4 r[8], o[8];
                const int p8 = it & 3;
                if (it < NB) {
                    const int tap = it / (4 * (CC / 8)), c8 = (it / 4) % (CC / 8);
                    const int yy = y + tap / 3 - 1, dx = tap % 3 - 1;
                    const bool row_ok = yy >= 0 && yy < a.H;
#pragma unroll
                    for (int i = 0; i < 8; ++i) {
                        const int x = xs + p8 * 8 + i, xx = x + dx;
                        r[i] = make_uint4(0u, 0u, 0u, 0u);
                        if (row_ok && x < a.W && xx >= 0 && xx < a.W)
                            r[i] = __ldg(reinterpret_cast<const uint4*>(
                                a.x.p + a.x.at(b, (size_t)yy * a.W + xx, 0) + ci0 + c8 * 8));
                    }
                    transpose8x8(r, o);
                    unsigned char* blk = stage + S::A_BYTES + tap * CC * 64;
#pragma unroll
                    for (int c = 0; c < 8; ++c) *sw64(blk, c8 * 8 + c, p8) = o[c];
                } else {
                    const int o8 = (it - NB) / 4;
#pragma unroll
                    for (int i = 0; i < 8; ++i) {
                        const int x = xs + p8 * 8 + i;
                        r[i] = make_uint4(0u, 0u, 0u, 0u);
                        if (x < a.W)
                            r[i] = __ldg(reinterpret_cast<const uint4*>(
                                a.dz.p + a.dz.at(b, (size_t)y * a.W + x, 0) + o8 * 8));
                    }
                    transpose8x8(r, o);
#pragma unroll
                    for (int c = 0; c < 8; ++c) *sw64(stage, o8 * 8 + c, p8) = o[c];
                    // the bias gradient: the same dz values summed per channel, pixel by pixel
#pragma unroll
                    for (int i = 0; i < 8; ++i) {
                        float f[8];
                        bf8_unpack(r[i], f);
#pragma unroll
                        for (int c = 0; c < 8; ++c) bsum[c] += f[c];
                    }
                }
            }
            asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
            __syncwarp();
            if (lane == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(s_addr(full + s)) : "memory");
            if (++s == kWgStages) { s = 0; ph ^= 1u; }
        }
        if (!ok && lane == 0) give_up(abort_flag, a.err);
        // bias partial sums of the slice: the four threads of an output-channel octet (lanes 4j .. 4j + 3,
        // pixels p8 = 0..3 of every stage) combine theirs in a fixed order; the group-0 CTA writes them
        // after the slice's weight sums
#pragma unroll
        for (int c = 0; c < 8; ++c) {
            bsum[c] += __shfl_xor_sync(0xffffffffu, bsum[c], 1);
            bsum[c] += __shfl_xor_sync(0xffffffffu, bsum[c], 2);
        }
        if (group == 0 && it >= NB && it < NB + na && (it & 3) == 0) {
            float* pb = a.part + ((size_t)slice * (a.cout * 9 * a.cin + a.cout)) + (size_t)a.cout * 9 * a.cin +
                        (it - NB) / 4 * 8;
#pragma unroll
            for (int c = 0; c < 8; ++c) pb[c] = bsum[c];
        }
        // ------------------------------------------------ accumulators -> partial sums
        int ready = 0;
        if (lane == 0) ready = mbar_wait(s_addr(done), 0, abort_flag, wait_ns) ? 1 : 0;
        ready = __shfl_sync(0xffffffffu, ready, 0);
        if (ready) {
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
            const int q = warp & 3, co = q * 32 + lane;
            constexpr int NCOL = (9 * CC + 31) / 32;   // 32-column chunks (CC = 16: the last one half used)
            float* prow = a.part + (size_t)slice * (a.cout * 9 * a.cin + a.cout) + (size_t)(co < a.cout ? co : 0) * 9 * a.cin;
            for (int cchunk = warp >> 2; cchunk < NCOL; cchunk += 2) {
                uint32_t v[32];
                tmem_ld32(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(cchunk * 32), v);
                asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
                if (co < a.cout) {
#pragma unroll
                    for (int j = 0; j < 32; ++j) {
                        const int col = cchunk * 32 + j;
                        if (col < 9 * CC) prow[(size_t)(col / CC) * a.cin + ci0 + col % CC] = __uint_as_float(v[j]);
                    }
                }
            }
        } else if (lane == 0) {
            give_up(abort_flag, a.err);
        }
    } else if (lane == 0) {
        // ------------------------------------------------ MMA issuer
        constexpr uint32_t IDESC = instr_desc(128, CC, false);
        constexpr uint32_t HI = (uint32_t)((8 * 64) >> 4) | (1u << 14) | (4u << 29);   // SBO 512 B, 64B swizzle
        int s = 0;
        uint32_t ph = 0;
        bool ok = true, issued = false;
        for (int st = 0; st < nst; ++st) {
            if (!mbar_wait(s_addr(full + s), ph, abort_flag, wait_ns)) { ok = false; break; }
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
            const uint32_t base = smem_base + s * S::STAGE;
            const uint32_t a_lo = ((base >> 4) & 0x3FFFu) | (1u << 16);
            const uint32_t b_lo = (((base + S::A_BYTES) >> 4) & 0x3FFFu) | (1u << 16);
#pragma unroll
            for (int tap = 0; tap < 9; ++tap) {
#pragma unroll
                for (int ks = 0; ks < 2; ++ks) {
                    const uint32_t av = a_lo + (uint32_t)((ks * 32) >> 4);
                    const uint32_t bv = b_lo + (uint32_t)((tap * CC * 64 + ks * 32) >> 4);
                    umma<false>(tmem + (uint32_t)(tap * CC), av, bv, HI, IDESC, (st > 0 || ks > 0) ? 1u : 0u);
                }
            }
            issued = true;
            mma_commit(s_addr(empty + s));
            if (++s == kWgStages) { s = 0; ph ^= 1u; }
        }
        if (ok) mma_commit(s_addr(done));   // every slice has at least one stage
        if (!ok) {
            give_up(abort_flag, a.err);
            if (issued) {
                mma_commit(s_addr(drain));
                const unsigned long long deadline = global_ns() + wait_ns;
                while (!mbar_test(s_addr(drain), 0) && global_ns() < deadline) {
                }
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    if (warp == 8)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(S::TMEM_COLS)
                     : "memory");
}

// dw[e] += sum over slices j = 0 .. slices-1 of part[j][e], in that order
__global__ void wgrad_reduce_kernel(const float* __restrict__ part, int slices, size_t n, float* __restrict__ dw) {
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
        float acc = 0.0f;
#pragma unroll 8
        for (int j = 0; j < slices; ++j) acc += __ldg(part + (size_t)j * n + e);
        dw[e] += acc;
    }
}

static int wgrad_slices(int cin, int cout) {
    const int groups = cin / (cin % 32 == 0 ? 32 : 16);
    const int sl = kWgMaxSlices / groups;
    (void)cout;
    return sl < 1 ? 1 : sl;
}

size_t wgrad_part_floats(int cin, int cout) { return (size_t)wgrad_slices(cin, cout) * (cout * 9 * cin + cout); }

template <int CC>
static cudaError_t run_wgrad(const WgradArgs& a, cudaStream_t s) {
    using S = WgShape<CC>;
    const int segs_per_row = (a.W + kWgSeg - 1) / kWgSeg;
    const long long nseg = (long long)a.B * a.H * segs_per_row;
    int slices = wgrad_slices(a.cin, a.cout);
    if (slices > nseg) slices = (int)nseg;
    const size_t n = (size_t)a.cout * 9 * a.cin + a.cout;   // weights, then the bias
    if ((size_t)slices * n > a.part_floats) return cudaErrorInvalidValue;
    auto kern = wgrad_tc_kernel<CC>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, S::SMEM);
    if (e != cudaSuccess) return e;
    kern<<<(a.cin / CC) * slices, kWgThreads, S::SMEM, s>>>(a, slices, segs_per_row);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    wgrad_reduce_kernel<<<(int)((n + 255) / 256), 256, 0, s>>>(a.part, slices, n, a.dw);
    return cudaGetLastError();
}

cudaError_t wgrad(const WgradArgs& a, cudaStream_t s) {
    // 16-byte loads of 8 channels: NHWC views (channels contiguous), 16-channel groups
    if (!view_ok(a.x) || !view_ok(a.dz) || a.x.grp != 8 || a.dz.grp != 8 || !a.part || !a.err || a.cin % 16 ||
        a.cout % 8 || a.cout > 128 || a.B < 1 || a.H < 1 || a.W < 1)
        return cudaErrorInvalidValue;
    return a.cin % 32 == 0 ? run_wgrad<32>(a, s) : run_wgrad<16>(a, s);
}

}  // namespace nn
}  // namespace sgi
