// sgi_cull.cuh - the culling passes of the GI stage as block-level device
// functions: the VPL visibility test and stable compaction
// (viscull_vpls.cs:47-120) and the two tile-culling stages
// (vpl_tiled_deferred_culling_stage1.cs:50-90, _stage2.cs:61-129).
//
// The kernels of sgi_kernels.cu launch them one pass per launch; the
// persistent multi-view kernel (sgi_persistent.cuh) runs them as work items.
// Every operation that decides a result is written with the correctly
// rounded x* operations of sgi_math.cuh, so the lists are identical in the
// exact and the tolerance build of the kernels that include this header.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "sgi_internal.h"
#include "sgi_math.cuh"
#include "sgi_shade_common.cuh"

namespace sgi {

// ------------------------------------------------------------- VPL cull --
// viscull_vpls.cs:63-75: a VPL is visible when the directional light's CSM
// does not shadow its position (1 - lit < 1).
SGI_D uint8_t vpl_visible(const sgi_vpl* __restrict__ vpls, int i, const sgi_csm& csm) {
    const float4 pos = __ldg(reinterpret_cast<const float4*>(vpls + i));
    const V3 p = v3(pos.x, pos.y, pos.z);
    const V3 L = v3(csm.light_direction[0], csm.light_direction[1], csm.light_direction[2]);
    const float shadowFactor = xsub(1.0f, infinite_shadow(csm, p, L, false));
    return shadowFactor < 1.0f ? 1 : 0;
}

// Stable compaction in ascending VPL index by one block of NT threads: ballot
// prefix within each warp, exclusive scan of the warp counts, running base
// across chunks of NT flags. Replaces the 8-thread atomicAdd loop of
// viscull_vpls.cs:85-98 (whose order is nondeterministic). With vpr given, the
// (position, radius) of each kept VPL is also written there for the tile cull.
// kCoherent: the flags were written by other blocks of the same launch, so they
// are read through L2 (ld.global.cg), not a read-only or L1 path.
template <int NT, bool kCoherent = false>
SGI_D void compact_vpls(const sgi_vpl* __restrict__ vpls, const sgi_atlas_entry* __restrict__ entries,
                        const uint8_t* __restrict__ flags, int n, int cap, sgi_vpl* __restrict__ cv,
                        sgi_atlas_entry* __restrict__ ce, int32_t* __restrict__ visible_index,
                        float4* __restrict__ vpr, int tid) {
    constexpr int kWarps = NT / 32;
    __shared__ int warp_count[kWarps];
    __shared__ int warp_base[kWarps];
    __shared__ int chunk_total;
    const int lane = tid & 31, warp = tid >> 5;
    int base = 0;
    for (int start = 0; start < n; start += NT) {
        const int i = start + tid;
        const bool f = i < n && (kCoherent ? __ldcg(flags + i) : flags[i]) != 0;
        const unsigned m = __ballot_sync(0xffffffffu, f);
        const int within = __popc(m & ((1u << lane) - 1u));
        if (lane == 0) warp_count[warp] = __popc(m);
        __syncthreads();
        if (warp == 0) {
            const int c = lane < kWarps ? warp_count[lane] : 0;
            int incl = c;
#pragma unroll
            for (int off = 1; off < 32; off <<= 1) {
                const int t = __shfl_up_sync(0xffffffffu, incl, off);
                if (lane >= off) incl += t;
            }
            if (lane < kWarps) warp_base[lane] = incl - c;
            if (lane == 31) chunk_total = incl;
        }
        __syncthreads();
        if (f) {
            const int k = base + warp_base[warp] + within;
            if (k < cap) {
                const float4* src = reinterpret_cast<const float4*>(vpls + i);
                float4* dst = reinterpret_cast<float4*>(cv + k);
                const float4 p = __ldg(src), c1 = __ldg(src + 1), c2 = __ldg(src + 2), c3 = __ldg(src + 3);
                dst[0] = p; dst[1] = c1; dst[2] = c2; dst[3] = c3;
                ce[k] = entries[i];
                visible_index[1 + k] = i;
                if (vpr) vpr[k] = make_float4(p.x, p.y, p.z, c3.x);
            }
        }
        base += chunk_total;
        __syncthreads();
    }
    if (tid == 0) visible_index[0] = base < cap ? base : cap;
}

// -------------------------------------------------------- tile stage 1 --
SGI_D float butterfly(float v) {
#pragma unroll
    for (int off = 16; off >= 1; off >>= 1) v = v + __shfl_xor_sync(0xffffffffu, v, off);
    return v;
}
// tile_size^2 = 32 x a power of two: sizes 8, 16, 32
__host__ __device__ __forceinline__ bool butterfly_tile_host(int ts) {
    const int n = ts * ts, nw = n >> 5;
    return (n & 31) == 0 && (nw & (nw - 1)) == 0;
}
SGI_D bool butterfly_tile(int ts) { return butterfly_tile_host(ts); }

// Per-tile mean world position and normalised mean normal, by the block of
// tile_size^2 threads (thread l = pixel l of the tile, row-major). For tile
// sizes 8, 16 and 32 the sums use the warp butterfly order (xor 16, 8, 4, 2,
// 1, then xor nw/2 .. 1 over the warp totals); otherwise (e.g. the reference's
// 5x5 tiles) thread 0 adds the pixels in their order in the tile, as
// vpl_tiled_deferred_culling_stage1.cs:73-81 does (seq: tile_size^2 x 6 floats
// of shared memory). Pixels outside the image add 0 and are left out of the
// count. The record is written by one thread to *out.
SGI_D void tile_mean(int W, int H, int ts, int tx, int ty, int l, const sgi_gbuffer& g, const sgi_camera& cam,
                     float* seq, sgi_tile_stage1* out) {
    __shared__ float wsum[32][6];
    const int nthreads = ts * ts;
    const int x = tx * ts + l % ts, y = ty * ts + l / ts;
    float v[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    if (x < W && y < H) {
        const size_t i = (size_t)y * W + x;
        const float u = xdiv(float(x) + 0.5f, float(W)), vv = xdiv(float(y) + 0.5f, float(H));
        const V3 p = world_from_depth(u, vv, __ldg(g.depth + i), cam.inv_proj_view);
        const V3 n = decode_normal(__ldg(g.normal + i));
        v[0] = p.x; v[1] = p.y; v[2] = p.z; v[3] = n.x; v[4] = n.y; v[5] = n.z;
    }
    float w[6];
    bool have = false;
    if (butterfly_tile(ts)) {
        const int lane = l & 31, warp = l >> 5, nw = nthreads >> 5;
#pragma unroll
        for (int c = 0; c < 6; ++c) v[c] = butterfly(v[c]);
        if (lane == 0) {
#pragma unroll
            for (int c = 0; c < 6; ++c) wsum[warp][c] = v[c];
        }
        __syncthreads();
        if (warp == 0) {
#pragma unroll
            for (int c = 0; c < 6; ++c) w[c] = lane < nw ? wsum[lane][c] : 0.0f;
            for (int off = nw >> 1; off >= 1; off >>= 1) {
#pragma unroll
                for (int c = 0; c < 6; ++c) w[c] = w[c] + __shfl_xor_sync(0xffffffffu, w[c], off);
            }
            have = lane == 0;
        }
    } else {
#pragma unroll
        for (int c = 0; c < 6; ++c) seq[l * 6 + c] = v[c];
        __syncthreads();
        if (l == 0) {
#pragma unroll
            for (int c = 0; c < 6; ++c) w[c] = 0.0f;
            for (int j = 0; j < nthreads; ++j) {
#pragma unroll
                for (int c = 0; c < 6; ++c) w[c] = w[c] + seq[j * 6 + c];
            }
            have = true;
        }
    }
    if (have) {
        const int cx = W - tx * ts < ts ? W - tx * ts : ts;
        const int cy = H - ty * ts < ts ? H - ty * ts : ts;
        const float cnt = float(cx * cy);
        const V3 ap = xdiv3(v3(w[0], w[1], w[2]), cnt);
        const V3 an = xnormalize(xdiv3(v3(w[3], w[4], w[5]), cnt));
        sgi_tile_stage1 o;
        o.average_position[0] = ap.x; o.average_position[1] = ap.y; o.average_position[2] = ap.z;
        o.average_position[3] = 1.0f;
        o.average_normal[0] = an.x; o.average_normal[1] = an.y; o.average_normal[2] = an.z;
        o.average_normal[3] = 1.0f;
        *out = o;
    }
}

// -------------------------------------------------------- tile stage 2 --
// vpl_tiled_deferred_culling_stage2.cs:61-129: for each tile the shader
// inserts the visible VPLs, in order, into a list sorted by key =
// distance / radius with a strict '<' (ties keep the earlier VPL) and keeps
// the first L. The result is the L smallest candidates by (key, index), in
// that order. One 256-thread block per tile computes that set with the keys
// in shared memory (nothing per (tile, VPL) reaches global memory):
//   1. every visible VPL's key (kNoKey when it is not a candidate) goes to
//      shared memory, and each candidate counts into a 256-bin histogram of
//      floor(ratio * 256) (ratio <= 1; the bins are ordered like the keys);
//   2. with more than L candidates, a block scan of the histogram finds the
//      bin b where the count reaches L: every candidate of a lower bin is
//      kept, and from bin b the need = L - (candidates below b) smallest by
//      (key, index), found by ranking bin b's members against each other;
//   3. the kept (key, index) pairs, at most 64, are sorted by one warp.
constexpr uint32_t kNoKey = 0xffffffffu;
constexpr int kCullThreads = 256;

SGI_D uint32_t order_key(float k) {     // float order -> uint order (-0 == +0)
    const uint32_t b = __float_as_uint(k == 0.0f ? 0.0f : k);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
SGI_D float key_value(uint32_t u) { return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u); }

// the histogram bin of a candidate's ratio (<= 1): non-decreasing in the ratio
SGI_D int ratio_bin(float ratio) {
    if (!(ratio > 0.0f)) return 0;
    const int b = (int)xmul(ratio, 256.0f);
    return b > 255 ? 255 : b;
}

SGI_D unsigned long long pair_key(uint32_t key, int index) {
    return ((unsigned long long)key << 32) | (uint32_t)index;
}

// One compare-exchange stage of a bitonic network over 64 elements held as
// k0 at position lane and k1 at position lane + 32.
SGI_D void bitonic_stage64(unsigned long long& k0, unsigned long long& k1, int size, int j, int lane) {
    const unsigned FULL = 0xffffffffu;
    if (j == 32) {   // partners are the two registers of this lane; size == 64 -> ascending
        if (k1 < k0) { const unsigned long long t = k0; k0 = k1; k1 = t; }
        return;
    }
#pragma unroll
    for (int r = 0; r < 2; ++r) {
        unsigned long long& k = r ? k1 : k0;
        const int pos = lane + 32 * r;
        const unsigned long long o = __shfl_xor_sync(FULL, k, j);
        const bool ascending = (pos & size) == 0;
        const bool lower = (pos & j) == 0;
        // the lower position keeps the min when ascending, the max otherwise
        if ((lower == ascending) ? (o < k) : (k < o)) k = o;
    }
}

// The list of one tile (mean position tp, mean normal tn) by a block of NT
// threads (128 or 256); cull_smem holds 2 x count uint32 (keys, bin members).
template <int NT = kCullThreads>
SGI_D void tile_cull(int L, V3 tp, V3 tn, const float4* __restrict__ vpr, int count, uint32_t* cull_smem,
                     int32_t* __restrict__ out, int tid) {
    static_assert(NT == 128 || NT == 256, "block size");
    constexpr int BPT = 256 / NT;   // histogram bins per thread
    __shared__ uint32_t hist[256];
    __shared__ unsigned long long kept[64];
    __shared__ int warp_sum[NT / 32];
    __shared__ int s_bin, s_need, s_nkept, s_nb, s_mc;
    const int lane = tid & 31, warp = tid >> 5;
    uint32_t* keys = cull_smem;
    uint32_t* members = cull_smem + count;
#pragma unroll
    for (int j = 0; j < BPT; ++j) hist[tid * BPT + j] = 0u;
    if (tid == 0) { s_nkept = 0; s_nb = 0; }
    __syncthreads();
    int mine = 0;
    for (int k = tid; k < count; k += NT) {
        const float4 v = __ldg(vpr + k);
        const V3 lmf = xsub3(v3(v.x, v.y, v.z), tp);
        const float side = xdot(tn, lmf);
        uint32_t u = kNoKey;
        if (!(side < 0.0f)) {
            const float ratio = xdiv(xlength(lmf), v.w);
            if (!(ratio > 1.0f) && ratio < kFloatMax) {
                u = order_key(ratio);
                ++mine;
                atomicAdd(&hist[ratio_bin(ratio)], 1u);
            }
        }
        keys[k] = u;
    }
    // candidates in the tile
    for (int off = 16; off >= 1; off >>= 1) mine += __shfl_xor_sync(0xffffffffu, mine, off);
    if (lane == 0) warp_sum[warp] = mine;
    __syncthreads();
    if (tid == 0) {
        int mc = 0;
        for (int w = 0; w < NT / 32; ++w) mc += warp_sum[w];
        s_mc = mc;
    }
    __syncthreads();
    const int mc = s_mc;
    const int take = mc < L ? mc : L;
    if (mc > L) {
        // inclusive scan of the histogram: bin b holds the L-th candidate (thread tid owns bins
        // tid * BPT .. + BPT - 1)
        uint32_t h[BPT], tot = 0;
#pragma unroll
        for (int j = 0; j < BPT; ++j) { h[j] = hist[tid * BPT + j]; tot += h[j]; }
        uint32_t incl = tot;
        for (int off = 1; off < 32; off <<= 1) {
            const uint32_t t = __shfl_up_sync(0xffffffffu, incl, off);
            if (lane >= off) incl += t;
        }
        if (lane == 31) warp_sum[warp] = (int)incl;
        __syncthreads();
        uint32_t run = incl - tot;   // candidates below this thread's first bin
        for (int w = 0; w < warp; ++w) run += (uint32_t)warp_sum[w];
#pragma unroll
        for (int j = 0; j < BPT; ++j) {
            if (run + h[j] >= (uint32_t)L && run < (uint32_t)L) { s_bin = tid * BPT + j; s_need = L - (int)run; }
            run += h[j];
        }
        __syncthreads();
    } else if (tid == 0) {
        s_bin = 256;   // every candidate is kept
        s_need = 0;
    }
    __syncthreads();
    const int bin = s_bin;
    // kept: candidates of lower bins; bin b's members are ranked below
    for (int k = tid; k < count; k += NT) {
        const uint32_t u = keys[k];
        if (u == kNoKey) continue;
        const int b = ratio_bin(key_value(u));
        if (b < bin) kept[atomicAdd(&s_nkept, 1)] = pair_key(u, k);
        else if (b == bin) members[atomicAdd(&s_nb, 1)] = (uint32_t)k;
    }
    __syncthreads();
    if (mc > L) {
        const int nb = s_nb, need = s_need;
        for (int m = tid; m < nb; m += NT) {
            const uint32_t k = members[m];
            const unsigned long long mk = pair_key(keys[k], (int)k);
            int rank = 0;
            for (int j = 0; j < nb; ++j) {
                const uint32_t kj = members[j];
                rank += pair_key(keys[kj], (int)kj) < mk ? 1 : 0;
            }
            if (rank < need) kept[atomicAdd(&s_nkept, 1)] = mk;
        }
        __syncthreads();
    }
    if (warp == 0) {
        unsigned long long k0 = lane < take ? kept[lane] : ~0ull;
        unsigned long long k1 = lane + 32 < take ? kept[lane + 32] : ~0ull;
        if (take > 1) {
            for (int size = 2; size <= 64; size <<= 1)
                for (int j = size >> 1; j >= 1; j >>= 1) bitonic_stage64(k0, k1, size, j, lane);
        }
        if (lane == 0) out[0] = take;
        if (lane < L) out[1 + lane] = lane < take ? (int32_t)(uint32_t)k0 : -1;
        if (lane + 32 < L) out[33 + lane] = lane + 32 < take ? (int32_t)(uint32_t)k1 : -1;
    }
    __syncthreads();   // the block's shared memory is free again when it returns
}

}  // namespace sgi
