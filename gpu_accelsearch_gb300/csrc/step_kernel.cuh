// step_kernel.cuh -- a launch group's power planes and harmonic sums in one
// persistent launch (k_step), the per-step work of AccelSearch.cu:203-247
// for every segment of the group.
//
// CTAs claim work items from one counter, in an order fixed by the group's
// size: for every segment j, its plane items (one template row of the
// largest segment length per item, or several rows of a smaller length
// side by side, each on its own named barrier) and, interleaved with the
// plane items of segment j + lag, the harmonic-sum tiles of segment j (the
// tiled sum of k_hsum_tile, same arithmetic).  A tile waits until every
// plane row of its segment is finished (a per-segment counter, release /
// acquire); those rows were all claimed before the tile, by CTAs that are
// running them and wait on nothing, so every wait ends.  Each wait is
// bounded all the same: a tile whose rows do not arrive within about 0.4 s
// sets bit 1 of the error word and is skipped; a tile whose copies do not
// land sets bit 0 and its CTA stops claiming.  The planes of a segment are
// summed shortly after they are written, while they are still in L2, and
// rows (FP32-bound) and tiles (memory-bound) of neighbouring segments run
// side by side on the SMs.
#pragma once

#include "search_kernels.cuh"

namespace accel {

// Index of the first item of block b (plane items of segment b, then the
// tiles of segment b - lag interleaved with them).
__device__ __forceinline__ long long step_block_start(const StepArgs& a, long long b) {
    const long long np = b < a.nseg ? b : a.nseg;
    const long long nt = b > a.lag ? b - a.lag : 0;
    return (long long)a.P * np + (long long)a.T * nt;
}

// kind 0: plane item idx of segment seg; kind 1: tile idx; -1: no work left.
struct StepItem {
    int kind, seg, idx;
};

__device__ __forceinline__ StepItem step_decode(const StepArgs& a, long long it) {
    StepItem r{-1, 0, 0};
    if (it >= a.nitems) return r;
    long long lo = 0, hi = (long long)a.nseg + a.lag;  // block: the last b with start(b) <= it
    while (hi - lo > 1) {
        const long long mid = (lo + hi) >> 1;
        if (step_block_start(a, mid) <= it) lo = mid;
        else hi = mid;
    }
    const long long b = lo, q = it - step_block_start(a, b);
    const long long np = b < a.nseg ? a.P : 0, nt = b >= a.lag ? a.T : 0;
    if (nt == 0) return StepItem{0, (int)b, (int)q};
    if (np == 0) return StepItem{1, (int)(b - a.lag), (int)q};
    // q spread evenly: tiles before position q = floor(q nt / (np + nt))
    const long long h0 = q * nt / (np + nt), h1 = (q + 1) * nt / (np + nt);
    if (h1 > h0) return StepItem{1, (int)(b - a.lag), (int)h0};
    return StepItem{0, (int)b, (int)(q - h0)};
}

// Rows [first, first + MMAX/M) of class c, M/16 threads per row.
template <int M, int MMAX, bool F16>
__device__ __forceinline__ void step_rows(const StepArgs& a, int c, int seg, int first, unsigned char* smem,
                                          const float2* __restrict__ tw) {
    constexpr int GT = M / 16, G = (MMAX / 16) / GT;
    static_assert(G == 1 || GT % 32 == 0, "named barriers need whole warps");
    const int g = threadIdx.x / GT, t = threadIdx.x % GT;
    const int row = first + g;
    if (row >= a.cls_ntpl[c]) return;  // the group's own barrier: nothing else waits for it
    int k = 0;
#pragma unroll 1
    while (k + 1 < a.cls_nh[c] && row >= a.cls_zbase[c][k + 1]) k++;
    const HarmPlan& H = a.hs.h[a.cls_h[c][k]];
    const int z = row - a.cls_zbase[c][k];
    const float2* __restrict__ D = a.dbuf + (long long)seg * a.dstride + H.doff;
    float* out = a.planes + (long long)seg * a.hs.pstride + H.poff + (long long)z * H.prow;
    float2* sm = reinterpret_cast<float2*>(smem) + (size_t)g * 2 * FftShape<M>::PADDED;
    float2 p[16];
    if constexpr (G == 1) plane_powers<M, F16, false>(H, D, z, sm, tw, p, t);
    else plane_powers<M, F16, false, GroupSync>(H, D, z, sm, tw, p, t, GroupSync{1 + g, GT});
    const int half_w = H.wmax >> 1;
#pragma unroll
    for (int e = 0; e < 16; e++) {
        const int i2 = t + e * GT - H.hw0;
        if (i2 >= 0 && i2 < half_w) *reinterpret_cast<float2*>(out + 2 * i2) = p[e];
    }
}

template <int MMAX, bool F16>
__device__ __forceinline__ int step_plane_item(const StepArgs& a, int seg, int pidx, unsigned char* smem,
                                               const float2* __restrict__ tw) {
    int c = 0;
#pragma unroll 1
    while (c + 1 < a.ncls && pidx >= a.cls_item0[c + 1]) c++;
    const int M = a.cls_M[c];
    const int per = MMAX / M;
    const int first = (pidx - a.cls_item0[c]) * per;
    if (M == MMAX) step_rows<MMAX, MMAX, F16>(a, c, seg, first, smem, tw);
    else if constexpr (MMAX / 2 >= 512) {
        if (M == MMAX / 2) step_rows<MMAX / 2, MMAX, F16>(a, c, seg, first, smem, tw);
        else if constexpr (MMAX / 4 >= 512) {
            if (M == MMAX / 4) step_rows<MMAX / 4, MMAX, F16>(a, c, seg, first, smem, tw);
            else if constexpr (MMAX / 8 >= 512) {
                if (M == MMAX / 8) step_rows<MMAX / 8, MMAX, F16>(a, c, seg, first, smem, tw);
            }
        }
    }
    return min(per, a.cls_ntpl[c] - first);
}

// Wait (thread 0) until *p >= target: acquire loads with the thread
// suspended between them; false after about 0.4 s.
__device__ __forceinline__ bool step_wait_count(const unsigned* p, unsigned target) {
#pragma unroll 1
    for (int it = 0; it < (1 << 22); it++) {
        unsigned v;
        asm volatile("ld.acquire.gpu.global.u32 %0, [%1];\n" : "=r"(v) : "l"(p) : "memory");
        if (v >= target) return true;
        __nanosleep(100);
    }
    return false;
}

template <int MMAX, int NH, bool F16>
__global__ void __launch_bounds__(MMAX / 16, 2) k_step(const StepArgs a, const float2* __restrict__ tw) {
    static_assert(MMAX / 16 == kTileI, "a tile takes one thread per column of the CTA");
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ __align__(16) TileShared<NH> S;
    __shared__ __align__(8) unsigned long long s_bar;
    __shared__ int s_item[4];
    const int tid = threadIdx.x;
    bool bar_init = true;
    unsigned parity = 0;
#pragma unroll 1
    for (;;) {
        if (tid == 0) {
            const StepItem w = step_decode(a, (long long)atomicAdd(a.next, 1u));
            s_item[0] = w.kind;
            s_item[1] = w.seg;
            s_item[2] = w.idx;
            s_item[3] = 1;
            if (w.kind == 1 && !step_wait_count(a.done + w.seg, (unsigned)a.rows)) {
                atomicOr(a.hs.err, 2ull);  // the segment's rows never arrived: skip the tile
                s_item[3] = 0;
            }
        }
        __syncthreads();
        const int kind = s_item[0], seg = s_item[1], idx = s_item[2], ok = s_item[3];
        if (kind < 0) break;
        if (kind == 0) {
            const int nrows = step_plane_item<MMAX, F16>(a, seg, idx, smem, tw);
            __threadfence();  // this thread's stores of the rows, before the count
            __syncthreads();
            if (tid == 0) atomicAdd(a.done + seg, (unsigned)nrows);
        } else {
            if (ok) {
                // the rows were written by other CTAs through the generic
                // proxy and this CTA's shared memory by its last plane item:
                // order both before the bulk copies (async proxy)
                if (tid < 32) asm volatile("fence.proxy.async;\n" ::: "memory");
                const int it = idx % a.nti, zt = idx / a.nti;
                if (!hsum_tile_body<NH, false>(a.hs, seg, zt * kTileZ, it * kTileI,
                                               reinterpret_cast<float*>(smem), S, &s_bar, bar_init, parity))
                    break;  // copies did not land: the barrier is unusable, stop claiming
                bar_init = false;
                parity ^= 1u;
            }
            __syncthreads();  // shared memory free for the next item
        }
    }
}

}  // namespace accel
