// search_kernels.cuh -- the per-step hot path (kernel templates; the
// instantiations live in search_*.cu).
//
//  k_prep   generate_harmonic_ffdot_data + perform_fft_harmonics
//           (bpd_search.cu:130-184, :228-240): gather the local Fourier
//           amplitudes, median-normalise the first numdata bins exactly as
//           the reference does (same float operations, exact lower median),
//           and FFT.  The reference FFTs the x2 zero-interleaved segment of
//           L points; its spectrum is the M = L/2 point spectrum of the
//           un-spread segment repeated twice, so only that is computed.
//  k_plane  perform_convolution + perform_inversefft + generatePowers
//           (bpd_search.cu:243-307, bpd_gpu_kernels.cu:39-116) fused: per
//           template, multiply by the folded template spectrum, two M-point
//           inverse FFTs in shared memory (even and odd outputs of the
//           L-point inverse), |y|^2 / L^2 for the valid window, and one
//           store of the powers.  Nothing but powers reaches global memory.
//  k_hsum   perform_harmonic_summing / addPowers (bpd_search.cu:310-360,
//           bpd_gpu_kernels.cu:119-170) with the reference's index
//           arithmetic, cumulative stage sums in registers, and the
//           candidate threshold the reference leaves as a stub
//           (bpd_candidates.cu:4-9), compacted with warp ballots.
#pragma once

#include "accel_internal.h"
#include "fft_smem.cuh"

namespace accel {



// ------------------------------------------------------------------ prep
template <int M>
__global__ void __launch_bounds__(M / 16) k_prep(const PrepArgs a, const float2* __restrict__ tw) {
    constexpr int T = M / 16;
    constexpr int PM = FftShape<M>::PADDED;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float2* sm = reinterpret_cast<float2*>(smem_raw);
    uint32_t* keys = reinterpret_cast<uint32_t*>(sm + PM);
    __shared__ int hist[256];
    __shared__ int bc[2];
    __shared__ float s_norm;

    const HarmPlan& H = a.h[blockIdx.x];
    const SegDesc sd = a.segs[blockIdx.y];
    const StepHarm g = step_harm(sd.startr, a.uselen, H.p, H.q, H.hw0);
    const int t = threadIdx.x;
    const int numdata = g.numdata < M ? g.numdata : M;  // host checks numdata <= M

    float2 x[1][16];
#pragma unroll
    for (int e = 0; e < 16; e++) {
        const int idx = t + e * T;
        const long long b = g.lobin + idx;
        float2 v = make_float2(0.f, 0.f);
        if (b >= 0 && b < sd.numbins) v = sd.spec[b];
        x[0][e] = v;
        if (idx < numdata) keys[idx] = __float_as_uint(power_exact(v));
    }
    __syncthreads();
    const uint32_t mk = block_select_u32(keys, numdata, (numdata - 1) / 2, hist, bc);
    if (t == 0) s_norm = rsqrt_norm((float)((double)__uint_as_float(mk) / kLn2), a.exact_rsqrt);
    __syncthreads();
    const float norm = s_norm;
#pragma unroll
    for (int e = 0; e < 16; e++) {
        if (t + e * T < numdata) {
            x[0][e].x = __fmul_rn(x[0][e].x, norm);
            x[0][e].y = __fmul_rn(x[0][e].y, norm);
        }
    }
    fft_run<M, -1, 1>(x, sm, tw, t);
    float2* out = a.dbuf + (long long)blockIdx.y * a.dstride + H.doff;
#pragma unroll
    for (int e = 0; e < 16; e++) out[t + e * T] = x[0][e];
}

// ----------------------------------------------------------------- plane
// Two layouts of the same work (chosen per context, see accel_set_tuning),
// both M/16 threads carrying 16 points each:
//   SPLIT = false: each thread carries the even and the odd transform at
//                  once (two shared buffers, twiddles formed once for both,
//                  128 registers: 2 CTAs per SM);
//   SPLIT = true:  the even transform, then the odd one, through one
//                  shared buffer (fewer registers and half the shared
//                  memory: 3 CTAs per SM).
template <bool SPLIT, int M> struct PlaneShape {
    static constexpr int THREADS = M / 16;
    static constexpr int BUFFERS = SPLIT ? 1 : 2;
    static constexpr int MINB = SPLIT ? (THREADS <= 256 ? 3 : 1) : (THREADS <= 256 ? 2 : 1);
};

// Template z's folded spectrum (half 0: A, half 1: B) at frequency idx.
template <int M, bool F16>
__device__ __forceinline__ float2 fold_at(const HarmPlan& H, int z, int half, int idx) {
    if constexpr (F16) {
        float2 w = __half22float2(H.fold16[(size_t)z * 2 * M + half * M + idx]);
        const float sc = H.f16scale[z];
        w.x *= sc;
        w.y *= sc;
        return w;
    } else {
        return __ldg(H.fold + (size_t)z * 2 * M + half * M + idx);
    }
}

// Row z of a harmonic's plane for one segment, both transforms at once:
// multiply the segment spectrum D by the folded template, run the inverse
// transforms and leave p[e] = (power of even output, power of odd output)
// at m = t + e*M/16.  The templates carry the 1/L normalisation, so |y|^2
// is the power.
template <int M, bool F16, bool SPLIT, class Sync = CtaSync>
__device__ __forceinline__ void plane_powers(const HarmPlan& H, const float2* __restrict__ D, int z,
                                             float2* sm, const float2* __restrict__ tw, float2 (&p)[16],
                                             int t, Sync sync = Sync()) {
    static_assert(!SPLIT, "the sequential layout stores each transform as it completes");
    constexpr int T = M / 16;
    float2 x[2][16];
#pragma unroll
    for (int e = 0; e < 16; e++) {
        const int idx = t + e * T;
        const float2 d = D[idx];
        x[0][e] = cmul(d, fold_at<M, F16>(H, z, 0, idx));
        x[1][e] = cmul(d, fold_at<M, F16>(H, z, 1, idx));
    }
    fft_run<M, +1, 2, Sync>(x, sm, tw, t, sync);
#pragma unroll
    for (int e = 0; e < 16; e++)
        p[e] = make_float2(fmaf(x[0][e].x, x[0][e].x, x[0][e].y * x[0][e].y),
                           fmaf(x[1][e].x, x[1][e].x, x[1][e].y * x[1][e].y));
}

// Stage the row's powers for columns [0, wmax) in shared memory (even and
// odd outputs interleaved) and return the float view.
template <int M>
__device__ __forceinline__ float* stage_row_powers(const HarmPlan& H, unsigned char* smem_raw,
                                                   const float2 (&p)[16], int t) {
    constexpr int T = M / 16;
    float* pw = reinterpret_cast<float*>(smem_raw);
    const int half_w = H.wmax >> 1;
    __syncthreads();  // every thread has finished reading the transform buffers
#pragma unroll
    for (int e = 0; e < 16; e++) {
        const int i2 = t + e * T - H.hw0;
        if (i2 >= 0 && i2 < half_w) *reinterpret_cast<float2*>(pw + 2 * i2) = p[e];
    }
    __syncthreads();
    return pw;
}

template <int M, bool F16, bool SPLIT>
__global__ void __launch_bounds__(PlaneShape<SPLIT, M>::THREADS, PlaneShape<SPLIT, M>::MINB)
    k_plane(const PlaneArgs a, const float2* __restrict__ tw) {
    constexpr int T = M / 16;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    // segments vary fastest across the grid, so that the CTAs resident at
    // one time share a few templates (read from DRAM once, then from L2)
    const int item = blockIdx.y;
    int hi = 0;
#pragma unroll 1
    while (hi + 1 < a.nh && item >= a.h[hi + 1].zbase) hi++;
    const HarmPlan& H = a.h[hi];
    const int z = item - H.zbase;
    const int seg = blockIdx.x;
    const int t = threadIdx.x;
    const float2* __restrict__ D = a.dbuf + (long long)seg * a.dstride + H.doff;
    float* row = a.planes + (long long)seg * a.pstride + H.poff + (long long)z * H.prow;
    const int half_w = H.wmax >> 1;
    if constexpr (!SPLIT) {
        // straight from registers: (even, odd) pairs as 8-byte stores
        float2 p[16];
        plane_powers<M, F16, false>(H, D, z, reinterpret_cast<float2*>(smem_raw), tw, p, t);
#pragma unroll
        for (int e = 0; e < 16; e++) {
            const int i2 = t + e * T - H.hw0;  // one unsigned compare for 0 <= i2 < half_w
            if ((unsigned)i2 < (unsigned)half_w) *reinterpret_cast<float2*>(row + 2 * i2) = p[e];
        }
    } else {
        // even transform, then odd, each stored as it completes (a loop, not
        // unrolled, so that nothing of the first stays live in the second)
#pragma unroll 1
        for (int half = 0; half < 2; half++) {
            float2 x[1][16];
#pragma unroll
            for (int e = 0; e < 16; e++) {
                const int idx = t + e * T;
                x[0][e] = cmul(D[idx], fold_at<M, F16>(H, z, half, idx));
            }
            fft_run<M, +1, 1>(x, reinterpret_cast<float2*>(smem_raw), tw, t);
#pragma unroll
            for (int e = 0; e < 16; e++) {
                const int i2 = t + e * T - H.hw0;
                if (i2 >= 0 && i2 < half_w) row[2 * i2 + half] = fmaf(x[0][e].x, x[0][e].x, x[0][e].y * x[0][e].y);
            }
        }
    }
}

// --------------------------------------------------- fundamental + harmonic sum
// The fundamental's row z of one segment: transform as in k_plane, then --
// instead of storing the row -- add the sub-harmonic powers gathered from
// their planes (computed by earlier k_plane launches of the same group) in
// the reference's order, check every stage against its cut and append the
// candidates.  The fundamental plane never reaches global memory.
__device__ __forceinline__ long long twice_r_shift(long long r2, int p, int lq) {
    return (2LL * r2 * p + (1LL << lq)) >> (lq + 1);
}
__device__ __forceinline__ int trunc_shift(int x, int k) {  // C division by 2^k
    return x >= 0 ? (x >> k) : -((-x) >> k);
}
__device__ __forceinline__ int sub_row(int zz, const HarmPlan& H) {
    const int d = trunc_shift(zz * H.p, H.lq) - H.zlo;
    return d >= 0 ? (d >> 1) : -((-d) >> 1);
}

// Warp-aggregated append of the lanes whose `hit` is set.
__device__ __forceinline__ void append_candidates(bool hit, int seg, int i, int z, int numharm, float s,
                                                  RawCand* cands, unsigned long long* ncand,
                                                  long long cap) {
    const unsigned m = __ballot_sync(0xffffffffu, hit);
    if (!m) return;
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(m) - 1;
    unsigned long long base = 0;
    if (lane == leader) base = atomicAdd(ncand, (unsigned long long)__popc(m));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (hit) {
        const unsigned long long slot = base + __popc(m & ((1u << lane) - 1u));
        if ((long long)slot < cap) {
            RawCand c;
            c.seg = seg;
            c.ridx = i;
            c.zidx = (int16_t)z;
            c.numharm = (int16_t)numharm;
            c.power = s;
            cands[slot] = c;
        }
    }
}

template <int M, bool F16>
__global__ void __launch_bounds__(PlaneShape<false, M>::THREADS, PlaneShape<false, M>::MINB)
    k_fund_sum(const FundArgs a, const float2* __restrict__ tw) {
    constexpr int THREADS = PlaneShape<false, M>::THREADS;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const HarmPlan& H0 = a.h[0];
    const int z = blockIdx.x;
    const int seg = blockIdx.y;
    float2 p[16];
    plane_powers<M, F16, false>(H0, a.dbuf + (long long)seg * a.dstride + H0.doff, z,
                                reinterpret_cast<float2*>(smem_raw), tw, p, (int)threadIdx.x);
    const float* pw = stage_row_powers<M>(H0, smem_raw, p, (int)threadIdx.x);

    const long long startr = a.segs[seg].startr;
    const float* __restrict__ P = a.planes + (long long)seg * a.pstride;
    const int zz = a.zlo0 + kDz * z;
    int rowoff[kMaxHarm];  // offset of the sub-harmonic row and its rlo*2
    long long rlo2[kMaxHarm];
#pragma unroll
    for (int h = 1; h < kMaxHarm; h++) {
        if (h < a.nh) {
            const HarmPlan& H = a.h[h];
            rowoff[h] = (int)H.poff + sub_row(zz, H) * H.prow;
            rlo2[h] = (twice_r_shift(2 * startr, H.p, H.lq) >> 1) << 1;
        }
    }
    const int U = a.uselen;
#pragma unroll 1
    for (int i0 = 0; i0 < U; i0 += THREADS) {
        const int i = i0 + threadIdx.x;
        const bool valid = i < U;
        float v[kMaxHarm];
        v[0] = valid ? pw[i] : 0.f;
#pragma unroll
        for (int h = 1; h < kMaxHarm; h++) {
            if (h < a.nh) {
                const HarmPlan& H = a.h[h];
                const int rind = (int)(unsigned short)(twice_r_shift(2 * startr + i, H.p, H.lq) - rlo2[h]);
                v[h] = valid ? P[rowoff[h] + rind] : 0.f;
            }
        }
        float s = 0.f;
#pragma unroll
        for (int h = 0; h < kMaxHarm; h++) {
            if (h < a.nh) {
                s = (h == 0) ? v[0] : s + v[h];
                const int st = a.stage_of[h];
                if (st >= 0) {
                    if (a.stage_out && valid)
                        a.stage_out[(((long long)seg * a.nstages + st) * a.numzs0 + z) * U + i] = s;
                    append_candidates(valid && s > a.cut[st], a.seg_base + seg, i, z, h + 1, s, a.cands,
                                      a.ncand, a.cap);
                }
            }
        }
    }
}

// ------------------------------------------------------------- tiled hsum
// Harmonic sum of one tile of kTileZ f-dot rows x kTileI columns of the
// fundamental plane.  The fundamental tile and, for every sub-harmonic, the
// rectangle of its plane that the tile's (zind, rind) indices touch are
// brought into shared memory by bulk asynchronous copies (cp.async.bulk,
// one per rectangle row, completing on one mbarrier), then every cell is
// summed from shared memory in the reference's harmonic order and checked
// against the stage cuts.
constexpr int kTileZ = kHsumTileZ;
constexpr int kTileI = kHsumTileI;
constexpr int kTileSmemFloats = kHsumTileFloats;   // 60 KB: fundamental tile + sub-tiles

__device__ __forceinline__ unsigned smem_addr(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_addr(bar)), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive(unsigned long long* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(smem_addr(bar)) : "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(unsigned long long* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}
// Wait for the barrier's phase with the thread suspended (no polling
// instructions), at most about 1 us per try; false after 2^15 tries (tens
// of milliseconds), far beyond any copy of a tile.
__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, unsigned parity) {
    unsigned done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(smem_addr(bar)), "r"(parity), "r"(1000u)
        : "memory");
    return done != 0;
}
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long* bar, unsigned parity) {
#pragma unroll 1
    for (int it = 0; it < (1 << 15); it++)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}
// One box of a 3-D tensor map (coordinates x = column, y = row, z =
// segment) into shared memory (128-byte aligned); elements past the
// tensor's edges arrive as zeros and count toward the transaction bytes.
__device__ __forceinline__ void tensor_copy_g2s(void* sdst, const CUtensorMap* map, int x, int y, int z,
                                                unsigned long long* bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
        "[%5];\n" ::"r"(smem_addr(sdst)),
        "l"(reinterpret_cast<unsigned long long>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_addr(bar))
        : "memory");
}

// bytes (a multiple of 16) from global to shared, both 16-byte aligned
__device__ __forceinline__ void bulk_copy_g2s(void* sdst, const void* gsrc, unsigned bytes,
                                              unsigned long long* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(
                     smem_addr(sdst)),
                 "l"(gsrc), "r"(bytes), "r"(smem_addr(bar))
                 : "memory");
}

// Stage index after harmonic h (bank order): stages end after 1, 2, 4, 8,
// 16 harmonics (bpd_search.cu:350), i.e. when h + 1 is a power of two.
__host__ __device__ constexpr int stage_after(int h) {
    return ((h + 1) & h) ? -1 : (h == 0 ? 0 : h == 1 ? 1 : h == 3 ? 2 : h == 7 ? 3 : 4);
}

// Static shared memory of one harmonic-sum tile of TZ f-dot rows.
template <int NH, int TZ = kTileZ> struct TileShared {
    int row[NH][TZ];      // byte offset of the row used by tile row zr
    int zf[NH], nzr[NH], r0[NH], c0[NH], w4[NH], off[NH];
    int cb[NH], crem[NH];  // column of tile column 0, and the rounding remainder
};

// One tile: segment seg, f-dot rows [z0, z0 + TZ), columns [i0, i0 +
// kTileI), by the CTA's kTileI threads.  The CTA's mbarrier `bar` is
// initialised here when init is set (its first use), else reused: the
// caller passes the parity of this use.  Returns false -- with the error
// word set -- when the copies did not land within the bounded wait; the
// barrier's state is then unknown and the CTA must not use it again.
// With tensor maps (maps != null, a.use_tmap): one box copy per harmonic
// instead of one bulk copy per rectangle row.
template <int NH, bool STAGE_OUT, int TZ = kTileZ>
__device__ __forceinline__ bool hsum_tile_body(const HsumArgs& a, int seg, int z0, int i0, float* tsm,
                                               TileShared<NH, TZ>& S, unsigned long long* bar, bool init,
                                               unsigned parity, const CUtensorMap* maps = nullptr) {
    static_assert(NH <= 32, "one lane per harmonic");
    static_assert(TZ % 4 == 0 && TZ <= kTileI, "rows in batches of four, one thread per row table entry");
    const int nz = min(TZ, a.numzs0 - z0);
    const int ni = min(kTileI, a.uselen - i0);
    const long long startr = a.segs[seg].startr;
    const float* __restrict__ P = a.planes + (long long)seg * a.pstride;
    const int tid = threadIdx.x;
    const int i = i0 + tid;
    const bool valid = tid < ni;

    // 1. warp 0: rectangles, lane h for harmonic h -- rows [zf, zf + nzr),
    //    4-aligned columns [c0, c0 + 4 w4) -- placed one after another in
    //    shared memory (warp prefix sums), then one bulk copy per row
    if (tid < 32) {
        int size = 0, nzr = 0;
        if (tid < NH) {
            const int h = tid;
            const HarmPlan& H = a.h[h];
            int rfirst = i0, rlast = i0 + ni - 1, zf = z0, zl = z0 + nz - 1;
            long long rlo2 = 0;
            if (h > 0) {
                rlo2 = (twice_r_shift(2 * startr, H.p, H.lq) >> 1) << 1;
                rfirst = (int)(unsigned short)(twice_r_shift(2 * startr + i0, H.p, H.lq) - rlo2);
                rlast = (int)(unsigned short)(twice_r_shift(2 * startr + i0 + ni - 1, H.p, H.lq) - rlo2);
                zf = sub_row(a.zlo0 + kDz * z0, H);
                zl = sub_row(a.zlo0 + kDz * (z0 + nz - 1), H);
            }
            const int c0 = rfirst & ~3;
            // rectangle row pitch: its own width, or the harmonic's box
            const int w4 = maps ? a.box_w4[h] : ((rlast - c0) >> 2) + 1;
            nzr = zl - zf + 1;
            S.zf[h] = zf;
            S.nzr[h] = nzr;
            S.c0[h] = c0;
            S.w4[h] = w4;
            size = 4 * nzr * w4;
            // twice_r_shift(2 startr + i0 + k) = (B + 2 k p) >> (lq + 1) with
            // B = 2 (2 startr + i0) p + 2^lq: split B once so that every
            // thread finishes in 32 bits (only the low 16 bits of the
            // difference to rlo2 matter, as in the reference's ushort)
            const long long B = 2LL * (2 * startr + i0) * H.p + (1LL << H.lq);
            S.cb[h] = (int)((B >> (H.lq + 1)) - rlo2) - c0;
            S.crem[h] = (int)(B & ((2LL << H.lq) - 1));
        }
        int incl = size, rincl = nzr;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int v = __shfl_up_sync(0xffffffffu, incl, o);
            const int w = __shfl_up_sync(0xffffffffu, rincl, o);
            if (tid >= o) {
                incl += v;
                rincl += w;
            }
        }
        if (tid < NH) {
            S.off[tid] = maps ? a.box_off[tid] : incl - size;
            S.r0[tid] = rincl - nzr;  // first copy index of harmonic tid
        }
        const int total_floats = __shfl_sync(0xffffffffu, incl, 31);
        const int total_rows = __shfl_sync(0xffffffffu, rincl, 31);
        if (tid == 0) {
            if (init) mbar_init(bar, 1);
            mbar_arrive_expect_tx(bar, (maps ? a.box_tx : 4u * (unsigned)total_floats) + a.test_extra_tx);
        }
        __syncwarp();
        if (maps) {
            // lane h: harmonic h's box from (c0, zf) of segment seg
            if (tid < NH) tensor_copy_g2s(tsm + S.off[tid], maps + tid, S.c0[tid], S.zf[tid], seg, bar);
        } else
        for (int j = tid; j < total_rows; j += 32) {
            int h = 0;
#pragma unroll
            for (int g = 1; g < NH; g++)
                if (j >= S.r0[g]) h = g;
            const HarmPlan& H = a.h[h];
            const int r = j - S.r0[h], w4 = S.w4[h];
            bulk_copy_g2s(tsm + S.off[h] + 4 * w4 * r, P + H.poff + (long long)(S.zf[h] + r) * H.prow + S.c0[h],
                          16u * (unsigned)w4, bar);
        }
    }
    __syncthreads();
    // 2. row table and this thread's column in every rectangle (while the
    //    copies fly)
    //    (rows past the plane's edge point at the rectangle's first row)
#pragma unroll
    for (int h = 0; h < NH; h++) {
        if (tid < TZ) {
            const int r = (tid >= nz) ? 0 : (h == 0) ? tid : sub_row(a.zlo0 + kDz * (z0 + tid), a.h[h]) - S.zf[h];
            S.row[h][tid] = 4 * (S.off[h] + 4 * S.w4[h] * r);
        }
    }
    int colb[NH];  // byte offset of this thread's column
#pragma unroll
    for (int h = 0; h < NH; h++) {
        if (h == 0) {
            colb[h] = valid ? 4 * tid : 0;  // lanes past the plane edge read column 0
        } else {
            const HarmPlan& H = a.h[h];
            const int c0 = S.c0[h];
            const int rind = (unsigned short)(S.cb[h] + c0 + ((S.crem[h] + 2 * tid * H.p) >> (H.lq + 1)));
            colb[h] = valid ? 4 * (rind - c0) : 0;
        }
    }
    float cut[kMaxStages];
#pragma unroll
    for (int st = 0; st < kMaxStages; st++) cut[st] = a.cut[st];
    // 3. wait for the copies (bounded; every thread agrees on the outcome)
    const bool landed = mbar_wait_bounded(bar, parity);
    if (!__syncthreads_and(landed)) {
        if (tid == 0) atomicOr(a.err, 1ull);
        mbar_wait_bounded(bar, parity);  // give copies still in flight a last chance to land
        return false;
    }

    // 4. sums in the reference's harmonic order, RB rows at a time (their
    //    row offsets in one vector load per harmonic); one warp vote per
    //    row over all stage tests, the per-stage appends only when some
    //    lane hit
    constexpr int RB = (NH <= 8 && !STAGE_OUT) ? 4 : 2;  // rows per batch (registers)
    const char* tb = reinterpret_cast<const char*>(tsm);
#pragma unroll 1
    for (int zq = 0; zq < nz; zq += RB) {
        int ro[NH][RB];
#pragma unroll
        for (int h = 0; h < NH; h++) {
            if constexpr (RB == 4) {
                const int4 v = *reinterpret_cast<const int4*>(&S.row[h][zq]);
                ro[h][0] = v.x;
                ro[h][1] = v.y;
                ro[h][2] = v.z;
                ro[h][3] = v.w;
            } else {
                const int2 v = *reinterpret_cast<const int2*>(&S.row[h][zq]);
                ro[h][0] = v.x;
                ro[h][1] = v.y;
            }
        }
#pragma unroll
        for (int k = 0; k < RB; k++) {
            const int zr = zq + k;
            const int z = z0 + zr;
            const bool live = valid && zr < nz;
            float s = 0.f, sst[kMaxStages];
            bool any = false;
#pragma unroll
            for (int h = 0; h < NH; h++) {
                const float v = *reinterpret_cast<const float*>(tb + ro[h][k] + colb[h]);
                s = (h == 0) ? v : s + v;
                const int st = stage_after(h);  // folds to a constant once h is unrolled
                if (st >= 0) {
                    sst[st] = s;
                    any |= s > cut[st];
                    if constexpr (STAGE_OUT) {
                        if (live)
                            a.stage_out[(((long long)seg * a.nstages + st) * a.numzs0 + z) * a.uselen + i] = s;
                    }
                }
            }
            if (__any_sync(0xffffffffu, live && any)) {
#pragma unroll
                for (int h = 0; h < NH; h++) {
                    const int st = stage_after(h);
                    if (st >= 0)
                        append_candidates(live && sst[st] > cut[st], a.seg_base + seg, i, z, h + 1, sst[st],
                                          a.cands, a.ncand, a.cap);
                }
            }
        }
    }
    return true;
}

template <int NH, bool STAGE_OUT, int TZ = kTileZ>
__global__ void __launch_bounds__(kTileI, TZ > 16 ? 2 : 4)
    k_hsum_tile(const HsumArgs a, const __grid_constant__ HsumMaps maps) {
    extern __shared__ __align__(128) float tsm[];
    __shared__ __align__(16) TileShared<NH, TZ> S;
    __shared__ __align__(8) unsigned long long s_bar;
    hsum_tile_body<NH, STAGE_OUT, TZ>(a, blockIdx.z, blockIdx.y * TZ, blockIdx.x * kTileI, tsm, S, &s_bar, true,
                                      0u, a.use_tmap ? maps.m : nullptr);
}

// ------------------------------------------------------- pipelined tiled hsum
// The same tiles and sums as k_hsum_tile, from one persistent CTA per SM
// with kPipeBufs tile buffers (each the plan's worst tile) in shared memory and specialised warps: one
// producer warp computes each tile's rectangles and issues its bulk copies
// (completing on the buffer's "full" mbarrier) as soon as the consumers
// have released the buffer (its "empty" mbarrier); 16 consumer warps, two
// threads per column and 8 rows each, sum the tiles in order.  DRAM reads
// of the next tiles overlap the additions of the current one.  Every wait
// is bounded; a warp that gives up sets the error word, lets the copies it
// knows of land, and leaves.
constexpr int kPipeBufs = kPipeBuffers;
constexpr int kPipeConsumers = 2 * kTileI;                 // 512 threads, 16 warps
constexpr int kPipeThreads = kPipeConsumers + 32 * kPipeBufs;  // + one producer warp per buffer

template <int NH, bool STAGE_OUT>
__global__ void __launch_bounds__(kPipeThreads, 1) k_hsum_pipe(const HsumArgs a, int ntiles, int bstride) {
    static_assert(NH <= 32, "one lane per harmonic");
    static_assert(kTileZ == 16 && kTileI == 256, "two threads per column, 8 rows each");
    extern __shared__ __align__(128) float tsm[];  // kPipeBufs buffers of bstride floats
    __shared__ __align__(16) int s_row[kPipeBufs][NH][kTileZ];  // byte offset of tile row zr's row
    __shared__ int s_c0[kPipeBufs][NH], s_cb[kPipeBufs][NH], s_crem[kPipeBufs][NH];
    __shared__ int s_tile[kPipeBufs][4];  // seg, z0, i0, nz | ni << 16
    __shared__ __align__(8) unsigned long long s_full[kPipeBufs], s_empty[kPipeBufs];
    const int tid = threadIdx.x;
    const int lane = tid & 31;
    const int G = gridDim.x;
    if (tid == 0)
        for (int b = 0; b < kPipeBufs; b++) {
            mbar_init(&s_full[b], 1);
            mbar_init(&s_empty[b], kPipeConsumers / 32);
        }
    __syncthreads();

    if (tid >= kPipeConsumers) {
        // ------------------------------------------------------ producers
        // producer warp b owns buffer b and fills it with tiles k = b,
        // b + kPipeBufs, ... of this CTA
        const int b = (tid - kPipeConsumers) >> 5;
        const int ntz = (a.numzs0 + kTileZ - 1) / kTileZ;
        const int nti = (a.uselen + kTileI - 1) / kTileI;
#pragma unroll 1
        for (int k = b; blockIdx.x + (long long)k * G < ntiles; k += kPipeBufs) {
            const int t = blockIdx.x + k * G;
            const unsigned use = (unsigned)(k / kPipeBufs);  // how often b was filled before
            if (use > 0 && !mbar_wait_bounded(&s_empty[b], (use - 1) & 1u)) {
                if (lane == 0) atomicOr(a.err, 1ull);
                mbar_wait_bounded(&s_full[b], (use - 1) & 1u);  // let the previous fill's copies land
                return;
            }
            const int it = t % nti, rest = t / nti;
            const int zt = rest % ntz, seg = rest / ntz;
            const int z0 = zt * kTileZ, i0 = it * kTileI;
            const int nz = min(kTileZ, a.numzs0 - z0), ni = min(kTileI, a.uselen - i0);
            const long long startr = a.segs[seg].startr;
            int size = 0, nzr = 0, zf = z0, c0 = 0, w4 = 0;
            if (lane < NH) {
                const int h = lane;
                const HarmPlan& H = a.h[h];
                int rfirst = i0, rlast = i0 + ni - 1, zl = z0 + nz - 1;
                long long rlo2 = 0;
                if (h > 0) {
                    rlo2 = (twice_r_shift(2 * startr, H.p, H.lq) >> 1) << 1;
                    rfirst = (int)(unsigned short)(twice_r_shift(2 * startr + i0, H.p, H.lq) - rlo2);
                    rlast = (int)(unsigned short)(twice_r_shift(2 * startr + i0 + ni - 1, H.p, H.lq) - rlo2);
                    zf = sub_row(a.zlo0 + kDz * z0, H);
                    zl = sub_row(a.zlo0 + kDz * (z0 + nz - 1), H);
                }
                c0 = rfirst & ~3;
                w4 = ((rlast - c0) >> 2) + 1;
                nzr = zl - zf + 1;
                size = 4 * nzr * w4;
                const long long B = 2LL * (2 * startr + i0) * H.p + (1LL << H.lq);
                s_c0[b][h] = c0;
                s_cb[b][h] = (int)((B >> (H.lq + 1)) - rlo2) - c0;
                s_crem[b][h] = (int)(B & ((2LL << H.lq) - 1));
            }
            int incl = size;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int v = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += v;
            }
            const int off = incl - size;
            const int total_floats = __shfl_sync(0xffffffffu, incl, 31);
            // row table: lane zr < 16 fills row zr of every harmonic (rows
            // past the plane's edge use the rectangle's first row)
#pragma unroll
            for (int h = 0; h < NH; h++) {
                const int offh = __shfl_sync(0xffffffffu, off, h), w4h = __shfl_sync(0xffffffffu, w4, h);
                const int zfh = __shfl_sync(0xffffffffu, zf, h);
                if (lane < kTileZ) {
                    const int r = (lane >= nz) ? 0 : (h == 0) ? lane : sub_row(a.zlo0 + kDz * (z0 + lane), a.h[h]) - zfh;
                    s_row[b][h][lane] = 4 * (offh + 4 * w4h * r);
                }
            }
            if (lane == 0) {
                s_tile[b][0] = seg;
                s_tile[b][1] = z0;
                s_tile[b][2] = i0;
                s_tile[b][3] = nz | (ni << 16);
            }
            __syncwarp();  // the tables above are released by lane 0's arrive
            if (lane == 0) mbar_arrive_expect_tx(&s_full[b], 4u * (unsigned)total_floats);
            __syncwarp();
            // copies: lane h brings rectangle h row by row
            if (lane < NH) {
                const HarmPlan& H = a.h[lane];
                const float* src = a.planes + (long long)seg * a.pstride + H.poff + (long long)zf * H.prow + c0;
                float* dst = tsm + b * bstride + off;
                for (int r = 0; r < nzr; r++)
                    bulk_copy_g2s(dst + 4 * w4 * r, src + (long long)r * H.prow, 16u * (unsigned)w4, &s_full[b]);
            }
        }
        return;
    }

    // --------------------------------------------------------- consumers
    const int c = tid & (kTileI - 1), rh = (tid / kTileI) * (kTileZ / 2);  // column, first row
    constexpr int RB = (NH <= 8 && !STAGE_OUT) ? 4 : 2;                      // rows per batch
    float cut[kMaxStages];
#pragma unroll
    for (int st = 0; st < kMaxStages; st++) cut[st] = a.cut[st];
    int k = 0;
#pragma unroll 1
    for (int t = blockIdx.x; t < ntiles; t += G, k++) {
        const int b = k % kPipeBufs;
        const unsigned parity = (unsigned)(k / kPipeBufs) & 1u;
        if (!mbar_wait_bounded(&s_full[b], parity)) {
            if (lane == 0) atomicOr(a.err, 1ull);
            mbar_wait_bounded(&s_full[b], parity);  // a last chance for the copies to land
            return;
        }
        const int seg = s_tile[b][0], z0 = s_tile[b][1], i0 = s_tile[b][2];
        const int nz = s_tile[b][3] & 0xffff, ni = s_tile[b][3] >> 16;
        const int i = i0 + c;
        const bool valid = c < ni;
        int colb[NH];
#pragma unroll
        for (int h = 0; h < NH; h++) {
            if (h == 0) {
                colb[h] = valid ? 4 * c : 0;
            } else {
                const HarmPlan& H = a.h[h];
                const int c0 = s_c0[b][h];
                const int rind = (unsigned short)(s_cb[b][h] + c0 + ((s_crem[b][h] + 2 * c * H.p) >> (H.lq + 1)));
                colb[h] = valid ? 4 * (rind - c0) : 0;
            }
        }
        const char* tb = reinterpret_cast<const char*>(tsm + b * bstride);
        int ro[NH][kTileZ / 2];
#pragma unroll
        for (int h = 0; h < NH; h++)
#pragma unroll
            for (int q = 0; q < kTileZ / 2; q += 4) {
                const int4 v = *reinterpret_cast<const int4*>(&s_row[b][h][rh + q]);
                ro[h][q] = v.x;
                ro[h][q + 1] = v.y;
                ro[h][q + 2] = v.z;
                ro[h][q + 3] = v.w;
            }
        float sums[kMaxStages][kTileZ / 2];
        // all reads of buffer b done before it is released
#pragma unroll
        for (int zz = 0; zz < kTileZ / 2; zz++) {
            float s = 0.f;
#pragma unroll
            for (int h = 0; h < NH; h++) {
                const float v = *reinterpret_cast<const float*>(tb + ro[h][zz] + colb[h]);
                s = (h == 0) ? v : s + v;
                const int st = stage_after(h);  // folds to a constant once h is unrolled
                if (st >= 0) sums[st][zz] = s;
            }
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(&s_empty[b]);
        if (rh < nz) {
#pragma unroll
            for (int zz = 0; zz < kTileZ / 2; zz++) {
                const int zr = rh + zz;
                const int z = z0 + zr;
                const bool live = valid && zr < nz;
                bool any = false;
#pragma unroll
                for (int st = 0; st < kMaxStages; st++) {
                    if (st < stage_after(NH - 1) + 1) {
                        any |= sums[st][zz] > cut[st];
                        if constexpr (STAGE_OUT) {
                            if (live)
                                a.stage_out[(((long long)seg * a.nstages + st) * a.numzs0 + z) * a.uselen + i] =
                                    sums[st][zz];
                        }
                    }
                }
                if (__any_sync(0xffffffffu, live && any)) {
#pragma unroll
                    for (int st = 0; st < kMaxStages; st++) {
                        if (st < stage_after(NH - 1) + 1)
                            append_candidates(live && sums[st][zz] > cut[st], a.seg_base + seg, i, z, 1 << st,
                                              sums[st][zz], a.cands, a.ncand, a.cap);
                    }
                }
            }
        }
    }
}

// ------------------------------------------------------------------ hsum
// One thread per fundamental column i, kHsumRows f-dot rows per block.  The
// reference's index arithmetic (twice_required_r, sub_zind) divides by
// powers of two only, so it is done with shifts here; the per-column
// sub-harmonic offsets are computed once per thread.
constexpr int kHsumCols = 128;
constexpr int kHsumRows = 32;

template <int NH>
__global__ void __launch_bounds__(kHsumCols) k_hsum(const HsumArgs a) {
    const int i = blockIdx.x * kHsumCols + threadIdx.x;
    const int seg = blockIdx.z;
    const bool valid = i < a.uselen;
    const long long startr = a.segs[seg].startr;
    const float* __restrict__ P = a.planes + (long long)seg * a.pstride;
    const int lane = threadIdx.x & 31;

    int roff[NH];
#pragma unroll
    for (int h = 1; h < NH; h++) {
        const HarmPlan& H = a.h[h];
        const long long rlo2 = (twice_r_shift(2 * startr, H.p, H.lq) >> 1) << 1;
        const int rind = (int)(unsigned short)(twice_r_shift(2 * startr + i, H.p, H.lq) - rlo2);
        roff[h] = (int)H.poff + rind;
    }
    const int z0 = blockIdx.y * kHsumRows;
    const int zend = min(z0 + kHsumRows, a.numzs0);
    const int base0 = (int)a.h[0].poff + i;
#pragma unroll 2
    for (int z = z0; z < zend; z++) {
        const int zz = a.zlo0 + kDz * z;
        float v[NH];
        v[0] = valid ? P[base0 + z * a.h[0].prow] : 0.f;
#pragma unroll
        for (int h = 1; h < NH; h++) {
            const HarmPlan& H = a.h[h];
            const int d = trunc_shift(zz * H.p, H.lq) - H.zlo;
            const int zind = d >= 0 ? (d >> 1) : -((-d) >> 1);
            v[h] = valid ? P[roff[h] + zind * H.prow] : 0.f;
        }
        float s = 0.f;
#pragma unroll
        for (int h = 0; h < NH; h++) {
            s = (h == 0) ? v[0] : s + v[h];
            const int st = stage_after(h);  // folds to a constant once h is unrolled
            if (st >= 0) {
                if (a.stage_out && valid)
                    a.stage_out[(((long long)seg * a.nstages + st) * a.numzs0 + z) * a.uselen + i] = s;
                const bool hit = valid && s > a.cut[st];
                const unsigned m = __ballot_sync(0xffffffffu, hit);
                if (m) {
                    unsigned long long base = 0;
                    const int leader = __ffs(m) - 1;
                    if (lane == leader) base = atomicAdd(a.ncand, (unsigned long long)__popc(m));
                    base = __shfl_sync(0xffffffffu, base, leader);
                    if (hit) {
                        const unsigned long long slot = base + __popc(m & ((1u << lane) - 1u));
                        if ((long long)slot < a.cap) {
                            RawCand c;
                            c.seg = a.seg_base + seg;
                            c.ridx = i;
                            c.zidx = (int16_t)z;
                            c.numharm = (int16_t)(h + 1);
                            c.power = s;
                            a.cands[slot] = c;
                        }
                    }
                }
            }
        }
    }
}

// -------------------------------------------------------------- launchers
template <int M> static int prep_m(const PrepArgs& a, int nseg, const float2* tw, cudaStream_t st) {
    size_t smem = sizeof(float2) * FftShape<M>::PADDED + sizeof(uint32_t) * M;
    static std::atomic<unsigned long long> attr{0};
    int dev = 0;
    if (attr_pending(attr, &dev)) {
        if (cudaFuncSetAttribute(k_prep<M>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
                cudaSuccess ||
            cudaFuncSetAttribute(k_prep<M>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                 carveout_for((const void*)k_prep<M>, M / 16, smem)) != cudaSuccess)
            return -1;
        attr_set(attr, dev);
    }
    k_prep<M><<<dim3(a.nh, nseg), M / 16, smem, st>>>(a, tw);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

template <int M, bool F16, bool SPLIT>
static int plane_m(const PlaneArgs& a, int nseg, const float2* tw, cudaStream_t st) {
    size_t smem = sizeof(float2) * FftShape<M>::PADDED * PlaneShape<SPLIT, M>::BUFFERS;
    static std::atomic<unsigned long long> attr{0};
    int dev = 0;
    if (attr_pending(attr, &dev)) {
        if (cudaFuncSetAttribute(k_plane<M, F16, SPLIT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem) != cudaSuccess ||
            cudaFuncSetAttribute(k_plane<M, F16, SPLIT>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                 carveout_for((const void*)k_plane<M, F16, SPLIT>, PlaneShape<SPLIT, M>::THREADS,
                                              smem)) != cudaSuccess)
            return -1;
        attr_set(attr, dev);
    }
    k_plane<M, F16, SPLIT><<<dim3(nseg, a.ntpl), PlaneShape<SPLIT, M>::THREADS, smem, st>>>(a, tw);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

template <int M>
static int plane_dispatch(const PlaneArgs& a, int nseg, const float2* tw, cudaStream_t st) {
    const bool h = a.use_fp16 != 0, sp = a.split != 0;
    if (h) return sp ? plane_m<M, true, true>(a, nseg, tw, st) : plane_m<M, true, false>(a, nseg, tw, st);
    return sp ? plane_m<M, false, true>(a, nseg, tw, st) : plane_m<M, false, false>(a, nseg, tw, st);
}

template <int M, bool F16>
static int fund_m(const FundArgs& a, int nseg, const float2* tw, cudaStream_t st) {
    size_t smem = sizeof(float2) * FftShape<M>::PADDED * 2;
    static std::atomic<unsigned long long> attr{0};
    int dev = 0;
    if (attr_pending(attr, &dev)) {
        if (cudaFuncSetAttribute(k_fund_sum<M, F16>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem) != cudaSuccess ||
            cudaFuncSetAttribute(k_fund_sum<M, F16>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                 carveout_for((const void*)k_fund_sum<M, F16>, PlaneShape<false, M>::THREADS,
                                              smem)) != cudaSuccess)
            return -1;
        attr_set(attr, dev);
    }
    k_fund_sum<M, F16><<<dim3(a.h[0].numzs, nseg), PlaneShape<false, M>::THREADS, smem, st>>>(a, tw);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

// The fused kernel always uses the two-transform layout (it stages the
// row's powers in shared memory, which the sequential layout keeps busy).
template <int M>
static int fund_dispatch(const FundArgs& a, int nseg, const float2* tw, cudaStream_t st) {
    return a.use_fp16 ? fund_m<M, true>(a, nseg, tw, st) : fund_m<M, false>(a, nseg, tw, st);
}

}  // namespace accel
