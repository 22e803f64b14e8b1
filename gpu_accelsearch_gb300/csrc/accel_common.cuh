// accel_common.cuh -- shared types, reference-exact arithmetic helpers and
// overlap-save geometry used by both host and device code.
//
// Geometry functions restate bpd_subharmonics.cu:10-19,31-45,60-67 and
// bpd_search.cu:72-127 in exact integer arithmetic.  The reference computes
// them in double precision, but every operand there is an integer, a
// half-integer or a dyadic fraction h/2^k, so the double results are exact
// and the integer forms below give identical values (checked against the
// reference in tests/test_native_cpu.py).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#ifndef ACCEL_HD
#define ACCEL_HD __host__ __device__ __forceinline__
#endif

namespace accel {

constexpr int kMaxHarm = 16;        // harmonics per bank (numharm <= 16)
constexpr int kMaxStages = 5;       // 1,2,4,8,16
constexpr int kNumBetween = 2;      // interbinning (bpd_common.h:30)
constexpr int kDz = 2;              // f-dot step (bpd_common.h:33)
constexpr double kLn2 = 0.693147180559945309417232121458;  // median -> mean of an exponential
constexpr int kFintBins = 16;       // NUMFINTBINS (bpd_common.h:45)
constexpr int kTwN = 8192;          // twiddle table length (max FFT points)
// Behind the kTwN-entry table: for every later-pass length NR of the
// shared-memory FFT, the base twiddles W^k, W^2k, W^4k, W^8k of pass index k
// (W = exp(2 pi i / NR)) side by side, four float2 per k, so that a thread
// fetches its pass's base twiddles with two 16-byte loads from consecutive
// memory instead of four scattered ones.  Sections: NR = 64, 128, 256 (16
// entries each), 512, 1024, 2048, 4096 (256 entries each).
ACCEL_HD constexpr int tw_pack_entries(int NR) { return NR <= 256 ? 16 : 256; }
ACCEL_HD constexpr int tw_pack_off(int NR) {  // in float2, from the start of the packed part
    return NR == 64 ? 0 : NR == 128 ? 64 : NR == 256 ? 128 : NR == 512 ? 192 : NR == 1024 ? 1216
         : NR == 2048 ? 2240 : 3264;           // NR == 4096
}
// Then, for the radix-16 pass with NR = 256 (16 distinct k, so one warp's
// loads of a slot fall in one 128-byte line), all fifteen powers W^jk,
// j = 1..15, slot-major: entry (j - 1) * 16 + k.
constexpr int kTwFull256 = 4288;    // offset of that section in the packed part
constexpr int kTwPacked = 4288 + 15 * 16;
constexpr int kTwTotal = kTwN + kTwPacked;
constexpr int kMinM = 64;           // smallest half-length FFT
constexpr int kMaxM = 8192;         // largest half-length FFT (L <= 16384)

// Short transforms: besides powers of two, the plane kernels take half
// lengths M = R * N2 with R = 5, 6 or 7 and N2 a power of two in
// [kMixedMinN2, kMixedMaxN2].  Such a transform is R transforms of N2
// points and one radix-R pass; its segment spectra and folded templates are
// stored in decimated order: position (k mod R) * N2 + k / R holds point k.
constexpr int kMixedMinN2 = 64;
constexpr int kMixedMaxN2 = 512;
// Behind the tables above, the twiddles of the radix-R pass of every short
// length, R = 5, 6, 7 and N2 = 64 .. 512 in turn: (R - 1) * N2 entries,
// entry (g - 1) * N2 + b = exp(2 pi i g b / (R N2)), so that the threads of
// consecutive butterflies b load consecutive addresses.
ACCEL_HD constexpr int tw_form_off(int R, int N2) {
    int off = kTwTotal;
    for (int r = 5; r <= 7; r++)
        for (int n = kMixedMinN2; n <= kMixedMaxN2; n *= 2) {
            if (r == R && n == N2) return off;
            off += (r - 1) * n;
        }
    return off;
}
constexpr int kTwAll = tw_form_off(8, 0);  // the end of the last section

// R of a plane-kernel half length M: 1 for a power of two, R for R * N2 as
// above, 0 for anything else.
ACCEL_HD int mixed_radix(int M) {
    if (M <= 0) return 0;
    if ((M & (M - 1)) == 0) return 1;
    for (int R = 5; R <= 7; R++) {
        if (M % R) continue;
        const int n2 = M / R;
        if ((n2 & (n2 - 1)) == 0 && n2 >= kMixedMinN2 && n2 <= kMixedMaxN2) return R;
    }
    return 0;
}

// Storage position of point k of a half length M transform (identity for a
// power of two).
ACCEL_HD int decimated_pos(int k, int M, int R) {
    if (R <= 1) return k;
    const int n2 = M / R;
    return (k % R) * n2 + k / R;
}

// ---------------------------------------------------------------- geometry
// z_response_halfwidth (bpd_subharmonics.cu:31-45) -- double arithmetic on
// purpose: the truncation points must match the reference.
ACCEL_HD int z_halfwidth(double z) {
    z = z < 0 ? -z : z;
    int m = (int)(z * (0.00089 * z + 0.3131) + kFintBins);
    m = (m < kFintBins) ? kFintBins : m;
    if (z > 100 && m > 0.6 * z) m = (int)(0.6 * z);
    return m;
}

// calc_required_z (bpd_subharmonics.cu:10-13): NEAREST_INT(z*h/(2H))*2,
// rounding halves away from zero.  Integer form: q = H is a power of two.
ACCEL_HD int required_z(int p, int q, int zfull) {
    // x = zfull * p / (2q); nearest int, ties away from zero
    long long num = (long long)zfull * p;     // x = num / (2q)
    long long den = 2LL * q;
    long long a = num < 0 ? -num : num;
    long long r = (2 * a + den) / (2 * den);  // floor(a/den + 1/2)
    return (int)(num < 0 ? -r : r) * kDz;
}

// (int)(2 * r * p/q + 0.5) for r = r2/2 >= 0 (calc_required_r before the
// final *0.5):  floor((2*r2*p + q) / (2q)).
ACCEL_HD long long twice_required_r(long long r2, int p, int q) {
    return (2LL * r2 * p + q) / (2LL * q);
}

ACCEL_HD long long next_pow2(long long x) {
    long long i = 1;
    while (i < x) i <<= 1;
    return i;
}

// Per-step, per-harmonic geometry (bpd_search.cu:72-127 and :138-144).
struct StepHarm {
    long long rlo;      // lowest full bin of this harmonic's window
    long long ceilhi;   // ceil(rhi)
    int numrs;          // powers per f-dot row
    long long lobin;    // first bin copied into the segment
    int numdata;        // bins copied and median-normalised
};

ACCEL_HD StepHarm step_harm(long long startr, int uselen, int p, int q, int hw0) {
    StepHarm g;
    long long a0 = twice_required_r(2 * startr, p, q);
    long long a1 = twice_required_r(2 * startr + uselen - 1, p, q);  // lastr = startr+U/2-1/2
    g.rlo = a0 >> 1;
    g.ceilhi = (a1 + 1) >> 1;
    if (p == 1 && q == 1) g.numrs = uselen;
    else g.numrs = (int)(2 * (g.ceilhi - g.rlo) + 2);  // odd 2d+1 rounded up to even
    g.lobin = g.rlo - hw0;
    g.numdata = (int)(g.ceilhi + hw0 - g.lobin + 1);
    return g;
}

// addPowers index arithmetic (bpd_gpu_kernels.cu:139-153):
// rind = (ushort)((subr - rlo_h) * 2), subr = (int)(2 rr f + 0.5) / 2,
// rr = startr + i/2.
ACCEL_HD int sub_rind(long long startr, int i, int p, int q, long long rlo_h) {
    long long a = twice_required_r(2 * startr + i, p, q);
    return (int)(unsigned short)(a - 2 * rlo_h);
}
// zind = (int)(((int)(zz * f) - zlo_h) * 0.5), zz = zlo0 + 2 z.
ACCEL_HD int sub_zind(int zz, int p, int q, int zlo_h) {
    int subz = (zz * p) / q;          // C division truncates like (int)(double)
    return (subz - zlo_h) / 2;        // (int)(x * 0.5) truncates toward zero too
}

// ---------------------------------------------------------------- numerics
#ifdef __CUDACC__
// inverse_square_root (bpd_math.c:94-105): magic constant and one Newton
// step, each operation rounded separately (no fused multiply-add).
__device__ __forceinline__ float rsqrt_magic(float x) {
    int i = __float_as_int(x);
    i = 0x5f3759df - (i >> 1);
    float y = __int_as_float(i);
    float h = __fmul_rn(0.5f, x);
    h = __fmul_rn(h, y);
    h = __fmul_rn(h, y);
    return __fmul_rn(y, __fsub_rn(1.5f, h));
}
// The normalisation factor 1/sqrt(x): the reference's approximation, or
// (exact) IEEE single precision.
__device__ __forceinline__ float rsqrt_norm(float x, int exact) {
    return exact ? __fdiv_rn(1.0f, __fsqrt_rn(x)) : rsqrt_magic(x);
}

// |a|^2 as the reference host code evaluates it: x*x + y*y, two rounded
// products and a rounded sum.
__device__ __forceinline__ float power_exact(float2 a) {
    return __fadd_rn(__fmul_rn(a.x, a.x), __fmul_rn(a.y, a.y));
}

__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }

// Exact k-th smallest (0-based) of n non-negative floats given as their bit
// patterns (monotone for x >= +0), by a 4-digit radix select over a
// 256-bin shared histogram.  All threads of the block must call it; `keys`
// and `hist` (256 ints) are shared memory.  Blocks of fewer than 32 threads
// (a single partial warp) are supported.  Returns the selected key.
__device__ __forceinline__ uint32_t block_select_u32(const uint32_t* keys, int n, int k,
                                                     int* hist, int* bcast) {
    uint32_t prefix = 0, mask = 0;
    const int tid = threadIdx.x, nt = blockDim.x;
    const int lane = tid & 31;
    const unsigned wmask = nt >= 32 ? 0xffffffffu : ((1u << nt) - 1u);
    for (int shift = 24; shift >= 0; shift -= 8) {
        for (int i = tid; i < 256; i += nt) hist[i] = 0;
        __syncthreads();
        for (int i0 = 0; i0 < n; i0 += nt) {
            int i = i0 + tid;
            bool act = false;
            uint32_t d = 0;
            if (i < n) {
                uint32_t key = keys[i];
                act = (key & mask) == prefix;
                d = (key >> shift) & 255u;
            }
            // aggregate equal digits within the warp before the atomic
            unsigned am = __ballot_sync(wmask, act);
            if (act) {
                unsigned peers = __match_any_sync(am, d);
                int leader = __ffs(peers) - 1;
                if (lane == leader) atomicAdd(&hist[d], __popc(peers));
            }
        }
        __syncthreads();
        if (nt >= 32) {
            if (tid < 32) {
                // each lane owns 8 consecutive bins; find the bin holding rank k
                int loc[8], s = 0;
                for (int j = 0; j < 8; j++) { loc[j] = hist[lane * 8 + j]; s += loc[j]; }
                int incl = s;
                for (int off = 1; off < 32; off <<= 1) {
                    int v = __shfl_up_sync(0xffffffffu, incl, off);
                    if (lane >= off) incl += v;
                }
                int excl = incl - s;
                if (k >= excl && k < incl) {
                    int c = excl;
                    for (int j = 0; j < 8; j++) {
                        if (k < c + loc[j]) { bcast[0] = lane * 8 + j; bcast[1] = k - c; break; }
                        c += loc[j];
                    }
                }
            }
        } else if (tid == 0) {
            int c = 0;
            for (int j = 0; j < 256; j++) {
                if (k < c + hist[j]) { bcast[0] = j; bcast[1] = k - c; break; }
                c += hist[j];
            }
        }
        __syncthreads();
        uint32_t digit = (uint32_t)bcast[0];
        k = bcast[1];
        prefix |= digit << shift;
        mask |= 255u << shift;
        __syncthreads();
    }
    return prefix;
}
#endif  // __CUDACC__

}  // namespace accel
