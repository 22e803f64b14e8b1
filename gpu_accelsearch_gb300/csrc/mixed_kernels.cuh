// mixed_kernels.cuh -- segment preparation and power planes of harmonics
// whose transforms have a short length M = R * N2 (fft_mixed.cuh) instead of
// the reference's power of two.
//
// The reference transforms each harmonic's segment at L_h = 2 M_h, the
// power of two above numdata (bpd_subharmonics.cu:60-67), and keeps the
// columns [2 hw0, 2 hw0 + numrs).  Those columns are a linear correlation of
// the first numdata bins with templates of halfwidth <= hw0, so any length
// M >= numdata gives the same values (up to FP32 rounding): the circular
// wrap of a shorter transform only reaches columns below 2 hw0.  At zmax
// 200 / 8 harmonics the 3/4, 5/8 and 7/8 harmonics fit 3/4, 5/8 and 7/8 of
// their power of two.
//
// Both kernels do exactly what k_prep and k_plane do (the same median
// normalisation, products, powers and stores), on the decimated storage
// order of the segment spectra and folded templates.  The plane kernels are
// instantiated in search_mixed{5,6,7}.cu, the preparation kernel (one for
// every short length) in search_mixed_prep.cu.
#pragma once

#include "fft_mixed.cuh"
#include "search_kernels.cuh"

namespace accel {

// Segment preparation of every short harmonic of a launch group in one
// launch (grid: harmonic x segment, kPrepShortThreads threads): each CTA
// runs the body of its harmonic's length.  Per length, the first
// roundup32(R N2/16) threads carry the R transforms (plus idle groups on
// zero data that fill their last warp, each with its own buffer) and
// synchronise on named barrier 1; all threads take part in the median and
// the radix-R pass.
constexpr int kPrepShortThreads = 256;

// Dynamic shared memory of the body for R * N2 points: GROUPS padded
// N2-point buffers and the median keys.
ACCEL_HD constexpr size_t prep_short_smem(int R, int N2) {
    return sizeof(float2) * (size_t)(((R * (N2 / 16) + 31) / 32 * 32) / (N2 / 16)) * (N2 + N2 / 16) +
           sizeof(uint32_t) * (size_t)(R * N2);
}
template <int R, int N2> struct MixedPrepShape {
    static constexpr int T2 = N2 / 16;
    static constexpr int FFT_THREADS = (R * T2 + 31) / 32 * 32;
    static constexpr int GROUPS = FFT_THREADS / T2;
    static constexpr int PM2 = FftShape<N2>::PADDED;
    static constexpr size_t SMEM = prep_short_smem(R, N2);
    static_assert(SMEM == sizeof(float2) * GROUPS * PM2 + sizeof(uint32_t) * R * N2, "layout");
    static_assert(FFT_THREADS <= kPrepShortThreads, "short transform fits the preparation CTA");
};

// generate_harmonic_ffdot_data + the forward transform of one harmonic's
// segment (bpd_search.cu:130-184, :228-240), as k_prep, into decimated order.
template <int R, int N2>
__device__ __forceinline__ void prep_short_body(const PrepArgs& a, const HarmPlan& H, const float2* __restrict__ tw,
                                                unsigned char* smem_raw, int* hist, int* bc, float* s_norm) {
    using S = MixedPrepShape<R, N2>;
    constexpr int T2 = S::T2, PM2 = S::PM2, M = R * N2;
    float2* sm = reinterpret_cast<float2*>(smem_raw);
    uint32_t* keys = reinterpret_cast<uint32_t*>(sm + S::GROUPS * PM2);
    const SegDesc sd = a.segs[blockIdx.y];
    const StepHarm g = step_harm(sd.startr, a.uselen, H.p, H.q, H.hw0);
    const int tid = threadIdx.x;
    const int grp = tid / T2, t = tid - grp * T2;
    const bool real = grp < R;
    const int numdata = g.numdata < M ? g.numdata : M;  // host checks numdata <= M

    float2 x[1][16];
#pragma unroll
    for (int e = 0; e < 16; e++) {
        const int idx = R * (t + e * T2) + grp;  // point of the segment
        float2 v = make_float2(0.f, 0.f);
        if (real) {
            const long long b = g.lobin + idx;
            if (b >= 0 && b < sd.numbins) v = sd.spec[b];
            if (idx < numdata) keys[idx] = __float_as_uint(power_exact(v));
        }
        x[0][e] = v;
    }
    __syncthreads();
    const uint32_t mk = block_select_u32(keys, numdata, (numdata - 1) / 2, hist, bc);
    if (tid == 0) *s_norm = rsqrt_norm((float)((double)__uint_as_float(mk) / kLn2), a.exact_rsqrt);
    __syncthreads();
    const float norm = *s_norm;
    if (tid < S::FFT_THREADS) {
#pragma unroll
        for (int e = 0; e < 16; e++) {
            if (real && R * (t + e * T2) + grp < numdata) {
                x[0][e].x = __fmul_rn(x[0][e].x, norm);
                x[0][e].y = __fmul_rn(x[0][e].y, norm);
            }
        }
        float2* buf = sm + grp * PM2;
        fft_run<N2, -1, 1, GroupSync>(x, buf, tw, t, GroupSync{1, S::FFT_THREADS});
#pragma unroll
        for (int e = 0; e < 16; e++) buf[fft_pad(t + e * T2)] = x[0][e];
    }
    __syncthreads();
    float2* out = a.dbuf + (long long)blockIdx.y * a.dstride + H.doff;
#pragma unroll 1
    for (int b = tid; b < N2; b += kPrepShortThreads) {
        float2 v[1][R];
        mixed_last_pass<R, N2, -1, 1, PM2>(v, sm, tw, b);
#pragma unroll
        for (int k1 = 0; k1 < R; k1++) {
            const int m = b + N2 * k1;
            out[(m % R) * N2 + m / R] = v[0][k1];
        }
    }
}

// perform_convolution + perform_inversefft + generatePowers of k_plane for a
// short transform: U rows (templates) per CTA, each by UNIT threads; the
// radix-R pass runs over all rows' butterflies and stores the powers of the
// valid window as (even, odd) pairs.
template <int R, int N2, bool F16>
__global__ void __launch_bounds__(MixedShape<R, N2>::THREADS, MixedShape<R, N2>::MINB)
    k_plane_mixed(const PlaneArgs a, const float2* __restrict__ tw) {
    using S = MixedShape<R, N2>;
    constexpr int T2 = S::T2, PM2 = S::PM2, M = S::M;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float2* sm = reinterpret_cast<float2*>(smem_raw);
    __shared__ float* s_row[S::U];
    __shared__ int s_lo[S::U], s_w[S::U];

    const int tid = threadIdx.x;
    const int seg = blockIdx.x;
    if (tid < S::FFT_THREADS) {
        const int u = tid / S::UNIT, ut = tid - u * S::UNIT;
        const int grp = ut / T2, t = ut - grp * T2;
        // segments vary fastest across the grid, as in k_plane
        int item = blockIdx.y * S::U + u;
        const bool live = item < a.ntpl;
        if (!live) item = a.ntpl - 1;  // a valid row, computed but not stored
        int hi = 0;
#pragma unroll 1
        while (hi + 1 < a.nh && item >= a.h[hi + 1].zbase) hi++;
        const HarmPlan& H = a.h[hi];
        const int z = item - H.zbase;
        if (ut == 0) {
            s_row[u] = a.planes + (long long)seg * a.pstride + H.poff + (long long)z * H.prow;
            s_lo[u] = H.hw0;
            s_w[u] = live ? (H.wmax >> 1) : 0;
        }
        const float2* __restrict__ D = a.dbuf + (long long)seg * a.dstride + H.doff;
        float2 x[2][16];
#pragma unroll
        for (int e = 0; e < 16; e++) {
            const int p = grp * N2 + t + e * T2;  // decimated position
            const float2 d = D[p];
            x[0][e] = cmul(d, fold_at<M, F16>(H, z, 0, p));
            x[1][e] = cmul(d, fold_at<M, F16>(H, z, 1, p));
        }
        float2* buf = sm + (u * R + grp) * S::GS;
        // the transforms' barriers: the whole CTA, or (with the extra warp)
        // named barrier 1 over the transforms' threads only
        if constexpr (S::EXTRA == 0) fft_run<N2, +1, 2>(x, buf, tw, t);
        else fft_run<N2, +1, 2, GroupSync>(x, buf, tw, t, GroupSync{1, S::FFT_THREADS});
#pragma unroll
        for (int e = 0; e < 16; e++) {
            const int i = fft_pad(t + e * T2);
            buf[i] = x[0][e];
            buf[PM2 + i] = x[1][e];
        }
    }
    __syncthreads();
#pragma unroll 1
    for (int j = tid; j < S::U * N2; j += S::THREADS) {
        const int uu = j / N2, b = j - uu * N2;
        float2 v[2][R];
        mixed_last_pass<R, N2, +1, 2, S::GS>(v, sm + uu * R * S::GS, tw, b);
        float* row = s_row[uu];
        const int lo = s_lo[uu], w = s_w[uu];
#pragma unroll
        for (int k1 = 0; k1 < R; k1++) {
            const int i2 = b + N2 * k1 - lo;  // one unsigned compare for 0 <= i2 < w
            if ((unsigned)i2 < (unsigned)w)
                *reinterpret_cast<float2*>(row + 2 * i2) =
                    make_float2(fmaf(v[0][k1].x, v[0][k1].x, v[0][k1].y * v[0][k1].y),
                                fmaf(v[1][k1].x, v[1][k1].x, v[1][k1].y * v[1][k1].y));
        }
    }
}

// -------------------------------------------------------------- launchers
template <int R, int N2, bool F16>
static int plane_mixed(const PlaneArgs& a, int nseg, const float2* tw, cudaStream_t st) {
    using S = MixedShape<R, N2>;
    const size_t smem = sizeof(float2) * S::U * R * S::GS;
    static std::atomic<unsigned long long> attr{0};
    int dev = 0;
    if (attr_pending(attr, &dev)) {
        if (cudaFuncSetAttribute(k_plane_mixed<R, N2, F16>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem) != cudaSuccess ||
            cudaFuncSetAttribute(k_plane_mixed<R, N2, F16>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                 carveout_for((const void*)k_plane_mixed<R, N2, F16>, S::THREADS, smem)) !=
                cudaSuccess)
            return -1;
        attr_set(attr, dev);
    }
    const int rows = (a.ntpl + S::U - 1) / S::U;
    k_plane_mixed<R, N2, F16><<<dim3(nseg, rows), S::THREADS, smem, st>>>(a, tw);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

// Dispatch on N2 for one R (the instantiating translation unit).
template <int R> static int plane_mixed_r(int N2, const PlaneArgs& a, int nseg, const float2* tw, cudaStream_t st) {
    const bool h = a.use_fp16 != 0;
    switch (N2) {
        case 64: return h ? plane_mixed<R, 64, true>(a, nseg, tw, st) : plane_mixed<R, 64, false>(a, nseg, tw, st);
        case 128: return h ? plane_mixed<R, 128, true>(a, nseg, tw, st) : plane_mixed<R, 128, false>(a, nseg, tw, st);
        case 256: return h ? plane_mixed<R, 256, true>(a, nseg, tw, st) : plane_mixed<R, 256, false>(a, nseg, tw, st);
        case 512: return h ? plane_mixed<R, 512, true>(a, nseg, tw, st) : plane_mixed<R, 512, false>(a, nseg, tw, st);
    }
    return -1;
}

}  // namespace accel
