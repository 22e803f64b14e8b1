// search.cu -- the per-step hot path.
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
#include "accel_internal.h"
#include "fft_smem.cuh"

namespace accel {

constexpr double kLn2 = 0.693147180559945309417232121458;

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
    const int numdata = g.numdata < M ? g.numdata : M;  // host checks next_pow2(numdata) == M

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
    if (t == 0) s_norm = rsqrt_magic((float)((double)__uint_as_float(mk) / kLn2));
    __syncthreads();
    const float norm = s_norm;
#pragma unroll
    for (int e = 0; e < 16; e++) {
        if (t + e * T < numdata) {
            x[0][e].x = __fmul_rn(x[0][e].x, norm);
            x[0][e].y = __fmul_rn(x[0][e].y, norm);
        }
    }
    fft_run<M, -1, 1>(x, sm, tw);
    float2* out = a.dbuf + (long long)blockIdx.y * a.dstride + H.doff;
#pragma unroll
    for (int e = 0; e < 16; e++) out[t + e * T] = x[0][e];
}

// ----------------------------------------------------------------- plane
template <int M, bool F16>
__global__ void __launch_bounds__(M / 16) k_plane(const PlaneArgs a, const float2* __restrict__ tw) {
    constexpr int T = M / 16;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float2* sm = reinterpret_cast<float2*>(smem_raw);

    const int item = blockIdx.x;
    int hi = 0;
#pragma unroll 1
    while (hi + 1 < a.nh && item >= a.h[hi + 1].zbase) hi++;
    const HarmPlan& H = a.h[hi];
    const int z = item - H.zbase;
    const int seg = blockIdx.y;
    const int t = threadIdx.x;
    const float2* D = a.dbuf + (long long)seg * a.dstride + H.doff;

    float2 x[2][16];
    if constexpr (F16) {
        const __half2* f = H.fold16 + (size_t)z * 2 * M;
        const float sc = H.f16scale[z];
#pragma unroll
        for (int e = 0; e < 16; e++) {
            const int idx = t + e * T;
            const float2 d = D[idx];
            float2 A = __half22float2(f[idx]);
            float2 B = __half22float2(f[M + idx]);
            A.x *= sc; A.y *= sc; B.x *= sc; B.y *= sc;
            x[0][e] = cmul(d, A);
            x[1][e] = cmul(d, B);
        }
    } else {
        const float2* f = H.fold + (size_t)z * 2 * M;
#pragma unroll
        for (int e = 0; e < 16; e++) {
            const int idx = t + e * T;
            const float2 d = D[idx];
            x[0][e] = cmul(d, __ldg(f + idx));
            x[1][e] = cmul(d, __ldg(f + M + idx));
        }
    }
    fft_run<M, +1, 2>(x, sm, tw);

    const float scale = 1.0f / (4.0f * (float)M * (float)M);  // 1 / L^2, exact
    float* row = a.planes + (long long)seg * a.pstride + H.poff + (long long)z * H.prow;
    const int half_w = H.wmax >> 1;
#pragma unroll
    for (int e = 0; e < 16; e++) {
        const int i2 = t + e * T - H.hw0;
        if (i2 >= 0 && i2 < half_w) {
            float2 p;
            p.x = fmaf(x[0][e].x, x[0][e].x, x[0][e].y * x[0][e].y) * scale;
            p.y = fmaf(x[1][e].x, x[1][e].x, x[1][e].y * x[1][e].y) * scale;
            *reinterpret_cast<float2*>(row + 2 * i2) = p;
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

__device__ __forceinline__ long long twice_r_shift(long long r2, int p, int lq) {
    return (2LL * r2 * p + (1LL << lq)) >> (lq + 1);
}
__device__ __forceinline__ int trunc_shift(int x, int k) {  // C division by 2^k
    return x >= 0 ? (x >> k) : -((-x) >> k);
}

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
            const int st = a.stage_of[h];
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
    static bool attr = false;
    if (!attr) {
        if (cudaFuncSetAttribute(k_prep<M>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
            cudaSuccess)
            return -1;
        attr = true;
    }
    k_prep<M><<<dim3(a.nh, nseg), M / 16, smem, st>>>(a, tw);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

template <int M, bool F16>
static int plane_m(const PlaneArgs& a, int nseg, const float2* tw, cudaStream_t st) {
    size_t smem = sizeof(float2) * FftShape<M>::PADDED * 2;
    static bool attr = false;
    if (!attr) {
        if (cudaFuncSetAttribute(k_plane<M, F16>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem) != cudaSuccess)
            return -1;
        attr = true;
    }
    k_plane<M, F16><<<dim3(a.ntpl, nseg), M / 16, smem, st>>>(a, tw);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int launch_prep(int M, const PrepArgs& a, int nseg, const float2* tw, cudaStream_t st) {
    switch (M) {
        case 64: return prep_m<64>(a, nseg, tw, st);
        case 128: return prep_m<128>(a, nseg, tw, st);
        case 256: return prep_m<256>(a, nseg, tw, st);
        case 512: return prep_m<512>(a, nseg, tw, st);
        case 1024: return prep_m<1024>(a, nseg, tw, st);
        case 2048: return prep_m<2048>(a, nseg, tw, st);
        case 4096: return prep_m<4096>(a, nseg, tw, st);
        case 8192: return prep_m<8192>(a, nseg, tw, st);
    }
    return -1;
}

int launch_plane(int M, const PlaneArgs& a, int nseg, const float2* tw, cudaStream_t st) {
    const bool h = a.use_fp16 != 0;
    switch (M) {
        case 64: return h ? plane_m<64, true>(a, nseg, tw, st) : plane_m<64, false>(a, nseg, tw, st);
        case 128: return h ? plane_m<128, true>(a, nseg, tw, st) : plane_m<128, false>(a, nseg, tw, st);
        case 256: return h ? plane_m<256, true>(a, nseg, tw, st) : plane_m<256, false>(a, nseg, tw, st);
        case 512: return h ? plane_m<512, true>(a, nseg, tw, st) : plane_m<512, false>(a, nseg, tw, st);
        case 1024: return h ? plane_m<1024, true>(a, nseg, tw, st) : plane_m<1024, false>(a, nseg, tw, st);
        case 2048: return h ? plane_m<2048, true>(a, nseg, tw, st) : plane_m<2048, false>(a, nseg, tw, st);
        case 4096: return h ? plane_m<4096, true>(a, nseg, tw, st) : plane_m<4096, false>(a, nseg, tw, st);
        case 8192: return h ? plane_m<8192, true>(a, nseg, tw, st) : plane_m<8192, false>(a, nseg, tw, st);
    }
    return -1;
}

int launch_hsum(const HsumArgs& a, int nseg, cudaStream_t st) {
    dim3 grid((a.uselen + kHsumCols - 1) / kHsumCols, (a.numzs0 + kHsumRows - 1) / kHsumRows, nseg);
    switch (a.nh) {
        case 1: k_hsum<1><<<grid, kHsumCols, 0, st>>>(a); break;
        case 2: k_hsum<2><<<grid, kHsumCols, 0, st>>>(a); break;
        case 4: k_hsum<4><<<grid, kHsumCols, 0, st>>>(a); break;
        case 8: k_hsum<8><<<grid, kHsumCols, 0, st>>>(a); break;
        case 16: k_hsum<16><<<grid, kHsumCols, 0, st>>>(a); break;
        default: return -1;
    }
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace accel
