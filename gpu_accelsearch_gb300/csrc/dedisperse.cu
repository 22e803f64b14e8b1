// dedisperse.cu -- incoherent dedispersion of a filterbank into DM trials
// (accel_dedisperse_delays, accel_dedisperse): the step upstream of the
// search that produces its input time series.  The reference takes series
// that are already dedispersed (its README names dedispersion as the step
// before it); this is the direct method in its textbook form:
//
//   out[d][t] = sum over channels c, in order, of in[c][t + delay[d][c]]
//   delay[d][c] = floor(kDM * DM_d * (f_c^-2 - f_ref^-2) / tsamp + 1/2)
//
// with the dispersion constant kDM = 4.148808e3 s MHz^2 pc^-1 cm^3, f_c the
// frequency of channel c (f_top + c * chan_bw) and f_ref the highest channel
// frequency, so that every delay is >= 0.
//
// Layout: filterbank channel-major [nchan][nsamp] float32 (time contiguous),
// output [ndm][nout] float32 with nout <= nsamp - max delay.  One CTA owns
// kDdD DM trials x kDdThreads*kDdPer consecutive output samples (each
// thread kDdPer samples kDdThreads apart, so every load of a warp is one
// contiguous run) and accumulates in registers over the channels in order
// (rounded float adds: the same sums as the host restatement).  The grid
// runs the DM tiles of one time window fastest, so the CTAs that read the
// same window of every channel run together and find it in L2.  The
// windowed form below (k_dedisperse_win) replaces it wherever a tile's
// delays lie close enough together for shared-memory windows.
#include <cmath>
#include <cstdint>
#include <vector>

#include "../../include/accelsearch.h"
#include "accel_internal.h"

namespace accel {

constexpr int kDdThreads = 256;
constexpr int kDdPer = 4;  // output samples per thread
constexpr int kDdD = 8;    // DM trials per CTA (a multiple of 4: int4 delay loads)
static_assert(kDdD % 4 == 0, "delays are loaded as int4");
constexpr double kDispConst = 4.148808e3;

__global__ void __launch_bounds__(kDdThreads) k_dedisperse(const float* __restrict__ in, int nchan, long long nsamp,
                                                           const int4* __restrict__ dtab, int ndm, int ndtile,
                                                           float* __restrict__ out, long long nout) {
    const long long bid = blockIdx.x;
    const int tile = (int)(bid % ndtile);
    const int d0 = tile * kDdD;
    const long long t0 = (bid / ndtile) * (long long)(kDdThreads * kDdPer) + threadIdx.x;
    const int nd = min(kDdD, ndm - d0);
    float acc[kDdD][kDdPer];
#pragma unroll
    for (int j = 0; j < kDdD; j++)
#pragma unroll
        for (int k = 0; k < kDdPer; k++) acc[j][k] = 0.f;
    // dtab row c: the delays of channel c for the tile's kDdD DM trials as
    // kDdD/4 int4 (padding trials have delay 0 and are not summed)
    constexpr int kQ = kDdD / 4;
    const int4* __restrict__ dt = dtab + (long long)kQ * tile;
    const long long dstride = (long long)kQ * ndtile;
#pragma unroll 4
    for (int c = 0; c < nchan; c++) {
        const float* __restrict__ row = in + (long long)c * nsamp;
        int dl[kDdD];
#pragma unroll
        for (int q = 0; q < kQ; q++) {
            const int4 v = __ldg(dt + c * dstride + q);
            dl[4 * q] = v.x;
            dl[4 * q + 1] = v.y;
            dl[4 * q + 2] = v.z;
            dl[4 * q + 3] = v.w;
        }
#pragma unroll
        for (int j = 0; j < kDdD; j++) {
            if (j < nd) {  // uniform over the CTA
#pragma unroll
                for (int k = 0; k < kDdPer; k++) {
                    const long long t = t0 + (long long)k * kDdThreads;
                    if (t < nout) acc[j][k] = __fadd_rn(acc[j][k], __ldg(row + t + dl[j]));
                }
            }
        }
    }
#pragma unroll
    for (int j = 0; j < kDdD; j++) {
        if (j < nd) {
#pragma unroll
            for (int k = 0; k < kDdPer; k++) {
                const long long t = t0 + (long long)k * kDdThreads;
                if (t < nout) out[(long long)(d0 + j) * nout + t] = acc[j][k];
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Windowed form (the default where its windows fit): a CTA owns kDwD DM
// trials x kDdThreads*kDdPer output samples.  For each chunk of kDwC
// channels it copies, per channel, the window of input samples its trials
// read -- [t0 + wmin_c, t0 + T + wmax_c) with wmin_c / wmax_c the smallest /
// largest delay of the tile's trials in channel c -- into shared memory by
// asynchronous copies (cp.async, 4 bytes each, zero-filled past the end of
// the series), double-buffered so that chunk k+1 lands while chunk k is
// summed; each sample copied once serves all kDwD trials.  The sums are
// the same rounded float adds in the same channel order as k_dedisperse.
constexpr int kDwD = 16;  // DM trials per CTA
constexpr int kDwC = 8;   // channels per chunk

__device__ __forceinline__ void cp_async4(float* dst, const float* src, bool valid) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(d), "l"(src), "r"(valid ? 4 : 0)
                 : "memory");
}

// rel [ndtile][nchan][kDwD]: delay - wmin of the tile's trials (0 for padding
// trials); wmin [ndtile][nchan]; every window fits wlen floats.
__global__ void __launch_bounds__(kDdThreads, 2)
    k_dedisperse_win(const float* __restrict__ in, int nchan, long long nsamp, const int* __restrict__ rel,
                     const int* __restrict__ wmin, int ndm, int ndtile, int wlen, float* __restrict__ out,
                     long long nout) {
    extern __shared__ __align__(16) float dsm[];  // [2][kDwC][wlen] windows, then [2][kDwC][kDwD] delays
    int* sdel = reinterpret_cast<int*>(dsm + 2 * kDwC * wlen);
    const long long bid = blockIdx.x;
    const int tile = (int)(bid % ndtile);
    const int d0 = tile * kDwD;
    const long long t0 = (bid / ndtile) * (long long)(kDdThreads * kDdPer);
    const int tid = threadIdx.x;
    const int nd = min(kDwD, ndm - d0);
    const int nchunk = (nchan + kDwC - 1) / kDwC;
    auto stage = [&](int k, int buf) {
        const int c0 = k * kDwC;
        for (int i = tid; i < kDwC * kDwD; i += kDdThreads) {
            const int c = c0 + i / kDwD;
            sdel[(buf * kDwC + i / kDwD) * kDwD + i % kDwD] =
                c < nchan ? rel[((long long)tile * nchan + c) * kDwD + i % kDwD] : 0;
        }
        for (int cc = 0; cc < kDwC; cc++) {
            const int c = c0 + cc;
            if (c >= nchan) break;
            const long long base = t0 + wmin[(long long)tile * nchan + c];
            const float* row = in + (long long)c * nsamp;
            float* dst = dsm + (buf * kDwC + cc) * wlen;
            for (int x = tid; x < wlen; x += kDdThreads) {
                const long long idx = base + x;
                const bool ok = idx < nsamp;
                cp_async4(dst + x, row + (ok ? idx : 0), ok);
            }
        }
        asm volatile("cp.async.commit_group;\n" ::: "memory");
    };
    float acc[kDwD][kDdPer];
#pragma unroll
    for (int j = 0; j < kDwD; j++)
#pragma unroll
        for (int q = 0; q < kDdPer; q++) acc[j][q] = 0.f;
    stage(0, 0);
#pragma unroll 1
    for (int k = 0; k < nchunk; k++) {
        const int buf = k & 1;
        if (k + 1 < nchunk) {
            stage(k + 1, buf ^ 1);
            asm volatile("cp.async.wait_group 1;\n" ::: "memory");  // chunk k has landed
        } else {
            asm volatile("cp.async.wait_group 0;\n" ::: "memory");
        }
        __syncthreads();
        const int ncc = min(kDwC, nchan - k * kDwC);
#pragma unroll 1
        for (int cc = 0; cc < ncc; cc++) {
            const float* w = dsm + (buf * kDwC + cc) * wlen + tid;
            const int* dl = sdel + (buf * kDwC + cc) * kDwD;
#pragma unroll
            for (int j = 0; j < kDwD; j++) {
                const int off = dl[j];
#pragma unroll
                for (int q = 0; q < kDdPer; q++) acc[j][q] = __fadd_rn(acc[j][q], w[off + q * kDdThreads]);
            }
        }
        __syncthreads();  // buffer buf is refilled by the next iteration's stage
    }
#pragma unroll
    for (int j = 0; j < kDwD; j++) {
        if (j < nd) {
#pragma unroll
            for (int q = 0; q < kDdPer; q++) {
                const long long t = t0 + tid + (long long)q * kDdThreads;
                if (t < nout) out[(long long)(d0 + j) * nout + t] = acc[j][q];
            }
        }
    }
}

}  // namespace accel

using namespace accel;

extern "C" {

int accel_dedisperse_delays(int nchan, double f_top_mhz, double chan_bw_mhz, double tsamp, const float* dms,
                            int ndm, int* delays, int* max_delay) {
    if (nchan < 1 || ndm < 1 || !dms || !delays || !(tsamp > 0.0) || !(f_top_mhz > 0.0) || chan_bw_mhz == 0.0)
        return set_error(ACCEL_ERR_INVALID, "accel_dedisperse_delays: bad argument");
    const double f_last = f_top_mhz + (nchan - 1) * chan_bw_mhz;
    if (!(f_last > 0.0)) return set_error(ACCEL_ERR_INVALID, "accel_dedisperse_delays: channel frequency <= 0");
    const double f_ref = std::max(f_top_mhz, f_last);
    const double inv_ref2 = 1.0 / (f_ref * f_ref);
    int mx = 0;
    for (int d = 0; d < ndm; d++) {
        if (!(dms[d] >= 0.0f)) return set_error(ACCEL_ERR_INVALID, "accel_dedisperse_delays: DM %d < 0", d);
        for (int c = 0; c < nchan; c++) {
            const double f = f_top_mhz + c * chan_bw_mhz;
            const double v = std::floor(kDispConst * (double)dms[d] * (1.0 / (f * f) - inv_ref2) / tsamp + 0.5);
            if (v > 2147483647.0) return set_error(ACCEL_ERR_INVALID, "accel_dedisperse_delays: delay overflow");
            delays[(long long)d * nchan + c] = (int)v;
            mx = std::max(mx, (int)v);
        }
    }
    if (max_delay) *max_delay = mx;
    return ACCEL_OK;
}

int accel_dedisperse(const float* filterbank_dev, int nchan, long long nsamp, const int* delays, int ndm,
                     float* out_dev, long long nout, void* cuda_stream) {
    if (!filterbank_dev || !out_dev || !delays || nchan < 1 || ndm < 1 || nsamp < 1 || nout < 1)
        return set_error(ACCEL_ERR_INVALID, "accel_dedisperse: bad argument");
    const long long nd = (long long)ndm * nchan;
    int mx = 0;
    for (long long i = 0; i < nd; i++) {
        if (delays[i] < 0) return set_error(ACCEL_ERR_INVALID, "accel_dedisperse: negative delay");
        mx = std::max(mx, delays[i]);
    }
    if (nout > nsamp - mx)
        return set_error(ACCEL_ERR_INVALID, "accel_dedisperse: %lld output samples need %lld input samples, have %lld",
                         nout, nout + mx, nsamp);
    cudaStream_t st = (cudaStream_t)cuda_stream;
    const long long ntt = (nout + kDdThreads * kDdPer - 1) / (kDdThreads * kDdPer);
    {
        // windowed kernel: per tile of kDwD trials and channel, the delays
        // relative to their smallest; the widest window sizes shared memory
        const int nwt = (ndm + kDwD - 1) / kDwD;
        std::vector<int> rel((size_t)nwt * nchan * kDwD, 0), wmn((size_t)nwt * nchan, 0);
        int spread = 0;
        for (int tl = 0; tl < nwt; tl++)
            for (int c = 0; c < nchan; c++) {
                int lo = INT32_MAX, hi = 0;
                for (int j = 0; j < kDwD && tl * kDwD + j < ndm; j++) {
                    const int v = delays[(long long)(tl * kDwD + j) * nchan + c];
                    lo = std::min(lo, v);
                    hi = std::max(hi, v);
                }
                wmn[(size_t)tl * nchan + c] = lo;
                spread = std::max(spread, hi - lo);
                for (int j = 0; j < kDwD && tl * kDwD + j < ndm; j++)
                    rel[((size_t)tl * nchan + c) * kDwD + j] = delays[(long long)(tl * kDwD + j) * nchan + c] - lo;
            }
        const int wlen = ((kDdThreads * kDdPer + spread) + 3) & ~3;
        const size_t smem = sizeof(float) * 2 * kDwC * (size_t)wlen + sizeof(int) * 2 * kDwC * kDwD;
        if (smem <= 100 * 1024 && (long long)nwt * ntt <= 0x7fffffffLL) {
            static std::atomic<unsigned long long> attr{0};
            int dev = 0;
            cudaError_t e = cudaSuccess;
            if (attr_pending(attr, &dev)) {
                e = cudaFuncSetAttribute(k_dedisperse_win, cudaFuncAttributeMaxDynamicSharedMemorySize, 100 * 1024);
                if (e == cudaSuccess)
                    e = cudaFuncSetAttribute(k_dedisperse_win, cudaFuncAttributePreferredSharedMemoryCarveout,
                                             cudaSharedmemCarveoutMaxShared);
                if (e == cudaSuccess) attr_set(attr, dev);
            }
            int* d_rel = nullptr;
            int* d_wmn = nullptr;
            if (e == cudaSuccess) e = cudaMallocAsync(reinterpret_cast<void**>(&d_rel), sizeof(int) * rel.size(), st);
            if (e == cudaSuccess) e = cudaMallocAsync(reinterpret_cast<void**>(&d_wmn), sizeof(int) * wmn.size(), st);
            // from pageable memory: staged before the call returns
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(d_rel, rel.data(), sizeof(int) * rel.size(), cudaMemcpyHostToDevice, st);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(d_wmn, wmn.data(), sizeof(int) * wmn.size(), cudaMemcpyHostToDevice, st);
            if (e == cudaSuccess) {
                k_dedisperse_win<<<(unsigned)(nwt * ntt), kDdThreads, smem, st>>>(filterbank_dev, nchan, nsamp, d_rel,
                                                                                 d_wmn, ndm, nwt, wlen, out_dev, nout);
                e = cudaGetLastError();
            }
            if (d_rel) {
                const cudaError_t ef = cudaFreeAsync(d_rel, st);
                if (e == cudaSuccess) e = ef;
            }
            if (d_wmn) {
                const cudaError_t ef = cudaFreeAsync(d_wmn, st);
                if (e == cudaSuccess) e = ef;
            }
            if (e != cudaSuccess) return set_error(ACCEL_ERR_CUDA, "accel_dedisperse: %s", cudaGetErrorString(e));
            return ACCEL_OK;
        }
    }
    // delays too far apart within a tile for the windows: one load per addition
    const int ndtile = (ndm + kDdD - 1) / kDdD;
    if ((long long)ndtile * ntt > 0x7fffffffLL) return set_error(ACCEL_ERR_UNSUPPORTED, "accel_dedisperse: grid too large");
    // the kernel's table: channel-major, each channel's delays of all DM
    // trials padded to whole tiles of kDdD (one 32-byte sector per tile)
    const long long pad = (long long)ndtile * kDdD;
    std::vector<int> tab((size_t)(pad * nchan), 0);
    for (int d = 0; d < ndm; d++)
        for (int c = 0; c < nchan; c++) tab[(size_t)c * pad + d] = delays[(long long)d * nchan + c];
    int* d_delays = nullptr;
    cudaError_t e = cudaMallocAsync(reinterpret_cast<void**>(&d_delays), sizeof(int) * tab.size(), st);
    if (e != cudaSuccess) return set_error(ACCEL_ERR_NOMEM, "accel_dedisperse: %s", cudaGetErrorString(e));
    // from pageable memory: staged before the call returns
    e = cudaMemcpyAsync(d_delays, tab.data(), sizeof(int) * tab.size(), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) {
        k_dedisperse<<<(unsigned)(ndtile * ntt), kDdThreads, 0, st>>>(
            filterbank_dev, nchan, nsamp, reinterpret_cast<const int4*>(d_delays), ndm, ndtile, out_dev, nout);
        e = cudaGetLastError();
    }
    const cudaError_t ef = cudaFreeAsync(d_delays, st);
    if (e == cudaSuccess) e = ef;
    if (e != cudaSuccess) return set_error(ACCEL_ERR_CUDA, "accel_dedisperse: %s", cudaGetErrorString(e));
    return ACCEL_OK;
}

}  // extern "C"
