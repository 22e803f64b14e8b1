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
// same window of every channel run together and find it in L2.
#include <cmath>
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
    const int ndtile = (ndm + kDdD - 1) / kDdD;
    const long long ntt = (nout + kDdThreads * kDdPer - 1) / (kDdThreads * kDdPer);
    if ((long long)ndtile * ntt > 0x7fffffffLL) return set_error(ACCEL_ERR_UNSUPPORTED, "accel_dedisperse: grid too large");
    cudaStream_t st = (cudaStream_t)cuda_stream;
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
