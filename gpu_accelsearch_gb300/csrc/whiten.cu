// whiten.cu -- red-noise removal (deredden, bpd_noise.c:12-92) on the GPU.
//
// The reference walks the spectrum serially: block medians of growing
// width (initialbuflen*ln(binnum), capped at maxbuflen), a linear slope
// between neighbouring block levels, and amplitude *= rsqrt(level).  The
// block boundaries are a serial recurrence and are planned on the host
// (plan_whiten_blocks in api.cu); everything else is parallel:
//   k_whiten_medians  one CTA per block: exact lower median of |A|^2
//                     (radix select), level = median / ln 2 in double;
//   k_whiten_scale    one CTA per write range: the range's level and slope
//                     from its two neighbouring blocks, then the scaling
//                     with the reference's float arithmetic.
// Results are bit-identical to the reference's host routine.
#include <cmath>
#include <mutex>

#include "../../include/accelsearch.h"
#include "accel_internal.h"

namespace accel {

constexpr double kLn2w = 0.693147180559945309417232121458;

__global__ void __launch_bounds__(256) k_whiten_medians(const int* __restrict__ bstart,
                                                        const int* __restrict__ blen,
                                                        const float2* __restrict__ spec, double* med) {
    extern __shared__ uint32_t keys[];
    __shared__ int hist[256];
    __shared__ int bc[2];
    const int b = blockIdx.x;
    const int s = bstart[b], n = blen[b];
    for (int i = threadIdx.x; i < n; i += blockDim.x) keys[i] = __float_as_uint(power_exact(spec[s + i]));
    __syncthreads();
    const uint32_t k = block_select_u32(keys, n, (n - 1) / 2, hist, bc);
    if (threadIdx.x == 0) med[b] = (double)__uint_as_float(k) / kLn2w;
}

// Write range r (0 <= r <= nb): r = 0 is the first half-block with a flat
// level; 1 <= r < nb interpolate from block r-1 towards block r; r = nb is
// the tail, continuing the last slope (1.0 when there was no second block).
__global__ void __launch_bounds__(256) k_whiten_scale(const int* __restrict__ bstart,
                                                      const int* __restrict__ blen,
                                                      const double* __restrict__ med, int nb,
                                                      float2* spec, unsigned numbins, int exact) {
    const int r = blockIdx.x;
    long long lo, hi;
    float mean_old, dslope;
    if (r == 0) {
        lo = 1;
        hi = bstart[0] + blen[0] / 2;
        mean_old = (float)med[0];
        dslope = 0.f;
        if (threadIdx.x == 0) spec[0] = make_float2(1.0f, 0.0f);
    } else if (r < nb) {
        lo = bstart[r - 1] + blen[r - 1] / 2;
        hi = bstart[r] + blen[r] / 2;
        mean_old = (float)med[r - 1];
        dslope = (float)((med[r] - (double)mean_old) / (0.5 * (blen[r - 1] + blen[r])));
    } else {
        lo = bstart[nb - 1] + blen[nb - 1] / 2;
        hi = numbins;
        mean_old = (float)med[nb - 1];
        if (nb >= 2) {
            const float mo = (float)med[nb - 2];
            dslope = (float)((med[nb - 1] - (double)mo) / (0.5 * (blen[nb - 2] + blen[nb - 1])));
        } else {
            dslope = 1.0f;
        }
    }
    const float flat = rsqrt_norm(mean_old, exact);
    for (long long ind = lo + threadIdx.x; ind < hi; ind += blockDim.x) {
        float norm;
        if (r == 0) norm = flat;
        else norm = rsqrt_norm(__fadd_rn(mean_old, __fmul_rn(dslope, (float)(ind - lo))), exact);
        float2 v = spec[ind];
        v.x = __fmul_rn(v.x, norm);
        v.y = __fmul_rn(v.y, norm);
        spec[ind] = v;
    }
}

// Warp-per-block forms of the two kernels for blocks of at most
// kWarpBlockMax bins (the reference's widths are at most 200): eight
// whitening blocks per CTA, no CTA-wide barriers.
constexpr int kWarpBlockMax = 1024;
constexpr int kWarpsPerCta = 8;

// Exact rank-k key of keys[0..n) by an 8-bit radix select within one warp
// (hist: 256 ints of this warp's shared memory).
__device__ __forceinline__ uint32_t warp_select_u32(const uint32_t* keys, int n, int k, int* hist) {
    const int lane = threadIdx.x & 31;
    uint32_t prefix = 0, mask = 0;
#pragma unroll 1
    for (int shift = 24; shift >= 0; shift -= 8) {
#pragma unroll
        for (int j = 0; j < 8; j++) hist[lane * 8 + j] = 0;
        __syncwarp();
        for (int i0 = 0; i0 < n; i0 += 32) {
            const int i = i0 + lane;
            bool act = false;
            uint32_t d = 0;
            if (i < n) {
                const uint32_t key = keys[i];
                act = (key & mask) == prefix;
                d = (key >> shift) & 255u;
            }
            // aggregate equal digits before the shared-memory atomic
            const unsigned am = __ballot_sync(0xffffffffu, act);
            if (act) {
                const unsigned peers = __match_any_sync(am, d);
                if (lane == __ffs(peers) - 1) atomicAdd(&hist[d], __popc(peers));
            }
        }
        __syncwarp();
        int loc[8], sum = 0;
#pragma unroll
        for (int j = 0; j < 8; j++) {
            loc[j] = hist[lane * 8 + j];
            sum += loc[j];
        }
        int incl = sum;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int v = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += v;
        }
        const int excl = incl - sum;
        int digit = 0, knew = 0;
        const bool mine = k >= excl && k < incl;
        if (mine) {
            int c = excl;
#pragma unroll
            for (int j = 0; j < 8; j++) {
                if (k >= c && k < c + loc[j]) {
                    digit = lane * 8 + j;
                    knew = k - c;
                }
                c += loc[j];
            }
        }
        const int src = __ffs(__ballot_sync(0xffffffffu, mine)) - 1;
        digit = __shfl_sync(0xffffffffu, digit, src);
        k = __shfl_sync(0xffffffffu, knew, src);
        prefix |= (uint32_t)digit << shift;
        mask |= 255u << shift;
        __syncwarp();
    }
    return prefix;
}

__global__ void __launch_bounds__(32 * kWarpsPerCta) k_whiten_medians_warp(const int* __restrict__ bstart,
                                                                           const int* __restrict__ blen,
                                                                           const float2* __restrict__ spec,
                                                                           double* med, int nblocks, int maxlen) {
    extern __shared__ uint32_t wsm[];  // per warp: 256 histogram ints, then maxlen keys
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int b = blockIdx.x * kWarpsPerCta + w;
    if (b >= nblocks) return;  // whole warps leave; nothing below synchronises the CTA
    int* hist = reinterpret_cast<int*>(wsm + (size_t)w * (256 + maxlen));
    uint32_t* keys = wsm + (size_t)w * (256 + maxlen) + 256;
    const int s = bstart[b], n = blen[b];
    for (int i = lane; i < n; i += 32) keys[i] = __float_as_uint(power_exact(spec[s + i]));
    __syncwarp();
    const uint32_t k = warp_select_u32(keys, n, (n - 1) / 2, hist);
    if (lane == 0) med[b] = (double)__uint_as_float(k) / kLn2w;
}

// Write range r as in k_whiten_scale, one warp per range.
__global__ void __launch_bounds__(32 * kWarpsPerCta) k_whiten_scale_warp(const int* __restrict__ bstart,
                                                                         const int* __restrict__ blen,
                                                                         const double* __restrict__ med, int nb,
                                                                         float2* spec, unsigned numbins,
                                                                         int exact) {
    const int r = blockIdx.x * kWarpsPerCta + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    if (r > nb) return;
    long long lo, hi;
    float mean_old, dslope;
    if (r == 0) {
        lo = 1;
        hi = bstart[0] + blen[0] / 2;
        mean_old = (float)med[0];
        dslope = 0.f;
        if (lane == 0) spec[0] = make_float2(1.0f, 0.0f);
    } else if (r < nb) {
        lo = bstart[r - 1] + blen[r - 1] / 2;
        hi = bstart[r] + blen[r] / 2;
        mean_old = (float)med[r - 1];
        dslope = (float)((med[r] - (double)mean_old) / (0.5 * (blen[r - 1] + blen[r])));
    } else {
        lo = bstart[nb - 1] + blen[nb - 1] / 2;
        hi = numbins;
        mean_old = (float)med[nb - 1];
        if (nb >= 2) {
            const float mo = (float)med[nb - 2];
            dslope = (float)((med[nb - 1] - (double)mo) / (0.5 * (blen[nb - 2] + blen[nb - 1])));
        } else {
            dslope = 1.0f;
        }
    }
    const float flat = rsqrt_norm(mean_old, exact);
    for (long long ind = lo + lane; ind < hi; ind += 32) {
        float norm;
        if (r == 0) norm = flat;
        else norm = rsqrt_norm(__fadd_rn(mean_old, __fmul_rn(dslope, (float)(ind - lo))), exact);
        float2 v = spec[ind];
        v.x = __fmul_rn(v.x, norm);
        v.y = __fmul_rn(v.y, norm);
        spec[ind] = v;
    }
}

// Block recurrence of deredden (bpd_noise.c:33-79): the first block holds
// initbuf bins from bin 1; each next block starts where the last ended and
// holds (int)(initbuf * ln(start)) bins, at most maxbuf; blocks continue
// while start + length < numbins.  Positions are carried in 64 bits so that
// no sum overflows near kMaxWhitenBins; the width is clamped before the
// conversion to int (same result wherever the reference's is defined).
long long whiten_blocks(long long numbins, int initbuf, int maxbuf, int* start, int* len, long long cap) {
    if (initbuf < 1 || maxbuf < 1 || numbins <= 1 + (long long)initbuf || numbins > kMaxWhitenBins) return -1;
    auto width = [&](long long at) {
        const double x = initbuf * std::log((double)at);
        return x >= (double)maxbuf ? maxbuf : (int)x;
    };
    long long n = 0, binnum = 1;
    int buflen = initbuf;
    for (;;) {
        if (n < cap) {
            start[n] = (int)binnum;
            len[n] = buflen;
        }
        n++;
        binnum += buflen;
        buflen = width(binnum);
        if (binnum + buflen >= numbins) break;
    }
    return n;
}

std::vector<std::pair<int, int>> plan_whiten_blocks(long long numbins, int initbuf, int maxbuf) {
    const long long n = whiten_blocks(numbins, initbuf, maxbuf, nullptr, nullptr, 0);
    std::vector<std::pair<int, int>> b;
    if (n <= 0) return b;
    std::vector<int> s((size_t)n), l((size_t)n);
    whiten_blocks(numbins, initbuf, maxbuf, s.data(), l.data(), n);
    b.reserve((size_t)n);
    for (long long i = 0; i < n; i++) b.push_back({s[i], l[i]});
    return b;
}

int launch_whiten(const int* d_bstart, const int* d_blen, int nblocks, double* d_med, float2* spec,
                  unsigned numbins, int maxlen, cudaStream_t st, int exact) {
    if (maxlen <= kWarpBlockMax) {
        const size_t smem = sizeof(uint32_t) * (size_t)kWarpsPerCta * (256 + maxlen);
        if (smem > 48 * 1024 &&
            cudaFuncSetAttribute(k_whiten_medians_warp, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem) != cudaSuccess)
            return -1;
        k_whiten_medians_warp<<<(nblocks + kWarpsPerCta - 1) / kWarpsPerCta, 32 * kWarpsPerCta, smem, st>>>(
            d_bstart, d_blen, spec, d_med, nblocks, maxlen);
        if (cudaGetLastError() != cudaSuccess) return -1;
        k_whiten_scale_warp<<<(nblocks + kWarpsPerCta) / kWarpsPerCta, 32 * kWarpsPerCta, 0, st>>>(
            d_bstart, d_blen, d_med, nblocks, spec, numbins, exact);
        return cudaGetLastError() == cudaSuccess ? 0 : -1;
    }
    size_t smem = sizeof(uint32_t) * (size_t)maxlen;
    if (smem > 48 * 1024) {
        if (cudaFuncSetAttribute(k_whiten_medians, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem) != cudaSuccess)
            return -1;
    }
    k_whiten_medians<<<nblocks, 256, smem, st>>>(d_bstart, d_blen, spec, d_med);
    if (cudaGetLastError() != cudaSuccess) return -1;
    k_whiten_scale<<<nblocks + 1, 256, 0, st>>>(d_bstart, d_blen, d_med, nblocks, spec, numbins, exact);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace accel

// --------------------------------------------------------------------------
// Allocation-free whitening (accel_whiten_noalloc).
//
// Same kernels as above; their scratch -- the block table (start, length)
// and the per-block levels -- lives in one file-scope device array instead
// of memory allocated by a context.  Every GPU that loads the library holds
// this array (2 MiB) until the process exits.  All calls share it, so calls
// whose GPU work overlaps race; every byte a call reads is written earlier
// by the same call (table copy, then medians), so nothing needs clearing.
namespace accel {
namespace {

constexpr int kNoAllocBlocks = 131072;
constexpr size_t kNoAllocBytes = (size_t)kNoAllocBlocks * (2 * sizeof(int) + sizeof(double));
static __device__ __align__(256) unsigned char g_whiten_scratch[kNoAllocBytes];

constexpr int kNoAllocDevices = 64;
std::mutex g_noalloc_mutex;
void* g_noalloc_addr[kNoAllocDevices];           // device address of g_whiten_scratch
int g_noalloc_start[kNoAllocBlocks];             // host staging of the block table
int g_noalloc_len[kNoAllocBlocks];

}  // namespace
}  // namespace accel

extern "C" int accel_whiten_noalloc(accel_complex* spec, long long numbins, int initbuf, int maxbuf,
                                    void* stream) {
    using namespace accel;
    if (!spec) return set_error(ACCEL_ERR_INVALID, "accel_whiten_noalloc: null spectrum");
    if (initbuf < 1 || maxbuf < 1 || maxbuf > 49152)
        return set_error(ACCEL_ERR_INVALID,
                         "accel_whiten_noalloc: block widths must be in [1, 49152]");
    if (numbins <= 1 + (long long)initbuf || numbins > kMaxWhitenBins)
        return set_error(ACCEL_ERR_INVALID, "accel_whiten_noalloc: %lld bins out of range (%d .. %lld)",
                         numbins, initbuf + 2, kMaxWhitenBins);
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess)
        return set_error(ACCEL_ERR_CUDA, "accel_whiten_noalloc: cudaGetDevice: %s", cudaGetErrorString(e));
    if (dev < 0 || dev >= kNoAllocDevices)
        return set_error(ACCEL_ERR_UNSUPPORTED, "accel_whiten_noalloc: device %d", dev);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    // The block table goes to the device by a copy from host arrays that the
    // next call overwrites: a captured copy would replay whatever table the
    // latest call left there, so calls inside a stream capture are refused.
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    e = cudaStreamIsCapturing(st, &cap);
    if (e != cudaSuccess || cap != cudaStreamCaptureStatusNone) {
        if (e != cudaSuccess) cudaGetLastError();
        return set_error(ACCEL_ERR_UNSUPPORTED, "accel_whiten_noalloc: not callable during stream capture");
    }
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_addr[dev]) {
        // once per device, with that device current: the array's device address
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_whiten_scratch);
        if (e != cudaSuccess || !p)
            return set_error(ACCEL_ERR_CUDA, "accel_whiten_noalloc: cudaGetSymbolAddress: %s",
                             cudaGetErrorString(e));
        g_noalloc_addr[dev] = p;
    }
    const long long nbl = whiten_blocks(numbins, initbuf, maxbuf, g_noalloc_start, g_noalloc_len, kNoAllocBlocks);
    const int nb = (int)nbl;
    if (nbl > kNoAllocBlocks)
        return set_error(ACCEL_ERR_INVALID,
                         "accel_whiten_noalloc: %lld bins need more than %d whitening blocks, the "
                         "size of the static scratch (about 1.2e7 bins with the default widths)",
                         numbins, kNoAllocBlocks);
    int maxlen = 0;
    for (int i = 0; i < nb; i++) maxlen = g_noalloc_len[i] > maxlen ? g_noalloc_len[i] : maxlen;
    char* base = static_cast<char*>(g_noalloc_addr[dev]);
    int* d_start = reinterpret_cast<int*>(base);
    int* d_len = reinterpret_cast<int*>(base + sizeof(int) * kNoAllocBlocks);
    double* d_med = reinterpret_cast<double*>(base + 2 * sizeof(int) * kNoAllocBlocks);
    // pageable source: the copies have left the host arrays when they return
    e = cudaMemcpyAsync(d_start, g_noalloc_start, sizeof(int) * nb, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(d_len, g_noalloc_len, sizeof(int) * nb, cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess)
        return set_error(ACCEL_ERR_CUDA, "accel_whiten_noalloc: block table copy: %s",
                         cudaGetErrorString(e));
    if (launch_whiten(d_start, d_len, nb, d_med, reinterpret_cast<float2*>(spec), (unsigned)numbins,
                      maxlen, st) != 0)
        return set_error(ACCEL_ERR_CUDA, "accel_whiten_noalloc: launch: %s",
                         cudaGetErrorString(cudaGetLastError()));
    return ACCEL_OK;
}
