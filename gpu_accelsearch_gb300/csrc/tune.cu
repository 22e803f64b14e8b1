// tune.cu -- the autotuner: picks the segment length and the launch shape
// (launch-group size, plane-kernel thread layout, harmonic-sum tile
// height) of a search by timing them on the GPU it will run on.
//
// For every candidate segment length it builds a context, whitens a seeded
// Gaussian spectrum generated on the device, and times accel_search_spectra
// over a fixed number of overlap-save steps with CUDA events, for every
// launch shape.  Throughput is counted in fundamental f-fdot cells per
// second, which is comparable across segment lengths.
#include <cmath>
#include <cstring>
#include <vector>

#include "../../include/accelsearch.h"
#include "accel_internal.h"

namespace accel {

__device__ __forceinline__ unsigned long long mix64(unsigned long long x) {
    x += 0x9e3779b97f4a7c15ULL;
    x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ULL;
    x = (x ^ (x >> 27)) * 0x94d049bb133111ebULL;
    return x ^ (x >> 31);
}

// Complex N(0,1) values from a counter-based hash and Box-Muller.
__global__ void k_noise_spectrum(float2* out, long long n, unsigned long long seed) {
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    unsigned long long h = mix64(seed ^ mix64((unsigned long long)i));
    float u1 = ((h >> 40) + 1) * (1.0f / 16777217.0f);
    float u2 = ((h >> 16) & 0xffffff) * (1.0f / 16777216.0f);
    float r = sqrtf(-2.0f * logf(u1));
    float s, c;
    sincospif(2.0f * u2, &s, &c);
    out[i] = make_float2(r * c, r * s);
}

int launch_noise_spectrum(float2* out, long long n, unsigned long long seed, cudaStream_t st) {
    k_noise_spectrum<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(out, n, seed);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace accel

extern "C" int accel_autotune(const accel_config* base, const int* fftlens, int nlens, int steps,
                              accel_config* best_cfg, accel_tuning* best_tuning, double* best_rate) {
    using namespace accel;
    if (!base || !fftlens || nlens <= 0 || steps <= 0 || !best_cfg || !best_tuning)
        return set_error(ACCEL_ERR_INVALID, "accel_autotune: bad argument");
    double best = -1.0;
    const int chunks[] = {16, 32, 64, 128, 256, 512};
    constexpr int kChunks = 6;
    for (int li = 0; li < nlens; li++) {
        accel_config cfg = *base;
        cfg.fftlen = fftlens[li];
        cfg.uselen = 0;
        cfg.chunk_segments = 8;
        accel_ctx* ctx = nullptr;
        int rc = accel_create(&cfg, &ctx);
        if (rc == ACCEL_ERR_UNSUPPORTED || rc == ACCEL_ERR_INVALID) continue;  // shape not buildable
        if (rc) return rc;
        const int U = accel_uselen(ctx);
        const long long rlo = 1000;
        const long long numbins = rlo + (long long)(steps + 1) * (U / 2) + 2;
        float2* spec = nullptr;
        cudaError_t e = cudaMalloc(&spec, sizeof(float2) * numbins);
        cudaStream_t st = nullptr;
        cudaEvent_t t0 = nullptr, t1 = nullptr;
        if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreate(&t0);
        if (e == cudaSuccess) e = cudaEventCreate(&t1);
        if (e != cudaSuccess) {
            accel_destroy(ctx);
            cudaFree(spec);
            return set_error(ACCEL_ERR_CUDA, "accel_autotune: %s", cudaGetErrorString(e));
        }
        accel_set_stream(ctx, st);
        rc = launch_noise_spectrum(spec, numbins, 0x5eedULL + li, st) ? ACCEL_ERR_CUDA : ACCEL_OK;
        if (!rc) rc = accel_whiten(ctx, reinterpret_cast<accel_complex*>(spec), numbins);
        const accel_complex* sp = reinterpret_cast<const accel_complex*>(spec);
        long long nsteps = 0;
        for (long long r = rlo; r + U / 2 < numbins; r += U / 2) nsteps++;
        accel_harmonic h0;
        accel_harmonic_info(ctx, 0, &h0);
        // best of two timed searches (after a warm one), in cells per second
        auto timed = [&](const accel_tuning& t, double* rate) -> int {
            int r = accel_set_tuning(ctx, &t);
            long long nc = 0;
            if (!r) r = accel_search_spectra(ctx, 1, &sp, &numbins, &rlo, &nc);  // warm
            if (r == ACCEL_ERR_CAPACITY) r = ACCEL_OK;
            if (r) return r;
            float best_ms = 1e30f;
            for (int rep = 0; rep < 2; rep++) {
                cudaEventRecord(t0, st);
                r = accel_search_spectra(ctx, 1, &sp, &numbins, &rlo, &nc);
                if (r == ACCEL_ERR_CAPACITY) r = ACCEL_OK;
                cudaEventRecord(t1, st);
                cudaEventSynchronize(t1);
                float ms = 0.f;
                cudaEventElapsedTime(&ms, t0, t1);
                if (ms < best_ms) best_ms = ms;
            }
            *rate = (double)nsteps * U * h0.numzs / (best_ms * 1e-3);
            return r;
        };
        const double best_before = best;
        accel_tuning best_here{};
        for (int combo = 0; combo < 4 && !rc; combo++) {
            for (int ci = 0; ci < kChunks && !rc; ci++) {
                if (ci > 0 && chunks[ci] > steps) break;  // the sample would fit in one group anyway
                accel_tuning t{};
                t.chunk_segments = chunks[ci];
                t.plane_split = combo & 1;
                t.fused_sum = combo >> 1;
                double rate = 0.0;
                rc = timed(t, &rate);
                if (rc) break;
                if (rate > best) {
                    best = rate;
                    *best_cfg = cfg;
                    best_cfg->chunk_segments = chunks[ci];
                    *best_tuning = t;
                    best_here = t;
                }
            }
        }
        // the tile height of the tiled harmonic sum, at the best shape of
        // this segment length when it is the best so far
        if (!rc && best > best_before && !best_here.fused_sum) {
            for (int tz : {8, 32}) {
                accel_tuning t = best_here;
                t.hsum_tile_rows = tz;
                double rate = 0.0;
                rc = timed(t, &rate);
                if (rc) break;
                if (rate > best) {
                    best = rate;
                    *best_tuning = t;
                }
            }
        }
        accel_destroy(ctx);
        cudaEventDestroy(t0);
        cudaEventDestroy(t1);
        cudaStreamDestroy(st);
        cudaFree(spec);
        if (rc) return rc;
    }
    if (best < 0) return set_error(ACCEL_ERR_UNSUPPORTED, "accel_autotune: no candidate could be built");
    if (best_rate) *best_rate = best;
    return ACCEL_OK;
}
