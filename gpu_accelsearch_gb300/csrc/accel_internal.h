// accel_internal.h -- types shared by the CUDA translation units of
// libaccelsearch.so.  Nothing here is part of the public C ABI
// (include/accelsearch.h).
#pragma once

#include <atomic>

#include <cuda.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <utility>
#include <vector>

#include "accel_common.cuh"

namespace accel {

// One harmonic of a template bank, as the kernels see it.
struct BankHarmDev {
    int harmnum, maxharm;   // fraction harmnum/maxharm of the fundamental
    int zmax;               // largest |z| of this harmonic's templates
    int numzs;              // templates, z = -zmax + 2 j
    int M;                  // half segment length (L = 2M)
    int hw0;                // halfwidth of the widest template (z = -zmax)
    int zlo;                // calc_required_z(f, -zmax_full)
    int tpl_base;           // first template index of this harmonic in the bank
    float2* kstd;           // [numzs][L]  FFT_L of the wrapped template
    float2* fold;           // [numzs][2M] A | B (see bank.cu)
    __half2* fold16;        // [numzs][2M] fold / scale, or null
    float* fold16_scale;    // [numzs]
};

// Per-segment descriptor: which whitened spectrum and where the step starts.
struct SegDesc {
    const float2* spec;     // whitened spectrum (bins [0, numbins) valid)
    long long numbins;      // N/2
    long long startr;       // first fundamental bin of the step
    int trial;              // caller's trial index
    int step;               // step index within the trial
};

// Per-harmonic plan of a search: bank data plus plane layout.
struct HarmPlan {
    int p, q;               // harmnum, maxharm
    int lq;                 // log2(q) (q is a power of two)
    int M;                  // half segment length
    int hw0, zlo, numzs;
    int wmax;               // columns written per f-dot row (max numrs over steps)
    int prow;               // row stride of the power plane (floats, multiple of 4)
    long long poff;         // offset of this plane inside a segment's plane block (floats)
    long long doff;         // offset of this harmonic's segment spectrum (float2)
    int zbase;              // prefix of numzs within the harmonic's M class
    const float2* fold;
    const __half2* fold16;
    const float* f16scale;
};

struct PrepArgs {
    HarmPlan h[kMaxHarm];
    int nh;                 // harmonics in this launch (one M class)
    int uselen;
    const SegDesc* segs;
    float2* dbuf;           // [nseg][dstride]
    long long dstride;
    int exact_rsqrt;        // IEEE 1/sqrt instead of the magic-constant one
};

struct PlaneArgs {
    HarmPlan h[kMaxHarm];
    int nh;                 // harmonics in this launch (one M class)
    int ntpl;               // sum of numzs over them
    const float2* dbuf;
    long long dstride;
    float* planes;          // [nseg][pstride]
    long long pstride;
    int use_fp16;
    int split;              // 1: even/odd transforms on separate threads
};

// Raw candidate as written by the harmonic-sum kernel (16 bytes).
struct RawCand {
    int32_t seg;            // segment index within the launch group
    int32_t ridx;           // fundamental r index, r = startr + ridx / 2
    int16_t zidx;           // fundamental z index, z = zlo0 + 2 zidx
    int16_t numharm;        // harmonics summed
    float power;
};

struct HsumArgs {
    HarmPlan h[kMaxHarm];
    int nh;                 // all harmonics of the bank, bank order
    int uselen;
    int numzs0, zlo0;
    int stage_of[kMaxHarm]; // stage index after harmonic h, or -1
    float cut[kMaxStages];
    const SegDesc* segs;
    const float* planes;
    long long pstride;
    RawCand* cands;
    unsigned long long* ncand;
    long long cap;
    int seg_base;           // added to the segment index stored in candidates
    float* stage_out;       // optional [nseg][nstages][numzs0][uselen]
    int nstages;
    unsigned long long* err;  // bit 0: a tile's copy wait timed out
    int tile_floats;          // largest shared-memory footprint of a tile (host-proven)
    unsigned test_extra_tx;   // 0, or (failure-detection test) bytes each tile expects
                              // beyond its copies, so that its bounded wait runs out
    // tensor path of the tiled sum (use_tmap): each harmonic's rectangle as
    // one box of box_h rows x 4 box_w4 columns at box_off floats (128-byte
    // aligned) in shared memory, box_tx bytes per tile in all
    int use_tmap;
    int box_w4[kMaxHarm], box_h[kMaxHarm], box_off[kMaxHarm];
    unsigned box_tx;
};

// Tensor maps of one plane buffer, harmonic by harmonic: 3-D (columns,
// f-dot rows, segments) views of each harmonic's planes for the tiled sum's
// box copies (kernel parameter space).
struct alignas(64) HsumMaps {
    CUtensorMap m[kMaxHarm];
};

// Fundamental plane fused with the harmonic sum (k_fund_sum).
struct FundArgs {
    HarmPlan h[kMaxHarm];   // all harmonics, bank order
    int nh;
    const float2* dbuf;
    long long dstride;
    const float* planes;    // sub-harmonic planes of the group
    long long pstride;
    int use_fp16;
    int split;
    int uselen;
    int numzs0, zlo0;
    int stage_of[kMaxHarm];
    float cut[kMaxStages];
    const SegDesc* segs;
    RawCand* cands;
    unsigned long long* ncand;
    long long cap;
    int seg_base;
    float* stage_out;       // optional [nseg][nstages][numzs0][uselen]
    int nstages;
};

// Kernel attributes (dynamic shared memory, carveout) are per device: a
// launcher keeps one bit per device it has configured.
inline bool attr_pending(const std::atomic<unsigned long long>& done, int* dev) {
    if (cudaGetDevice(dev) != cudaSuccess) *dev = 64;
    return *dev >= 64 || !((done.load() >> *dev) & 1ull);
}
inline void attr_set(std::atomic<unsigned long long>& done, int dev) {
    if (dev < 64) done.fetch_or(1ull << dev);
}

// The smallest shared-memory carveout (percent of the SM's shared memory)
// that holds as many CTAs of `kernel` as its registers and threads allow:
// the rest of the unified L1/shared array stays L1 for the kernel's global
// loads (the plane kernel: 2 CTAs of 70 KB take the 164 KB configuration,
// leaving 92 KB of L1 instead of 28 KB at the largest carveout).
inline int carveout_for(const void* kernel, int threads, size_t dyn_smem) {
    cudaFuncAttributes fa{};
    int dev = 0, smem_sm = 0, reserved = 0, regs_sm = 0, thr_sm = 0;
    if (cudaFuncGetAttributes(&fa, kernel) != cudaSuccess || cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&regs_sm, cudaDevAttrMaxRegistersPerMultiprocessor, dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&thr_sm, cudaDevAttrMaxThreadsPerMultiProcessor, dev) != cudaSuccess ||
        smem_sm <= 0 || threads <= 0) {
        cudaGetLastError();
        return 100;
    }
    const int regs = ((fa.numRegs + 7) & ~7) * threads;  // per CTA, in units of 8 registers a thread
    int ctas = std::min(thr_sm / threads, regs > 0 ? regs_sm / regs : 32);
    ctas = std::max(1, std::min(ctas, 32));
    const double need = (double)ctas * ((double)dyn_smem + fa.sharedSizeBytes + reserved);
    // the shared-memory capacities an SM of this family can be configured to
    // (KB); the percent just below the chosen one lands on it whether the
    // hint is rounded up or to the nearest capacity
    if (smem_sm != 228 * 1024) return 100;
    const int caps[] = {0, 8, 16, 32, 64, 100, 132, 164, 196, 228};
    for (int cap : caps)
        if (cap * 1024.0 >= need) return cap == 228 ? 100 : std::max(1, (int)std::floor(100.0 * cap / 228.0));
    return 100;
}

// Candidate refinement (k_optimize in bank.cu): one CTA per candidate.
struct OptCand {
    double r, z;            // fundamental-plane frequency and f-dot of the candidate
    int numharm;            // harmonics k r / numharm, k = 1..numharm, are summed
    int trial;
    long long lobin[kMaxHarm];  // harmonic k's segment in the candidate's step:
    int numdata[kMaxHarm];      // its median sets the power normalisation
};
struct OptOut {
    double r, z, power;     // refined position and summed power
    float harm[kMaxHarm];   // power of harmonic k at the refined position
};
struct OptArgs {
    const float2* const* spec;   // [ntrials] whitened spectra (device)
    const long long* numbins;    // [ntrials]
    const OptCand* in;
    OptOut* out;
    int n;
    int refine;                  // 0: evaluate at the given position only
    int maxdata;                 // largest numdata (shared-memory keys)
    int exact_rsqrt;
};

// ---- launchers (return 0 or -1 after a launch error) ----
int launch_fund_sum(const FundArgs& a, int nseg, const float2* tw, cudaStream_t st);
int launch_twiddles(float2* tw, cudaStream_t st);
int launch_optimize(const OptArgs& a, cudaStream_t st);
int launch_bank_build(const BankHarmDev* hd_dev, const BankHarmDev* hd_host, int nh, int ntpl,
                      float2* resp, int rstride, bool fp16, cudaStream_t st);
int launch_prep(int M, const PrepArgs& a, int nseg, const float2* tw, cudaStream_t st);
int launch_plane(int M, const PlaneArgs& a, int nseg, const float2* tw, cudaStream_t st);
int launch_hsum(const HsumArgs& a, int nseg, cudaStream_t st);
int launch_hsum_tile(const HsumArgs& a, int nseg, int tile_rows, const HsumMaps* maps, cudaStream_t st);
int launch_hsum_pipe(const HsumArgs& a, int nseg, cudaStream_t st);
// Tile geometry of launch_hsum_tile (the host proves the shared-memory bound).
constexpr int kHsumTileZ = 16;
constexpr int kHsumTileI = 256;
constexpr int kHsumTileFloats = 15360;
// Shared-memory bound of a tile of tz f-dot rows (floats): 60 KB for 8 and
// 16 rows, 112 KB for 32 (two CTAs per SM).
constexpr int hsum_tile_floats_max(int tz) { return tz > 16 ? 28672 : kHsumTileFloats; }
constexpr int kHsumTileRows[3] = {8, 16, 32};  // tile heights of launch_hsum_tile
constexpr int kPipeBuffers = 4;   // tile buffers of the pipelined harmonic sum
constexpr int kPipeSmemMax = 222 * 1024;  // their dynamic shared memory (227 KB less the static tables)

// A launch group's plane rows and harmonic-sum tiles in one persistent
// launch (k_step, step_kernel.cuh).
constexpr int kStepClasses = 4;
constexpr int kStepLag = 1;  // tiles of segment j run beside the rows of segment j + kStepLag

struct StepArgs {
    HsumArgs hs;                            // bank-order harmonics, planes, cuts, candidates, error word
    const float2* dbuf;                     // segment spectra [nseg][dstride]
    long long dstride;
    float* planes;                          // == hs.planes, written by the plane items
    int ncls;                               // plane classes (segment lengths M), largest first
    int cls_M[kStepClasses];
    int cls_nh[kStepClasses];
    int cls_h[kStepClasses][kMaxHarm];      // bank index of each harmonic of the class
    int cls_zbase[kStepClasses][kMaxHarm];  // its first row within the class
    int cls_ntpl[kStepClasses];             // rows of the class
    int cls_item0[kStepClasses + 1];        // first plane item of each class within a segment
    int P, T;                               // plane items and sum tiles per segment
    int rows;                               // plane rows per segment
    int nti;                                // tiles across the columns
    int nseg, lag;                          // lag <= nseg
    long long nitems;
    unsigned* next;                         // work counter, zero at launch
    unsigned* done;                         // [nseg] plane rows finished, zero at launch
};
int launch_step(const StepArgs& a, int mmax, int use_fp16, const float2* tw, cudaStream_t st);

// Record an error message for accel_last_error() and return `code`.
int set_error(int code, const char* fmt, ...);

// whitening
struct WhitenPlan;
int launch_whiten(const int* d_bstart, const int* d_blen, int nblocks, double* d_med, float2* spec,
                  unsigned numbins, int maxlen, cudaStream_t st, int exact_rsqrt = 0);
// Largest spectrum the whitening takes: block starts and lengths are int
// (as in the reference's recurrence) and every block lies below numbins.
constexpr long long kMaxWhitenBins = 0x7fffffffLL;
// Block recurrence of deredden (bpd_noise.c:33-79) in 64-bit arithmetic:
// writes the first min(count, cap) blocks to start/len (either may be null
// when cap is 0) and returns the number of blocks, or -1 when numbins,
// initbuf or maxbuf is out of range.
long long whiten_blocks(long long numbins, int initbuf, int maxbuf, int* start, int* len, long long cap);
std::vector<std::pair<int, int>> plan_whiten_blocks(long long numbins, int initbuf, int maxbuf);

}  // namespace accel
