// context.h -- the search context (accel_ctx) and the host-side driver
// functions shared by api.cu (the accel_* C ABI) and server.cu (the
// request server).  Internal to libaccelsearch.so.
#pragma once

#include <cufft.h>

#include <algorithm>
#include <map>
#include <string>
#include <vector>

#include "../../include/accelsearch.h"
#include "accel_internal.h"

namespace accel {

struct WhitenPlanDev {
    int nb = 0, maxlen = 0;
    int* d_start = nullptr;
    int* d_len = nullptr;
    double* d_med = nullptr;
    long long last_use = 0;
};

// Real-to-complex transforms of any even length from power-of-two C2C
// plans (rfft.cu).  One thread uses an engine at a time.
struct R2CEngine {
    std::map<long long, cufftHandle> plans;  // C2C plans by power-of-two length
    R2CEngine() = default;
    R2CEngine(const R2CEngine&) = delete;
    R2CEngine& operator=(const R2CEngine&) = delete;
    ~R2CEngine();
};
// spec[0 .. n/2] = the DFT of the n real samples of x (device, n even), on
// stream st: 0, -1 on a CUDA or cuFFT error, -2 when scratch memory runs out.
int r2c_any(R2CEngine& e, const float* x, long long n, float2* spec, cudaStream_t st);

struct TrialBuf {
    long long n = 0;            // allocated samples
    long long numbins = 0;      // whitened bins of the last search
    float* series = nullptr;
    float2* spec = nullptr;
};

}  // namespace accel

using namespace accel;  // internal header: the context is written in the library's own types

struct accel_ctx {
    accel_config cfg{};
    int last_trials = 0;        // trials of the last accel_search
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    int uselen = 0, nh = 0, nstages = 0, numzs0 = 0, zlo0 = 0;

    // bank
    BankHarmDev bh[kMaxHarm]{};
    BankHarmDev* d_bh = nullptr;
    void* bank_mem = nullptr;
    int ntpl = 0;
    float2* tw = nullptr;

    // plan
    HarmPlan hp[kMaxHarm]{};
    int stage_of[kMaxHarm]{};
    std::vector<int> mvals;
    long long dstride = 0, pstride = 0;
    float cuts[kMaxStages]{};

    // work buffers
    int chunk = 1;
    int plane_split = 0;
    int fused_sum = 0;
    int overlap = 1;          // sum of group k on stream2 while group k+1 is transformed
    cudaStream_t stream2 = nullptr;
    cudaStream_t copy_stream = nullptr;       // host-to-device copies of the series
    std::vector<cudaEvent_t> copy_ev;         // one per trial: its series has landed
    float* planes2 = nullptr; // second plane buffer for the overlap
    cudaEvent_t ev_fork = nullptr, ev_plane[2] = {nullptr, nullptr}, ev_sum[2] = {nullptr, nullptr};
    bool tile_ok = false;     // the tiled harmonic sum fits its shared buffer
    int hsum_tiled = 1;
    int hsum_pipe = 0;      // persistent pipelined tile kernel
    int persistent = 0;     // plane rows and sum tiles of a group in one launch (k_step)
    unsigned* d_step = nullptr;  // k_step's work counter and per-segment row counts
    int wait_test = 0;      // failure-detection test: every tile's copy wait runs out
    // CUDA graph of a device-resident search: recorded on two non-blocking
    // capture streams standing in for stream/stream2, launched on stream
    int use_graph = 1;
    bool capturing = false;   // launches are being recorded, not run
    cudaStream_t gcap = nullptr, gcap2 = nullptr;
    cudaGraphExec_t gexec = nullptr;
    int tile_floats = 0;
    int tile_floats_h[3] = {0, 0, 0};     // worst tile of 8, 16, 32 rows (floats)
    bool tile_ok_h[3] = {false, false, false};
    int tile_rows = 16;                   // height of the tiled sum's tiles
    // tensor path of the tiled sum: per tile height, each harmonic's box
    // (the largest rectangle of any tile), and the tensor maps of the two
    // plane buffers
    int hsum_tensor = 1;                  // box copies where the plan allows them
    int tbox_w4[3][kMaxHarm]{}, tbox_h[3][kMaxHarm]{}, tbox_off[3][kMaxHarm]{};
    int tbox_floats[3] = {0, 0, 0};
    unsigned tbox_tx[3] = {0, 0, 0};
    bool tbox_ok[3] = {false, false, false};
    HsumMaps tmaps[2][3]{};               // [plane buffer][tile height]
    bool tmaps_ok[2][3] = {};
    float2* dbuf = nullptr;
    float* planes = nullptr;
    SegDesc* d_segs = nullptr;
    SegDesc* h_segs = nullptr;  // pinned
    long long segs_cap = 0;
    RawCand* d_cands = nullptr;
    unsigned long long* d_ncand = nullptr;
    unsigned long long* h_ncand = nullptr;  // pinned
    RawCand* h_raw = nullptr;               // pinned read-back of the raw candidates
    long long h_raw_cap = 0;
    long long cand_cap = 0;

    std::map<unsigned, WhitenPlanDev> wplans;  // by spectrum length, at most kWhitenPlans
    long long wplan_clock = 0;
    R2CEngine r2c;  // the trials' real-to-complex transforms
    std::vector<TrialBuf> trials;

    std::vector<accel_candidate> results;
    unsigned long long last_raw = 0;

    // accounting
    bool profiling = false;
    struct Ev { int kind; cudaEvent_t a, b; };
    std::vector<Ev> pending;
    std::vector<cudaEvent_t> evpool;
    accel_stats stats{};
    cudaEvent_t ev_begin = nullptr, ev_end = nullptr;  // bracket each search call
};

namespace accel {

int ensure_device(accel_ctx* c);
int ensure_segs(accel_ctx* c, long long n);
int do_whiten(accel_ctx* c, float2* spec, unsigned numbins);
int do_rfft(accel_ctx* c, const float* series, long long n, float2* spec);
int run_group(accel_ctx* c, const SegDesc* d_segs, int nseg, int seg_base, float* stage_out,
              const float2* dh_in, float* planes_out, bool do_prep, bool do_plane, bool do_sum,
              bool fused = false, cudaStream_t sum_stream = nullptr);
void prof_collect(accel_ctx* c);
double sigma_of_power_host(double power, int numharm, double numindep);

}  // namespace accel
