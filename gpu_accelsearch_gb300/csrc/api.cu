// api.cu -- host side of libaccelsearch.so: the accel_* C ABI, the search
// context (template bank, plans, work buffers) and the overlap-save driver.
//
// The reference drives one DM trial from main() (AccelSearch.cu:48-281): a
// host loop over steps, each step a synchronous H2D copy of host-prepared
// segments and a sequence of launches.  Here a search call takes any number
// of trials, keeps their spectra on the device, and runs the steps of all
// of them in launch groups of `chunk` segments: segment preparation, the
// fused plane kernel and the harmonic sum, with no host round trip.
#include <cudaTypedefs.h>
#include <cufft.h>

#include <algorithm>
#include <functional>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <thread>
#include <vector>

#include "../../include/accelsearch.h"
#include "accel_internal.h"
#include "context.h"

using namespace accel;

namespace {

thread_local std::string g_err;

int set_err(int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_err = buf;
    return code;
}

#define CK(x)                                                                                    \
    do {                                                                                         \
        cudaError_t e_ = (x);                                                                    \
        if (e_ != cudaSuccess)                                                                   \
            return set_err(ACCEL_ERR_CUDA, "%s failed: %s", #x, cudaGetErrorString(e_));         \
    } while (0)

#define CKL(x, what)                                                                             \
    do {                                                                                         \
        if ((x) != 0) {                                                                          \
            cudaError_t e_ = cudaGetLastError();                                                 \
            return set_err(ACCEL_ERR_CUDA, "%s launch failed: %s", what, cudaGetErrorString(e_)); \
        }                                                                                        \
    } while (0)

// ---- Gamma(n,1) tail and Gaussian equivalents (candidate cut and sigma)
double log_gamma_q(int n, double x) {  // log P(Gamma(n,1) > x)
    double term = 1.0, s = 1.0;
    for (int k = 1; k < n; k++) {
        term *= x / k;
        s += term;
    }
    return -x + std::log(s);
}
double log_gauss_tail(double sigma) {  // log P(N(0,1) > sigma)
    if (sigma < 30.0) return std::log(0.5 * std::erfc(sigma / std::sqrt(2.0)));
    // asymptotic expansion beyond double erfc's range
    double s2 = sigma * sigma;
    return -0.5 * s2 - std::log(sigma * std::sqrt(2.0 * M_PI)) + std::log1p(-1.0 / s2 + 3.0 / (s2 * s2));
}
double power_cut(double sigma, int numharm, double numindep) {
    double logp = log_gauss_tail(sigma) - std::log(numindep > 1.0 ? numindep : 1.0);
    double lo = 0.0, hi = 4096.0;
    for (int it = 0; it < 200; it++) {
        double mid = 0.5 * (lo + hi);
        if (log_gamma_q(numharm, mid) > logp) lo = mid;
        else hi = mid;
    }
    return 0.5 * (lo + hi);
}
// Equivalent Gaussian significance: solve log Q(sigma) = logp with Newton
// steps on log Q, whose derivative is -phi(s)/Q(s) (the inverse Mills ratio).
double sigma_of_power(double power, int numharm, double numindep) {
    const double logp = log_gamma_q(numharm, power) + std::log(numindep > 1.0 ? numindep : 1.0);
    if (logp >= std::log(0.5)) return 0.0;
    double s = std::sqrt(-2.0 * logp);  // asymptotic start, slightly above the root
    for (int it = 0; it < 50; it++) {
        const double f = log_gauss_tail(s) - logp;
        const double lphi = -0.5 * s * s - 0.5 * std::log(2.0 * M_PI);
        const double d = -std::exp(lphi - log_gauss_tail(s));  // d/ds log Q(s)
        const double step = f / d;
        s -= step;
        if (s < 0.0) s = 0.0;
        if (std::fabs(step) < 1e-10 * (1.0 + s)) break;
    }
    return s;
}
}  // namespace



namespace accel {

int ensure_device(accel_ctx* c) {
    CK(cudaSetDevice(c->device));
    return ACCEL_OK;
}

enum { K_PREP = 0, K_PLANE = 1, K_HSUM = 2, K_WHITEN = 3, K_RFFT = 4, K_FUND = 5, K_STEP = 6 };

cudaEvent_t take_event(accel_ctx* c) {
    cudaEvent_t e = nullptr;
    if (!c->evpool.empty()) {
        e = c->evpool.back();
        c->evpool.pop_back();
    } else {
        cudaEventCreate(&e);
    }
    return e;
}

// Bracket `nlaunch` kernel launches of one kind with events (when profiling).
struct ProfScope {
    accel_ctx* c;
    int kind;
    cudaStream_t st;
    cudaEvent_t a = nullptr;
    ProfScope(accel_ctx* c_, int kind_, int nlaunch, cudaStream_t st_ = nullptr)
        : c(c_), kind(kind_), st(st_ ? st_ : c_->stream) {
        if (kind != K_RFFT) c->stats.launches += nlaunch;
        c->stats.kind_launches[kind] += nlaunch;
        if (c->profiling) {
            a = take_event(c);
            record(a);
        }
    }
    // inside a graph capture the events become event-record nodes, timed
    // when the graph runs
    void record(cudaEvent_t e) const {
        if (c->capturing) cudaEventRecordWithFlags(e, st, cudaEventRecordExternal);
        else cudaEventRecord(e, st);
    }
    ~ProfScope() {
        if (a) {
            cudaEvent_t b = take_event(c);
            record(b);
            c->pending.push_back({kind, a, b});
        }
    }
};

// Fold finished event pairs into the stats (the stream must be idle).
void prof_collect(accel_ctx* c) {
    for (auto& e : c->pending) {
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, e.a, e.b) == cudaSuccess) c->stats.kind_ms[e.kind] += ms;
        c->evpool.push_back(e.a);
        c->evpool.push_back(e.b);
    }
    c->pending.clear();
}

// Shortest half length of a plane-kernel transform (a power of two, or
// R * N2 with R = 5, 6, 7: accel_common.cuh) that holds the harmonic's
// segment of numdata bins at every step phase (the geometry repeats with
// period q in startr); M (the reference's power of two) if none is shorter.
// The powers kept, columns [hw0, hw0 + numrs/2) of the even and odd
// outputs, are a linear correlation of the first numdata bins with
// templates of halfwidth <= hw0, which any length >= numdata gives.
int short_half_length(int M, int U, int p, int q, int hw0) {
    int need = 0;
    for (long long s = 0; s < 4LL * q; s++) need = std::max(need, step_harm(1000000 + s, U, p, q, hw0).numdata);
    int best = M;
    for (int R = 5; R <= 7; R++)
        for (int n2 = kMixedMinN2; n2 <= kMixedMaxN2; n2 *= 2)
            if (R * n2 >= need && R * n2 < best && mixed_radix(R * n2) == R) best = R * n2;
    return best;
}

int build_bank(accel_ctx* c) {
    int info_zmax = c->cfg.zmax, numharm = c->cfg.numharm, U = c->uselen;
    // bank order: stage by stage, odd harmonics (bpd_subharmonics.cu:319-354)
    int stages = 0;
    while ((1 << stages) < numharm) stages++;
    stages += 1;
    int n = 0, tb = 0, rmax = 0;
    size_t bytes = 0;
    for (int st = 0; st < stages; st++) {
        int maxh = st < 1 ? 1 : (1 << st);
        for (int h = 1; h <= maxh; h += 2) {
            BankHarmDev& b = c->bh[n];
            b.harmnum = h;
            b.maxharm = maxh;
            b.zmax = required_z(h, maxh, info_zmax);
            b.numzs = (b.zmax / kDz) * 2 + 1;
            int hwz = z_halfwidth((double)required_z(h, maxh, info_zmax));
            long long L = next_pow2((long long)(U * h) / maxh + 2 + 2 * kNumBetween * hwz);
            if (L < 2 * kMinM || L > 2 * kMaxM)
                return set_err(ACCEL_ERR_UNSUPPORTED,
                               "harmonic %d/%d needs an FFT of %lld points; supported 128..16384", h,
                               maxh, L);
            b.M = (int)(L / 2);
            b.hw0 = z_halfwidth((double)(-b.zmax));
            b.zlo = required_z(h, maxh, -info_zmax);
            // (the fundamental keeps its power of two: the fused sum's kernel
            // takes powers of two only)
            if (c->cfg.short_transforms && n > 0) b.M = short_half_length(b.M, U, h, maxh, b.hw0);
            b.tpl_base = tb;
            tb += b.numzs;
            int hwmax = b.hw0;
            rmax = std::max(rmax, 4 * hwmax);
            bytes += (size_t)b.numzs * L * sizeof(float2) * 2;  // kstd + fold
            if (c->cfg.template_fp16) bytes += (size_t)b.numzs * L * sizeof(__half2) + b.numzs * sizeof(float);
            bytes = (bytes + 255) & ~(size_t)255;
            n++;
        }
    }
    if (tb > 65535)  // the plane kernels index templates by blockIdx.y
        return set_err(ACCEL_ERR_UNSUPPORTED, "template bank of %d rows exceeds 65535", tb);
    c->nh = n;
    c->ntpl = tb;
    c->nstages = stages;
    CK(cudaMalloc(&c->bank_mem, bytes));
    char* p = (char*)c->bank_mem;
    for (int h = 0; h < n; h++) {
        BankHarmDev& b = c->bh[h];
        size_t L = 2 * (size_t)b.M;
        b.kstd = (float2*)p;
        p += b.numzs * L * sizeof(float2);
        b.fold = (float2*)p;
        p += b.numzs * L * sizeof(float2);
        if (c->cfg.template_fp16) {
            b.fold16 = (__half2*)p;
            p += b.numzs * L * sizeof(__half2);
            b.fold16_scale = (float*)p;
            p += b.numzs * sizeof(float);
        }
        p = (char*)c->bank_mem + ((p - (char*)c->bank_mem + 255) & ~(size_t)255);
    }
    CK(cudaMalloc(&c->d_bh, sizeof(BankHarmDev) * n));
    CK(cudaMemcpyAsync(c->d_bh, c->bh, sizeof(BankHarmDev) * n, cudaMemcpyHostToDevice, c->stream));
    float2* resp = nullptr;
    CK(cudaMalloc(&resp, sizeof(float2) * (size_t)tb * rmax));
    CK(cudaMemsetAsync(resp, 0, sizeof(float2) * (size_t)tb * rmax, c->stream));
    CKL(launch_bank_build(c->d_bh, c->bh, n, tb, resp, rmax, c->cfg.template_fp16 != 0, c->stream),
        "template bank");
    CK(cudaStreamSynchronize(c->stream));
    CK(cudaFree(resp));
    return ACCEL_OK;
}

int build_plan(accel_ctx* c) {
    const int U = c->uselen;
    long long doff = 0, poff = 0;
    int stage = 0;
    for (int h = 0; h < c->nh; h++) {
        const BankHarmDev& b = c->bh[h];
        HarmPlan& P = c->hp[h];
        P.p = b.harmnum;
        P.q = b.maxharm;
        P.lq = 0;
        while ((1 << P.lq) < P.q) P.lq++;
        P.M = b.M;
        P.hw0 = b.hw0;
        P.zlo = b.zlo;
        P.numzs = b.numzs;
        P.fold = b.fold;
        P.fold16 = b.fold16;
        P.f16scale = b.fold16_scale;
        // widest window over all step phases (the geometry repeats with period q in startr)
        int wmax = 0;
        for (long long s = 0; s < 4LL * P.q; s++) {
            StepHarm g = step_harm(1000000 + s, U, P.p, P.q, P.hw0);
            wmax = std::max(wmax, g.numrs);
            const bool fits = c->cfg.short_transforms ? g.numdata <= P.M : next_pow2(g.numdata) == P.M;
            if (!fits || mixed_radix(P.M) == 0)
                return set_err(ACCEL_ERR_INVALID,
                               "harmonic %d/%d: segment of %d bins does not fit half length %d", P.p,
                               P.q, g.numdata, P.M);
        }
        if (P.hw0 + wmax / 2 > P.M)
            return set_err(ACCEL_ERR_INVALID, "harmonic %d/%d: window exceeds segment", P.p, P.q);
        P.wmax = wmax;
        P.prow = (wmax + 3) & ~3;
        P.poff = poff;
        poff += (long long)P.prow * P.numzs;
        P.doff = doff;
        doff += P.M;
        c->stage_of[h] = (((h + 1) & h) == 0) ? stage++ : -1;
    }
    c->dstride = (doff + 31) & ~31LL;
    c->pstride = (poff + 63) & ~63LL;
    if (c->pstride >= (1LL << 31))
        return set_err(ACCEL_ERR_UNSUPPORTED, "power planes of one step exceed 2^31 floats");
    c->numzs0 = c->hp[0].numzs;
    c->zlo0 = c->hp[0].zlo;
    // zind must stay inside each harmonic's plane for every fundamental row
    for (int h = 1; h < c->nh; h++) {
        for (int z = 0; z < c->numzs0; z++) {
            int zi = sub_zind(c->zlo0 + kDz * z, c->hp[h].p, c->hp[h].q, c->hp[h].zlo);
            if (zi < 0 || zi >= c->hp[h].numzs)
                return set_err(ACCEL_ERR_INVALID, "f-dot index out of range for harmonic %d", h);
        }
    }
    c->mvals.clear();
    for (int h = 0; h < c->nh; h++)
        if (std::find(c->mvals.begin(), c->mvals.end(), c->hp[h].M) == c->mvals.end())
            c->mvals.push_back(c->hp[h].M);
    // power-of-two classes first: the short ones share one preparation launch
    // issued after them
    std::stable_partition(c->mvals.begin(), c->mvals.end(), [](int M) { return mixed_radix(M) == 1; });
    for (int s = 0; s < c->nstages; s++)
        c->cuts[s] = (float)power_cut(c->cfg.sigma, 1 << s, c->cfg.numindep);
    // Largest shared-memory footprint of a k_hsum_tile tile of each height,
    // over every tile position and every step phase (the geometry repeats
    // with period q in startr), with the kernel's own index arithmetic.
    int qmax = 1;
    for (int h = 0; h < c->nh; h++) qmax = std::max(qmax, c->hp[h].q);
    for (int k = 0; k < 3; k++) {
        const int TZ = kHsumTileRows[k];
        int worst = 0;
        int bw4[kMaxHarm] = {}, bh[kMaxHarm] = {};  // largest rectangle of each harmonic
        for (long long ph = 0; ph < 4LL * qmax && worst < (1 << 30); ph++) {
            const long long startr = 1000000 + ph;
            for (int z0 = 0; z0 < c->numzs0; z0 += TZ) {
                const int nz = std::min(TZ, c->numzs0 - z0);
                for (int i0 = 0; i0 < U; i0 += kHsumTileI) {
                    const int ni = std::min(kHsumTileI, U - i0);
                    int off = 0;
                    for (int h = 0; h < c->nh; h++) {
                        const HarmPlan& H = c->hp[h];
                        int rfirst = i0, rlast = i0 + ni - 1, zf = z0, zl = z0 + nz - 1;
                        if (h > 0) {
                            const long long rlo = twice_required_r(2 * startr, H.p, H.q) >> 1;
                            rfirst = sub_rind(startr, i0, H.p, H.q, rlo);
                            rlast = sub_rind(startr, i0 + ni - 1, H.p, H.q, rlo);
                            zf = sub_zind(c->zlo0 + kDz * z0, H.p, H.q, H.zlo);
                            zl = sub_zind(c->zlo0 + kDz * (z0 + nz - 1), H.p, H.q, H.zlo);
                        }
                        const int c0 = rfirst & ~3;
                        const int w4 = ((rlast - c0) >> 2) + 1;
                        if (zl < zf || rlast < rfirst || zf < 0 || zl >= H.numzs || (rlast | 3) >= H.prow) {
                            off = 1 << 30;  // never use the tiled kernel for this plan
                            break;
                        }
                        off += 4 * (zl - zf + 1) * w4;
                        bw4[h] = std::max(bw4[h], w4);
                        bh[h] = std::max(bh[h], zl - zf + 1);
                    }
                    worst = std::max(worst, off);
                }
            }
        }
        c->tile_floats_h[k] = worst;
        c->tile_ok_h[k] = worst <= hsum_tile_floats_max(TZ);
        // boxes of the tensor path: every harmonic's largest rectangle, at
        // 128-byte aligned offsets; a box dimension is at most 256 elements
        int at = 0;
        unsigned tx = 0;
        bool fits = c->tile_ok_h[k];
        for (int h = 0; h < c->nh; h++) {
            c->tbox_w4[k][h] = bw4[h];
            c->tbox_h[k][h] = bh[h];
            c->tbox_off[k][h] = at;
            at += (4 * bw4[h] * bh[h] + 31) & ~31;
            tx += 16u * (unsigned)(bw4[h] * bh[h]);
            fits = fits && bw4[h] >= 1 && 4 * bw4[h] <= 256 && bh[h] >= 1 && bh[h] <= 256;
        }
        c->tbox_floats[k] = at;
        c->tbox_tx[k] = tx;
        c->tbox_ok[k] = fits && at <= hsum_tile_floats_max(TZ);
    }
    c->tile_floats = c->tile_floats_h[1];  // 16 rows: the pipelined and persistent sums
    c->tile_ok = c->tile_ok_h[1];
    return ACCEL_OK;
}

// cuTensorMapEncodeTiled from the driver (no link against libcuda), or null.
PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess) {
            cudaGetLastError();
            return (PFN_cuTensorMapEncodeTiled_v12000) nullptr;
        }
        return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }();
    return fn;
}

// Tensor maps of the tiled sum's boxes for both plane buffers: harmonic h
// as a 3-D tensor (prow_h columns, numzs_h rows, chunk segments; strides
// prow_h and pstride floats) starting at its plane offset.  A plan, height
// or buffer whose maps cannot be made takes the per-row bulk copies.
void encode_hsum_maps(accel_ctx* c) {
    PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
    float* bufs[2] = {c->planes, c->planes2};
    for (int b = 0; b < 2; b++)
        for (int k = 0; k < 3; k++) {
            bool ok = enc && bufs[b] && c->tbox_ok[k];
            for (int h = 0; h < c->nh && ok; h++) {
                const HarmPlan& H = c->hp[h];
                const cuuint64_t dim[3] = {(cuuint64_t)H.prow, (cuuint64_t)H.numzs, (cuuint64_t)c->chunk};
                const cuuint64_t stride[2] = {(cuuint64_t)H.prow * 4, (cuuint64_t)c->pstride * 4};
                const cuuint32_t box[3] = {(cuuint32_t)(4 * c->tbox_w4[k][h]), (cuuint32_t)c->tbox_h[k][h], 1};
                const cuuint32_t estr[3] = {1, 1, 1};
                ok = enc(&c->tmaps[b][k].m[h], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, bufs[b] + H.poff, dim, stride,
                         box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                         CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
            }
            c->tmaps_ok[b][k] = ok;
        }
}

int alloc_work(accel_ctx* c) {
    long long plane_bytes = c->pstride * 4;
    int chunk = c->cfg.chunk_segments;
    if (chunk <= 0) {
        chunk = (int)std::max(1LL, std::min(512LL, (8LL << 30) / plane_bytes));  // up to 8 GB of planes
    }
    c->chunk = chunk;
    CK(cudaMalloc(&c->dbuf, sizeof(float2) * c->dstride * chunk));
    CK(cudaMalloc(&c->planes, sizeof(float) * c->pstride * chunk));
    CK(cudaMalloc(&c->planes2, sizeof(float) * c->pstride * chunk));
    CK(cudaStreamCreate(&c->stream2));
    CK(cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming));
    for (int b = 0; b < 2; b++) {
        CK(cudaEventCreateWithFlags(&c->ev_plane[b], cudaEventDisableTiming));
        CK(cudaEventCreateWithFlags(&c->ev_sum[b], cudaEventDisableTiming));
    }
    CK(cudaMalloc(&c->d_step, sizeof(unsigned) * ((size_t)chunk + 1)));
    c->cand_cap = c->cfg.cand_capacity > 0 ? c->cfg.cand_capacity : (1LL << 22);
    CK(cudaMalloc(&c->d_cands, sizeof(RawCand) * c->cand_cap));
    // [0] candidate count, [1] kernel error bits
    CK(cudaMalloc(&c->d_ncand, 2 * sizeof(unsigned long long)));
    CK(cudaMallocHost(&c->h_ncand, 2 * sizeof(unsigned long long)));
    encode_hsum_maps(c);
    return ACCEL_OK;
}

int ensure_segs(accel_ctx* c, long long n) {
    if (n <= c->segs_cap) return ACCEL_OK;
    if (c->d_segs) cudaFree(c->d_segs);
    if (c->h_segs) cudaFreeHost(c->h_segs);
    c->d_segs = nullptr;
    c->h_segs = nullptr;
    long long cap = std::max(n, 2 * c->segs_cap);
    CK(cudaMalloc(&c->d_segs, sizeof(SegDesc) * cap));
    CK(cudaMallocHost(&c->h_segs, sizeof(SegDesc) * cap));
    c->segs_cap = cap;
    return ACCEL_OK;
}

// Whitening block plan of a spectrum length on the device, cached per
// length.  The cache keeps the kWhitenPlans most recently used lengths (a
// request server sees a new length with almost every request); buffers are
// allocated and freed in stream order on the context's stream, so neither
// a new length nor an eviction waits for the device.
constexpr size_t kWhitenPlans = 64;

int whiten_plan(accel_ctx* c, unsigned numbins, WhitenPlanDev** out) {
    auto it = c->wplans.find(numbins);
    if (it != c->wplans.end()) {
        it->second.last_use = ++c->wplan_clock;
        *out = &it->second;
        return ACCEL_OK;
    }
    if (numbins <= (unsigned)(1 + c->cfg.whiten_initbuf))
        return set_err(ACCEL_ERR_INVALID, "spectrum of %u bins is too short to whiten", numbins);
    if ((long long)numbins > kMaxWhitenBins)
        return set_err(ACCEL_ERR_INVALID, "spectrum of %u bins exceeds the whitening limit of %lld", numbins,
                       kMaxWhitenBins);
    if (c->wplans.size() >= kWhitenPlans) {
        auto lru = c->wplans.begin();
        for (auto e = c->wplans.begin(); e != c->wplans.end(); ++e)
            if (e->second.last_use < lru->second.last_use) lru = e;
        CK(cudaFreeAsync(lru->second.d_start, c->stream));
        CK(cudaFreeAsync(lru->second.d_len, c->stream));
        CK(cudaFreeAsync(lru->second.d_med, c->stream));
        c->wplans.erase(lru);
    }
    auto blocks = plan_whiten_blocks(numbins, c->cfg.whiten_initbuf, c->cfg.whiten_maxbuf);
    WhitenPlanDev w;
    w.nb = (int)blocks.size();
    std::vector<int> s(w.nb), l(w.nb);
    for (int i = 0; i < w.nb; i++) {
        s[i] = blocks[i].first;
        l[i] = blocks[i].second;
        w.maxlen = std::max(w.maxlen, l[i]);
    }
    CK(cudaMallocAsync(reinterpret_cast<void**>(&w.d_start), sizeof(int) * w.nb, c->stream));
    CK(cudaMallocAsync(reinterpret_cast<void**>(&w.d_len), sizeof(int) * w.nb, c->stream));
    CK(cudaMallocAsync(reinterpret_cast<void**>(&w.d_med), sizeof(double) * w.nb, c->stream));
    // from pageable memory: staged before the call returns, so the vectors
    // may go out of scope
    CK(cudaMemcpyAsync(w.d_start, s.data(), sizeof(int) * w.nb, cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(w.d_len, l.data(), sizeof(int) * w.nb, cudaMemcpyHostToDevice, c->stream));
    w.last_use = ++c->wplan_clock;
    auto r = c->wplans.emplace(numbins, w);
    *out = &r.first->second;
    return ACCEL_OK;
}

int do_whiten(accel_ctx* c, float2* spec, unsigned numbins) {
    WhitenPlanDev* w = nullptr;
    int rc = whiten_plan(c, numbins, &w);
    if (rc) return rc;
    ProfScope ps(c, K_WHITEN, 2);
    CKL(launch_whiten(w->d_start, w->d_len, w->nb, w->d_med, spec, numbins, w->maxlen, c->stream,
                      c->cfg.exact_rsqrt),
        "whitening");
    return ACCEL_OK;
}

int do_rfft(accel_ctx* c, const float* series, long long n, float2* spec) {
    ProfScope ps(c, K_RFFT, 1);
    const int r = r2c_any(c->r2c, series, n, spec, c->stream);
    if (r == -2) return set_err(ACCEL_ERR_NOMEM, "real-to-complex transform of %lld samples: scratch memory", n);
    if (r) return set_err(ACCEL_ERR_CUDA, "real-to-complex transform of %lld samples failed", n);
    return ACCEL_OK;
}

// Launch one group of nseg prepared segment descriptors (device array).
// fused: the fundamental's plane is not stored; k_fund_sum adds the
// sub-harmonic planes to it row by row (the search path).  Otherwise every
// plane is stored and, with do_sum, k_hsum sums them (the stage API).
int run_group(accel_ctx* c, const SegDesc* d_segs, int nseg, int seg_base, float* stage_out,
              const float2* dh_in, float* planes_out, bool do_prep, bool do_plane, bool do_sum,
              bool fused, cudaStream_t sum_stream) {
    if (!sum_stream) sum_stream = c->stream;
    float2* dbuf = dh_in ? const_cast<float2*>(dh_in) : c->dbuf;
    float* planes = planes_out ? planes_out : c->planes;
    bool short_prepped = !do_prep;
    for (int M : c->mvals) {
        if (mixed_radix(M) > 1 && !short_prepped) {
            // the segments of every short-transform harmonic in one launch,
            // after the power-of-two classes' planes (the fundamental's
            // first): by then the previous group's harmonic sum on the other
            // stream has usually left the SMs
            short_prepped = true;
            PrepArgs ps{};
            int k = 0;
            for (int h = 0; h < c->nh; h++)
                if (mixed_radix(c->hp[h].M) > 1) ps.h[k++] = c->hp[h];
            ps.nh = k;
            ps.uselen = c->uselen;
            ps.exact_rsqrt = c->cfg.exact_rsqrt;
            ps.segs = d_segs;
            ps.dbuf = dbuf;
            ps.dstride = c->dstride;
            ProfScope pscope(c, K_PREP, 1);
            CKL(launch_prep(M, ps, nseg, c->tw, c->stream), "segment preparation");
        }
        PrepArgs pa{};
        PlaneArgs la{};
        int k = 0, kp = 0, zb = 0;
        for (int h = 0; h < c->nh; h++) {
            if (c->hp[h].M != M) continue;
            pa.h[k++] = c->hp[h];
            if (fused && h == 0) continue;
            la.h[kp] = c->hp[h];
            la.h[kp].zbase = zb;
            zb += c->hp[h].numzs;
            kp++;
        }
        pa.nh = k;
        pa.uselen = c->uselen;
        pa.exact_rsqrt = c->cfg.exact_rsqrt;
        pa.segs = d_segs;
        pa.dbuf = dbuf;
        pa.dstride = c->dstride;
        la.nh = kp;
        la.ntpl = zb;
        la.dbuf = dbuf;
        la.dstride = c->dstride;
        la.planes = planes;
        la.pstride = c->pstride;
        la.use_fp16 = c->cfg.template_fp16;
        la.split = c->plane_split;
        if (do_prep && mixed_radix(M) == 1) {
            ProfScope ps(c, K_PREP, 1);
            CKL(launch_prep(M, pa, nseg, c->tw, c->stream), "segment preparation");
        }
        if (do_plane && kp > 0) {
            ProfScope ps(c, K_PLANE, 1);
            CKL(launch_plane(M, la, nseg, c->tw, c->stream), "power plane");
        }
    }
    if (fused) {
        FundArgs fa{};
        for (int h = 0; h < c->nh; h++) {
            fa.h[h] = c->hp[h];
            fa.stage_of[h] = c->stage_of[h];
        }
        fa.nh = c->nh;
        fa.dbuf = dbuf;
        fa.dstride = c->dstride;
        fa.planes = planes;
        fa.pstride = c->pstride;
        fa.use_fp16 = c->cfg.template_fp16;
        fa.split = c->plane_split;
        fa.uselen = c->uselen;
        fa.numzs0 = c->numzs0;
        fa.zlo0 = c->zlo0;
        for (int s = 0; s < c->nstages; s++) fa.cut[s] = c->cuts[s];
        fa.segs = d_segs;
        fa.cands = c->d_cands;
        fa.ncand = c->d_ncand;
        fa.cap = c->cand_cap;
        fa.seg_base = seg_base;
        fa.stage_out = stage_out;
        fa.nstages = c->nstages;
        ProfScope ps(c, K_FUND, 1);
        c->stats.segments += nseg;
        c->stats.cells += (long long)nseg * c->uselen * c->numzs0;
        CKL(launch_fund_sum(fa, nseg, c->tw, c->stream), "fundamental plane and harmonic sum");
    } else if (do_sum) {
        HsumArgs ha{};
        for (int h = 0; h < c->nh; h++) {
            ha.h[h] = c->hp[h];
            ha.stage_of[h] = c->stage_of[h];
        }
        ha.nh = c->nh;
        ha.uselen = c->uselen;
        ha.numzs0 = c->numzs0;
        ha.zlo0 = c->zlo0;
        for (int s = 0; s < c->nstages; s++) ha.cut[s] = c->cuts[s];
        ha.segs = d_segs;
        ha.planes = planes;
        ha.pstride = c->pstride;
        ha.cands = c->d_cands;
        ha.ncand = c->d_ncand;
        ha.cap = c->cand_cap;
        ha.seg_base = seg_base;
        ha.stage_out = stage_out;
        ha.nstages = c->nstages;
        ha.err = c->d_ncand + 1;
        ha.tile_floats = c->tile_floats;
        ha.test_extra_tx = c->wait_test ? 16u : 0u;
        ProfScope ps(c, K_HSUM, 1, sum_stream);
        c->stats.segments += nseg;
        c->stats.cells += (long long)nseg * c->uselen * c->numzs0;
        if (c->tile_ok && c->hsum_tiled && c->hsum_pipe && 4LL * ((c->tile_floats + 31) & ~31) * kPipeBuffers <= kPipeSmemMax)
            CKL(launch_hsum_pipe(ha, nseg, sum_stream), "harmonic sum (tiled, pipelined)");
        else if (c->tile_ok && c->hsum_tiled) {
            // the tuned tile height where its tiles fit, else 16 rows
            int k = c->tile_rows == 8 ? 0 : c->tile_rows == 32 ? 2 : 1;
            if (!c->tile_ok_h[k]) k = 1;
            ha.tile_floats = c->tile_floats_h[k];
            // one box copy per harmonic where the planes are one of the
            // context's two buffers and their maps exist
            const int b = planes == c->planes ? 0 : planes == c->planes2 ? 1 : -1;
            const HsumMaps* maps = nullptr;
            if (c->hsum_tensor && b >= 0 && c->tmaps_ok[b][k]) {
                maps = &c->tmaps[b][k];
                ha.use_tmap = 1;
                for (int h = 0; h < c->nh; h++) {
                    ha.box_w4[h] = c->tbox_w4[k][h];
                    ha.box_h[h] = c->tbox_h[k][h];
                    ha.box_off[h] = c->tbox_off[k][h];
                }
                ha.box_tx = c->tbox_tx[k];
                ha.tile_floats = c->tbox_floats[k];
            }
            CKL(launch_hsum_tile(ha, nseg, kHsumTileRows[k], maps, sum_stream), "harmonic sum (tiled)");
        }
        else
            CKL(launch_hsum(ha, nseg, sum_stream), "harmonic sum");
    }
    return ACCEL_OK;
}

// Whether the persistent plane-and-sum kernel can take this plan: the
// tiled sum applies, the largest segment length is 8192 (256 threads, one
// per tile column), and every class is one of 4096, 2048, 1024, 512 points
// (at most four classes).
bool step_plan_ok(const accel_ctx* c) {
    if (!c->tile_ok || !c->hsum_tiled || c->fused_sum || !c->d_step) return false;
    if (c->mvals.empty() || c->mvals.size() > (size_t)kStepClasses) return false;
    int mmax = 0;
    for (int M : c->mvals) {
        if (M != 4096 && M != 2048 && M != 1024 && M != 512) return false;
        mmax = std::max(mmax, M);
    }
    return mmax == 4096;
}

// One launch group as a single persistent launch: plane rows and harmonic-
// sum tiles of its segments from one work queue (k_step).  The segments'
// spectra must have been prepared (k_prep) on the same stream before.
int run_step(accel_ctx* c, const SegDesc* d_segs, int nseg, int seg_base) {
    StepArgs sa{};
    HsumArgs& ha = sa.hs;
    for (int h = 0; h < c->nh; h++) {
        ha.h[h] = c->hp[h];
        ha.stage_of[h] = c->stage_of[h];
    }
    ha.nh = c->nh;
    ha.uselen = c->uselen;
    ha.numzs0 = c->numzs0;
    ha.zlo0 = c->zlo0;
    for (int s = 0; s < c->nstages; s++) ha.cut[s] = c->cuts[s];
    ha.segs = d_segs;
    ha.planes = c->planes;
    ha.pstride = c->pstride;
    ha.cands = c->d_cands;
    ha.ncand = c->d_ncand;
    ha.cap = c->cand_cap;
    ha.seg_base = seg_base;
    ha.stage_out = nullptr;
    ha.nstages = c->nstages;
    ha.err = c->d_ncand + 1;
    ha.tile_floats = c->tile_floats;
    ha.test_extra_tx = c->wait_test ? 16u : 0u;
    sa.dbuf = c->dbuf;
    sa.dstride = c->dstride;
    sa.planes = c->planes;
    int mmax = 0;
    for (int M : c->mvals) mmax = std::max(mmax, M);
    // classes largest first, harmonics of a class in bank order
    std::vector<int> ms(c->mvals);
    std::sort(ms.begin(), ms.end(), std::greater<int>());
    sa.ncls = (int)ms.size();
    int items = 0, rows = 0;
    for (int k = 0; k < sa.ncls; k++) {
        sa.cls_M[k] = ms[k];
        int n = 0, zb = 0;
        for (int h = 0; h < c->nh; h++) {
            if (c->hp[h].M != ms[k]) continue;
            sa.cls_h[k][n] = h;
            sa.cls_zbase[k][n] = zb;
            zb += c->hp[h].numzs;
            n++;
        }
        sa.cls_nh[k] = n;
        sa.cls_ntpl[k] = zb;
        sa.cls_item0[k] = items;
        const int per = mmax / ms[k];
        items += (zb + per - 1) / per;
        rows += zb;
    }
    sa.cls_item0[sa.ncls] = items;
    sa.P = items;
    sa.nti = (c->uselen + kHsumTileI - 1) / kHsumTileI;
    sa.T = sa.nti * ((c->numzs0 + kHsumTileZ - 1) / kHsumTileZ);
    sa.rows = rows;
    sa.nseg = nseg;
    sa.lag = std::min(kStepLag, nseg);
    sa.nitems = (long long)(sa.P + sa.T) * nseg;
    if (sa.nitems >= (1LL << 31)) return set_err(ACCEL_ERR_UNSUPPORTED, "launch group of %d segments too large", nseg);
    sa.next = c->d_step;
    sa.done = c->d_step + 1;
    CK(cudaMemsetAsync(c->d_step, 0, sizeof(unsigned) * (size_t)(nseg + 1), c->stream));
    ProfScope ps(c, K_STEP, 1);
    c->stats.segments += nseg;
    c->stats.cells += (long long)nseg * c->uselen * c->numzs0;
    CKL(launch_step(sa, mmax, c->cfg.template_fp16, c->tw, c->stream), "persistent plane and sum");
    return ACCEL_OK;
}

// Record the launches that issue() makes into a CUDA graph and launch it on
// the context's stream.  issue() runs against two non-blocking capture
// streams standing in for stream and stream2, so that nothing else ordered
// with the legacy default stream can join the capture.  The executable
// graph is kept: a later capture of the same shape (same launch groups and
// kernels, other arguments) updates it in place, any other is instantiated
// anew.
int launch_as_graph(accel_ctx* c, const std::function<int()>& issue) {
    if (!c->gcap) CK(cudaStreamCreateWithFlags(&c->gcap, cudaStreamNonBlocking));
    if (!c->gcap2) CK(cudaStreamCreateWithFlags(&c->gcap2, cudaStreamNonBlocking));
    cudaStream_t s0 = c->stream, s1 = c->stream2;
    c->stream = c->gcap;
    c->stream2 = s1 ? c->gcap2 : nullptr;
    cudaError_t e = cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeRelaxed);
    if (e != cudaSuccess) {
        c->stream = s0;
        c->stream2 = s1;
        return set_err(ACCEL_ERR_CUDA, "cudaStreamBeginCapture failed: %s", cudaGetErrorString(e));
    }
    c->capturing = true;
    const int rc = issue();
    cudaGraph_t g = nullptr;
    e = cudaStreamEndCapture(c->stream, &g);
    c->capturing = false;
    c->stream = s0;
    c->stream2 = s1;
    if (rc || e != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        cudaGetLastError();
        return rc ? rc : set_err(ACCEL_ERR_CUDA, "graph capture failed: %s", cudaGetErrorString(e));
    }
    bool built = false;
    if (c->gexec) {
        cudaGraphExecUpdateResultInfo info;
        if (cudaGraphExecUpdate(c->gexec, g, &info) != cudaSuccess) {
            cudaGetLastError();  // not an error: the shape changed, instantiate anew
            cudaGraphExecDestroy(c->gexec);
            c->gexec = nullptr;
        }
    }
    if (!c->gexec) {
        e = cudaGraphInstantiate(&c->gexec, g, 0);
        if (e != cudaSuccess) {
            c->gexec = nullptr;
            cudaGraphDestroy(g);
            return set_err(ACCEL_ERR_CUDA, "cudaGraphInstantiate failed: %s", cudaGetErrorString(e));
        }
        built = true;
    }
    cudaGraphDestroy(g);
    CK(cudaGraphLaunch(c->gexec, c->stream));
    c->stats.graph_launches++;
    if (built) c->stats.graph_builds++;
    return ACCEL_OK;
}

// Segment table: one entry per (trial, step), trial-major.
struct SegSpan {
    std::vector<int> trial, step;
};

// prepare(t), when given, is called on the main stream before the first
// launch group that holds a segment of trial t (trials in order), so that a
// trial's transform and whitening are issued just ahead of its search.
int run_search(accel_ctx* c, int ntrials, float2* const* spec, const long long* numbins,
               const long long* rlo, const std::function<int(int)>& prepare) {
    long long total = 0;
    const long long half = (unsigned short)(c->uselen / 2);
    std::vector<long long> nsteps(ntrials);
    for (int i = 0; i < ntrials; i++) {
        long long s = 0;
        for (long long r = rlo[i]; r + half < numbins[i]; r += half) s++;
        nsteps[i] = s;
        total += s;
    }
    int rc = ensure_segs(c, std::max(total, 1LL));
    if (rc) return rc;
    long long k = 0;
    for (int i = 0; i < ntrials; i++)
        for (long long s = 0; s < nsteps[i]; s++, k++) {
            SegDesc& d = c->h_segs[k];
            d.spec = spec[i];
            d.numbins = numbins[i];
            d.startr = rlo[i] + s * half;
            d.trial = i;
            d.step = (int)s;
        }
    // everything from clearing the candidate count to the last harmonic sum:
    // launched directly, or recorded into the context's CUDA graph
    auto issue = [&]() -> int {
        CK(cudaMemsetAsync(c->d_ncand, 0, 2 * sizeof(unsigned long long), c->stream));
        if (total > 0)
            CK(cudaMemcpyAsync(c->d_segs, c->h_segs, sizeof(SegDesc) * total, cudaMemcpyHostToDevice,
                               c->stream));
        const bool persistent = c->persistent && step_plan_ok(c);
        const bool overlap = !persistent && c->overlap && !c->fused_sum && c->planes2 && c->stream2;
        if (overlap) {
            // fork: stream2 starts after everything queued so far on the main stream
            CK(cudaEventRecord(c->ev_fork, c->stream));
            CK(cudaStreamWaitEvent(c->stream2, c->ev_fork, 0));
        }
        int prepared = 0;  // trials [0, prepared) have been prepared
        auto prepare_upto = [&](int last) -> int {
            for (; prepare && prepared <= last && prepared < ntrials; prepared++) {
                const int r = prepare(prepared);
                if (r) return r;
            }
            return ACCEL_OK;
        };
        for (long long g = 0, k = 0; g < total; g += c->chunk, k++) {
            int n = (int)std::min<long long>(c->chunk, total - g);
            rc = prepare_upto(c->h_segs[g + n - 1].trial);
            if (rc) return rc;
            if (persistent) {
                rc = run_group(c, c->d_segs + g, n, (int)g, nullptr, nullptr, nullptr, true, false, false, false);
                if (!rc) rc = run_step(c, c->d_segs + g, n, (int)g);
                if (rc) return rc;
                continue;
            }
            if (!overlap) {
                rc = run_group(c, c->d_segs + g, n, (int)g, nullptr, nullptr, nullptr, true, true, true,
                               c->fused_sum != 0);
                if (rc) return rc;
                continue;
            }
            // group k: planes into buffer k%2 on the main stream, summed on stream2
            const int b = (int)(k & 1);
            float* pb = b ? c->planes2 : c->planes;
            if (k >= 2) CK(cudaStreamWaitEvent(c->stream, c->ev_sum[b], 0));  // buffer b free again
            rc = run_group(c, c->d_segs + g, n, (int)g, nullptr, nullptr, pb, true, true, false);
            if (rc) return rc;
            CK(cudaEventRecord(c->ev_plane[b], c->stream));
            CK(cudaStreamWaitEvent(c->stream2, c->ev_plane[b], 0));
            rc = run_group(c, c->d_segs + g, n, (int)g, nullptr, nullptr, pb, false, false, true, false,
                           c->stream2);
            if (rc) return rc;
            CK(cudaEventRecord(c->ev_sum[b], c->stream2));
        }
        rc = prepare_upto(ntrials - 1);
        if (rc) return rc;
        if (overlap) {
            // join: the main stream continues after the last sum
            CK(cudaEventRecord(c->ev_fork, c->stream2));
            CK(cudaStreamWaitEvent(c->stream, c->ev_fork, 0));
        }
        return ACCEL_OK;
    };
    rc = (c->use_graph && !prepare) ? launch_as_graph(c, issue) : issue();
    if (rc) return rc;
    CK(cudaMemcpyAsync(c->h_ncand, c->d_ncand, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                       c->stream));
    CK(cudaStreamSynchronize(c->stream));
    if (c->h_ncand[1])
        return set_err(ACCEL_ERR_CUDA,
                       "harmonic sum: a bounded wait timed out (error bits %llx: 1 a tile's copies, 2 a "
                       "segment's plane rows)",
                       c->h_ncand[1]);
    unsigned long long nraw = *c->h_ncand;
    c->last_raw = nraw;
    long long keep = (long long)std::min<unsigned long long>(nraw, (unsigned long long)c->cand_cap);
    if (keep > c->h_raw_cap) {
        // pinned, so that the read-back is one asynchronous DMA
        const long long cap = std::max(keep, 2 * c->h_raw_cap);
        CK(cudaStreamSynchronize(c->stream));
        cudaFreeHost(c->h_raw);
        c->h_raw = nullptr;
        c->h_raw_cap = 0;
        CK(cudaMallocHost(&c->h_raw, sizeof(RawCand) * cap));
        c->h_raw_cap = cap;
    }
    const RawCand* raw = c->h_raw;
    if (keep > 0)
        CK(cudaMemcpyAsync(c->h_raw, c->d_cands, sizeof(RawCand) * keep, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaEventRecord(c->ev_end, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    {
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, c->ev_begin, c->ev_end) == cudaSuccess) c->stats.search_ms += ms;
        c->stats.searches++;
    }
    prof_collect(c);
    // Candidates in (trial, step, numharm, z, r) order.  Segment k holds
    // (trial, step) in increasing order, so a counting sort by segment and
    // a sort of each segment's few candidates by (numharm, z, r) give that
    // order (no two candidates share all five keys); the conversion (sigma
    // by Newton steps) and the per-segment sorts run on host threads.
    c->results.clear();
    std::vector<long long> off(total + 1, 0);
    for (long long j = 0; j < keep; j++) {
        if (raw[j].seg < 0 || raw[j].seg >= total)
            return set_err(ACCEL_ERR_CUDA, "candidate %lld names segment %d of %lld", j, raw[j].seg, total);
        off[raw[j].seg + 1]++;
    }
    for (long long s = 0; s < total; s++) off[s + 1] += off[s];
    std::vector<long long> at(off.begin(), off.end() - 1);
    std::vector<int> order(keep);
    for (long long j = 0; j < keep; j++) order[at[raw[j].seg]++] = (int)j;
    c->results.resize(keep);
    accel_candidate* out = c->results.data();
    const double numindep = c->cfg.numindep;
    auto convert = [&](long long s0, long long s1) {
        for (long long s = s0; s < s1; s++) {
            const SegDesc& d = c->h_segs[s];
            for (long long q = off[s]; q < off[s + 1]; q++) {
                const RawCand& r = raw[order[q]];
                accel_candidate& o = out[q];
                o.trial = d.trial;
                o.step = d.step;
                o.r = (double)d.startr + 0.5 * r.ridx;
                o.z = (double)(c->zlo0 + kDz * r.zidx);
                o.numharm = r.numharm;
                o.power = r.power;
                o.sigma = (float)sigma_of_power(r.power, r.numharm, numindep);
            }
            std::sort(out + off[s], out + off[s + 1], [](const accel_candidate& a, const accel_candidate& b) {
                if (a.numharm != b.numharm) return a.numharm < b.numharm;
                if (a.z != b.z) return a.z < b.z;
                return a.r < b.r;
            });
        }
    };
    const int nthr = keep < 16384 ? 1 : (int)std::min<unsigned>(16u, std::max(1u, std::thread::hardware_concurrency()));
    // segment ranges holding about keep / nthr candidates each; a range a
    // thread could not be started for is converted here
    std::vector<std::thread> pool;
    long long s0 = 0;
    for (int t = 0; t < nthr && s0 < total; t++) {
        const long long goal = keep * (t + 1) / nthr;
        long long s1 = t == nthr - 1 ? total
                                     : (long long)(std::upper_bound(off.begin(), off.end(), goal) - off.begin()) - 1;
        s1 = std::min(std::max(s1, s0 + 1), total);
        bool started = false;
        if (t + 1 < nthr) {
            try {
                pool.emplace_back(convert, s0, s1);
                started = true;
            } catch (...) {
            }
        }
        if (!started) convert(s0, s1);
        s0 = s1;
    }
    for (std::thread& th : pool) th.join();
    if (nraw > (unsigned long long)c->cand_cap)
        return set_err(ACCEL_ERR_CAPACITY, "%llu candidates exceed the capacity of %lld", nraw,
                       c->cand_cap);
    return ACCEL_OK;
}

void free_ctx(accel_ctx* c) {
    if (!c) return;
    cudaSetDevice(c->device);
    for (auto& kv : c->r2c.plans) cufftDestroy(kv.second);
    c->r2c.plans.clear();
    for (auto& e : c->pending) {
        cudaEventDestroy(e.a);
        cudaEventDestroy(e.b);
    }
    for (auto e : c->evpool) cudaEventDestroy(e);
    if (c->ev_begin) cudaEventDestroy(c->ev_begin);
    if (c->ev_end) cudaEventDestroy(c->ev_end);
    for (auto& kv : c->wplans) {
        cudaFree(kv.second.d_start);
        cudaFree(kv.second.d_len);
        cudaFree(kv.second.d_med);
    }
    for (auto& t : c->trials) {
        cudaFree(t.series);
        cudaFree(t.spec);
    }
    cudaFree(c->bank_mem);
    cudaFree(c->d_bh);
    cudaFree(c->tw);
    cudaFree(c->dbuf);
    cudaFree(c->planes);
    cudaFree(c->planes2);
    cudaFree(c->d_step);
    if (c->gexec) cudaGraphExecDestroy(c->gexec);
    if (c->gcap) cudaStreamDestroy(c->gcap);
    if (c->gcap2) cudaStreamDestroy(c->gcap2);
    if (c->stream2) cudaStreamDestroy(c->stream2);
    if (c->copy_stream) cudaStreamDestroy(c->copy_stream);
    for (cudaEvent_t e : c->copy_ev) cudaEventDestroy(e);
    if (c->ev_fork) cudaEventDestroy(c->ev_fork);
    for (int b = 0; b < 2; b++) {
        if (c->ev_plane[b]) cudaEventDestroy(c->ev_plane[b]);
        if (c->ev_sum[b]) cudaEventDestroy(c->ev_sum[b]);
    }
    cudaFree(c->d_segs);
    cudaFreeHost(c->h_segs);
    cudaFree(c->d_cands);
    cudaFree(c->d_ncand);
    cudaFreeHost(c->h_ncand);
    cudaFreeHost(c->h_raw);
    if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
    delete c;
}

}  // namespace accel

namespace accel {
int set_error(int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_err = buf;
    return code;
}
}  // namespace accel

// =================================================================== C ABI
extern "C" {

const char* accel_version(void) { return "gpu_accelsearch_gb300 0.1 (sm_103a)"; }
const char* accel_last_error(void) { return g_err.c_str(); }

void accel_config_init(accel_config* cfg) {
    if (!cfg) return;
    std::memset(cfg, 0, sizeof(*cfg));
    cfg->zmax = 200;
    cfg->numharm = 8;
    cfg->fftlen = 8192;
    cfg->uselen = 0;
    cfg->whiten_initbuf = 6;
    cfg->whiten_maxbuf = 200;
    cfg->sigma = 6.0;
    cfg->numindep = 1.0;
    cfg->template_fp16 = 0;
    cfg->chunk_segments = 0;
    cfg->cand_capacity = 0;
    cfg->device = 0;
}

int accel_create(const accel_config* cfg, accel_ctx** out) {
    if (!cfg || !out) return set_err(ACCEL_ERR_INVALID, "null argument");
    *out = nullptr;
    if (cfg->zmax < 0 || (cfg->zmax & 1)) return set_err(ACCEL_ERR_INVALID, "zmax must be even and >= 0");
    if (cfg->numharm < 1 || cfg->numharm > kMaxHarm || (cfg->numharm & (cfg->numharm - 1)))
        return set_err(ACCEL_ERR_INVALID, "numharm must be 1, 2, 4, 8 or 16");
    if (cfg->fftlen < 2 * kMinM || cfg->fftlen > 2 * kMaxM || (cfg->fftlen & (cfg->fftlen - 1)))
        return set_err(ACCEL_ERR_UNSUPPORTED, "fftlen must be a power of two in [128, 16384]");
    if (cfg->whiten_initbuf < 1 || cfg->whiten_maxbuf < 1)
        return set_err(ACCEL_ERR_INVALID, "whitening block widths must be positive");
    int U = cfg->uselen;
    if (U <= 0) U = (cfg->fftlen - 2 - 2 * kNumBetween * z_halfwidth((double)cfg->zmax)) & ~1;
    if (U < 2 || (U & 1) || U >= 65536)
        return set_err(ACCEL_ERR_INVALID, "uselen %d must be even, positive and < 65536", U);
    if (next_pow2((long long)U + 2 + 2 * kNumBetween * z_halfwidth((double)cfg->zmax)) != cfg->fftlen)
        return set_err(ACCEL_ERR_INVALID, "uselen %d does not give segment length %d", U, cfg->fftlen);
    accel_ctx* c = new accel_ctx();
    c->cfg = *cfg;
    c->device = cfg->device;
    c->uselen = U;
    int rc = ensure_device(c);
    if (!rc) {
        // a blocking stream: ordered with the legacy default stream, where
        // callers (PyTorch by default) produce the inputs they pass in
        cudaError_t e = cudaStreamCreate(&c->stream);
        if (e != cudaSuccess) rc = set_err(ACCEL_ERR_CUDA, "stream: %s", cudaGetErrorString(e));
        c->own_stream = true;
    }
    if (!rc) {
        cudaError_t e = cudaMalloc(&c->tw, sizeof(float2) * kTwAll);
        if (e != cudaSuccess) rc = set_err(ACCEL_ERR_NOMEM, "twiddles: %s", cudaGetErrorString(e));
        else if (launch_twiddles(c->tw, c->stream) != 0) rc = set_err(ACCEL_ERR_CUDA, "twiddle launch");
    }
    if (!rc && (cudaEventCreate(&c->ev_begin) != cudaSuccess || cudaEventCreate(&c->ev_end) != cudaSuccess))
        rc = set_err(ACCEL_ERR_CUDA, "event creation failed");
    if (!rc) rc = build_bank(c);
    if (!rc) rc = build_plan(c);
    if (!rc) rc = alloc_work(c);
    if (rc) {
        free_ctx(c);
        return rc;
    }
    *out = c;
    return ACCEL_OK;
}

int accel_destroy(accel_ctx* c) {
    free_ctx(c);
    return ACCEL_OK;
}

int accel_set_stream(accel_ctx* c, void* s) {
    if (!c) return set_err(ACCEL_ERR_INVALID, "null context");
    // work already issued on the old stream finishes first: buffers it uses
    // may be freed in stream order on the new one (whitening-plan eviction)
    if (c->stream) cudaStreamSynchronize(c->stream);
    if (c->own_stream && c->stream) {
        cudaStreamDestroy(c->stream);
        c->own_stream = false;
        c->stream = nullptr;
    }
    if (s) {
        c->stream = (cudaStream_t)s;
    } else {
        CK(cudaStreamCreate(&c->stream));
        c->own_stream = true;
    }
    return ACCEL_OK;
}

int accel_synchronize(accel_ctx* c) {
    if (!c) return set_err(ACCEL_ERR_INVALID, "null context");
    CK(cudaStreamSynchronize(c->stream));
    if (c->stream2) CK(cudaStreamSynchronize(c->stream2));
    return ACCEL_OK;
}

int accel_profile(accel_ctx* c, int enable) {
    if (!c) return set_err(ACCEL_ERR_INVALID, "null context");
    c->profiling = enable != 0;
    return ACCEL_OK;
}

int accel_get_stats(accel_ctx* c, accel_stats* out) {
    if (!c || !out) return set_err(ACCEL_ERR_INVALID, "null argument");
    CK(cudaStreamSynchronize(c->stream));
    prof_collect(c);
    *out = c->stats;
    return ACCEL_OK;
}

int accel_reset_stats(accel_ctx* c) {
    if (!c) return set_err(ACCEL_ERR_INVALID, "null context");
    CK(cudaStreamSynchronize(c->stream));
    prof_collect(c);
    c->stats = accel_stats{};
    return ACCEL_OK;
}

int accel_get_tuning(const accel_ctx* c, accel_tuning* t) {
    if (!c || !t) return set_err(ACCEL_ERR_INVALID, "null argument");
    std::memset(t, 0, sizeof(*t));
    t->chunk_segments = c->chunk;
    t->plane_split = c->plane_split;
    t->fused_sum = c->fused_sum;
    t->hsum_rowwise = !c->hsum_tiled;
    t->serial_sum = !c->overlap;
    t->hsum_pipelined = c->hsum_pipe;
    t->graph = c->use_graph;
    t->persistent = c->persistent;
    t->hsum_tile_rows = c->tile_rows;
    t->wait_test = c->wait_test;
    t->hsum_row_copies = !c->hsum_tensor;
    return ACCEL_OK;
}

int accel_set_tuning(accel_ctx* c, const accel_tuning* t) {
    if (!c || !t) return set_err(ACCEL_ERR_INVALID, "null argument");
    if (t->chunk_segments < 1 || t->chunk_segments > 65535)
        return set_err(ACCEL_ERR_INVALID, "chunk_segments must be in [1, 65535]");
    if (t->hsum_tile_rows != 0 && t->hsum_tile_rows != 8 && t->hsum_tile_rows != 16 && t->hsum_tile_rows != 32)
        return set_err(ACCEL_ERR_INVALID, "hsum_tile_rows must be 8, 16 or 32");
    int rc = ensure_device(c);
    if (rc) return rc;
    c->plane_split = t->plane_split != 0;
    c->fused_sum = t->fused_sum != 0;
    c->hsum_tiled = t->hsum_rowwise == 0;
    c->overlap = t->serial_sum == 0;
    c->hsum_pipe = t->hsum_pipelined != 0;
    c->use_graph = t->graph != 0;
    c->persistent = t->persistent != 0;
    c->tile_rows = t->hsum_tile_rows ? t->hsum_tile_rows : 16;
    c->wait_test = t->wait_test != 0;
    c->hsum_tensor = t->hsum_row_copies == 0;
    if (t->chunk_segments != c->chunk) {
        CK(cudaStreamSynchronize(c->stream));
        CK(cudaStreamSynchronize(c->stream2));
        cudaFree(c->dbuf);
        cudaFree(c->planes);
        cudaFree(c->planes2);
        cudaFree(c->d_step);
        c->dbuf = nullptr;
        c->planes = nullptr;
        c->planes2 = nullptr;
        c->d_step = nullptr;
        c->chunk = t->chunk_segments;
        CK(cudaMalloc(&c->dbuf, sizeof(float2) * c->dstride * c->chunk));
        CK(cudaMalloc(&c->planes, sizeof(float) * c->pstride * c->chunk));
        CK(cudaMalloc(&c->planes2, sizeof(float) * c->pstride * c->chunk));
        CK(cudaMalloc(&c->d_step, sizeof(unsigned) * ((size_t)c->chunk + 1)));
        encode_hsum_maps(c);
    }
    return ACCEL_OK;
}

int accel_num_harmonics(const accel_ctx* c) { return c ? c->nh : 0; }
int accel_num_stages(const accel_ctx* c) { return c ? c->nstages : 0; }
int accel_uselen(const accel_ctx* c) { return c ? c->uselen : 0; }

int accel_harmonic_info(const accel_ctx* c, int h, accel_harmonic* o) {
    if (!c || !o || h < 0 || h >= c->nh) return set_err(ACCEL_ERR_INVALID, "bad harmonic index");
    const BankHarmDev& b = c->bh[h];
    o->harmnum = b.harmnum;
    o->maxharm = b.maxharm;
    o->zmax = b.zmax;
    o->numzs = b.numzs;
    o->fftlen = 2 * b.M;
    o->halfwidth = b.hw0;
    o->zlo = b.zlo;
    o->plane_width = c->hp[h].wmax;
    return ACCEL_OK;
}

int accel_get_power_cuts(const accel_ctx* c, float* cuts) {
    if (!c || !cuts) return set_err(ACCEL_ERR_INVALID, "null argument");
    for (int s = 0; s < c->nstages; s++) cuts[s] = c->cuts[s];
    return ACCEL_OK;
}

int accel_set_power_cuts(accel_ctx* c, const float* cuts) {
    if (!c || !cuts) return set_err(ACCEL_ERR_INVALID, "null argument");
    for (int s = 0; s < c->nstages; s++) c->cuts[s] = cuts[s];
    return ACCEL_OK;
}

}  // extern "C"

namespace accel {
double sigma_of_power_host(double power, int numharm, double numindep) {
    return sigma_of_power(power, numharm, numindep);
}
}  // namespace accel

extern "C" {

double accel_power_cut(double sigma, int numharm, double numindep) {
    return power_cut(sigma, numharm, numindep);
}

double accel_sigma_of_power(double power, int numharm, double numindep) {
    return sigma_of_power(power, numharm, numindep);
}

long long accel_first_bin(long long nsamples, double dt) {
    // AccelSearch.cu:101: long * float evaluated in single precision
    return (long long)std::floor(1.0 * (double)((float)nsamples * (float)dt));
}

long long accel_step_count(const accel_ctx* c, long long nsamples, double dt) {
    if (!c) return -1;
    const long long half = (unsigned short)(c->uselen / 2);
    long long rlo = accel_first_bin(nsamples, dt), numbins = nsamples / 2, s = 0;
    for (long long r = rlo; r + half < numbins; r += half) s++;
    return s;
}

int accel_step_harmonic(long long startr, int uselen, int harmnum, int maxharm, int hw0, long long* out) {
    if (!out || harmnum < 1 || maxharm < 1 || uselen < 2) return set_err(ACCEL_ERR_INVALID, "bad argument");
    StepHarm g = step_harm(startr, uselen, harmnum, maxharm, hw0);
    out[0] = g.rlo;
    out[1] = g.ceilhi;
    out[2] = g.numrs;
    out[3] = g.lobin;
    out[4] = g.numdata;
    return ACCEL_OK;
}

int accel_harmonic_indices(long long startr, int uselen, int harmnum, int maxharm, int hw0, int zlo0,
                           int zlo_h, int nr, int nz, int* rind, int* zind) {
    if (harmnum < 1 || maxharm < 1 || nr < 0 || nz < 0) return set_err(ACCEL_ERR_INVALID, "bad argument");
    StepHarm g = step_harm(startr, uselen, harmnum, maxharm, hw0);
    for (int i = 0; rind && i < nr; i++) rind[i] = sub_rind(startr, i, harmnum, maxharm, g.rlo);
    for (int z = 0; zind && z < nz; z++) zind[z] = sub_zind(zlo0 + kDz * z, harmnum, maxharm, zlo_h);
    return ACCEL_OK;
}

int accel_whiten(accel_ctx* c, accel_complex* spec, long long numbins) {
    if (!c || !spec || numbins <= 0) return set_err(ACCEL_ERR_INVALID, "bad argument");
    if (numbins > kMaxWhitenBins)
        return set_err(ACCEL_ERR_INVALID, "accel_whiten: %lld bins exceed the limit of %lld", numbins,
                       kMaxWhitenBins);
    int rc = ensure_device(c);
    if (rc) return rc;
    return do_whiten(c, reinterpret_cast<float2*>(spec), (unsigned)numbins);
}

int accel_whiten_blocks(long long numbins, int initbuf, int maxbuf, int* start, int* len, long long cap,
                        long long* nblocks) {
    if (!nblocks || cap < 0 || (cap > 0 && (!start || !len))) return set_err(ACCEL_ERR_INVALID, "bad argument");
    const long long n = whiten_blocks(numbins, initbuf, maxbuf, start, len, cap);
    if (n < 0)
        return set_err(ACCEL_ERR_INVALID, "accel_whiten_blocks: %lld bins or widths %d/%d out of range", numbins,
                       initbuf, maxbuf);
    *nblocks = n;
    return ACCEL_OK;
}

int accel_rfft(accel_ctx* c, const float* series, long long n, accel_complex* spec) {
    if (!c || !series || !spec || n < 2 || (n & 1)) return set_err(ACCEL_ERR_INVALID, "bad argument");
    int rc = ensure_device(c);
    if (rc) return rc;
    return do_rfft(c, series, n, reinterpret_cast<float2*>(spec));
}

int accel_search(accel_ctx* c, int ntrials, const float* const* series, const long long* nsamples,
                 const double* dt, int on_device, long long* ncand) {
    if (!c || ntrials < 0 || (ntrials > 0 && (!series || !nsamples || !dt)))
        return set_err(ACCEL_ERR_INVALID, "bad argument");
    int rc = ensure_device(c);
    if (rc) return rc;
    if ((int)c->trials.size() < ntrials) c->trials.resize(ntrials);
    if (!on_device) {
        // the series are copied on their own stream, so that trial i+1 lands
        // while trial i is transformed and whitened
        if (!c->copy_stream) CK(cudaStreamCreate(&c->copy_stream));
        while ((int)c->copy_ev.size() < ntrials) {
            cudaEvent_t e;
            CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
            c->copy_ev.push_back(e);
        }
    }
    CK(cudaEventRecord(c->ev_begin, c->stream));
    if (!on_device) CK(cudaStreamWaitEvent(c->copy_stream, c->ev_begin, 0));
    std::vector<float2*> specs(ntrials);
    std::vector<long long> nb(ntrials), rlo(ntrials);
    for (int i = 0; i < ntrials; i++) {
        long long n = nsamples[i];
        if (n < 4 || (n & 1) || n / 2 > 0x7fffffffLL)
            return set_err(ACCEL_ERR_INVALID, "trial %d: sample count %lld must be even and >= 4", i, n);
        TrialBuf& t = c->trials[i];
        if (t.n < n) {
            CK(cudaStreamSynchronize(c->stream));
            if (c->copy_stream) CK(cudaStreamSynchronize(c->copy_stream));
            cudaFree(t.series);
            cudaFree(t.spec);
            t.series = nullptr;
            t.spec = nullptr;
            t.n = 0;
            CK(cudaMalloc(&t.series, sizeof(float) * n));
            CK(cudaMalloc(&t.spec, sizeof(float2) * (n / 2 + 1)));
            t.n = n;
        }
    }
    for (int i = 0; i < ntrials; i++) {
        TrialBuf& t = c->trials[i];
        specs[i] = t.spec;
        nb[i] = nsamples[i] / 2;
        t.numbins = nsamples[i] / 2;
        rlo[i] = accel_first_bin(nsamples[i], dt[i]);
    }
    // From host memory, a trial's R2C and whitening are issued just before
    // the first launch group that needs it, so that the copies of later
    // trials overlap the search; series already on the device are all
    // prepared first.  The copies are issued kCopyAhead trials ahead of the
    // trial being prepared rather than all before the first launch group:
    // with every copy of a 256-trial batch queued up front, the device time
    // of host-fed searches on a GB300 grew from call to call (1.53 to 1.60 s
    // over 16 calls, while copies of the same pinned buffers slowed down);
    // issued a few trials ahead it stays within 0.3 % of the search from
    // device-resident series.  The host still runs far ahead of the GPU, so
    // the copies stay ahead of the search.
    constexpr int kCopyAhead = 8;
    int copied = 0;  // copies of trials [0, copied) have been issued
    auto copy_upto = [&](int last) -> int {
        for (; copied <= last && copied < ntrials; copied++) {
            CK(cudaMemcpyAsync(c->trials[copied].series, series[copied], sizeof(float) * nsamples[copied],
                               cudaMemcpyHostToDevice, c->copy_stream));
            CK(cudaEventRecord(c->copy_ev[copied], c->copy_stream));
        }
        return ACCEL_OK;
    };
    auto prepare = [&](int i) -> int {
        TrialBuf& t = c->trials[i];
        const float* src = series[i];
        if (!on_device) {
            const int r = copy_upto(i + kCopyAhead);
            if (r) return r;
            CK(cudaStreamWaitEvent(c->stream, c->copy_ev[i], 0));
            src = t.series;
        }
        int r = do_rfft(c, src, nsamples[i], t.spec);
        if (!r) r = do_whiten(c, t.spec, (unsigned)(nsamples[i] / 2));
        return r;
    };
    c->last_trials = ntrials;
    if (on_device) {
        for (int i = 0; i < ntrials && !rc; i++) rc = prepare(i);
        if (rc) return rc;
        rc = run_search(c, ntrials, specs.data(), nb.data(), rlo.data(), nullptr);
    } else {
        rc = run_search(c, ntrials, specs.data(), nb.data(), rlo.data(), prepare);
    }
    if (ncand) *ncand = (long long)c->last_raw;
    return rc;
}

int accel_search_spectra(accel_ctx* c, int ntrials, const accel_complex* const* wspec,
                         const long long* numbins, const long long* rlo, long long* ncand) {
    if (!c || ntrials < 0 || (ntrials > 0 && (!wspec || !numbins || !rlo)))
        return set_err(ACCEL_ERR_INVALID, "bad argument");
    int rc = ensure_device(c);
    if (rc) return rc;
    CK(cudaEventRecord(c->ev_begin, c->stream));
    std::vector<float2*> specs(ntrials);
    for (int i = 0; i < ntrials; i++) specs[i] = (float2*)wspec[i];
    rc = run_search(c, ntrials, specs.data(), numbins, rlo, nullptr);
    if (ncand) *ncand = (long long)c->last_raw;
    return rc;
}

int accel_candidates(accel_ctx* c, accel_candidate* out, long long cap, long long* n) {
    if (!c) return set_err(ACCEL_ERR_INVALID, "null context");
    long long m = std::min<long long>(cap, (long long)c->results.size());
    if (out && m > 0) std::memcpy(out, c->results.data(), sizeof(accel_candidate) * m);
    if (n) *n = (long long)c->results.size();
    return ACCEL_OK;
}

int accel_layout(const accel_ctx* c, long long* dstride, long long* doff, long long* pstride,
                 long long* poff, int* prow) {
    if (!c) return set_err(ACCEL_ERR_INVALID, "null context");
    if (dstride) *dstride = c->dstride;
    if (pstride) *pstride = c->pstride;
    for (int h = 0; h < c->nh; h++) {
        if (doff) doff[h] = c->hp[h].doff;
        if (poff) poff[h] = c->hp[h].poff;
        if (prow) prow[h] = c->hp[h].prow;
    }
    return ACCEL_OK;
}

static int stage_segs(accel_ctx* c, const float2* spec, long long numbins, const long long* startr, int nseg) {
    int rc = ensure_segs(c, nseg);
    if (rc) return rc;
    for (int s = 0; s < nseg; s++) {
        SegDesc& d = c->h_segs[s];
        d.spec = spec;
        d.numbins = numbins;
        d.startr = startr[s];
        d.trial = 0;
        d.step = s;
    }
    CK(cudaMemcpyAsync(c->d_segs, c->h_segs, sizeof(SegDesc) * nseg, cudaMemcpyHostToDevice, c->stream));
    return ACCEL_OK;
}

int accel_prepare_segments(accel_ctx* c, const accel_complex* wspec, long long numbins,
                           const long long* startr, int nseg, accel_complex* dhalf) {
    if (!c || !wspec || !startr || !dhalf || nseg <= 0) return set_err(ACCEL_ERR_INVALID, "bad argument");
    int rc = ensure_device(c);
    if (!rc) rc = stage_segs(c, (const float2*)wspec, numbins, startr, nseg);
    if (!rc) rc = run_group(c, c->d_segs, nseg, 0, nullptr, (float2*)dhalf, nullptr, true, false, false);
    if (!rc) CK(cudaStreamSynchronize(c->stream));
    return rc;
}

int accel_power_planes(accel_ctx* c, const accel_complex* dhalf, int nseg, float* planes) {
    if (!c || !dhalf || !planes || nseg <= 0) return set_err(ACCEL_ERR_INVALID, "bad argument");
    int rc = ensure_device(c);
    if (!rc) rc = run_group(c, c->d_segs, nseg, 0, nullptr, (const float2*)dhalf, planes, false, true, false);
    if (!rc) CK(cudaStreamSynchronize(c->stream));
    return rc;
}

int accel_sum_harmonics(accel_ctx* c, const float* planes, const long long* startr, int nseg,
                        float* stage_out, long long* ncand) {
    if (!c || !planes || !startr || nseg <= 0) return set_err(ACCEL_ERR_INVALID, "bad argument");
    if (reinterpret_cast<uintptr_t>(planes) & 15)
        return set_err(ACCEL_ERR_INVALID, "planes must be 16-byte aligned");
    int rc = ensure_device(c);
    if (!rc) rc = stage_segs(c, nullptr, 0, startr, nseg);
    if (!rc) CK(cudaMemsetAsync(c->d_ncand, 0, 2 * sizeof(unsigned long long), c->stream));
    if (!rc) rc = run_group(c, c->d_segs, nseg, 0, stage_out, nullptr, const_cast<float*>(planes), false, false, true);
    if (!rc) {
        CK(cudaMemcpyAsync(c->h_ncand, c->d_ncand, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                           c->stream));
        CK(cudaStreamSynchronize(c->stream));
        if (c->h_ncand[1])
            return set_err(ACCEL_ERR_CUDA, "harmonic sum: a tile's copy wait timed out");
        if (ncand) *ncand = (long long)*c->h_ncand;
    }
    return rc;
}

int accel_bank_spectra(const accel_ctx* c, int h, accel_complex* kstd, accel_complex* fold) {
    if (!c || h < 0 || h >= c->nh) return set_err(ACCEL_ERR_INVALID, "bad harmonic index");
    const BankHarmDev& b = c->bh[h];
    size_t n = (size_t)b.numzs * 2 * b.M;
    CK(cudaSetDevice(c->device));
    if (kstd) CK(cudaMemcpy(kstd, b.kstd, sizeof(float2) * n, cudaMemcpyDeviceToHost));
    if (fold) {
        // the device copy is scaled by 1/L; A and B are returned unscaled
        CK(cudaMemcpy(fold, b.fold, sizeof(float2) * n, cudaMemcpyDeviceToHost));
        const float L = 2.0f * (float)b.M;
        for (size_t i = 0; i < n; i++) {
            fold[i].x *= L;
            fold[i].y *= L;
        }
    }
    return ACCEL_OK;
}

}  // extern "C"
