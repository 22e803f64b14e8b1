// server.cu -- continuous-batching request server (accel_server_*).
//
// Requests are single DM-trial time series.
//   * An admission thread admits queued requests in arrival order while
//     their device memory (series + spectrum) fits the HBM budget and the
//     active limit: it copies the series in through pinned staging buffers
//     and runs the R2C transform and whitening on its own stream, records
//     an event and hands the request to the scheduler.
//   * The scheduler thread orders its stream after each handed-over
//     request's event and builds each launch group from the active requests
//     of one template bank (one bank per zmax, created on first use),
//     shortest remaining work first -- the bank holding the request with
//     the least work left, then that bank's requests in the same order, as
//     many steps of each as the group has room for -- except that while
//     requests have waited longer than max_wait_s since submission, every
//     other group serves them first, oldest first.  A request admitted while
//     others are in flight joins the very next group that has room, so its
//     work overlaps with theirs on the device; a short request overtakes a
//     long one instead of sharing the GPU with it step by step, and the
//     wait limit keeps long requests from starving while arrivals continue;
//   * keeps further launch groups queued on the GPU while it reads back
//     the oldest (kFlightDepth in flight, one buffer set more per bank),
//     and completes a request when its last step
//     has been summed: candidates are kept for accel_server_result, its
//     device memory is released and its latency (submission to completion)
//     recorded.
// Each segment is computed independently of the others in its group, so a
// request's result does not depend on what it was batched with.
//
// Almost every request of a serving stream has a length of its own.  The
// R2C transform therefore runs on power-of-two cuFFT plans only (rfft.cu):
// making a cuFFT plan per length took 6-19 ms of host time per request on
// the planner threads of an earlier design and, while it ran, held up every
// CUDA call of the scheduler (kernel launches 0.5 ms instead of 18 us per
// launch group), leaving the GPU waiting between groups.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include "context.h"

namespace {

using Clock = std::chrono::steady_clock;

// Launch groups launched and not yet read back: the host reads the oldest
// once this many are queued, so the GPU still has the others to run.
constexpr int kFlightDepth = 3;

struct Request {
    long long id = 0;
    const float* host = nullptr;
    long long n = 0;
    double dt = 0;
    int zmax = 0;
    long long numbins = 0, rlo = 0, nsteps = 0, next_step = 0, done_steps = 0;
    float* d_series = nullptr;
    float2* d_spec = nullptr;
    double bytes = 0;
    int state = 0;  // 0 queued, 1 active, 2 done, 3 failed
    bool prepared = false;  // its ready event has completed (seen from the host)
    int rc = ACCEL_OK;
    cudaEvent_t ready = nullptr;  // end of its copy, R2C and whitening (admission stream)
    cudaEvent_t ev_prep = nullptr;  // start of its R2C (after the copy): GPU time of the preparation
    std::vector<accel_candidate> cands;
    // submission, admission start, admission's host work done, first launch
    // group issued, completion (accel_server_timing)
    Clock::time_point t_submit, t_admit, t_prepared, t_first, t_done;
};

// Candidates read back with a launch group's count (pinned, asynchronous);
// a group with more reads the rest afterwards.
constexpr int kCandStage = 8192;

// Device and pinned host buffers of one launch group in flight.
struct GroupBuf {
    SegDesc* d_segs = nullptr;
    SegDesc* h_segs = nullptr;                // pinned
    RawCand* d_cands = nullptr;
    RawCand* h_cands = nullptr;               // pinned, kCandStage
    unsigned long long* d_ncand = nullptr;    // count, error word
    unsigned long long* h_ncand = nullptr;    // pinned
    cudaEvent_t ev0 = nullptr, ev1 = nullptr; // the group's kernels
    cudaEvent_t done = nullptr;               // and its count read-back
};

struct Group {
    accel_ctx* ctx = nullptr;
    std::vector<Request*> active;
    GroupBuf buf[kFlightDepth + 1];  // launch groups of this bank take them in turn
    int next_buf = 0;
};

// A launched group whose candidates have not been read yet.
struct Flight {
    int zmax = -1, b = 0, n = 0, rc = ACCEL_OK;
    bool after_idle = false;  // launched after every earlier group had been read back
    std::vector<std::pair<Request*, long long>> owner;  // per segment: request, step
};

// Series reach the device through two pinned staging buffers: the
// admission thread copies a chunk of the caller's (pageable) memory into one
// with the CPU while the other's DMA runs.  (A copy straight from pageable
// memory makes the driver stage it, holding up the scheduler's launches.)
constexpr long long kStageFloats = 1LL << 22;  // 16 MB per buffer

}  // namespace

struct accel_server {
    accel_server_config cfg{};
    cudaStream_t stream = nullptr;   // launch groups (scheduler thread)
    cudaStream_t astream = nullptr;  // copies, R2C and whitening (admission thread)
    float* stage[2] = {nullptr, nullptr};            // pinned staging (admission thread)
    cudaEvent_t stage_ev[2] = {nullptr, nullptr};    // each buffer's last DMA
    bool stage_used[2] = {false, false};
    accel_ctx* wctx = nullptr;       // R2C engine and whitening plans of the admission thread
    std::thread worker, admitter;
    bool admitter_done = false;
    std::deque<Request*> ready;      // admitted and prepared, not yet with the scheduler
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    bool stop = false;
    std::deque<Request*> pending;
    std::map<long long, std::unique_ptr<Request>> reqs;
    std::map<int, Group> groups;
    long long next_id = 1;
    double bytes_in_use = 0;
    accel_server_stats st{};
    std::deque<Flight> flights;  // launched groups not yet read back, oldest first
    cudaEvent_t last_ev1 = nullptr;  // end of the last group read back (its buffer is not reused before the next read)
    bool late_turn = true;       // the next group serves the late requests (when there are any)
};

namespace {

double request_bytes(long long n) { return 4.0 * n + 8.0 * (n / 2 + 1); }

// Whether a request's copy, transform and whitening have finished on the
// admission stream, seen from the host: a launch group takes a request only
// then, so that the group stream never waits on the admission stream (for
// a large request, milliseconds of copy and transform) before a group that
// may not even hold it.  (An error there is sticky: the group that takes
// the request reports it.)
bool is_prepared(accel_server* s, Request* r) {
    if (!r->prepared && cudaEventQuery(r->ready) != cudaErrorNotReady) {
        r->prepared = true;
        float ms = 0.f;
        if (r->ev_prep && cudaEventElapsedTime(&ms, r->ev_prep, r->ready) == cudaSuccess) {
            std::lock_guard<std::mutex> lk(s->mu);
            s->st.prep_gpu_ms += ms;
        }
    }
    return r->prepared;
}

Request* first_unprepared(accel_server* s) {
    for (auto& kv : s->groups)
        for (Request* r : kv.second.active)
            if (r->next_step < r->nsteps && !r->prepared) return r;
    return nullptr;
}

void finish(accel_server* s, Request* r, int rc, cudaStream_t st) {
    if (r->d_series) cudaFreeAsync(r->d_series, st);
    if (r->d_spec) cudaFreeAsync(r->d_spec, st);
    if (r->ready) cudaEventDestroy(r->ready);
    if (r->ev_prep) cudaEventDestroy(r->ev_prep);
    r->ready = nullptr;
    r->ev_prep = nullptr;
    r->d_series = nullptr;
    r->d_spec = nullptr;
    r->rc = rc;
    r->t_done = Clock::now();
    std::lock_guard<std::mutex> lk(s->mu);
    s->bytes_in_use -= r->bytes;
    r->state = rc == ACCEL_OK ? 2 : 3;
    s->st.completed++;
    s->st.active--;
    s->cv_done.notify_all();
    s->cv_work.notify_all();  // budget freed: the admission thread may admit more
}

void free_group(Group& g) {
    for (GroupBuf& b : g.buf) {
        cudaFree(b.d_segs);
        cudaFreeHost(b.h_segs);
        cudaFree(b.d_cands);
        cudaFreeHost(b.h_cands);
        cudaFree(b.d_ncand);
        cudaFreeHost(b.h_ncand);
        if (b.ev0) cudaEventDestroy(b.ev0);
        if (b.ev1) cudaEventDestroy(b.ev1);
        if (b.done) cudaEventDestroy(b.done);
        b = GroupBuf{};
    }
    accel_destroy(g.ctx);
    g.ctx = nullptr;
}

accel_ctx* group_ctx(accel_server* s, int zmax, int* rc) {
    Group& g = s->groups[zmax];
    if (g.ctx) return g.ctx;
    accel_config cfg;
    accel_config_init(&cfg);
    cfg.zmax = zmax;
    cfg.numharm = s->cfg.numharm;
    cfg.fftlen = s->cfg.fftlen;
    cfg.sigma = s->cfg.sigma;
    cfg.chunk_segments = std::max(s->cfg.chunk_segments, s->cfg.max_chunk_segments);
    cfg.device = s->cfg.device;
    *rc = accel_create(&cfg, &g.ctx);
    if (*rc) {
        g.ctx = nullptr;
        return nullptr;
    }
    accel_set_stream(g.ctx, s->stream);
    accel_tuning t;
    accel_get_tuning(g.ctx, &t);
    t.serial_sum = 1;
    accel_set_tuning(g.ctx, &t);
    for (GroupBuf& b : g.buf) {
        const int cap = g.ctx->chunk;
        if (cudaMalloc(&b.d_segs, sizeof(SegDesc) * cap) != cudaSuccess ||
            cudaMallocHost(&b.h_segs, sizeof(SegDesc) * cap) != cudaSuccess ||
            cudaMalloc(&b.d_cands, sizeof(RawCand) * g.ctx->cand_cap) != cudaSuccess ||
            cudaMallocHost(&b.h_cands, sizeof(RawCand) * kCandStage) != cudaSuccess ||
            cudaMalloc(&b.d_ncand, 2 * sizeof(unsigned long long)) != cudaSuccess ||
            cudaMallocHost(&b.h_ncand, 2 * sizeof(unsigned long long)) != cudaSuccess ||
            cudaEventCreate(&b.ev0) != cudaSuccess || cudaEventCreate(&b.ev1) != cudaSuccess ||
            cudaEventCreateWithFlags(&b.done, cudaEventDisableTiming) != cudaSuccess) {
            *rc = set_error(ACCEL_ERR_NOMEM, "server: launch-group buffers");
            free_group(g);
            return nullptr;
        }
    }
    return g.ctx;
}


// Copy in, transform and whiten one admitted request (admission thread,
// admission stream), then record its event.
int admit(accel_server* s, Request* r) {
    int rc = ACCEL_OK;
    if (cudaMallocAsync(&r->d_series, sizeof(float) * r->n, s->astream) != cudaSuccess ||
        cudaMallocAsync(&r->d_spec, sizeof(float2) * (r->n / 2 + 1), s->astream) != cudaSuccess)
        return set_error(ACCEL_ERR_NOMEM, "request %lld: device allocation", r->id);
    if (s->stage[0] && s->stage[1]) {
        int k = 0;
        for (long long off = 0; off < r->n; off += kStageFloats, k ^= 1) {
            const long long m = std::min(kStageFloats, r->n - off);
            if (s->stage_used[k] && cudaEventSynchronize(s->stage_ev[k]) != cudaSuccess)
                return set_error(ACCEL_ERR_CUDA, "request %lld: staging", r->id);
            std::memcpy(s->stage[k], r->host + off, sizeof(float) * m);
            if (cudaMemcpyAsync(r->d_series + off, s->stage[k], sizeof(float) * m, cudaMemcpyHostToDevice,
                                s->astream) != cudaSuccess ||
                cudaEventRecord(s->stage_ev[k], s->astream) != cudaSuccess)
                return set_error(ACCEL_ERR_CUDA, "request %lld: copy", r->id);
            s->stage_used[k] = true;
        }
    } else if (cudaMemcpyAsync(r->d_series, r->host, sizeof(float) * r->n, cudaMemcpyHostToDevice, s->astream) !=
               cudaSuccess) {
        return set_error(ACCEL_ERR_CUDA, "request %lld: copy", r->id);
    }
    // the same transform as the context path (so a request's result equals
    // accel_search's), on the admission stream
    if (cudaEventCreate(&r->ev_prep) != cudaSuccess || cudaEventCreate(&r->ready) != cudaSuccess ||
        cudaEventRecord(r->ev_prep, s->astream) != cudaSuccess)
        return set_error(ACCEL_ERR_CUDA, "request %lld: event", r->id);
    rc = do_rfft(s->wctx, r->d_series, r->n, r->d_spec);
    if (!rc) rc = do_whiten(s->wctx, r->d_spec, (unsigned)r->numbins);
    if (!rc && cudaEventRecord(r->ready, s->astream) != cudaSuccess)
        rc = set_error(ACCEL_ERR_CUDA, "request %lld: event", r->id);
    return rc;
}

// Scheduling order.  late_first: requests past the wait limit first,
// oldest first, then the least work left (steps x fundamental cells per
// step); otherwise the least work left for every request.  Ties by
// submission.
struct Prio {
    bool late;
    double key;
    long long id;
    bool operator<(const Prio& o) const {
        if (late != o.late) return late;
        if (key != o.key) return key < o.key;
        return id < o.id;
    }
};
bool is_late(const accel_server* s, const Request* r, Clock::time_point now) {
    const double lim = s->cfg.max_wait_s > 0 ? s->cfg.max_wait_s : 1.0;
    return std::chrono::duration<double>(now - r->t_submit).count() > lim;
}
Prio prio(const accel_server* s, const Request* r, const accel_ctx* c, Clock::time_point now, bool late_first) {
    if (late_first && is_late(s, r, now))
        return Prio{true, -std::chrono::duration<double>(now - r->t_submit).count(), r->id};
    return Prio{false, (double)(r->nsteps - r->next_step) * c->uselen * c->numzs0, r->id};
}

// Build and launch one group from the active requests of bank zmax:
// shortest remaining work first (ties: earlier submission), every step of
// a request before the next one's.  The candidate count is copied back
// asynchronously; complete_group reads the rest.  Returns a flight with
// n == 0 when the bank had no step left to issue.
Flight launch_group(accel_server* s, int zmax, bool late_first) {
    Flight f;
    f.zmax = zmax;
    Group& g = s->groups[zmax];
    accel_ctx* c = g.ctx;
    if (!c || g.active.empty()) return f;
    f.b = g.next_buf;
    GroupBuf& B = g.buf[f.b];
    // group size: chunk_segments, or with max_chunk_segments a third of the
    // bank's prepared backlog (three groups are kept in flight) within
    // [chunk_segments, max_chunk_segments]
    int cap = std::min(s->cfg.chunk_segments, c->chunk);
    if (s->cfg.max_chunk_segments > cap) {
        long long backlog = 0;
        for (Request* r : g.active)
            if (r->prepared) backlog += r->nsteps - r->next_step;
        cap = (int)std::max<long long>(cap, std::min<long long>(backlog / kFlightDepth, c->chunk));
    }
    const long long half = (unsigned short)(c->uselen / 2);
    std::vector<Request*> order(g.active);
    const auto now = Clock::now();
    std::stable_sort(order.begin(), order.end(), [&](const Request* a, const Request* b) {
        return prio(s, a, c, now, late_first) < prio(s, b, c, now, late_first);
    });
    for (Request* r : order) {
        if (r->next_step >= r->nsteps || !is_prepared(s, r)) continue;
        // (its event has completed: this orders the group after it at no cost)
        if (r->next_step == 0 && cudaStreamWaitEvent(s->stream, r->ready, 0) != cudaSuccess)
            f.rc = set_error(ACCEL_ERR_CUDA, "request %lld: stream wait", r->id);
        while ((int)f.owner.size() < cap && r->next_step < r->nsteps) {
            if (r->next_step == 0) r->t_first = now;
            SegDesc& d = B.h_segs[f.owner.size()];
            d.spec = r->d_spec;
            d.numbins = r->numbins;
            d.startr = r->rlo + r->next_step * half;
            d.trial = (int)(r->id & 0x7fffffff);
            d.step = (int)r->next_step;
            f.owner.push_back({r, r->next_step});
            r->next_step++;
        }
    }
    f.n = (int)f.owner.size();
    if (f.n == 0) return f;
    g.next_buf = (g.next_buf + 1) % (kFlightDepth + 1);
    if (cudaMemcpyAsync(B.d_segs, B.h_segs, sizeof(SegDesc) * f.n, cudaMemcpyHostToDevice, s->stream) ||
        cudaMemsetAsync(B.d_ncand, 0, 2 * sizeof(unsigned long long), s->stream))
        f.rc = set_error(ACCEL_ERR_CUDA, "server: group upload");
    cudaEventRecord(B.ev0, s->stream);
    if (!f.rc) {
        // the harmonic sums append to the context's candidate buffer: this group's
        RawCand* own_c = c->d_cands;
        unsigned long long* own_n = c->d_ncand;
        c->d_cands = B.d_cands;
        c->d_ncand = B.d_ncand;
        f.rc = run_group(c, B.d_segs, f.n, 0, nullptr, nullptr, nullptr, true, true, true, c->fused_sum != 0);
        c->d_cands = own_c;
        c->d_ncand = own_n;
    }
    cudaEventRecord(B.ev1, s->stream);
    if (!f.rc && (cudaMemcpyAsync(B.h_ncand, B.d_ncand, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                                  s->stream) != cudaSuccess ||
                  cudaMemcpyAsync(B.h_cands, B.d_cands, sizeof(RawCand) * std::min<long long>(kCandStage, c->cand_cap),
                                  cudaMemcpyDeviceToHost, s->stream) != cudaSuccess))
        f.rc = set_error(ACCEL_ERR_CUDA, "server: group count");
    cudaEventRecord(B.done, s->stream);
    return f;
}

// Wait for a launched group, read its candidates, hand them to their
// requests and complete the requests whose last step it held.
void complete_group(accel_server* s, Flight& f) {
    Group& g = s->groups[f.zmax];
    accel_ctx* c = g.ctx;
    GroupBuf& B = g.buf[f.b];
    const long long half = (unsigned short)(c->uselen / 2);
    int rc = f.rc;
    std::vector<RawCand> raw;
    const auto tw = Clock::now();
    if (!rc && cudaEventSynchronize(B.done) != cudaSuccess) rc = set_error(ACCEL_ERR_CUDA, "server: group");
    {
        const double ms = std::chrono::duration<double, std::milli>(Clock::now() - tw).count();
        std::lock_guard<std::mutex> lk(s->mu);
        s->st.wait_ms += ms;
        s->st.groups++;
        s->st.group_segments += f.n;
    }
    if (!rc) {
        // the group stream between the previous group's kernels and this
        // one's: the GPU waiting on the host (or, after the queue had
        // drained, on arrivals)
        float gap = 0.f;
        if (s->last_ev1 && cudaEventElapsedTime(&gap, s->last_ev1, B.ev0) == cudaSuccess && gap > 0.f) {
            std::lock_guard<std::mutex> lk(s->mu);
            (f.after_idle ? s->st.idle_ms : s->st.gap_ms) += gap;
        }
        s->last_ev1 = B.ev1;
    } else {
        s->last_ev1 = nullptr;
    }
    if (!rc && B.h_ncand[1]) rc = set_error(ACCEL_ERR_CUDA, "server: a harmonic-sum tile's copy wait timed out");
    if (!rc) {
        const long long nr = (long long)std::min<unsigned long long>(B.h_ncand[0], (unsigned long long)c->cand_cap);
        raw.resize(nr);
        const long long ns = std::min<long long>(nr, kCandStage);
        if (ns > 0) std::memcpy(raw.data(), B.h_cands, sizeof(RawCand) * ns);
        // (the group's kernels are done; a copy on the group stream would wait
        // for the groups queued behind it)
        if (nr > ns && cudaMemcpy(raw.data() + ns, B.d_cands + ns, sizeof(RawCand) * (nr - ns),
                                  cudaMemcpyDeviceToHost) != cudaSuccess)
            rc = set_error(ACCEL_ERR_CUDA, "server: candidates");
        if (B.h_ncand[0] > (unsigned long long)c->cand_cap) rc = set_error(ACCEL_ERR_CAPACITY, "server: candidates");
        float ms = 0.f;
        cudaEventElapsedTime(&ms, B.ev0, B.ev1);
        std::lock_guard<std::mutex> lk(s->mu);  // accel_server_get_stats reads under mu
        s->st.gpu_ms += ms;
        s->st.cells += (long long)f.n * c->uselen * c->numzs0;
    }
    for (const RawCand& x : raw) {
        Request* r = f.owner[x.seg].first;
        if (r->state != 1) continue;
        accel_candidate o;
        o.trial = (int)(r->id & 0x7fffffff);
        o.step = (int)f.owner[x.seg].second;
        o.r = (double)(r->rlo + o.step * half) + 0.5 * x.ridx;
        o.z = (double)(c->zlo0 + kDz * x.zidx);
        o.numharm = x.numharm;
        o.power = x.power;
        o.sigma = (float)sigma_of_power_host(x.power, x.numharm, c->cfg.numindep);
        r->cands.push_back(o);
    }
    for (auto& so : f.owner) {
        Request* r = so.first;
        if (r->state != 1) continue;
        if (rc != ACCEL_OK) {
            finish(s, r, rc, s->stream);
            continue;
        }
        if (++r->done_steps == r->nsteps) {
            std::sort(r->cands.begin(), r->cands.end(), [](const accel_candidate& a, const accel_candidate& b) {
                if (a.step != b.step) return a.step < b.step;
                if (a.numharm != b.numharm) return a.numharm < b.numharm;
                if (a.z != b.z) return a.z < b.z;
                return a.r < b.r;
            });
            finish(s, r, ACCEL_OK, s->stream);
        }
    }
    std::vector<Request*> keep;
    for (Request* r : g.active)
        if (r->state == 1) keep.push_back(r);
    g.active.swap(keep);
}

// Admission thread: admits queued requests in arrival order while the HBM
// budget and the active limit allow, stopping at the first request they
// cannot take; prepares each on the admission stream and hands it to the
// scheduler.
void admitter_loop(accel_server* s) {
    cudaSetDevice(s->cfg.device);
    for (;;) {
        std::vector<Request*> admitted;
        {
            std::unique_lock<std::mutex> lk(s->mu);
            auto can_admit = [&] {
                if (s->pending.empty()) return false;
                if (s->cfg.max_active > 0 && s->st.active >= s->cfg.max_active) return false;
                return s->bytes_in_use + s->pending.front()->bytes <= s->cfg.hbm_budget_bytes;
            };
            s->cv_work.wait(lk, [&] { return (s->stop && s->pending.empty()) || can_admit(); });
            if (s->stop && s->pending.empty()) {
                s->admitter_done = true;
                s->cv_work.notify_all();
                return;
            }
            while (!s->pending.empty()) {
                Request* r = s->pending.front();
                if (s->cfg.max_active > 0 && s->st.active >= s->cfg.max_active) break;
                if (s->bytes_in_use + r->bytes > s->cfg.hbm_budget_bytes) break;
                s->pending.pop_front();
                s->bytes_in_use += r->bytes;
                s->st.admitted++;
                s->st.active++;
                s->st.queued--;
                r->state = 1;
                admitted.push_back(r);
            }
        }
        for (Request* r : admitted) {
            const auto ta = Clock::now();
            r->t_admit = ta;
            const int rc = admit(s, r);
            {
                r->t_prepared = Clock::now();
                const double ms = std::chrono::duration<double, std::milli>(r->t_prepared - ta).count();
                std::lock_guard<std::mutex> lk(s->mu);
                s->st.admit_ms += ms;
            }
            if (rc) {
                finish(s, r, rc, s->astream);
                continue;
            }
            {
                std::lock_guard<std::mutex> lk(s->mu);
                s->ready.push_back(r);
            }
            s->cv_work.notify_all();
        }
    }
}

// Scheduler thread: takes prepared requests, builds and launches groups.
void worker_loop(accel_server* s) {
    cudaSetDevice(s->cfg.device);
    for (;;) {
        std::vector<Request*> incoming;
        {
            std::unique_lock<std::mutex> lk(s->mu);
            s->cv_work.wait(lk, [&] {
                if (!s->flights.empty() || !s->ready.empty()) return true;
                for (auto& kv : s->groups)
                    if (!kv.second.active.empty()) return true;
                return s->stop && s->admitter_done;
            });
            bool any_active = false;
            for (auto& kv : s->groups) any_active |= !kv.second.active.empty();
            if (s->stop && s->admitter_done && s->ready.empty() && !any_active && s->flights.empty()) return;
            incoming.assign(s->ready.begin(), s->ready.end());
            s->ready.clear();
        }
        for (Request* r : incoming) {
            int rc = ACCEL_OK;
            accel_ctx* c = group_ctx(s, r->zmax, &rc);
            if (!c || rc) {
                finish(s, r, rc ? rc : ACCEL_ERR_CUDA, s->stream);
                continue;
            }
            const long long half = (unsigned short)(c->uselen / 2);
            r->nsteps = 0;
            for (long long x = r->rlo; x + half < r->numbins; x += half) r->nsteps++;
            if (r->nsteps == 0) {
                finish(s, r, ACCEL_OK, s->stream);
                continue;
            }
            s->groups[r->zmax].active.push_back(r);
        }
        // while requests past the wait limit exist, every other launch
        // group serves them (oldest first) and the others stay shortest
        // remaining work first: late requests get at least half of the GPU
        // and short ones keep flowing
        int zmax = -1;
        Prio best{};
        const auto now = Clock::now();
        bool any_late = false;
        for (auto& kv : s->groups)
            for (Request* r : kv.second.active)
                any_late |= r->next_step < r->nsteps && is_late(s, r, now) && is_prepared(s, r);
        const bool late_first = any_late && s->late_turn;
        if (any_late) s->late_turn = !s->late_turn;
        for (auto& kv : s->groups) {
            accel_ctx* c = kv.second.ctx;
            for (Request* r : kv.second.active) {
                if (r->next_step >= r->nsteps || !is_prepared(s, r)) continue;
                const Prio p = prio(s, r, c, now, late_first);
                if (zmax < 0 || p < best) {
                    zmax = kv.first;
                    best = p;
                }
            }
        }
        // launch the next group, then read back the oldest one once
        // kFlightDepth are queued (or nothing new could be launched): the
        // host's candidate handling and the next groups' set-up overlap the
        // GPU's work
        const auto tg = Clock::now();
        Flight next;
        if (zmax >= 0) next = launch_group(s, zmax, late_first);
        const double launch_ms = std::chrono::duration<double, std::milli>(Clock::now() - tg).count();
        const bool launched = next.n > 0;
        if (launched) {
            next.after_idle = s->flights.empty();
            s->flights.push_back(std::move(next));
        }
        if (!s->flights.empty() && ((int)s->flights.size() >= kFlightDepth || !launched)) {
            complete_group(s, s->flights.front());
            s->flights.pop_front();
        } else if (!launched && s->flights.empty()) {
            // nothing to launch or read: wait for a request still being prepared
            if (Request* r = first_unprepared(s)) cudaEventSynchronize(r->ready);
        }
        {
            const double ms = std::chrono::duration<double, std::milli>(Clock::now() - tg).count();
            std::lock_guard<std::mutex> lk(s->mu);
            s->st.group_ms += ms;
            s->st.launch_ms += launch_ms;
        }
    }
}

}  // namespace

extern "C" {

void accel_server_config_init(accel_server_config* c) {
    if (!c) return;
    std::memset(c, 0, sizeof(*c));
    c->hbm_budget_bytes = 150e9;
    c->max_active = 0;
    c->fftlen = 8192;
    c->numharm = 8;
    c->sigma = 6.0;
    c->chunk_segments = 128;
    c->device = 0;
    c->max_wait_s = 1.0;
}

int accel_server_create(const accel_server_config* cfg, accel_server** out) {
    if (!cfg || !out) return set_error(ACCEL_ERR_INVALID, "null argument");
    if (cfg->hbm_budget_bytes <= 0) return set_error(ACCEL_ERR_INVALID, "hbm_budget_bytes must be positive");
    *out = nullptr;
    accel_server* s = new accel_server();
    s->cfg = *cfg;
    if (s->cfg.chunk_segments <= 0) s->cfg.chunk_segments = 128;
    if (!(s->cfg.max_wait_s > 0)) s->cfg.max_wait_s = 1.0;
    cudaError_t e = cudaSetDevice(cfg->device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->astream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        if (s->stream) cudaStreamDestroy(s->stream);
        delete s;
        return set_error(ACCEL_ERR_CUDA, "accel_server_create: %s", cudaGetErrorString(e));
    }
    // R2C and whitening for the admission thread: a context of its own (its
    // transform plans and whitening plans are not shared with the
    // scheduler's contexts), on its stream
    accel_config wc;
    accel_config_init(&wc);
    wc.zmax = 0;
    wc.numharm = 1;
    wc.fftlen = 128;
    wc.chunk_segments = 1;
    wc.device = cfg->device;
    int rc = accel_create(&wc, &s->wctx);
    if (!rc) rc = accel_set_stream(s->wctx, s->astream);
    if (rc) {
        if (s->wctx) accel_destroy(s->wctx);
        cudaStreamDestroy(s->astream);
        cudaStreamDestroy(s->stream);
        delete s;
        return rc;
    }
    // pinned staging for the series copies (without it: copies from pageable memory)
    for (int k = 0; k < 2; k++) {
        if (cudaMallocHost(&s->stage[k], sizeof(float) * kStageFloats) != cudaSuccess ||
            cudaEventCreateWithFlags(&s->stage_ev[k], cudaEventDisableTiming) != cudaSuccess) {
            cudaGetLastError();
            if (s->stage[k]) cudaFreeHost(s->stage[k]);
            s->stage[k] = nullptr;
        }
    }
    s->admitter = std::thread(admitter_loop, s);
    s->worker = std::thread(worker_loop, s);
    *out = s;
    return ACCEL_OK;
}

int accel_server_destroy(accel_server* s) {
    if (!s) return ACCEL_OK;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
    }
    s->cv_work.notify_all();
    if (s->admitter.joinable()) s->admitter.join();
    if (s->worker.joinable()) s->worker.join();
    cudaStreamSynchronize(s->stream);
    cudaStreamSynchronize(s->astream);
    for (auto& kv : s->groups) free_group(kv.second);
    for (auto& kv : s->reqs) {
        if (kv.second->d_series) cudaFree(kv.second->d_series);
        if (kv.second->d_spec) cudaFree(kv.second->d_spec);
        if (kv.second->ready) cudaEventDestroy(kv.second->ready);
    }
    accel_destroy(s->wctx);
    for (int k = 0; k < 2; k++) {
        if (s->stage[k]) cudaFreeHost(s->stage[k]);
        if (s->stage_ev[k]) cudaEventDestroy(s->stage_ev[k]);
    }
    cudaStreamDestroy(s->astream);
    cudaStreamDestroy(s->stream);
    delete s;
    return ACCEL_OK;
}

int accel_server_submit(accel_server* s, const float* series, long long n, double dt, int zmax, long long* id) {
    if (!s || !series || n < 4 || (n & 1) || n > 0x7fffffffLL || zmax < 0 || (zmax & 1))
        return set_error(ACCEL_ERR_INVALID, "accel_server_submit: bad argument");
    auto r = std::make_unique<Request>();
    r->host = series;
    r->n = n;
    r->dt = dt;
    r->zmax = zmax;
    r->numbins = n / 2;
    r->rlo = accel_first_bin(n, dt);
    r->bytes = request_bytes(n);
    r->t_submit = Clock::now();
    if (r->bytes > s->cfg.hbm_budget_bytes)
        return set_error(ACCEL_ERR_BUDGET, "request of %.3g bytes exceeds the HBM budget of %.3g", r->bytes,
                         s->cfg.hbm_budget_bytes);
    {
        std::lock_guard<std::mutex> lk(s->mu);
        r->id = s->next_id++;
        if (id) *id = r->id;
        s->pending.push_back(r.get());
        s->reqs[r->id] = std::move(r);
        s->st.submitted++;
        s->st.queued++;
    }
    s->cv_work.notify_all();
    return ACCEL_OK;
}

int accel_server_wait(accel_server* s, long long id, double timeout_s, int* done) {
    if (!s) return set_error(ACCEL_ERR_INVALID, "null server");
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->reqs.find(id);
    if (it == s->reqs.end()) return set_error(ACCEL_ERR_INVALID, "unknown request %lld", id);
    Request* r = it->second.get();
    auto pred = [&] { return r->state >= 2; };
    if (timeout_s < 0) s->cv_done.wait(lk, pred);
    else s->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), pred);
    if (done) *done = r->state >= 2;
    return r->state == 3 ? r->rc : ACCEL_OK;
}

int accel_server_result(accel_server* s, long long id, accel_candidate* out, long long cap, long long* n,
                        double* latency_ms) {
    if (!s) return set_error(ACCEL_ERR_INVALID, "null server");
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->reqs.find(id);
    if (it == s->reqs.end()) return set_error(ACCEL_ERR_INVALID, "unknown request %lld", id);
    Request* r = it->second.get();
    if (r->state < 2) return set_error(ACCEL_ERR_INVALID, "request %lld is not finished", id);
    if (n) *n = (long long)r->cands.size();
    if (latency_ms)
        *latency_ms = std::chrono::duration<double, std::milli>(r->t_done - r->t_submit).count();
    const long long m = std::min<long long>(cap, (long long)r->cands.size());
    if (out && m > 0) std::memcpy(out, r->cands.data(), sizeof(accel_candidate) * m);
    return r->state == 3 ? r->rc : ACCEL_OK;
}

int accel_server_timing(accel_server* s, long long id, double* out_ms) {
    if (!s || !out_ms) return set_error(ACCEL_ERR_INVALID, "null argument");
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->reqs.find(id);
    if (it == s->reqs.end()) return set_error(ACCEL_ERR_INVALID, "unknown request %lld", id);
    const Request* r = it->second.get();
    if (r->state != 2) return set_error(ACCEL_ERR_INVALID, "request %lld has not completed", id);
    auto ms = [](Clock::time_point a, Clock::time_point b) {
        return std::chrono::duration<double, std::milli>(b - a).count();
    };
    out_ms[0] = ms(r->t_submit, r->t_admit);
    out_ms[1] = ms(r->t_admit, r->t_prepared);
    out_ms[2] = r->nsteps ? ms(r->t_prepared, r->t_first) : 0.0;
    out_ms[3] = r->nsteps ? ms(r->t_first, r->t_done) : ms(r->t_prepared, r->t_done);
    return ACCEL_OK;
}

int accel_server_release(accel_server* s, long long id) {
    if (!s) return set_error(ACCEL_ERR_INVALID, "null server");
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->reqs.find(id);
    if (it == s->reqs.end()) return set_error(ACCEL_ERR_INVALID, "unknown request %lld", id);
    if (it->second->state < 2) return set_error(ACCEL_ERR_INVALID, "request %lld is not finished", id);
    s->reqs.erase(it);
    return ACCEL_OK;
}

int accel_server_get_stats(accel_server* s, accel_server_stats* out) {
    if (!s || !out) return set_error(ACCEL_ERR_INVALID, "null argument");
    std::lock_guard<std::mutex> lk(s->mu);
    *out = s->st;
    out->bytes_in_use = s->bytes_in_use;
    return ACCEL_OK;
}

}  // extern "C"
