// server.cu -- continuous-batching request server (accel_server_*).
//
// Requests are single DM-trial time series.
//   * An admission thread admits queued requests in arrival order, as their
//     R2C plans are ready, while their device memory (series + spectrum)
//     fits the HBM budget and the active limit: it copies the series in and
//     runs the R2C transform and whitening on its own stream, records an
//     event and hands the request to the scheduler.  (Copies from pageable
//     host memory block the calling thread; on their own thread they no
//     longer hold up the launches.)
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
// Planner threads make each request's cuFFT R2C plan when the request is
// submitted (making a plan for a new length costs about 2 ms of host time,
// and almost every request of a serving stream has a new length), without
// work area: the worker runs every transform on one stream with one shared
// work area.  A queued request is admitted once its plan is ready.  Plans
// no queued or active request needs are destroyed once more than
// kPlanCache of them exist.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <set>
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
    int rc = ACCEL_OK;
    cudaEvent_t ready = nullptr;  // end of its copy, R2C and whitening (admission stream)
    std::vector<accel_candidate> cands;
    Clock::time_point t_submit, t_done;
};

// Device and pinned host buffers of one launch group in flight.
struct GroupBuf {
    SegDesc* d_segs = nullptr;
    SegDesc* h_segs = nullptr;                // pinned
    RawCand* d_cands = nullptr;
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
    std::vector<std::pair<Request*, long long>> owner;  // per segment: request, step
};

struct R2CPlan {
    cufftHandle plan = 0;
    size_t work = 0;  // work-area bytes
    bool ok = false;
};

constexpr size_t kPlanCache = 256;
constexpr int kPlanners = 4;

}  // namespace

struct accel_server {
    accel_server_config cfg{};
    cudaStream_t stream = nullptr;   // launch groups (scheduler thread)
    cudaStream_t astream = nullptr;  // copies, R2C and whitening (admission thread)
    accel_ctx* wctx = nullptr;       // whitening plans of the admission thread
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
    // R2C plans by series length (planner thread; guarded by plan_mu)
    std::vector<std::thread> planners;    // kPlanners threads
    std::mutex plan_mu;
    std::condition_variable plan_cv;
    bool plan_stop = false;
    bool plan_evict = false;              // a cached plan lost its last user
    std::deque<long long> plan_queue;
    std::map<long long, R2CPlan> plans;
    std::map<long long, int> plan_users;  // queued or active requests per length
    std::set<long long> planning;         // lengths queued or being planned
    void* work = nullptr;                 // shared cuFFT work area (worker thread)
    size_t work_bytes = 0;
    double bytes_in_use = 0;
    accel_server_stats st{};
    std::deque<Flight> flights;  // launched groups not yet read back, oldest first
    bool late_turn = true;       // the next group serves the late requests (when there are any)
};

namespace {

double request_bytes(long long n) { return 4.0 * n + 8.0 * (n / 2 + 1); }

void release_plan(accel_server* s, long long n) {
    bool wake = false;
    {
        std::lock_guard<std::mutex> lk(s->plan_mu);
        auto it = s->plan_users.find(n);
        if (it != s->plan_users.end() && --it->second <= 0) {
            s->plan_users.erase(it);
            wake = s->plan_evict = s->plans.size() > kPlanCache;
        }
    }
    if (wake) s->plan_cv.notify_all();
}

void finish(accel_server* s, Request* r, int rc, cudaStream_t st) {
    if (r->d_series) cudaFreeAsync(r->d_series, st);
    if (r->d_spec) cudaFreeAsync(r->d_spec, st);
    if (r->ready) cudaEventDestroy(r->ready);
    r->ready = nullptr;
    r->d_series = nullptr;
    r->d_spec = nullptr;
    release_plan(s, r->n);
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
    cfg.chunk_segments = s->cfg.chunk_segments;
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
    if (cudaMemcpyAsync(r->d_series, r->host, sizeof(float) * r->n, cudaMemcpyHostToDevice, s->astream) !=
        cudaSuccess)
        return set_error(ACCEL_ERR_CUDA, "request %lld: copy", r->id);
    R2CPlan pl;
    {
        std::unique_lock<std::mutex> lk(s->plan_mu);
        s->plan_cv.wait(lk, [&] { return s->plans.count(r->n) != 0; });
        pl = s->plans[r->n];
    }
    if (!pl.ok) return set_error(ACCEL_ERR_CUDA, "request %lld: cuFFT plan for %lld samples", r->id, r->n);
    if (pl.work > s->work_bytes) {
        // grow the shared work area (transforms in flight use the old one)
        if (cudaStreamSynchronize(s->astream) != cudaSuccess)
            return set_error(ACCEL_ERR_CUDA, "request %lld: stream", r->id);
        cudaFree(s->work);
        s->work = nullptr;
        s->work_bytes = 0;
        if (cudaMalloc(&s->work, pl.work) != cudaSuccess)
            return set_error(ACCEL_ERR_NOMEM, "request %lld: cuFFT work area", r->id);
        s->work_bytes = pl.work;
    }
    if (cufftSetWorkArea(pl.plan, s->work) != CUFFT_SUCCESS || cufftSetStream(pl.plan, s->astream) != CUFFT_SUCCESS ||
        cufftExecR2C(pl.plan, r->d_series, reinterpret_cast<cufftComplex*>(r->d_spec)) != CUFFT_SUCCESS)
        return set_error(ACCEL_ERR_CUDA, "request %lld: R2C", r->id);
    rc = do_whiten(s->wctx, r->d_spec, (unsigned)r->numbins);
    if (!rc && (cudaEventCreateWithFlags(&r->ready, cudaEventDisableTiming) != cudaSuccess ||
                cudaEventRecord(r->ready, s->astream) != cudaSuccess))
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
    const int cap = c->chunk;
    const long long half = (unsigned short)(c->uselen / 2);
    std::vector<Request*> order(g.active);
    const auto now = Clock::now();
    std::stable_sort(order.begin(), order.end(), [&](const Request* a, const Request* b) {
        return prio(s, a, c, now, late_first) < prio(s, b, c, now, late_first);
    });
    for (Request* r : order) {
        while ((int)f.owner.size() < cap && r->next_step < r->nsteps) {
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
    if (!f.rc && cudaMemcpyAsync(B.h_ncand, B.d_ncand, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                                 s->stream) != cudaSuccess)
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
    if (!rc && cudaEventSynchronize(B.done) != cudaSuccess) rc = set_error(ACCEL_ERR_CUDA, "server: group");
    if (!rc && B.h_ncand[1]) rc = set_error(ACCEL_ERR_CUDA, "server: a harmonic-sum tile's copy wait timed out");
    if (!rc) {
        const long long nr = (long long)std::min<unsigned long long>(B.h_ncand[0], (unsigned long long)c->cand_cap);
        raw.resize(nr);
        if (nr > 0 && cudaMemcpy(raw.data(), B.d_cands, sizeof(RawCand) * nr, cudaMemcpyDeviceToHost) != cudaSuccess)
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

// Makes the R2C plans of submitted lengths; destroys plans no request
// needs while more than kPlanCache exist.
void planner_loop(accel_server* s) {
    cudaSetDevice(s->cfg.device);
    for (;;) {
        long long n = -1;
        std::vector<cufftHandle> drop;
        {
            std::unique_lock<std::mutex> lk(s->plan_mu);
            s->plan_cv.wait(lk, [&] { return s->plan_stop || !s->plan_queue.empty() || s->plan_evict; });
            s->plan_evict = false;
            if (!s->plan_queue.empty()) {
                n = s->plan_queue.front();
                s->plan_queue.pop_front();
            } else if (s->plan_stop) {
                return;
            }
            for (auto it = s->plans.begin(); it != s->plans.end() && s->plans.size() > kPlanCache;) {
                if (s->plan_users.count(it->first) == 0) {
                    if (it->second.ok) drop.push_back(it->second.plan);
                    it = s->plans.erase(it);
                } else {
                    ++it;
                }
            }
        }
        for (cufftHandle h : drop) cufftDestroy(h);
        if (n < 0) continue;
        R2CPlan pl;
        cufftResult e = cufftCreate(&pl.plan);
        if (e == CUFFT_SUCCESS) e = cufftSetAutoAllocation(pl.plan, 0);
        if (e == CUFFT_SUCCESS) e = cufftMakePlan1d(pl.plan, (int)n, CUFFT_R2C, 1, &pl.work);
        pl.ok = e == CUFFT_SUCCESS;
        if (!pl.ok && pl.plan) {
            cufftDestroy(pl.plan);
            pl.plan = 0;
        }
        {
            std::lock_guard<std::mutex> lk(s->plan_mu);
            s->plans[n] = pl;
            s->planning.erase(n);
        }
        s->plan_cv.notify_all();
        { std::lock_guard<std::mutex> lk(s->mu); }  // the worker waits on cv_work under mu
        s->cv_work.notify_all();
    }
}

// Admission thread: admits queued requests in arrival order as their R2C
// plans become ready (a request whose plan is still being made does not
// hold back the ones behind it) while the HBM budget and the active limit
// allow, stopping at the first request they cannot take; prepares each
// on the admission stream and hands it to the scheduler.
void admitter_loop(accel_server* s) {
    cudaSetDevice(s->cfg.device);
    for (;;) {
        std::vector<Request*> admitted;
        {
            std::unique_lock<std::mutex> lk(s->mu);
            // lock order: mu, then plan_mu
            auto plan_ready = [&](const Request* r) {
                std::lock_guard<std::mutex> pk(s->plan_mu);
                return s->plans.count(r->n) != 0;
            };
            auto can_admit = [&] {
                for (const Request* r : s->pending) {
                    if (s->cfg.max_active > 0 && s->st.active >= s->cfg.max_active) return false;
                    if (s->bytes_in_use + r->bytes > s->cfg.hbm_budget_bytes) return false;
                    if (plan_ready(r)) return true;
                }
                return false;
            };
            s->cv_work.wait(lk, [&] { return (s->stop && s->pending.empty()) || can_admit(); });
            if (s->stop && s->pending.empty()) {
                s->admitter_done = true;
                s->cv_work.notify_all();
                return;
            }
            for (auto it = s->pending.begin(); it != s->pending.end();) {
                Request* r = *it;
                if (s->cfg.max_active > 0 && s->st.active >= s->cfg.max_active) break;
                if (s->bytes_in_use + r->bytes > s->cfg.hbm_budget_bytes) break;
                if (!plan_ready(r)) {
                    ++it;
                    continue;
                }
                it = s->pending.erase(it);
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
            const int rc = admit(s, r);
            {
                const double ms = std::chrono::duration<double, std::milli>(Clock::now() - ta).count();
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
            // the group stream waits for the request's copy, R2C and whitening
            if (c && cudaStreamWaitEvent(s->stream, r->ready, 0) != cudaSuccess)
                rc = set_error(ACCEL_ERR_CUDA, "request %lld: stream wait", r->id);
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
                any_late |= r->next_step < r->nsteps && is_late(s, r, now);
        const bool late_first = any_late && s->late_turn;
        if (any_late) s->late_turn = !s->late_turn;
        for (auto& kv : s->groups) {
            accel_ctx* c = kv.second.ctx;
            for (Request* r : kv.second.active) {
                if (r->next_step >= r->nsteps) continue;
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
        const bool launched = next.n > 0;
        if (launched) s->flights.push_back(std::move(next));
        if (!s->flights.empty() && ((int)s->flights.size() >= kFlightDepth || !launched)) {
            complete_group(s, s->flights.front());
            s->flights.pop_front();
        }
        {
            const double ms = std::chrono::duration<double, std::milli>(Clock::now() - tg).count();
            std::lock_guard<std::mutex> lk(s->mu);
            s->st.group_ms += ms;
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
    // whitening for the admission thread: a context of its own (its plans
    // cache is not shared with the scheduler's contexts), on its stream
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
    for (int i = 0; i < kPlanners; i++) s->planners.emplace_back(planner_loop, s);
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
    {
        std::lock_guard<std::mutex> lk(s->plan_mu);
        s->plan_stop = true;
        s->plan_queue.clear();
    }
    s->plan_cv.notify_all();
    for (std::thread& t : s->planners)
        if (t.joinable()) t.join();
    cudaStreamSynchronize(s->stream);
    cudaStreamSynchronize(s->astream);
    for (auto& kv : s->plans)
        if (kv.second.ok) cufftDestroy(kv.second.plan);
    cudaFree(s->work);
    for (auto& kv : s->groups) free_group(kv.second);
    for (auto& kv : s->reqs) {
        if (kv.second->d_series) cudaFree(kv.second->d_series);
        if (kv.second->d_spec) cudaFree(kv.second->d_spec);
        if (kv.second->ready) cudaEventDestroy(kv.second->ready);
    }
    accel_destroy(s->wctx);
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
        // the planner makes this length's R2C plan while the request waits
        std::lock_guard<std::mutex> lk(s->plan_mu);
        s->plan_users[n]++;
        if (s->plans.count(n) == 0 && s->planning.insert(n).second) s->plan_queue.push_back(n);
    }
    s->plan_cv.notify_all();
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
