// server.cu -- continuous-batching request server (accel_server_*).
//
// Requests are single DM-trial time series.  A scheduler thread
//   * admits queued requests in arrival order while their device memory
//     (series + spectrum) fits the HBM budget and the active limit, copies
//     the series in, and runs the R2C transform and whitening on the device;
//   * builds each launch group from the active requests of one template
//     bank (one bank per zmax, created on first use), shortest remaining
//     work first: the bank holding the active request with the least work
//     left, then that bank's requests in order of remaining steps, as many
//     steps of each as the group has room for.  A request admitted while
//     others are in flight joins the very next group that has room, so its
//     work overlaps with theirs on the device, and a short request overtakes
//     a long one instead of sharing the GPU with it step by step;
//   * completes a request when its last step has been summed: candidates
//     are kept for accel_server_result, its device memory is released and
//     its latency (submission to completion) recorded.
// Each segment is computed independently of the others in its group, so a
// request's result does not depend on what it was batched with.
//
// A planner thread makes each request's cuFFT R2C plan when the request is
// submitted (making a plan for a new length costs about 2 ms of host time,
// and almost every request of a serving stream has a new length), without
// work area: the worker runs every transform on one stream with one shared
// work area.  Plans no queued or active request needs are destroyed once
// more than kPlanCache of them exist.
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
    std::vector<accel_candidate> cands;
    Clock::time_point t_submit, t_done;
};

struct Group {
    accel_ctx* ctx = nullptr;
    std::vector<Request*> active;
};

struct R2CPlan {
    cufftHandle plan = 0;
    size_t work = 0;  // work-area bytes
    bool ok = false;
};

constexpr size_t kPlanCache = 256;

}  // namespace

struct accel_server {
    accel_server_config cfg{};
    cudaStream_t stream = nullptr;
    std::thread worker;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    bool stop = false;
    std::deque<Request*> pending;
    std::map<long long, std::unique_ptr<Request>> reqs;
    std::map<int, Group> groups;
    long long next_id = 1;
    // R2C plans by series length (planner thread; guarded by plan_mu)
    std::thread planner;
    std::mutex plan_mu;
    std::condition_variable plan_cv;
    bool plan_stop = false;
    bool plan_evict = false;              // a cached plan lost its last user
    std::deque<long long> plan_queue;
    std::map<long long, R2CPlan> plans;
    std::map<long long, int> plan_users;  // queued or active requests per length
    void* work = nullptr;                 // shared cuFFT work area (worker thread)
    size_t work_bytes = 0;
    double bytes_in_use = 0;
    accel_server_stats st{};
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    std::vector<std::pair<Request*, long long>> seg_owner;  // per segment of the current group
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

void finish(accel_server* s, Request* r, int rc) {
    if (r->d_series) cudaFreeAsync(r->d_series, s->stream);
    if (r->d_spec) cudaFreeAsync(r->d_spec, s->stream);
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
    return g.ctx;
}

// Copy in, transform and whiten one admitted request (worker thread).
int admit(accel_server* s, Request* r) {
    int rc = ACCEL_OK;
    accel_ctx* c = group_ctx(s, r->zmax, &rc);
    if (!c) return rc;
    if (cudaMallocAsync(&r->d_series, sizeof(float) * r->n, s->stream) != cudaSuccess ||
        cudaMallocAsync(&r->d_spec, sizeof(float2) * (r->n / 2 + 1), s->stream) != cudaSuccess)
        return set_error(ACCEL_ERR_NOMEM, "request %lld: device allocation", r->id);
    if (cudaMemcpyAsync(r->d_series, r->host, sizeof(float) * r->n, cudaMemcpyHostToDevice, s->stream) !=
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
        if (cudaStreamSynchronize(s->stream) != cudaSuccess)
            return set_error(ACCEL_ERR_CUDA, "request %lld: stream", r->id);
        cudaFree(s->work);
        s->work = nullptr;
        s->work_bytes = 0;
        if (cudaMalloc(&s->work, pl.work) != cudaSuccess)
            return set_error(ACCEL_ERR_NOMEM, "request %lld: cuFFT work area", r->id);
        s->work_bytes = pl.work;
    }
    if (cufftSetWorkArea(pl.plan, s->work) != CUFFT_SUCCESS || cufftSetStream(pl.plan, s->stream) != CUFFT_SUCCESS ||
        cufftExecR2C(pl.plan, r->d_series, reinterpret_cast<cufftComplex*>(r->d_spec)) != CUFFT_SUCCESS)
        return set_error(ACCEL_ERR_CUDA, "request %lld: R2C", r->id);
    rc = do_whiten(c, r->d_spec, (unsigned)r->numbins);
    if (!rc) {
        const long long half = (unsigned short)(c->uselen / 2);
        r->nsteps = 0;
        for (long long x = r->rlo; x + half < r->numbins; x += half) r->nsteps++;
    }
    return rc;
}

// One launch group from the active requests of group zmax.  Returns false
// when the group had no steps left.
bool run_one_group(accel_server* s, int zmax) {
    Group& g = s->groups[zmax];
    accel_ctx* c = g.ctx;
    if (!c || g.active.empty()) return false;
    const int cap = c->chunk;
    if (ensure_segs(c, cap)) return false;
    const long long half = (unsigned short)(c->uselen / 2);
    s->seg_owner.clear();
    // shortest remaining work first (ties: earlier submission), every step
    // of a request before the next one's
    std::vector<Request*> order(g.active);
    std::stable_sort(order.begin(), order.end(), [](const Request* a, const Request* b) {
        return a->nsteps - a->next_step < b->nsteps - b->next_step;
    });
    for (Request* r : order) {
        while ((int)s->seg_owner.size() < cap && r->next_step < r->nsteps) {
            SegDesc& d = c->h_segs[s->seg_owner.size()];
            d.spec = r->d_spec;
            d.numbins = r->numbins;
            d.startr = r->rlo + r->next_step * half;
            d.trial = (int)(r->id & 0x7fffffff);
            d.step = (int)r->next_step;
            s->seg_owner.push_back({r, r->next_step});
            r->next_step++;
        }
    }
    const int n = (int)s->seg_owner.size();
    if (n == 0) return false;
    int rc = ACCEL_OK;
    if (cudaMemcpyAsync(c->d_segs, c->h_segs, sizeof(SegDesc) * n, cudaMemcpyHostToDevice, s->stream) ||
        cudaMemsetAsync(c->d_ncand, 0, 2 * sizeof(unsigned long long), s->stream))
        rc = set_error(ACCEL_ERR_CUDA, "server: group upload");
    cudaEventRecord(s->ev0, s->stream);
    if (!rc) rc = run_group(c, c->d_segs, n, 0, nullptr, nullptr, nullptr, true, true, true, c->fused_sum != 0);
    cudaEventRecord(s->ev1, s->stream);
    std::vector<RawCand> raw;
    if (!rc) {
        if (cudaMemcpyAsync(c->h_ncand, c->d_ncand, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                            s->stream) != cudaSuccess ||
            cudaStreamSynchronize(s->stream) != cudaSuccess)
            rc = set_error(ACCEL_ERR_CUDA, "server: group");
        else if (c->h_ncand[1])
            rc = set_error(ACCEL_ERR_CUDA, "server: a harmonic-sum tile's copy wait timed out");
    }
    if (!rc) {
        const long long nr = (long long)std::min<unsigned long long>(*c->h_ncand, (unsigned long long)c->cand_cap);
        raw.resize(nr);
        if (nr > 0 && cudaMemcpy(raw.data(), c->d_cands, sizeof(RawCand) * nr, cudaMemcpyDeviceToHost) != cudaSuccess)
            rc = set_error(ACCEL_ERR_CUDA, "server: candidates");
        if (*c->h_ncand > (unsigned long long)c->cand_cap) rc = set_error(ACCEL_ERR_CAPACITY, "server: candidates");
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, s->ev0, s->ev1) == cudaSuccess) s->st.gpu_ms += ms;
        s->st.cells += (long long)n * c->uselen * c->numzs0;
    }
    for (const RawCand& x : raw) {
        Request* r = s->seg_owner[x.seg].first;
        accel_candidate o;
        o.trial = (int)(r->id & 0x7fffffff);
        o.step = (int)s->seg_owner[x.seg].second;
        o.r = (double)(r->rlo + o.step * half) + 0.5 * x.ridx;
        o.z = (double)(c->zlo0 + kDz * x.zidx);
        o.numharm = x.numharm;
        o.power = x.power;
        o.sigma = (float)sigma_of_power_host(x.power, x.numharm, c->cfg.numindep);
        r->cands.push_back(o);
    }
    for (auto& so : s->seg_owner) so.first->done_steps++;
    std::vector<Request*> keep;
    for (Request* r : g.active) {
        if (rc != ACCEL_OK && r->next_step > 0 && r->state == 1) {
            finish(s, r, rc);
        } else if (r->done_steps >= r->nsteps) {
            std::sort(r->cands.begin(), r->cands.end(), [](const accel_candidate& a, const accel_candidate& b) {
                if (a.step != b.step) return a.step < b.step;
                if (a.numharm != b.numharm) return a.numharm < b.numharm;
                if (a.z != b.z) return a.z < b.z;
                return a.r < b.r;
            });
            finish(s, r, ACCEL_OK);
        } else {
            keep.push_back(r);
        }
    }
    g.active.swap(keep);
    return true;
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
        }
        s->plan_cv.notify_all();
    }
}

void worker_loop(accel_server* s) {
    cudaSetDevice(s->cfg.device);
    for (;;) {
        std::vector<Request*> admitted;
        {
            std::unique_lock<std::mutex> lk(s->mu);
            s->cv_work.wait(lk, [&] {
                if (s->stop || !s->pending.empty()) return true;
                for (auto& kv : s->groups)
                    if (!kv.second.active.empty()) return true;
                return false;
            });
            bool any_active = false;
            for (auto& kv : s->groups) any_active |= !kv.second.active.empty();
            if (s->stop && s->pending.empty() && !any_active) return;
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
            int rc = admit(s, r);
            s->st.admit_ms += std::chrono::duration<double, std::milli>(Clock::now() - ta).count();
            if (rc) {
                finish(s, r, rc);
                continue;
            }
            if (r->nsteps == 0) {
                finish(s, r, ACCEL_OK);
                continue;
            }
            s->groups[r->zmax].active.push_back(r);
        }
        // the bank holding the active request with the least work left
        // (steps x fundamental cells per step; ties: earlier submission)
        int zmax = -1;
        double best = 0.0;
        long long best_id = 0;
        for (auto& kv : s->groups) {
            accel_ctx* c = kv.second.ctx;
            for (Request* r : kv.second.active) {
                if (r->next_step >= r->nsteps) continue;
                const double w = (double)(r->nsteps - r->next_step) * c->uselen * c->numzs0;
                if (zmax < 0 || w < best || (w == best && r->id < best_id)) {
                    zmax = kv.first;
                    best = w;
                    best_id = r->id;
                }
            }
        }
        if (zmax < 0) continue;  // (a group completes every request whose steps it issued)
        const auto tg = Clock::now();
        run_one_group(s, zmax);
        s->st.group_ms += std::chrono::duration<double, std::milli>(Clock::now() - tg).count();
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
}

int accel_server_create(const accel_server_config* cfg, accel_server** out) {
    if (!cfg || !out) return set_error(ACCEL_ERR_INVALID, "null argument");
    if (cfg->hbm_budget_bytes <= 0) return set_error(ACCEL_ERR_INVALID, "hbm_budget_bytes must be positive");
    *out = nullptr;
    accel_server* s = new accel_server();
    s->cfg = *cfg;
    if (s->cfg.chunk_segments <= 0) s->cfg.chunk_segments = 128;
    cudaError_t e = cudaSetDevice(cfg->device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreate(&s->ev0);
    if (e == cudaSuccess) e = cudaEventCreate(&s->ev1);
    if (e != cudaSuccess) {
        delete s;
        return set_error(ACCEL_ERR_CUDA, "accel_server_create: %s", cudaGetErrorString(e));
    }
    s->planner = std::thread(planner_loop, s);
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
    if (s->worker.joinable()) s->worker.join();
    {
        std::lock_guard<std::mutex> lk(s->plan_mu);
        s->plan_stop = true;
        s->plan_queue.clear();
    }
    s->plan_cv.notify_all();
    if (s->planner.joinable()) s->planner.join();
    cudaStreamSynchronize(s->stream);
    for (auto& kv : s->plans)
        if (kv.second.ok) cufftDestroy(kv.second.plan);
    cudaFree(s->work);
    for (auto& kv : s->groups) accel_destroy(kv.second.ctx);
    for (auto& kv : s->reqs) {
        if (kv.second->d_series) cudaFree(kv.second->d_series);
        if (kv.second->d_spec) cudaFree(kv.second->d_spec);
    }
    cudaEventDestroy(s->ev0);
    cudaEventDestroy(s->ev1);
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
        if (s->plan_users[n]++ == 0 && s->plans.count(n) == 0 &&
            std::find(s->plan_queue.begin(), s->plan_queue.end(), n) == s->plan_queue.end())
            s->plan_queue.push_back(n);
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
