// optimize.cu -- host side of candidate refinement and properties
// (accel_optimize_candidates; the kernel is k_optimize in bank.cu).
#include <algorithm>
#include <cmath>
#include <numeric>
#include <vector>

#include "../../include/accelsearch.h"
#include "context.h"

extern "C" int accel_trial_spectrum(accel_ctx* c, int trial, const accel_complex** spec, long long* numbins) {
    if (!c || !spec || !numbins) return set_error(ACCEL_ERR_INVALID, "accel_trial_spectrum: null argument");
    if (trial < 0 || trial >= c->last_trials || trial >= (int)c->trials.size())
        return set_error(ACCEL_ERR_INVALID, "accel_trial_spectrum: trial %d not in the last search", trial);
    *spec = reinterpret_cast<const accel_complex*>(c->trials[trial].spec);
    *numbins = c->trials[trial].numbins;
    return ACCEL_OK;
}

extern "C" int accel_optimize_candidates(accel_ctx* c, int ntrials, const accel_complex* const* wspec,
                                         const long long* numbins, const long long* rlo, const double* tobs,
                                         const accel_candidate* in, long long n, int refine,
                                         accel_optimized* out) {
    if (!c || ntrials < 1 || !wspec || !numbins || !rlo || !tobs || n < 0 || (n > 0 && (!in || !out)))
        return set_error(ACCEL_ERR_INVALID, "accel_optimize_candidates: bad argument");
    if (n > 0x7fffffffLL) return set_error(ACCEL_ERR_INVALID, "accel_optimize_candidates: too many candidates");
    for (int t = 0; t < ntrials; t++)
        if (!wspec[t] || numbins[t] < 1 || !(tobs[t] > 0.0))
            return set_error(ACCEL_ERR_INVALID, "accel_optimize_candidates: trial %d", t);
    int rc = ensure_device(c);
    if (rc) return rc;
    std::vector<OptCand> cand((size_t)n);
    int maxdata = 1;
    for (long long i = 0; i < n; i++) {
        const accel_candidate& x = in[i];
        if (x.trial < 0 || x.trial >= ntrials || x.numharm < 1 || x.numharm > c->nh ||
            (x.numharm & (x.numharm - 1)) || x.step < 0 || !std::isfinite(x.r) || !std::isfinite(x.z))
            return set_error(ACCEL_ERR_INVALID, "accel_optimize_candidates: candidate %lld", i);
        OptCand& o = cand[i];
        o.r = x.r;
        o.z = x.z;
        o.numharm = x.numharm;
        o.trial = x.trial;
        // harmonic k of H is the bank's harmonic p/q = k/H in lowest terms;
        // its segment in the candidate's step is the search's (A6/A7)
        const long long startr = rlo[x.trial] + (long long)x.step * (c->uselen / 2);
        for (int k = 1; k <= x.numharm; k++) {
            const int g = std::gcd(k, x.numharm), p = k / g, q = x.numharm / g;
            int h = 0;
            while (h < c->nh && !(c->hp[h].p == p && c->hp[h].q == q)) h++;
            if (h == c->nh) return set_error(ACCEL_ERR_INVALID, "accel_optimize_candidates: harmonic %d/%d", p, q);
            const StepHarm sh = step_harm(startr, c->uselen, p, q, c->hp[h].hw0);
            o.lobin[k - 1] = sh.lobin;
            o.numdata[k - 1] = std::min(sh.numdata, c->hp[h].M);
            maxdata = std::max(maxdata, o.numdata[k - 1]);
        }
    }
    if (n == 0) return ACCEL_OK;
    const float2** d_spec = nullptr;
    long long* d_nb = nullptr;
    OptCand* d_in = nullptr;
    OptOut* d_out = nullptr;
    std::vector<OptOut> res((size_t)n);
    cudaError_t e = cudaMalloc(&d_spec, sizeof(float2*) * ntrials);
    if (e == cudaSuccess) e = cudaMalloc(&d_nb, sizeof(long long) * ntrials);
    if (e == cudaSuccess) e = cudaMalloc(&d_in, sizeof(OptCand) * n);
    if (e == cudaSuccess) e = cudaMalloc(&d_out, sizeof(OptOut) * n);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(d_spec, wspec, sizeof(float2*) * ntrials, cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(d_nb, numbins, sizeof(long long) * ntrials, cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(d_in, cand.data(), sizeof(OptCand) * n, cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) {
        OptArgs a{};
        a.spec = d_spec;
        a.numbins = d_nb;
        a.in = d_in;
        a.out = d_out;
        a.n = (int)n;
        a.refine = refine != 0;
        a.maxdata = maxdata;
        a.exact_rsqrt = c->cfg.exact_rsqrt;
        if (launch_optimize(a, c->stream) != 0) e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaGetLastError();
    }
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(res.data(), d_out, sizeof(OptOut) * n, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    cudaFree(d_spec);
    cudaFree(d_nb);
    cudaFree(d_in);
    cudaFree(d_out);
    if (e != cudaSuccess)
        return set_error(ACCEL_ERR_CUDA, "accel_optimize_candidates: %s", cudaGetErrorString(e));
    for (long long i = 0; i < n; i++) {
        const OptOut& o = res[i];
        accel_optimized& y = out[i];
        y.cand = in[i];
        y.cand.r = o.r;
        y.cand.z = o.z;
        y.cand.power = (float)o.power;
        y.cand.sigma = (float)sigma_of_power_host(o.power, in[i].numharm, c->cfg.numindep);
        y.r_grid = in[i].r;
        y.z_grid = in[i].z;
        for (int k = 0; k < 16; k++) y.harm_power[k] = k < kMaxHarm ? o.harm[k] : 0.f;
        const double T = tobs[in[i].trial];
        y.f = o.r / T;
        y.fdot = o.z / (T * T);
        y.period = y.f != 0.0 ? 1.0 / y.f : 0.0;
        y.pdot = y.f != 0.0 ? -y.fdot / (y.f * y.f) : 0.0;
    }
    return ACCEL_OK;
}
