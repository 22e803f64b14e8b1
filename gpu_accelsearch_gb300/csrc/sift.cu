// sift.cu -- candidate sifting on the host: the reference's candidate
// post-processing stubs (sortCandidates, eliminateHarmonics,
// bpd_candidates.cu:15-33, called at AccelSearch.cu:290-305) implemented
// as one pass over a candidate list.
//
// Per trial, independently:
//   1. order by sigma (descending; ties by power, then r, z, numharm);
//   2. keep a candidate only if no kept candidate is strictly closer than
//      min_dr bins in r (any z, any number of harmonics): the strongest
//      cell of a cluster of threshold crossings stands for the cluster;
//   3. with maxharm > 1, drop a kept candidate whose r is within harm_dr
//      bins of (a/b) times the r of a stronger kept candidate, for
//      1 <= a, b <= maxharm, a != b (a harmonic or sub-harmonic of it).
// The output is ordered by trial, then sigma as in step 1.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <iterator>
#include <numeric>
#include <set>
#include <utility>
#include <vector>

#include "../../include/accelsearch.h"
#include "accel_internal.h"

namespace {

bool stronger(const accel_candidate& a, const accel_candidate& b) {
    if (a.sigma != b.sigma) return a.sigma > b.sigma;
    if (a.power != b.power) return a.power > b.power;
    if (a.r != b.r) return a.r < b.r;
    if (a.z != b.z) return a.z < b.z;
    return a.numharm < b.numharm;
}

// Is there a kept r strictly closer than d to x?  (The window is widened so
// that rounding of x -+ d cannot hide a neighbour; the test itself is the
// exact |r - x| < d.)
bool closer_than(const std::multiset<double>& s, double x, double d) {
    const double w = d * (1.0 + 1e-9) + 1e-9;
    for (auto it = s.lower_bound(x - w); it != s.end() && *it <= x + w; ++it)
        if (std::fabs(*it - x) < d) return true;
    return false;
}
// Is there a kept r with |x - (a/b) r| <= d?
bool harmonic_of(const std::multiset<double>& s, double x, int a, int b, double d) {
    const double c = x * b / a, w = d * b / a * (1.0 + 1e-9) + 1e-9;
    for (auto it = s.lower_bound(c - w); it != s.end() && *it <= c + w; ++it)
        if (std::fabs(x - (double)a / b * *it) <= d) return true;
    return false;
}

}  // namespace

extern "C" int accel_sift_candidates(const accel_candidate* in, long long n, double min_dr, int maxharm,
                                     double harm_dr, accel_candidate* out, long long cap, long long* nout) {
    using accel::set_error;
    if (n < 0 || (n > 0 && !in) || !nout || cap < 0 || (cap > 0 && !out))
        return set_error(ACCEL_ERR_INVALID, "accel_sift_candidates: bad argument");
    if (!(min_dr >= 0.0) || !(harm_dr >= 0.0) || maxharm < 1 || maxharm > 64)
        return set_error(ACCEL_ERR_INVALID, "accel_sift_candidates: min_dr and harm_dr >= 0, maxharm in [1, 64]");
    std::vector<long long> idx(n);
    std::iota(idx.begin(), idx.end(), 0LL);
    std::stable_sort(idx.begin(), idx.end(), [&](long long x, long long y) {
        if (in[x].trial != in[y].trial) return in[x].trial < in[y].trial;
        return stronger(in[x], in[y]);
    });
    // harmonic ratios a/b in lowest terms, a != b
    std::vector<std::pair<int, int>> ratios;
    for (int a = 1; a <= maxharm; a++)
        for (int b = 1; b <= maxharm; b++)
            if (a != b && std::gcd(a, b) == 1) ratios.push_back({a, b});
    std::vector<accel_candidate> kept;
    long long t0 = 0;
    while (t0 < n) {
        long long t1 = t0;
        while (t1 < n && in[idx[t1]].trial == in[idx[t0]].trial) t1++;
        // 2. clusters: the strongest of every min_dr neighbourhood
        std::multiset<double> seen;
        std::vector<accel_candidate> group;
        for (long long k = t0; k < t1; k++) {
            const accel_candidate& c = in[idx[k]];
            // strictly closer than min_dr to a stronger one: part of its cluster
            if (min_dr > 0.0 && closer_than(seen, c.r, min_dr)) continue;
            seen.insert(c.r);
            group.push_back(c);
        }
        // 3. harmonics of stronger survivors
        std::multiset<double> final_r;
        for (const accel_candidate& c : group) {
            bool harmonic = false;
            if (maxharm > 1) {
                for (const auto& ab : ratios) {
                    if (harmonic_of(final_r, c.r, ab.first, ab.second, harm_dr)) {
                        harmonic = true;
                        break;
                    }
                }
            }
            if (!harmonic) {
                final_r.insert(c.r);
                kept.push_back(c);
            }
        }
        t0 = t1;
    }
    *nout = (long long)kept.size();
    const long long m = std::min<long long>(cap, (long long)kept.size());
    if (m > 0) std::memcpy(out, kept.data(), sizeof(accel_candidate) * (size_t)m);
    return ACCEL_OK;
}
