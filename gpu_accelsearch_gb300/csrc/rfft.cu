// rfft.cu -- real-to-complex FFT of any even length N from power-of-two
// cuFFT plans only (the search's transform of a DM trial; the reference
// makes a cuFFT R2C plan of the trial's own length, bpd_fft.cu:4-48).
//
// The N real samples are read as K = N/2 complex values z[n] = x[2n] +
// i x[2n+1].  Z = DFT_K(z) is one power-of-two C2C transform when K is a
// power of two; when K = m L with L a power of two and an odd m <= 15, m
// transforms of L points (the samples j, j + m, j + 2m, ...) combined by
//     Z[k] = sum_j exp(-2 pi i j k / K) Y_j[k mod L]
// (one Cooley-Tukey step); else Bluestein's chirp-z form: with
// w[m] = exp(i pi m^2/K),
//     Z[k] = conj(w[k]) sum_n (z[n] conj(w[n])) w[k - n],
// a linear convolution done by power-of-two transforms of P >= 2K - 1
// points.  Every phase is a multiple of pi/K reduced exactly to r in
// [0, 2K) (m^2 mod 2K in integers) and evaluated as the double-precision
// product of two table entries, exp(i pi q S/K) exp(i pi t/K) with
// r = q S + t, S ~ sqrt(2K): four double operations per value instead of a
// double sincos (double precision runs at a small fraction of the FP32
// rate), rounded once to float.  The N/2 + 1 bins follow from the
// transforms of the even and odd samples, E[k] = (Z[k] + conj Z[K-k]) / 2
// and O[k] = (Z[k] - conj Z[K-k]) / (2i):
//     X[k] = E[k] + exp(-2 pi i k / N) O[k],   k = 0 .. K   (Z[K] = Z[0]).
// A plan per power of two serves every length, so a stream of trials of
// many lengths (the serving path) makes no new cuFFT plan per trial --
// making one costs milliseconds of host time and holds up every other
// thread's CUDA calls while it runs.
#include <map>

#include "context.h"

namespace accel {

namespace {

__device__ __forceinline__ float2 cmulc(float2 a, float2 b) {  // a * conj(b)
    return make_float2(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}

// Phase tables of exp(i pi r / K): lo[t] for t < S, hi[q] = exp(i pi q S/K)
// for q < ceil(2K/S), in double precision and rounded to float.
__global__ void k_phase_tables(double2* __restrict__ lo, double2* __restrict__ hi, float2* __restrict__ flo,
                               float2* __restrict__ fhi, long long K, int S, int nq) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double s, c;
    if (i < S) {
        sincospi((double)i / (double)K, &s, &c);
        lo[i] = make_double2(c, s);
        flo[i] = make_float2((float)c, (float)s);
    } else if (i < S + nq) {
        sincospi((double)(i - S) * (double)S / (double)K, &s, &c);
        hi[i - S] = make_double2(c, s);
        fhi[i - S] = make_float2((float)c, (float)s);
    }
}

struct Phase {
    const double2* lo;
    const double2* hi;
    const float2* flo;
    const float2* fhi;
    unsigned S;
    // exp(i pi r / K) for 0 <= r < 2K: in double, and (f) in float
    __device__ __forceinline__ double2 operator()(unsigned r) const {
        const double2 a = hi[r / S], b = lo[r % S];
        return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
    }
    __device__ __forceinline__ float2 f(unsigned r) const {
        const float2 a = __ldg(fhi + r / S), b = __ldg(flo + r % S);
        return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
    }
};

// T[j L + l] = z[j + m l]: the m subsequences of stride m, each contiguous
__global__ void k_ct_split(const float2* __restrict__ z, float2* __restrict__ T, int m, long long L) {
    const long long K = (long long)m * L;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < K;
         i += (long long)gridDim.x * blockDim.x) {
        const long long j = i / L, l = i - j * L;
        T[i] = z[j + (long long)m * l];
    }
}

// Z[k] = sum_j exp(-2 pi i j k / K) Y_j[k mod L], Y_j = T[j L .. j L + L)
__global__ void k_ct_combine(const float2* __restrict__ T, float2* __restrict__ Z, int m, long long L,
                             Phase ph) {
    const long long K = (long long)m * L;
    const unsigned long long K2 = 2ull * (unsigned long long)K;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < K;
         k += (long long)gridDim.x * blockDim.x) {
        const long long l = k & (L - 1);
        float2 acc = T[l];
        unsigned long long r = 0;  // 2 j k mod 2K, a multiple of pi/K
        for (int j = 1; j < m; j++) {
            r += 2ull * (unsigned long long)k;
            if (r >= K2) r -= K2;
            const float2 w = ph.f((unsigned)r);  // exp(+i pi r/K); the transform uses its conjugate
            const float2 y = T[(long long)j * L + l];
            acc.x += y.x * w.x + y.y * w.y;
            acc.y += y.y * w.x - y.x * w.y;
        }
        Z[k] = acc;
    }
}

// The chirp w[m] = exp(i pi m^2 / K) for m in [0, K), wrapped into b (b[m]
// and b[P - m], zero elsewhere), and a[n] = z[n] conj(w[n]) for n < K,
// zero up to P.
__global__ void k_chirp(const float2* __restrict__ z, float2* __restrict__ a, float2* __restrict__ b, long long K,
                        long long P, Phase ph) {
    const unsigned long long K2 = 2ull * (unsigned long long)K;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < P;
         i += (long long)gridDim.x * blockDim.x) {
        long long m = -1;
        if (i < K) m = i;
        else if (i > P - K) m = P - i;
        float2 w = make_float2(0.f, 0.f);
        if (m >= 0) {
            const double2 v = ph((unsigned)(((unsigned long long)m * (unsigned long long)m) % K2));
            w = make_float2((float)v.x, (float)v.y);
        }
        b[i] = w;
        a[i] = i < K ? cmulc(z[i], w) : make_float2(0.f, 0.f);
    }
}

__global__ void k_pointwise(float2* __restrict__ a, const float2* __restrict__ fb, long long P) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < P;
         i += (long long)gridDim.x * blockDim.x) {
        const float2 x = a[i], y = fb[i];
        a[i] = make_float2(x.x * y.x - x.y * y.y, x.x * y.y + x.y * y.x);
    }
}

// Z[k] = conj(w[k]) y[k] / P (y: the unnormalised inverse transform)
__global__ void k_chirp_out(const float2* __restrict__ y, const float2* __restrict__ b, float2* __restrict__ Z,
                            long long K, float inv_p) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < K;
         i += (long long)gridDim.x * blockDim.x) {
        const float2 v = cmulc(y[i], b[i]);
        Z[i] = make_float2(v.x * inv_p, v.y * inv_p);
    }
}

// In place over X[0 .. K]: Z[k] in X[k] on entry (k < K); thread k <= K/2
// writes X[k] and X[K - k].
__global__ void k_r2c_unpack(float2* __restrict__ X, long long K, Phase ph) {
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k <= K / 2;
         k += (long long)gridDim.x * blockDim.x) {
        const float2 zk = X[k];
        if (k == 0) {
            X[0] = make_float2(zk.x + zk.y, 0.f);
            X[K] = make_float2(zk.x - zk.y, 0.f);
            continue;
        }
        const float2 zc = X[K - k];
        // E = (Z[k] + conj Z[K-k]) / 2, O = (Z[k] - conj Z[K-k]) / (2i)
        const float2 e = make_float2(0.5f * (zk.x + zc.x), 0.5f * (zk.y - zc.y));
        const float2 o = make_float2(0.5f * (zk.y + zc.y), -0.5f * (zk.x - zc.x));
        const double2 v = ph((unsigned)k);  // exp(+i pi k / K) = exp(2 pi i k / N)
        const float2 t = make_float2((float)v.x, -(float)v.y);  // exp(-2 pi i k / N)
        const float2 to = make_float2(t.x * o.x - t.y * o.y, t.x * o.y + t.y * o.x);
        X[k] = make_float2(e.x + to.x, e.y + to.y);
        if (2 * k != K) {
            // X[K-k] = conj(E) - conj(t) conj(O) = conj(E - t O)
            X[K - k] = make_float2(e.x - to.x, -(e.y - to.y));
        }
    }
}

// Largest odd factor taken by the Cooley-Tukey step (its combine reads m
// values per output)
constexpr long long kCtMaxOdd = 15;

int grid_for(long long n) {
    long long g = (n + 255) / 256;
    return (int)(g < 152 * 16 ? (g < 1 ? 1 : g) : 152 * 16);
}

}  // namespace

int r2c_aligned(R2CEngine& e, const float* x, long long n, float2* out, cudaStream_t st);
static int r2c_tables(R2CEngine& e, const float2* z, long long K, float2* out, const Phase& ph, cudaStream_t st);

R2CEngine::~R2CEngine() {
    for (auto& kv : plans) cufftDestroy(kv.second);
}

// The forward/inverse C2C plan of P points (a power of two), made once.
static int c2c_plan(R2CEngine& e, long long P, cufftHandle* out) {
    auto it = e.plans.find(P);
    if (it != e.plans.end()) {
        *out = it->second;
        return 0;
    }
    cufftHandle h;
    if (cufftCreate(&h) != CUFFT_SUCCESS) return -1;
    long long n = P;
    size_t work = 0;
    if (cufftMakePlanMany64(h, 1, &n, nullptr, 1, P, nullptr, 1, P, CUFFT_C2C, 1, &work) != CUFFT_SUCCESS) {
        cufftDestroy(h);
        return -1;
    }
    e.plans[P] = h;
    *out = h;
    return 0;
}

int r2c_any(R2CEngine& e, const float* x, long long n, float2* out, cudaStream_t st) {
    if (n < 2 || (n & 1)) return -1;
    // the samples as complex pairs need an 8-byte aligned series: a caller's
    // device row at an odd float offset is copied first
    float* al = nullptr;
    if (reinterpret_cast<uintptr_t>(x) & 7) {
        if (cudaMallocAsync(&al, sizeof(float) * n, st) != cudaSuccess) return -2;
        if (cudaMemcpyAsync(al, x, sizeof(float) * n, cudaMemcpyDeviceToDevice, st) != cudaSuccess) {
            cudaFreeAsync(al, st);
            return -1;
        }
        x = al;
    }
    const int rc = r2c_aligned(e, x, n, out, st);
    if (al) cudaFreeAsync(al, st);
    return rc;
}

int r2c_aligned(R2CEngine& e, const float* x, long long n, float2* out, cudaStream_t st) {
    const long long K = n / 2;
    const float2* z = reinterpret_cast<const float2*>(x);
    // phase tables for multiples of pi/K
    int S = 1;
    while ((long long)S * S < 2 * K) S <<= 1;
    const int nq = (int)((2 * K + S - 1) / S);
    double2* tab = nullptr;
    if (cudaMallocAsync(&tab, (sizeof(double2) + sizeof(float2)) * (S + nq), st) != cudaSuccess) return -2;
    float2* ftab = reinterpret_cast<float2*>(tab + S + nq);
    k_phase_tables<<<(S + nq + 255) / 256, 256, 0, st>>>(tab, tab + S, ftab, ftab + S, K, S, nq);
    const Phase ph{tab, tab + S, ftab, ftab + S, (unsigned)S};
    const int rc = cudaGetLastError() != cudaSuccess ? -1 : r2c_tables(e, z, K, out, ph, st);
    cudaFreeAsync(tab, st);
    return rc;
}

int r2c_tables(R2CEngine& e, const float2* z, long long K, float2* out, const Phase& ph, cudaStream_t st) {
    if ((K & (K - 1)) == 0) {
        cufftHandle h;
        if (c2c_plan(e, K, &h) || cufftSetStream(h, st) != CUFFT_SUCCESS ||
            cufftExecC2C(h, reinterpret_cast<cufftComplex*>(const_cast<float2*>(z)),
                         reinterpret_cast<cufftComplex*>(out), CUFFT_FORWARD) != CUFFT_SUCCESS)
            return -1;
    } else if ((K >> __builtin_ctzll(K)) <= kCtMaxOdd) {
        const int m = (int)(K >> __builtin_ctzll(K));
        const long long L = K / m;
        cufftHandle h = 0;
        if (L > 1 && (c2c_plan(e, L, &h) || cufftSetStream(h, st) != CUFFT_SUCCESS)) return -1;
        float2* T = nullptr;
        if (cudaMallocAsync(&T, sizeof(float2) * K, st) != cudaSuccess) return -2;
        int rc = 0;
        k_ct_split<<<grid_for(K), 256, 0, st>>>(z, T, m, L);
        if (cudaGetLastError() != cudaSuccess) rc = -1;
        for (int j = 0; j < m && !rc && L > 1; j++)
            if (cufftExecC2C(h, reinterpret_cast<cufftComplex*>(T + (long long)j * L),
                             reinterpret_cast<cufftComplex*>(T + (long long)j * L), CUFFT_FORWARD) != CUFFT_SUCCESS)
                rc = -1;
        if (!rc) {
            k_ct_combine<<<grid_for(K), 256, 0, st>>>(T, out, m, L, ph);
            if (cudaGetLastError() != cudaSuccess) rc = -1;
        }
        cudaFreeAsync(T, st);
        if (rc) return rc;
    } else {
        long long P = 1;
        while (P < 2 * K - 1) P <<= 1;
        cufftHandle h;
        if (c2c_plan(e, P, &h) || cufftSetStream(h, st) != CUFFT_SUCCESS) return -1;
        float2 *a = nullptr, *b = nullptr;
        if (cudaMallocAsync(&a, sizeof(float2) * P, st) != cudaSuccess) return -2;
        if (cudaMallocAsync(&b, sizeof(float2) * P, st) != cudaSuccess) {
            cudaFreeAsync(a, st);
            return -2;
        }
        int rc = 0;
        k_chirp<<<grid_for(P), 256, 0, st>>>(z, a, b, K, P, ph);
        if (cudaGetLastError() != cudaSuccess) rc = -1;
        // the chirp's transform out of place: b keeps w for k_chirp_out
        float2* fb = nullptr;
        if (!rc && cudaMallocAsync(&fb, sizeof(float2) * P, st) != cudaSuccess) rc = -2;
        if (!rc && (cufftExecC2C(h, reinterpret_cast<cufftComplex*>(b), reinterpret_cast<cufftComplex*>(fb),
                                 CUFFT_FORWARD) != CUFFT_SUCCESS ||
                    cufftExecC2C(h, reinterpret_cast<cufftComplex*>(a), reinterpret_cast<cufftComplex*>(a),
                                 CUFFT_FORWARD) != CUFFT_SUCCESS))
            rc = -1;
        if (!rc) {
            k_pointwise<<<grid_for(P), 256, 0, st>>>(a, fb, P);
            if (cudaGetLastError() != cudaSuccess) rc = -1;
        }
        if (!rc && cufftExecC2C(h, reinterpret_cast<cufftComplex*>(a), reinterpret_cast<cufftComplex*>(a),
                                CUFFT_INVERSE) != CUFFT_SUCCESS)
            rc = -1;
        if (!rc) {
            k_chirp_out<<<grid_for(K), 256, 0, st>>>(a, b, out, K, (float)(1.0 / (double)P));
            if (cudaGetLastError() != cudaSuccess) rc = -1;
        }
        if (fb) cudaFreeAsync(fb, st);
        cudaFreeAsync(a, st);
        cudaFreeAsync(b, st);
        if (rc) return rc;
    }
    k_r2c_unpack<<<grid_for(K / 2 + 1), 256, 0, st>>>(out, K, ph);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace accel
