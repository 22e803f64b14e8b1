// fft_mixed.cuh -- complex FP32 FFTs of M = R * N2 points (R = 5, 6, 7; N2 a
// power of two, 64..512) in shared memory, for the short transforms of the
// plane kernels.  Decimation in time:
//
//   X[k2 + N2 k1] = sum_g W_R^(g k1) (W_M^(g k2) Y_g[k2]),
//   Y_g = the N2-point transform of x[R n + g], n < N2,
//
// so the R transforms Y_g run side by side on the radix-16 Stockham engine
// of fft_smem.cuh (N2/16 threads each, one barrier per pass for all of
// them), leave their outputs in shared memory, and a last radix-R pass
// combines them: one butterfly per k2, its R outputs in natural order
// (X[k2], X[k2 + N2], ...), so consecutive threads produce consecutive
// points of each of the R output blocks.  The inputs are taken in
// decimated order -- position g N2 + n holds point R n + g -- so that the
// N2/16 threads of a transform load consecutive addresses.
//
// The radix-R butterflies: R = 5 and 7 pair x_n with x_(R-n) (real cosine
// and sine weights, (R-1)/2 of each per output pair); R = 6 is two
// 3-point transforms and the 6th roots of unity.
#pragma once

#include "fft_smem.cuh"

namespace accel {

constexpr int cgcd(int a, int b) { return b == 0 ? a : cgcd(b, a % b); }

// cos(2 pi m / R), sin(2 pi m / R) for R = 5, 7 (m < R; constant after
// unrolling).
template <int R> __device__ __forceinline__ float root_cos(int m) {
    if constexpr (R == 5) {
        return m == 0 ? 1.f : (m == 1 || m == 4) ? 0.309016994374947424102f : -0.809016994374947424102f;
    } else {
        return m == 0 ? 1.f
             : (m == 1 || m == 6) ? 0.623489801858733530525f
             : (m == 2 || m == 5) ? -0.222520933956314404289f
                                  : -0.900968867902419126236f;
    }
}
template <int R> __device__ __forceinline__ float root_sin(int m) {
    if constexpr (R == 5) {
        return m == 0 ? 0.f : m == 1 ? 0.951056516295153572116f : m == 2 ? 0.587785252292473129169f
             : m == 3 ? -0.587785252292473129169f : -0.951056516295153572116f;
    } else {
        return m == 0 ? 0.f : m == 1 ? 0.781831482468029808708f : m == 2 ? 0.974927912181823607018f
             : m == 3 ? 0.433883739117558120476f : m == 4 ? -0.433883739117558120476f
             : m == 5 ? -0.974927912181823607018f : -0.781831482468029808708f;
    }
}

__device__ __forceinline__ float2 cscale(float s, float2 a) { return make_float2(s * a.x, s * a.y); }

// X_k = sum_n v_n exp(DIR 2 pi i n k / R), in place, R odd (5 or 7):
// with s_n = v_n + v_(R-n), d_n = v_n - v_(R-n),
// X_k, X_(R-k) = v_0 + sum_n s_n cos(2 pi n k / R) +- DIR i sum_n d_n sin(2 pi n k / R).
template <int R, int DIR> __device__ __forceinline__ void dft_odd(float2* v) {
    constexpr int H = (R - 1) / 2;
    float2 s[H + 1], d[H + 1];
    float2 x0 = v[0], sum = v[0];
#pragma unroll
    for (int n = 1; n <= H; n++) {
        s[n] = cadd(v[n], v[R - n]);
        d[n] = csub(v[n], v[R - n]);
        sum = cadd(sum, s[n]);
    }
#pragma unroll
    for (int k = 1; k <= H; k++) {
        float2 a = x0, b = cscale(root_sin<R>(k % R), d[1]);
        a = cfma(root_cos<R>(k % R), s[1], a);
#pragma unroll
        for (int n = 2; n <= H; n++) {
            a = cfma(root_cos<R>((n * k) % R), s[n], a);
            b = cfma(root_sin<R>((n * k) % R), d[n], b);
        }
        const float2 ib = mul_i<DIR>(b);
        v[k] = cadd(a, ib);
        v[R - k] = csub(a, ib);
    }
    v[0] = sum;
}

// 3 points: X_1, X_2 = v_0 - s/2 +- DIR i (sqrt3/2) d, s = v_1 + v_2, d = v_1 - v_2.
template <int DIR> __device__ __forceinline__ void dft3(float2* v) {
    const float S3 = 0.866025403784438646764f;
    const float2 s = cadd(v[1], v[2]), d = csub(v[1], v[2]);
    const float2 t = cfma(-0.5f, s, v[0]);
    const float2 w = cscale(S3, mul_i<DIR>(d));
    v[0] = cadd(v[0], s);
    v[1] = cadd(t, w);
    v[2] = csub(t, w);
}

// 6 points as 3-point transforms of the even (E) and odd (O) points:
// X_k = E_k + w^k O_k, X_(k+3) = E_k - w^k O_k (k < 3), w = exp(DIR 2 pi i / 6)
// = 1/2 + DIR i sqrt3/2, w^2 = -1/2 + DIR i sqrt3/2.
template <int DIR> __device__ __forceinline__ void dft6(float2* v) {
    const float S3 = 0.866025403784438646764f;
    float2 e[3] = {v[0], v[2], v[4]};
    float2 o[3] = {v[1], v[3], v[5]};
    dft3<DIR>(e);
    dft3<DIR>(o);
    const float2 t1 = cfma(S3, mul_i<DIR>(o[1]), cscale(0.5f, o[1]));
    const float2 t2 = cfma(S3, mul_i<DIR>(o[2]), cscale(-0.5f, o[2]));
    v[0] = cadd(e[0], o[0]), v[3] = csub(e[0], o[0]);
    v[1] = cadd(e[1], t1), v[4] = csub(e[1], t1);
    v[2] = cadd(e[2], t2), v[5] = csub(e[2], t2);
}

template <int R, int DIR> __device__ __forceinline__ void dft_radix(float2* v) {
    static_assert(R == 5 || R == 6 || R == 7, "radix of the last pass");
    if constexpr (R == 6) dft6<DIR>(v);
    else dft_odd<R, DIR>(v);
}

// Thread layout of a short transform.  UNIT threads carry one transform
// (R groups of N2/16, 16 points each); CTAs of the plane kernel hold U
// transforms of different rows so that they are whole warps.  For R = 7
// one more warp joins the radix-7 pass only: the U N2 butterflies then
// divide evenly among the threads (2 each) instead of leaving a third
// round to two of seven warps.
template <int R, int N2> struct MixedShape {
    static_assert(R >= 5 && R <= 7 && N2 >= kMixedMinN2 && N2 <= kMixedMaxN2 && (N2 & (N2 - 1)) == 0,
                  "short transform shape");
    static constexpr int M = R * N2;
    static constexpr int T2 = N2 / 16;                  // threads per N2-point transform
    static constexpr int UNIT = R * T2;                 // threads per M-point transform
    static constexpr int U = 32 / cgcd(UNIT, 32);       // transforms per plane CTA
    static constexpr int FFT_THREADS = U * UNIT;        // a multiple of 32
    static constexpr int EXTRA = R == 7 ? 32 : 0;       // threads of the last pass only
    static constexpr int THREADS = FFT_THREADS + EXTRA;
    static_assert(EXTRA == 0 || (U * N2) % THREADS == 0, "the last pass divides evenly");
    static constexpr int PM2 = FftShape<N2>::PADDED;    // one padded N2-point buffer
    // float2 from one group's pair of buffers to the next: with fewer than 16
    // threads per group, the groups sharing a half-warp start T2 float2
    // apart modulo 16 (different banks)
    static constexpr int GS = 2 * PM2 + (T2 >= 16 ? 0 : (T2 - (2 * PM2) % 16 + 16) % 16);
    static constexpr int MINB = THREADS >= 512 ? 1 : 512 / THREADS;  // >= 16 warps per SM
};

// Twiddle W_M^(g k2) of the radix-R pass (exp(DIR 2 pi i g k2 / M)), g >= 1.
template <int R, int N2, int DIR>
__device__ __forceinline__ float2 mixed_twiddle(const float2* __restrict__ tw, int g, int k2) {
    return twid<DIR>(tw + tw_form_off(R, N2), (g - 1) * N2 + k2);
}

// The radix-R pass of butterfly b (0 <= b < N2) over NB transforms whose
// N2-point outputs Y_g lie in shared memory at buf + g GS + nb PM2 (padded
// index): leaves X[b + N2 k1] in v[nb][k1].
template <int R, int N2, int DIR, int NB, int GS>
__device__ __forceinline__ void mixed_last_pass(float2 (&v)[NB][R], const float2* buf,
                                                const float2* __restrict__ tw, int b) {
    constexpr int PM2 = FftShape<N2>::PADDED;
    const float2* p = buf + fft_pad(b);
#pragma unroll
    for (int g = 0; g < R; g++)
#pragma unroll
        for (int nb = 0; nb < NB; nb++) v[nb][g] = p[g * GS + nb * PM2];
#pragma unroll
    for (int g = 1; g < R; g++) {
        const float2 w = mixed_twiddle<R, N2, DIR>(tw, g, b);
#pragma unroll
        for (int nb = 0; nb < NB; nb++) v[nb][g] = cmul(v[nb][g], w);
    }
#pragma unroll
    for (int nb = 0; nb < NB; nb++) dft_radix<R, DIR>(v[nb]);
}

}  // namespace accel
