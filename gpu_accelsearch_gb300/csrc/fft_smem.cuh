// fft_smem.cuh -- complex FP32 FFT of M = 2^k points (64 <= M <= 8192) in
// shared memory, Stockham auto-sort, radix-16 passes plus one radix-2/4/8
// pass.  T = M/16 threads each hold 16 points in registers; register e of
// thread t is point t + e*T both on entry (time order) and on exit
// (frequency order), so loads from and stores to global memory coalesce.
// Between passes the points go through shared memory (one element of
// padding every 16 keeps the stride-16 stores free of bank conflicts).
//
// NB independent transforms of the same length are done side by side by
// the same threads (one barrier per pass for all of them).
//
// Twiddles come from a table tw[m] = exp(+2 pi i m / kTwN) in global
// memory (computed once from double precision); the forward direction uses
// its conjugate.
#pragma once

#include "accel_common.cuh"

namespace accel {

__device__ __forceinline__ int fft_pad(int i) { return i + (i >> 4); }
template <int M> struct FftShape {
    static constexpr int T = M / 16;
    static constexpr int PADDED = M + M / 16;
};

// x * (DIR * i)
template <int DIR> __device__ __forceinline__ float2 mul_i(float2 a) {
    return DIR > 0 ? make_float2(-a.y, a.x) : make_float2(a.y, -a.x);
}

template <int DIR> __device__ __forceinline__ void dft2(float2* v) {
    float2 a = v[0], b = v[1];
    v[0] = cadd(a, b);
    v[1] = csub(a, b);
}

template <int DIR> __device__ __forceinline__ void dft4(float2* v) {
    float2 s02 = cadd(v[0], v[2]), d02 = csub(v[0], v[2]);
    float2 s13 = cadd(v[1], v[3]), d13 = mul_i<DIR>(csub(v[1], v[3]));
    v[0] = cadd(s02, s13);
    v[2] = csub(s02, s13);
    v[1] = cadd(d02, d13);
    v[3] = csub(d02, d13);
}

// W8^k for direction DIR, k = 1,3 (k=2 is DIR*i)
template <int DIR> __device__ __forceinline__ float2 w8_1(float2 a) {
    const float s = 0.70710678118654752440f;  // (1 + DIR i)/sqrt2
    return DIR > 0 ? make_float2(s * (a.x - a.y), s * (a.x + a.y))
                   : make_float2(s * (a.x + a.y), s * (a.y - a.x));
}
template <int DIR> __device__ __forceinline__ float2 w8_3(float2 a) {
    const float s = 0.70710678118654752440f;  // (-1 + DIR i)/sqrt2
    return DIR > 0 ? make_float2(-s * (a.x + a.y), s * (a.x - a.y))
                   : make_float2(s * (a.y - a.x), -s * (a.x + a.y));
}

template <int DIR> __device__ __forceinline__ void dft8(float2* v) {
    float2 e[4] = {v[0], v[2], v[4], v[6]};
    float2 o[4] = {v[1], v[3], v[5], v[7]};
    dft4<DIR>(e);
    dft4<DIR>(o);
    o[1] = w8_1<DIR>(o[1]);
    o[2] = mul_i<DIR>(o[2]);
    o[3] = w8_3<DIR>(o[3]);
#pragma unroll
    for (int k = 0; k < 4; k++) {
        v[k] = cadd(e[k], o[k]);
        v[k + 4] = csub(e[k], o[k]);
    }
}

template <int DIR> __device__ __forceinline__ void dft16(float2* v) {
    float2 e[8], o[8];
#pragma unroll
    for (int k = 0; k < 8; k++) { e[k] = v[2 * k]; o[k] = v[2 * k + 1]; }
    dft8<DIR>(e);
    dft8<DIR>(o);
    const float c1 = 0.92387953251128675613f, s1 = 0.38268343236508977173f;
    const float c2 = 0.70710678118654752440f;
    // W16^k = cos(2 pi k/16) + DIR i sin(2 pi k/16)
    const float wr[8] = {1.f, c1, c2, s1, 0.f, -s1, -c2, -c1};
    const float wi[8] = {0.f, s1, c2, c1, 1.f, c1, c2, s1};
#pragma unroll
    for (int k = 1; k < 8; k++) {
        float2 w = make_float2(wr[k], DIR * wi[k]);
        o[k] = cmul(o[k], w);
    }
#pragma unroll
    for (int k = 0; k < 8; k++) {
        v[k] = cadd(e[k], o[k]);
        v[k + 8] = csub(e[k], o[k]);
    }
}

template <int R, int DIR> __device__ __forceinline__ void dft(float2* v) {
    if constexpr (R == 2) dft2<DIR>(v);
    else if constexpr (R == 4) dft4<DIR>(v);
    else if constexpr (R == 8) dft8<DIR>(v);
    else dft16<DIR>(v);
}

template <int DIR> __device__ __forceinline__ float2 twid(const float2* __restrict__ tw, int idx) {
    float2 w = __ldg(tw + idx);
    return DIR > 0 ? w : make_float2(w.x, -w.y);
}

// v[r] *= W^{r k} with W = exp(DIR 2 pi i / NR).  Table lookups for
// r = 1,2,4,8; the rest are at most two products away.
template <int R, int DIR>
__device__ __forceinline__ void apply_twiddles(float2* v, const float2* __restrict__ tw, int k, int NR) {
    const int step = kTwN / NR;
    const int base = k * step;
    float2 w1 = twid<DIR>(tw, base);
    v[1] = cmul(v[1], w1);
    if constexpr (R >= 4) {
        float2 w2 = twid<DIR>(tw, 2 * base);
        float2 w3 = cmul(w2, w1);
        v[2] = cmul(v[2], w2);
        v[3] = cmul(v[3], w3);
        if constexpr (R >= 8) {
            float2 w4 = twid<DIR>(tw, 4 * base);
            v[4] = cmul(v[4], w4);
            v[5] = cmul(v[5], cmul(w4, w1));
            v[6] = cmul(v[6], cmul(w4, w2));
            v[7] = cmul(v[7], cmul(w4, w3));
            if constexpr (R >= 16) {
                float2 w8 = twid<DIR>(tw, 8 * base);
                v[8] = cmul(v[8], w8);
                v[9] = cmul(v[9], cmul(w8, w1));
                v[10] = cmul(v[10], cmul(w8, w2));
                v[11] = cmul(v[11], cmul(w8, w3));
                float2 w12 = cmul(w8, w4);
                v[12] = cmul(v[12], w12);
                v[13] = cmul(v[13], cmul(w12, w1));
                v[14] = cmul(v[14], cmul(w12, w2));
                v[15] = cmul(v[15], cmul(w12, w3));
            }
        }
    }
}

// Base twiddles W^k, W^2k, W^4k, W^8k of one radix-16 pass, loaded ahead of
// time so that the table lookups are off the pass's critical path.
struct Tw16 {
    float2 w1, w2, w4, w8;
};
template <int DIR>
__device__ __forceinline__ Tw16 load_tw16(const float2* __restrict__ tw, int k, int NR) {
    const int base = k * (kTwN / NR);
    Tw16 r;
    r.w1 = twid<DIR>(tw, base);
    r.w2 = twid<DIR>(tw, 2 * base);
    r.w4 = twid<DIR>(tw, 4 * base);
    r.w8 = twid<DIR>(tw, 8 * base);
    return r;
}
__device__ __forceinline__ void apply_tw16(float2* v, const Tw16& p) {
    const float2 w3 = cmul(p.w2, p.w1);
    v[1] = cmul(v[1], p.w1);
    v[2] = cmul(v[2], p.w2);
    v[3] = cmul(v[3], w3);
    v[4] = cmul(v[4], p.w4);
    v[5] = cmul(v[5], cmul(p.w4, p.w1));
    v[6] = cmul(v[6], cmul(p.w4, p.w2));
    v[7] = cmul(v[7], cmul(p.w4, w3));
    v[8] = cmul(v[8], p.w8);
    v[9] = cmul(v[9], cmul(p.w8, p.w1));
    v[10] = cmul(v[10], cmul(p.w8, p.w2));
    v[11] = cmul(v[11], cmul(p.w8, w3));
    const float2 w12 = cmul(p.w8, p.w4);
    v[12] = cmul(v[12], w12);
    v[13] = cmul(v[13], cmul(w12, p.w1));
    v[14] = cmul(v[14], cmul(w12, p.w2));
    v[15] = cmul(v[15], cmul(w12, w3));
}

// One Stockham pass of radix R over NB transforms.  FIRST: input already in
// registers (time order).  LAST: output left in registers (frequency order).
// PRE: twiddles of a radix-16 pass supplied by the caller (Q == 1).
template <int M, int R, int NS, bool FIRST, bool LAST, int DIR, int NB>
__device__ __forceinline__ void fft_pass(float2 (&a)[NB][16], float2* sm,
                                         const float2* __restrict__ tw, int t,
                                         const Tw16* pre = nullptr) {
    constexpr int T = M / 16;
    constexpr int Q = 16 / R;
    constexpr int PM = FftShape<M>::PADDED;
    if constexpr (!FIRST) {
#pragma unroll
        for (int nb = 0; nb < NB; nb++)
#pragma unroll
            for (int q = 0; q < Q; q++)
#pragma unroll
                for (int r = 0; r < R; r++)
                    a[nb][q + r * Q] = sm[nb * PM + fft_pad(t + q * T + r * (M / R))];
        __syncthreads();
    }
#pragma unroll
    for (int q = 0; q < Q; q++) {
        const int b = t + q * T;
        const int k = b & (NS - 1);
#pragma unroll
        for (int nb = 0; nb < NB; nb++) {
            float2 v[R];
#pragma unroll
            for (int r = 0; r < R; r++) v[r] = a[nb][q + r * Q];
            if constexpr (NS > 1) {
                if constexpr (R == 16) {
                    if (pre) apply_tw16(v, *pre);
                    else apply_twiddles<R, DIR>(v, tw, k, NS * R);
                } else {
                    apply_twiddles<R, DIR>(v, tw, k, NS * R);
                }
            }
            dft<R, DIR>(v);
            if constexpr (LAST) {
#pragma unroll
                for (int r = 0; r < R; r++) a[nb][q + r * Q] = v[r];
            } else {
                const int j = (b / NS) * (NS * R) + k;
#pragma unroll
                for (int r = 0; r < R; r++) sm[nb * PM + fft_pad(j + r * NS)] = v[r];
            }
        }
    }
    if constexpr (!LAST) __syncthreads();
}

// Full transform: radix-16 passes, the leftover factor (2, 4 or 8) last.
// t is the thread's index within the group of M/16 threads doing the
// transform(s); sm must hold NB * FftShape<M>::PADDED float2.  The
// twiddles of the radix-16 passes after the first are loaded up front.
// Shared memory may be rewritten as soon as this returns.
template <int M, int DIR, int NB>
__device__ __forceinline__ void fft_run(float2 (&a)[NB][16], float2* sm, const float2* __restrict__ tw,
                                        int t) {
    static_assert(M >= kMinM && M <= kMaxM && (M & (M - 1)) == 0, "M must be a power of two");
    if constexpr (M == 64) {
        fft_pass<M, 16, 1, true, false, DIR, NB>(a, sm, tw, t);
        fft_pass<M, 4, 16, false, true, DIR, NB>(a, sm, tw, t);
    } else if constexpr (M == 128) {
        fft_pass<M, 16, 1, true, false, DIR, NB>(a, sm, tw, t);
        fft_pass<M, 8, 16, false, true, DIR, NB>(a, sm, tw, t);
    } else if constexpr (M == 256) {
        const Tw16 p1 = load_tw16<DIR>(tw, t & 15, 256);
        fft_pass<M, 16, 1, true, false, DIR, NB>(a, sm, tw, t);
        fft_pass<M, 16, 16, false, true, DIR, NB>(a, sm, tw, t, &p1);
    } else if constexpr (M == 512 || M == 1024 || M == 2048) {
        constexpr int RL = M / 256;
        const Tw16 p1 = load_tw16<DIR>(tw, t & 15, 256);
        fft_pass<M, 16, 1, true, false, DIR, NB>(a, sm, tw, t);
        fft_pass<M, 16, 16, false, false, DIR, NB>(a, sm, tw, t, &p1);
        fft_pass<M, RL, 256, false, true, DIR, NB>(a, sm, tw, t);
    } else if constexpr (M == 4096) {
        const Tw16 p1 = load_tw16<DIR>(tw, t & 15, 256);
        const Tw16 p2 = load_tw16<DIR>(tw, t & 255, 4096);
        fft_pass<M, 16, 1, true, false, DIR, NB>(a, sm, tw, t);
        fft_pass<M, 16, 16, false, false, DIR, NB>(a, sm, tw, t, &p1);
        fft_pass<M, 16, 256, false, true, DIR, NB>(a, sm, tw, t, &p2);
    } else {  // 8192
        const Tw16 p1 = load_tw16<DIR>(tw, t & 15, 256);
        const Tw16 p2 = load_tw16<DIR>(tw, t & 255, 4096);
        fft_pass<M, 16, 1, true, false, DIR, NB>(a, sm, tw, t);
        fft_pass<M, 16, 16, false, false, DIR, NB>(a, sm, tw, t, &p1);
        fft_pass<M, 16, 256, false, false, DIR, NB>(a, sm, tw, t, &p2);
        fft_pass<M, 2, 4096, false, true, DIR, NB>(a, sm, tw, t);
    }
}

}  // namespace accel
