// fft_smem.cuh -- complex FP32 FFT of M = 2^k points (64 <= M <= 8192) in
// shared memory, Stockham auto-sort, radix-16 passes plus one radix-2/4/8
// pass.  T = M/16 threads each hold 16 points in registers; register e of
// thread t is point t + e*T both on entry (time order) and on exit
// (frequency order), so loads from and stores to global memory coalesce.
// Between passes the points go through shared memory (one element of
// padding every 16 keeps the stride-16 stores free of bank conflicts; the
// padding of every offset that is a multiple of 16 is a constant, so each
// access costs one base index per pass and an immediate offset).
//
// NB independent transforms of the same length are done side by side by
// the same threads (one barrier per pass for all of them), each through its
// own padded buffer: a transform's butterflies run while the other's
// shared-memory stores and loads are still in flight.
//
// Twiddles come from a table tw[m] = exp(+2 pi i m / kTwN) in global
// memory (computed once from double precision); the forward direction uses
// its conjugate.
#pragma once

#include "accel_common.cuh"

namespace accel {

__device__ __forceinline__ int fft_pad(int i) { return i + (i >> 4); }

// Barrier between passes: the whole CTA (the default), or a named barrier
// over the group of threads doing one transform (several transforms of a
// smaller size side by side in one CTA, each group on its own barrier).
struct CtaSync {
    __device__ __forceinline__ void operator()() const { __syncthreads(); }
};
struct GroupSync {
    int id, nthreads;  // barrier 1..15, a multiple of 32 threads
    __device__ __forceinline__ void operator()() const {
        asm volatile("bar.sync %0, %1;\n" ::"r"(id), "r"(nthreads) : "memory");
    }
};
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

__device__ __forceinline__ float2 cfma(float s, float2 a, float2 b) {  // s a + b
    return make_float2(fmaf(s, a.x, b.x), fmaf(s, a.y, b.y));
}


// 8 points as 2 x 4; the twiddles W8^1 = s (1 + i'), W8^3 = s (-1 + i')
// (i' = DIR i, s = 1/sqrt2) applied by the fused multiply-adds of the last
// layer: 52 floating-point instructions instead of 56.
template <int DIR> __device__ __forceinline__ void dft8(float2* v) {
    const float S = 0.70710678118654752440f;
    float2 e[4] = {v[0], v[2], v[4], v[6]};
    float2 o[4] = {v[1], v[3], v[5], v[7]};
    dft4<DIR>(e);
    dft4<DIR>(o);
    const float2 p1 = cadd(o[1], mul_i<DIR>(o[1])), p3 = csub(mul_i<DIR>(o[3]), o[3]);
    const float2 o2 = mul_i<DIR>(o[2]);
    v[0] = cadd(e[0], o[0]), v[4] = csub(e[0], o[0]);
    v[1] = cfma(S, p1, e[1]), v[5] = cfma(-S, p1, e[1]);
    v[2] = cadd(e[2], o2), v[6] = csub(e[2], o2);
    v[3] = cfma(S, p3, e[3]), v[7] = cfma(-S, p3, e[3]);
}

// 16 points as 4 x 4: x[4 n1 + n2] -> X[k1 + 4 k2].  DFT4 over n1 for each
// n2, twiddles W16^(n2 k1), DFT4 over n2 for each k1.  Each nontrivial
// twiddle is written as a real scale times a factor with a unit component
// -- W^2 = s (1 + i'), W^6 = s (-1 + i'), W^1 = c (1 + t i'), W^3 =
// c (t + i'), W^9 = -c (1 + t i') with i' = DIR i, s = 1/sqrt2,
// c = cos(pi/8), t = tan(pi/8) -- and the scale is applied by the fused
// multiply-adds of the second DFT4 layer, whose two inputs of a pair carry
// the same scale: 144 floating-point instructions per 16 points instead of
// 160 with the twiddles multiplied out.
template <int DIR> __device__ __forceinline__ void dft16(float2* v) {
    const float C = 0.92387953251128675613f, S = 0.70710678118654752440f, TN = 0.41421356237309504880f;
    float2 y[4][4];  // y[n2][k1]
#pragma unroll
    for (int n2 = 0; n2 < 4; n2++) {
        float2 u[4] = {v[n2], v[n2 + 4], v[n2 + 8], v[n2 + 12]};
        dft4<DIR>(u);
#pragma unroll
        for (int k1 = 0; k1 < 4; k1++) y[n2][k1] = u[k1];
    }
    {  // k1 = 0: no twiddles
        float2 u[4] = {y[0][0], y[1][0], y[2][0], y[3][0]};
        dft4<DIR>(u);
        v[0] = u[0], v[4] = u[1], v[8] = u[2], v[12] = u[3];
    }
    {  // k1 = 1: W^1 = c (1 + t i'), W^2 = s (1 + i'), W^3 = c (t + i')
        const float2 p2 = cadd(y[2][1], mul_i<DIR>(y[2][1]));
        const float2 s02 = cfma(S, p2, y[0][1]), d02 = cfma(-S, p2, y[0][1]);
        const float2 i1 = mul_i<DIR>(y[1][1]), i3 = mul_i<DIR>(y[3][1]);
        const float2 a1 = cfma(TN, i1, y[1][1]), a3 = cfma(TN, y[3][1], i3);
        const float2 s13 = cadd(a1, a3), d13 = mul_i<DIR>(csub(a1, a3));
        v[1] = cfma(C, s13, s02), v[9] = cfma(-C, s13, s02);
        v[5] = cfma(C, d13, d02), v[13] = cfma(-C, d13, d02);
    }
    {  // k1 = 2: W^2 = s (1 + i'), W^4 = i', W^6 = s (-1 + i')
        const float2 i2 = mul_i<DIR>(y[2][2]);
        const float2 s02 = cadd(y[0][2], i2), d02 = csub(y[0][2], i2);
        const float2 a = csub(y[1][2], y[3][2]), ib = mul_i<DIR>(cadd(y[1][2], y[3][2]));
        const float2 s13 = cadd(a, ib), d13 = csub(ib, a);
        v[2] = cfma(S, s13, s02), v[10] = cfma(-S, s13, s02);
        v[6] = cfma(S, d13, d02), v[14] = cfma(-S, d13, d02);
    }
    {  // k1 = 3: W^3 = c (t + i'), W^6 = s (-1 + i'), W^9 = -c (1 + t i')
        const float2 p2 = csub(mul_i<DIR>(y[2][3]), y[2][3]);
        const float2 s02 = cfma(S, p2, y[0][3]), d02 = cfma(-S, p2, y[0][3]);
        const float2 i1 = mul_i<DIR>(y[1][3]), i3 = mul_i<DIR>(y[3][3]);
        const float2 a1 = cfma(TN, y[1][3], i1), a3 = cfma(TN, i3, y[3][3]);
        const float2 s13 = csub(a1, a3), d13 = mul_i<DIR>(cadd(a1, a3));
        v[3] = cfma(C, s13, s02), v[11] = cfma(-C, s13, s02);
        v[7] = cfma(C, d13, d02), v[15] = cfma(-C, d13, d02);
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

// The base twiddles W^k, W^2k, W^4k, W^8k (W = exp(DIR 2 pi i / NR)) of
// pass index k: from the packed section of NR (two 16-byte loads of
// consecutive memory) or, for NR = kTwN, from the table itself.
struct Tw16 {
    float2 w1, w2, w4, w8;
};
template <int DIR>
__device__ __forceinline__ Tw16 load_tw16(const float2* __restrict__ tw, int k, int NR) {
    Tw16 r;
    if (NR == kTwN) {
        r.w1 = twid<DIR>(tw, k);
        r.w2 = twid<DIR>(tw, (2 * k) & (kTwN - 1));
        r.w4 = twid<DIR>(tw, (4 * k) & (kTwN - 1));
        r.w8 = twid<DIR>(tw, (8 * k) & (kTwN - 1));
        return r;
    }
    const float4* p = reinterpret_cast<const float4*>(tw + kTwN + tw_pack_off(NR)) + 2 * k;
    const float4 a = __ldg(p), b = __ldg(p + 1);
    const float sg = DIR > 0 ? 1.f : -1.f;
    r.w1 = make_float2(a.x, sg * a.y);
    r.w2 = make_float2(a.z, sg * a.w);
    r.w4 = make_float2(b.x, sg * b.y);
    r.w8 = make_float2(b.z, sg * b.w);
    return r;
}

// v[nb][r] *= W^{r k} with W = exp(DIR 2 pi i / NR), for every transform nb.
// Base powers from load_tw16; the rest are one product away.
template <int R, int DIR, int NB>
__device__ __forceinline__ void apply_twiddles(float2 (&v)[NB][R], const float2* __restrict__ tw, int k,
                                               int NR) {
    static_assert(R <= 8, "radix-16 passes use apply_tw16");
    const Tw16 b = load_tw16<DIR>(tw, k, NR);
    float2 w[R];
    w[1] = b.w1;
    if constexpr (R >= 4) {
        w[2] = b.w2;
        w[3] = cmul(w[2], w[1]);
        if constexpr (R >= 8) {
            w[4] = b.w4;
            w[5] = cmul(w[4], w[1]);
            w[6] = cmul(w[4], w[2]);
            w[7] = cmul(w[4], w[3]);
        }
    }
#pragma unroll
    for (int nb = 0; nb < NB; nb++)
#pragma unroll
        for (int r = 1; r < R; r++) v[nb][r] = cmul(v[nb][r], w[r]);
}

// v[nb][r] *= W^{rk} for the radix-16 pass with NR = 256, every power from
// its own table entry (no products).
template <int DIR, int NB>
__device__ __forceinline__ void apply_tw16_full256(float2 (&v)[NB][16], const float2* __restrict__ tw, int k) {
    const float2* f = tw + kTwN + kTwFull256 + k;
#pragma unroll
    for (int r = 1; r < 16; r++) {
        const float2 w = twid<DIR>(f, (r - 1) * 16);
#pragma unroll
        for (int nb = 0; nb < NB; nb++) v[nb][r] = cmul(v[nb][r], w);
    }
}

template <int NB>
__device__ __forceinline__ void apply_tw16(float2 (&v)[NB][16], const Tw16& p) {
    float2 w[16];
    w[1] = p.w1;
    w[2] = p.w2;
    w[3] = cmul(p.w2, p.w1);
    w[4] = p.w4;
    w[5] = cmul(p.w4, p.w1);
    w[6] = cmul(p.w4, p.w2);
    w[7] = cmul(p.w4, w[3]);
    w[8] = p.w8;
    w[9] = cmul(p.w8, p.w1);
    w[10] = cmul(p.w8, p.w2);
    w[11] = cmul(p.w8, w[3]);
    w[12] = cmul(p.w8, p.w4);
    w[13] = cmul(w[12], p.w1);
    w[14] = cmul(w[12], p.w2);
    w[15] = cmul(w[12], w[3]);
#pragma unroll
    for (int nb = 0; nb < NB; nb++)
#pragma unroll
        for (int r = 1; r < 16; r++) v[nb][r] = cmul(v[nb][r], w[r]);
}

// Padded shared-memory index of point t + q T + r M/R, the point a pass
// loads into its register q + r Q: for M >= 256 the offset is a multiple of
// 16, so its padding is a constant.
template <int M, int R>
__device__ __forceinline__ int fft_load_index(int tp, int t, int q, int r) {
    constexpr int T = M / 16;
    const int o = q * T + r * (M / R);
    if constexpr (T % 16 == 0 && (M / R) % 16 == 0) return tp + o + (o >> 4);
    else return fft_pad(t + o);
}

// One Stockham pass of radix R over NB transforms.  FIRST: input already in
// registers (time order).  LAST: output left in registers (frequency order).
// PRE: twiddles of a radix-16 pass supplied by the caller (Q == 1).
template <int M, int R, int NS, bool FIRST, bool LAST, int DIR, int NB, class Sync = CtaSync>
__device__ __forceinline__ void fft_pass(float2 (&a)[NB][16], float2* sm,
                                         const float2* __restrict__ tw, int t,
                                         const Tw16* pre = nullptr, Sync sync = Sync()) {
    constexpr int T = M / 16;
    constexpr int Q = 16 / R;
    constexpr int PM = FftShape<M>::PADDED;
    // the stores of a pass go to j + r NS with j a multiple of 16 (first
    // pass) or NS a multiple of 16: constant padding again
    static_assert(LAST || (NS == 1 && R == 16) || NS % 16 == 0, "store offsets must pad by a constant");
    if constexpr (!FIRST) {
        const int tp = fft_pad(t);
#pragma unroll
        for (int nb = 0; nb < NB; nb++)
#pragma unroll
            for (int q = 0; q < Q; q++)
#pragma unroll
                for (int r = 0; r < R; r++) a[nb][q + r * Q] = sm[nb * PM + fft_load_index<M, R>(tp, t, q, r)];
        sync();
    }
#pragma unroll
    for (int q = 0; q < Q; q++) {
        const int b = t + q * T;
        const int k = b & (NS - 1);
        float2 v[NB][R];
#pragma unroll
        for (int nb = 0; nb < NB; nb++)
#pragma unroll
            for (int r = 0; r < R; r++) v[nb][r] = a[nb][q + r * Q];
        if constexpr (NS > 1) {
            // each twiddle is formed once and applied to every transform
            if constexpr (R == 16 && NS == 16) {
                apply_tw16_full256<DIR, NB>(v, tw, k);
            } else if constexpr (R == 16) {
                if (pre) apply_tw16<NB>(v, *pre);
                else apply_tw16<NB>(v, load_tw16<DIR>(tw, k, NS * R));
            } else {
                apply_twiddles<R, DIR, NB>(v, tw, k, NS * R);
            }
        }
        const int jp = fft_pad((b / NS) * (NS * R) + k);
#pragma unroll
        for (int nb = 0; nb < NB; nb++) {
            dft<R, DIR>(v[nb]);
#pragma unroll
            for (int r = 0; r < R; r++) {
                if constexpr (LAST) a[nb][q + r * Q] = v[nb][r];
                else sm[nb * PM + jp + r * NS + ((r * NS) >> 4)] = v[nb][r];
            }
        }
    }
    if constexpr (!LAST) sync();
}

// Full transform: radix-16 passes, the leftover factor (2, 4 or 8) last.
// t is the thread's index within the group of M/16 threads doing the
// transform(s); sm (16-byte aligned) must hold NB * FftShape<M>::PADDED
// float2, one padded buffer per transform.  The twiddles of the radix-16 passes after the
// first are loaded up front.  Shared memory may be rewritten as soon as
// this returns.
template <int M, int DIR, int NB, class Sync = CtaSync>
__device__ __forceinline__ void fft_run(float2 (&a)[NB][16], float2* sm, const float2* __restrict__ tw,
                                        int t, Sync sync = Sync()) {
    static_assert(M >= kMinM && M <= kMaxM && (M & (M - 1)) == 0, "M must be a power of two");
    if constexpr (M == 64) {
        fft_pass<M, 16, 1, true, false, DIR, NB, Sync>(a, sm, tw, t, nullptr, sync);
        fft_pass<M, 4, 16, false, true, DIR, NB, Sync>(a, sm, tw, t, nullptr, sync);
    } else if constexpr (M == 128) {
        fft_pass<M, 16, 1, true, false, DIR, NB, Sync>(a, sm, tw, t, nullptr, sync);
        fft_pass<M, 8, 16, false, true, DIR, NB, Sync>(a, sm, tw, t, nullptr, sync);
    } else if constexpr (M == 256) {
        fft_pass<M, 16, 1, true, false, DIR, NB, Sync>(a, sm, tw, t, nullptr, sync);
        fft_pass<M, 16, 16, false, true, DIR, NB, Sync>(a, sm, tw, t, nullptr, sync);
    } else if constexpr (M == 512 || M == 1024 || M == 2048) {
        constexpr int RL = M / 256;
        fft_pass<M, 16, 1, true, false, DIR, NB, Sync>(a, sm, tw, t, nullptr, sync);
        fft_pass<M, 16, 16, false, false, DIR, NB, Sync>(a, sm, tw, t, nullptr, sync);
        fft_pass<M, RL, 256, false, true, DIR, NB, Sync>(a, sm, tw, t, nullptr, sync);
    } else if constexpr (M == 4096) {
        const Tw16 p2 = load_tw16<DIR>(tw, t & 255, 4096);
        fft_pass<M, 16, 1, true, false, DIR, NB, Sync>(a, sm, tw, t, nullptr, sync);
        fft_pass<M, 16, 16, false, false, DIR, NB, Sync>(a, sm, tw, t, nullptr, sync);
        fft_pass<M, 16, 256, false, true, DIR, NB, Sync>(a, sm, tw, t, &p2, sync);
    } else {  // 8192
        const Tw16 p2 = load_tw16<DIR>(tw, t & 255, 4096);
        fft_pass<M, 16, 1, true, false, DIR, NB, Sync>(a, sm, tw, t, nullptr, sync);
        fft_pass<M, 16, 16, false, false, DIR, NB, Sync>(a, sm, tw, t, nullptr, sync);
        fft_pass<M, 16, 256, false, false, DIR, NB, Sync>(a, sm, tw, t, &p2, sync);
        fft_pass<M, 2, 4096, false, true, DIR, NB, Sync>(a, sm, tw, t, nullptr, sync);
    }
}

}  // namespace accel
