// search_mixed_prep.cu -- segment preparation of the short transforms: one
// kernel for every short harmonic of a launch group (mixed_kernels.cuh).
#include "mixed_kernels.cuh"

namespace accel {

constexpr size_t cmax(size_t a, size_t b) { return a > b ? a : b; }
template <int R> constexpr size_t prep_short_smem_r() {
    return cmax(cmax(MixedPrepShape<R, 64>::SMEM, MixedPrepShape<R, 128>::SMEM),
                cmax(MixedPrepShape<R, 256>::SMEM, MixedPrepShape<R, 512>::SMEM));
}
constexpr size_t kPrepShortSmem = cmax(prep_short_smem_r<5>(), cmax(prep_short_smem_r<6>(), prep_short_smem_r<7>()));

// One CTA per (short harmonic, segment): the body of the harmonic's length.
__global__ void __launch_bounds__(kPrepShortThreads) k_prep_short(const PrepArgs a, const float2* __restrict__ tw) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int hist[256];
    __shared__ int bc[2];
    __shared__ float s_norm;
    const HarmPlan& H = a.h[blockIdx.x];
    const int R = mixed_radix(H.M), N2 = R > 1 ? H.M / R : 0;
#define ACCEL_PREP_FORM(r, n)                                                      \
    if (R == r && N2 == n) {                                                       \
        prep_short_body<r, n>(a, H, tw, smem_raw, hist, bc, &s_norm);              \
        return;                                                                    \
    }
    ACCEL_PREP_FORM(5, 64) ACCEL_PREP_FORM(5, 128) ACCEL_PREP_FORM(5, 256) ACCEL_PREP_FORM(5, 512)
    ACCEL_PREP_FORM(6, 64) ACCEL_PREP_FORM(6, 128) ACCEL_PREP_FORM(6, 256) ACCEL_PREP_FORM(6, 512)
    ACCEL_PREP_FORM(7, 64) ACCEL_PREP_FORM(7, 128) ACCEL_PREP_FORM(7, 256) ACCEL_PREP_FORM(7, 512)
#undef ACCEL_PREP_FORM
}

int launch_prep_short(const PrepArgs& a, int nseg, const float2* tw, cudaStream_t st) {
    static std::atomic<unsigned long long> attr{0};
    int dev = 0;
    if (attr_pending(attr, &dev)) {
        if (cudaFuncSetAttribute(k_prep_short, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kPrepShortSmem) !=
                cudaSuccess ||
            cudaFuncSetAttribute(k_prep_short, cudaFuncAttributePreferredSharedMemoryCarveout,
                                 carveout_for((const void*)k_prep_short, kPrepShortThreads, kPrepShortSmem)) !=
                cudaSuccess)
            return -1;
        attr_set(attr, dev);
    }
    // the largest body of this launch's harmonics (CTAs that need less fit
    // beside the harmonic sums of the other stream)
    size_t smem = 0;
    for (int h = 0; h < a.nh; h++) {
        const int R = mixed_radix(a.h[h].M);
        if (R < 5) return -1;
        smem = cmax(smem, prep_short_smem(R, a.h[h].M / R));
    }
    k_prep_short<<<dim3(a.nh, nseg), kPrepShortThreads, smem, st>>>(a, tw);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace accel
