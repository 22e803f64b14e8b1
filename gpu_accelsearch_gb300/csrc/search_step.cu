// search_step.cu -- instantiations and launcher of the persistent
// plane-and-sum kernel (k_step).
#include "step_kernel.cuh"

namespace accel {

template <int MMAX, int NH, bool F16>
static int step_launch(const StepArgs& a, const float2* tw, cudaStream_t st) {
    const size_t smem = sizeof(float2) * 2 * FftShape<MMAX>::PADDED;  // >= every tile of the plan
    static std::atomic<unsigned long long> attr{0};
    static int per_sm[64] = {0};
    int dev = 0;
    if (attr_pending(attr, &dev)) {
        if (cudaFuncSetAttribute(k_step<MMAX, NH, F16>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
                cudaSuccess ||
            cudaFuncSetAttribute(k_step<MMAX, NH, F16>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                 cudaSharedmemCarveoutMaxShared) != cudaSuccess)
            return -1;
        int nb = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_step<MMAX, NH, F16>, MMAX / 16, smem) !=
                cudaSuccess ||
            nb < 1)
            return -1;
        if (dev >= 0 && dev < 64) per_sm[dev] = nb;
        attr_set(attr, dev);
    }
    int sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return -1;
    const int nb = (dev >= 0 && dev < 64 && per_sm[dev] > 0) ? per_sm[dev] : 1;
    const long long grid = std::min<long long>(a.nitems, (long long)nb * sms);
    k_step<MMAX, NH, F16><<<(unsigned)grid, MMAX / 16, smem, st>>>(a, tw);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

template <int MMAX, bool F16>
static int step_nh(const StepArgs& a, const float2* tw, cudaStream_t st) {
    switch (a.hs.nh) {
        case 1: return step_launch<MMAX, 1, F16>(a, tw, st);
        case 2: return step_launch<MMAX, 2, F16>(a, tw, st);
        case 4: return step_launch<MMAX, 4, F16>(a, tw, st);
        case 8: return step_launch<MMAX, 8, F16>(a, tw, st);
        case 16: return step_launch<MMAX, 16, F16>(a, tw, st);
    }
    return -1;
}

int launch_step(const StepArgs& a, int mmax, int use_fp16, const float2* tw, cudaStream_t st) {
    if (mmax != 4096) return -1;  // one thread per tile column: 256 threads
    return use_fp16 ? step_nh<4096, true>(a, tw, st) : step_nh<4096, false>(a, tw, st);
}

}  // namespace accel
