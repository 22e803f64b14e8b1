// search.cu -- kernel instantiations (segment preparation and harmonic sum; dispatch).
#include "search_kernels.cuh"

#include <algorithm>

namespace accel {

int launch_prep_short(const PrepArgs& a, int nseg, const float2* tw, cudaStream_t st);
int launch_plane_r5(int N2, const PlaneArgs& a, int nseg, const float2* tw, cudaStream_t st);
int launch_plane_r6(int N2, const PlaneArgs& a, int nseg, const float2* tw, cudaStream_t st);
int launch_plane_r7(int N2, const PlaneArgs& a, int nseg, const float2* tw, cudaStream_t st);

int launch_prep(int M, const PrepArgs& a, int nseg, const float2* tw, cudaStream_t st) {
    if (mixed_radix(M) > 1) return launch_prep_short(a, nseg, tw, st);  // any short harmonics
    switch (M) {
        case 64: return prep_m<64>(a, nseg, tw, st);
        case 128: return prep_m<128>(a, nseg, tw, st);
        case 256: return prep_m<256>(a, nseg, tw, st);
        case 512: return prep_m<512>(a, nseg, tw, st);
        case 1024: return prep_m<1024>(a, nseg, tw, st);
        case 2048: return prep_m<2048>(a, nseg, tw, st);
        case 4096: return prep_m<4096>(a, nseg, tw, st);
        case 8192: return prep_m<8192>(a, nseg, tw, st);
    }
    return -1;
}

int launch_hsum(const HsumArgs& a, int nseg, cudaStream_t st) {
    dim3 grid((a.uselen + kHsumCols - 1) / kHsumCols, (a.numzs0 + kHsumRows - 1) / kHsumRows, nseg);
    switch (a.nh) {
        case 1: k_hsum<1><<<grid, kHsumCols, 0, st>>>(a); break;
        case 2: k_hsum<2><<<grid, kHsumCols, 0, st>>>(a); break;
        case 4: k_hsum<4><<<grid, kHsumCols, 0, st>>>(a); break;
        case 8: k_hsum<8><<<grid, kHsumCols, 0, st>>>(a); break;
        case 16: k_hsum<16><<<grid, kHsumCols, 0, st>>>(a); break;
        default: return -1;
    }
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

template <int NH, bool SO, int TZ>
static int hsum_tile_nh(const HsumArgs& a, dim3 grid, size_t smem, const HsumMaps& maps, cudaStream_t st) {
    static std::atomic<unsigned long long> attr{0};
    int dev = 0;
    if (attr_pending(attr, &dev)) {
        if (cudaFuncSetAttribute(k_hsum_tile<NH, SO, TZ>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)(sizeof(float) * hsum_tile_floats_max(TZ))) != cudaSuccess ||
            cudaFuncSetAttribute(k_hsum_tile<NH, SO, TZ>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                 cudaSharedmemCarveoutMaxShared) != cudaSuccess)
            return -1;
        attr_set(attr, dev);
    }
    k_hsum_tile<NH, SO, TZ><<<grid, kTileI, smem, st>>>(a, maps);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

template <int NH, bool SO>
static int hsum_tile_tz(const HsumArgs& a, int tz, dim3 grid, size_t smem, const HsumMaps& maps, cudaStream_t st) {
    switch (tz) {
        case 8: return hsum_tile_nh<NH, SO, 8>(a, grid, smem, maps, st);
        case 16: return hsum_tile_nh<NH, SO, 16>(a, grid, smem, maps, st);
        case 32: return hsum_tile_nh<NH, SO, 32>(a, grid, smem, maps, st);
    }
    return -1;
}

template <int NH, bool SO>
static int hsum_pipe_nh(const HsumArgs& a, int ntiles, cudaStream_t st) {
    static std::atomic<unsigned long long> attr{0};
    int dev = 0;
    // buffers of the plan's worst tile, 128-byte aligned
    const int bstride = (a.tile_floats > 0 && a.tile_floats <= kTileSmemFloats) ? ((a.tile_floats + 31) & ~31)
                                                                                 : kTileSmemFloats;
    const size_t smem = sizeof(float) * (size_t)bstride * kPipeBufs;
    if (smem > (size_t)kPipeSmemMax) return -1;  // the caller checks this before choosing the kernel
    if (attr_pending(attr, &dev)) {
        if (cudaFuncSetAttribute(k_hsum_pipe<NH, SO>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 kPipeSmemMax) != cudaSuccess ||
            cudaFuncSetAttribute(k_hsum_pipe<NH, SO>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                 cudaSharedmemCarveoutMaxShared) != cudaSuccess)
            return -1;
        attr_set(attr, dev);
    }
    int sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return -1;
    const int grid = std::max(1, std::min(ntiles, sms));
    k_hsum_pipe<NH, SO><<<grid, kPipeThreads, smem, st>>>(a, ntiles, bstride);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int launch_hsum_pipe(const HsumArgs& a, int nseg, cudaStream_t st) {
    const long long nt = (long long)((a.uselen + kTileI - 1) / kTileI) * ((a.numzs0 + kTileZ - 1) / kTileZ) * nseg;
    if (nt >= (1LL << 31)) return -1;
    const int ntiles = (int)nt;
    const bool so = a.stage_out != nullptr;
    switch (a.nh) {
        case 1: return so ? hsum_pipe_nh<1, true>(a, ntiles, st) : hsum_pipe_nh<1, false>(a, ntiles, st);
        case 2: return so ? hsum_pipe_nh<2, true>(a, ntiles, st) : hsum_pipe_nh<2, false>(a, ntiles, st);
        case 4: return so ? hsum_pipe_nh<4, true>(a, ntiles, st) : hsum_pipe_nh<4, false>(a, ntiles, st);
        case 8: return so ? hsum_pipe_nh<8, true>(a, ntiles, st) : hsum_pipe_nh<8, false>(a, ntiles, st);
        case 16: return so ? hsum_pipe_nh<16, true>(a, ntiles, st) : hsum_pipe_nh<16, false>(a, ntiles, st);
    }
    return -1;
}

int launch_hsum_tile(const HsumArgs& a0, int nseg, int tz, const HsumMaps* maps, cudaStream_t st) {
    static const HsumMaps no_maps{};
    HsumArgs a = a0;
    if (!maps) a.use_tmap = 0;
    const HsumMaps& m = maps ? *maps : no_maps;
    dim3 grid((a.uselen + kTileI - 1) / kTileI, (a.numzs0 + tz - 1) / tz, nseg);
    // the plan's own worst tile of this height (host-proven to fit): a
    // smaller footprint fits more CTAs per SM (4 instead of 3 at zmax 200,
    // 8 harmonics, 16 rows)
    const int fmax = hsum_tile_floats_max(tz);
    const int floats = (a.tile_floats > 0 && a.tile_floats <= fmax) ? ((a.tile_floats + 3) & ~3) : fmax;
    const size_t smem = sizeof(float) * floats;
    const bool so = a.stage_out != nullptr;
    switch (a.nh) {
        case 1: return so ? hsum_tile_tz<1, true>(a, tz, grid, smem, m, st) : hsum_tile_tz<1, false>(a, tz, grid, smem, m, st);
        case 2: return so ? hsum_tile_tz<2, true>(a, tz, grid, smem, m, st) : hsum_tile_tz<2, false>(a, tz, grid, smem, m, st);
        case 4: return so ? hsum_tile_tz<4, true>(a, tz, grid, smem, m, st) : hsum_tile_tz<4, false>(a, tz, grid, smem, m, st);
        case 8: return so ? hsum_tile_tz<8, true>(a, tz, grid, smem, m, st) : hsum_tile_tz<8, false>(a, tz, grid, smem, m, st);
        case 16: return so ? hsum_tile_tz<16, true>(a, tz, grid, smem, m, st) : hsum_tile_tz<16, false>(a, tz, grid, smem, m, st);
    }
    return -1;
}

int launch_plane_lo(int M, const PlaneArgs& a, int nseg, const float2* tw, cudaStream_t st);
int launch_plane_hi(int M, const PlaneArgs& a, int nseg, const float2* tw, cudaStream_t st);
int launch_fund_sum_lo(const FundArgs& a, int nseg, const float2* tw, cudaStream_t st);
int launch_fund_sum_hi(const FundArgs& a, int nseg, const float2* tw, cudaStream_t st);

int launch_plane(int M, const PlaneArgs& a, int nseg, const float2* tw, cudaStream_t st) {
    switch (mixed_radix(M)) {  // short transforms
        case 5: return launch_plane_r5(M / 5, a, nseg, tw, st);
        case 6: return launch_plane_r6(M / 6, a, nseg, tw, st);
        case 7: return launch_plane_r7(M / 7, a, nseg, tw, st);
    }
    return M >= 2048 ? launch_plane_hi(M, a, nseg, tw, st) : launch_plane_lo(M, a, nseg, tw, st);
}

int launch_fund_sum(const FundArgs& a, int nseg, const float2* tw, cudaStream_t st) {
    return a.h[0].M >= 2048 ? launch_fund_sum_hi(a, nseg, tw, st) : launch_fund_sum_lo(a, nseg, tw, st);
}

}  // namespace accel
