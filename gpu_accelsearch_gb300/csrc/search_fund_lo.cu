// search_fund_lo.cu -- kernel instantiations (fundamental plane + harmonic sum, M <= 1024).
#include "search_kernels.cuh"

namespace accel {

int launch_fund_sum_lo(const FundArgs& a, int nseg, const float2* tw, cudaStream_t st) {
    switch (a.h[0].M) {
        case 64: return fund_dispatch<64>(a, nseg, tw, st);
        case 128: return fund_dispatch<128>(a, nseg, tw, st);
        case 256: return fund_dispatch<256>(a, nseg, tw, st);
        case 512: return fund_dispatch<512>(a, nseg, tw, st);
        case 1024: return fund_dispatch<1024>(a, nseg, tw, st);
    }
    return -1;
}

}  // namespace accel
