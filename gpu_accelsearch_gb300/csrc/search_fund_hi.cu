// search_fund_hi.cu -- kernel instantiations (fundamental plane + harmonic sum, M >= 2048).
#include "search_kernels.cuh"

namespace accel {

int launch_fund_sum_hi(const FundArgs& a, int nseg, const float2* tw, cudaStream_t st) {
    switch (a.h[0].M) {
        case 2048: return fund_dispatch<2048>(a, nseg, tw, st);
        case 4096: return fund_dispatch<4096>(a, nseg, tw, st);
        case 8192: return fund_dispatch<8192>(a, nseg, tw, st);
    }
    return -1;
}

}  // namespace accel
