// search_plane_hi.cu -- kernel instantiations (power planes, M >= 2048).
#include "search_kernels.cuh"

namespace accel {

int launch_plane_hi(int M, const PlaneArgs& a, int nseg, const float2* tw, cudaStream_t st) {
    switch (M) {
        case 2048: return plane_dispatch<2048>(a, nseg, tw, st);
        case 4096: return plane_dispatch<4096>(a, nseg, tw, st);
        case 8192: return plane_dispatch<8192>(a, nseg, tw, st);
    }
    return -1;
}

}  // namespace accel
