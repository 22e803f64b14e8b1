// search_plane_lo.cu -- kernel instantiations (power planes, M <= 1024).
#include "search_kernels.cuh"

namespace accel {

int launch_plane_lo(int M, const PlaneArgs& a, int nseg, const float2* tw, cudaStream_t st) {
    switch (M) {
        case 64: return plane_dispatch<64>(a, nseg, tw, st);
        case 128: return plane_dispatch<128>(a, nseg, tw, st);
        case 256: return plane_dispatch<256>(a, nseg, tw, st);
        case 512: return plane_dispatch<512>(a, nseg, tw, st);
        case 1024: return plane_dispatch<1024>(a, nseg, tw, st);
    }
    return -1;
}

}  // namespace accel
