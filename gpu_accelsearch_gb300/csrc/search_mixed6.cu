// search_mixed6.cu -- instantiations of the short-transform plane kernels
// with a radix-6 last pass (half lengths 6 * 64 .. 6 * 512).
#include "mixed_kernels.cuh"

namespace accel {

int launch_plane_r6(int N2, const PlaneArgs& a, int nseg, const float2* tw, cudaStream_t st) {
    return plane_mixed_r<6>(N2, a, nseg, tw, st);
}

}  // namespace accel
