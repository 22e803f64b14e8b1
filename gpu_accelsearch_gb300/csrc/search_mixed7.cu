// search_mixed7.cu -- instantiations of the short-transform plane kernels
// with a radix-7 last pass (half lengths 7 * 64 .. 7 * 512).
#include "mixed_kernels.cuh"

namespace accel {

int launch_plane_r7(int N2, const PlaneArgs& a, int nseg, const float2* tw, cudaStream_t st) {
    return plane_mixed_r<7>(N2, a, nseg, tw, st);
}

}  // namespace accel
