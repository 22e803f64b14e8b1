// search_mixed5.cu -- instantiations of the short-transform plane kernels
// with a radix-5 last pass (half lengths 5 * 64 .. 5 * 512).
#include "mixed_kernels.cuh"

namespace accel {

int launch_plane_r5(int N2, const PlaneArgs& a, int nseg, const float2* tw, cudaStream_t st) {
    return plane_mixed_r<5>(N2, a, nseg, tw, st);
}

}  // namespace accel
