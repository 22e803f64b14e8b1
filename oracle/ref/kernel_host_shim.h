/*
 * kernel_host_shim.h -- force-included when the reference's
 * source/bpd_gpu_kernels.cu is compiled as host C++ (oracle/ref/Makefile,
 * target kernels).  The reference's three kernels use no shared memory, no
 * barriers and no atomics, so each thread of a launch is a plain call of the
 * kernel body with the thread's indices set; kernels_host.cpp walks a
 * launch's grid that way.  This header only makes __global__ an ordinary
 * function and supplies the index variables; the kernel source is compiled
 * as it lies.
 */
#ifndef ORACLE_KERNEL_HOST_SHIM_H_
#define ORACLE_KERNEL_HOST_SHIM_H_
#include <cuda_runtime.h>
#include <vector_types.h>
#undef __global__
#define __global__
extern thread_local uint3 threadIdx, blockIdx;
extern thread_local dim3 blockDim, gridDim;
#endif
