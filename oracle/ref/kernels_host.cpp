/*
 * kernels_host.cpp -- runs the reference's own kernels (convolveSignal,
 * generatePowers, addPowers of source/bpd_gpu_kernels.cu, compiled as host
 * C++ with kernel_host_shim.h) on the CPU, one call of the kernel body per
 * thread of the launch, over the launch geometry the caller gives (the
 * reference's own launches are bpd_search.cu:249, :301, :333).  Used only by
 * tests/golden/make_plane_golden.py to produce golden planes from the
 * reference's kernel code; nothing here is part of the product.
 */
#include <cuda_runtime.h>
#include <cufft.h>
#include <vector_types.h>

thread_local uint3 threadIdx, blockIdx;
thread_local dim3 blockDim, gridDim;

void convolveSignal(int kernelTotalNumzs, int fftlen, cufftComplex *data, cufftComplex *kernels,
                    int kernelTemplateLength, cufftComplex *outputdata);
void generatePowers(int kernelTotalNumzs, int numrs, int fftlen, cufftComplex *data, float scale,
                    float *outputdata);
void addPowers(int fundamental_numzs, int fundamental_numrs, int subharm_fftlen, int fundamental_zlo,
               int subharm_zlo, int subharm_rlo, double harmonicFraction, cufftComplex *data, float scale,
               float *output_powers, int fullrlo);

template <class F> static void walk(unsigned gx, unsigned gy, unsigned bx, F body)
{
    gridDim = dim3(gx, gy, 1);
    blockDim = dim3(bx, 1, 1);
    for (unsigned y = 0; y < gy; y++)
        for (unsigned x = 0; x < gx; x++)
            for (unsigned t = 0; t < bx; t++) {
                blockIdx = make_uint3(x, y, 0);
                threadIdx = make_uint3(t, 0, 0);
                body();
            }
}

extern "C" {
void ref_launch_convolve(unsigned gx, unsigned gy, unsigned bx, int numzs, int fftlen, float *data,
                         float *kernels, int kernelTemplateLength, float *out)
{
    walk(gx, gy, bx, [&] {
        convolveSignal(numzs, fftlen, (cufftComplex *)data, (cufftComplex *)kernels, kernelTemplateLength,
                       (cufftComplex *)out);
    });
}

void ref_launch_powers(unsigned gx, unsigned gy, unsigned bx, int numzs, int numrs, int fftlen, float *data,
                       float scale, float *out)
{
    walk(gx, gy, bx, [&] { generatePowers(numzs, numrs, fftlen, (cufftComplex *)data, scale, out); });
}

void ref_launch_add_powers(unsigned gx, unsigned gy, unsigned bx, int fnumzs, int fnumrs, int sfftlen, int fzlo,
                           int szlo, int srlo, double frac, float *data, float scale, float *out, int fullrlo)
{
    walk(gx, gy, bx, [&] {
        addPowers(fnumzs, fnumrs, sfftlen, fzlo, szlo, srlo, frac, (cufftComplex *)data, scale, out, fullrlo);
    });
}
}
