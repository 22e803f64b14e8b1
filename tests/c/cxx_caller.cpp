// A C++ caller of the reference pipeline API under its own C++ linkage
// (compiled by the CPU test test_cxx_linkage_cpu.py, once against
// include/bpd_compat_cxx.h and, where the reference checkout is present,
// once against the reference's own headers): it takes the address of every
// function the reference's headers declare -- so the link fails if the
// library lacks one -- and prints the answers of the host-only ones.
#include <cstdio>
#include <cstdlib>

#ifdef WITH_REFERENCE_HEADERS
extern "C" {
#include "bpd_common.h"
#include "bpd_math.h"
#include "bpd_noise.h"
#include "bpd_data.h"
}
#include "bpd_cudacommon.cuh"
#include "bpd_fft.cuh"
#include "bpd_subharmonics.cuh"
#include "bpd_search.cuh"
#include "bpd_candidates.cuh"
#else
#include "bpd_compat_cxx.h"
#endif

int main() {
    void* fns[] = {
        (void*)&createSubharmonicInfo, (void*)&calc_required_z, (void*)&calc_required_r,
        (void*)&index_from_r, (void*)&index_from_z, (void*)&getTotalHarmonics,
        (void*)&realToComplexFFT, (void*)&complexToComplexFFT, (void*)&inverseComplexToComplexFFT,
        (void*)&deredden, (void*)&get_fourier_amplitudes, (void*)&spreadData,
        (void*)&generate_harmonics_ffdot, (void*)&generate_harmonic_ffdot_data,
        (void*)&perform_fft_harmonics, (void*)&perform_convolution, (void*)&perform_inversefft,
        (void*)&generate_fundamental_powers, (void*)&perform_harmonic_summing,
        (void*)&initialize_cuda_plans, (void*)&free_cuda_plans, (void*)&search_ffdot_powers,
        (void*)&sortCandidates, (void*)&eliminateHarmonics, (void*)&optimizeCandidates,
        (void*)&calculateProperties, (void*)&__checkCudaErrors, (void*)&gpuAssert,
        (void*)&checkGPUMemory, (void*)&readData, (void*)&fast_median, (void*)&inverse_square_root,
        (void*)&fast_log2, (void*)&toNearestInt, (void*)&get2PowerNGreaterThan, (void*)&logMessage};
    int n = 0;
    for (void* f : fns) n += f != nullptr;
    printf("functions %d\n", n);
    printf("required_z %d %d %d\n", calc_required_z(0.75, 200.0), calc_required_z(0.125, -200.0),
           calc_required_z(0.375, 300.0));
    printf("required_r %.3f %.3f\n", calc_required_r(0.375, 1234.5), calc_required_r(0.875, 99999.25));
    printf("index %d %d\n", index_from_r(1000.5, 990.0), index_from_z(-10.0, -200.0));
    printf("total_harmonics %d %d\n", getTotalHarmonics(4), getTotalHarmonics(5));
    printf("log2 %d %d\n", fast_log2(8), fast_log2(1000));
    float a[7] = {5, 1, 4, 2, 7, 3, 6};
    printf("median %.1f\n", fast_median(a, 7));
    printf("rsqrt %.9g\n", inverse_square_root(2.0f));
    cufftComplex spec[6];
    for (int i = 0; i < 6; i++) spec[i] = make_float2((float)i + 1.0f, -(float)i);
    cufftComplex* amps = get_fourier_amplitudes(98, 10, spec, 6, 100);  // bins 98..107 of bins 100..105
    printf("amps");
    for (int i = 0; i < 10; i++) printf(" %.0f", amps[i].x);
    printf("\n");
    cufftComplex spread[12];
    for (int i = 0; i < 12; i++) spread[i] = make_float2(-1.f, -1.f);
    spreadData(amps + 2, 5, 2, 1u, spread);  // 5 values, every second slot from 1
    printf("spread");
    for (int i = 0; i < 12; i++) printf(" %.0f", spread[i].x);
    printf("\n");
    free(amps);
    sortCandidates();
    eliminateHarmonics();
    return 0;
}
