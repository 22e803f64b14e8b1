/*
 * bpd_compat_cxx.h -- the reference pipeline API with the reference's own
 * C++ linkage.  C++ only.
 *
 * The reference compiles its pipeline as CUDA C++ and its driver includes
 * the headers bpd_search.cuh, bpd_subharmonics.cuh, bpd_fft.cuh,
 * bpd_candidates.cuh and bpd_cudacommon.cuh outside any extern "C"
 * (AccelSearch.cu:8-13), so an object compiled against them refers to
 * C++-mangled names (createSubharmonicInfo(int, int) is
 * _Z21createSubharmonicInfoii).  libaccelsearch.so exports every function
 * below under exactly those names, as thin wrappers over the C-linkage
 * drop-in layer of bpd_compat.h: such an object -- the reference's own
 * driver included -- links against -laccelsearch with no source change.
 * This header restates those declarations (it replaces the reference's
 * headers for a caller that has none of them) with cufftComplex and the
 * reference's struct names, which fix the mangled names.
 *
 * Semantics are those of bpd_compat.h: no pipeline function exits the
 * process; a failure sets accel_compat_status() (and accel_last_error()).
 * The reference's error-check utilities (bpd_cudacommon.cuh:21-23) read it:
 * __checkCudaErrors also reports a failed drop-in call at the caller's next
 * check, and then exits like the reference's (so do gpuAssert and
 * throwError, which exist to end the caller's process).
 */
#ifndef BPD_COMPAT_CXX_H_
#define BPD_COMPAT_CXX_H_

#ifndef __cplusplus
#error "bpd_compat_cxx.h declares C++-linkage functions; C callers use bpd_compat.h"
#endif

#include <cuda_runtime.h>
#include <cufft.h>

#define BPD_COMPAT_TYPES_ONLY
#include "bpd_compat.h"
#undef BPD_COMPAT_TYPES_ONLY

/* headers/bpd_subharmonics.cuh:27-33 */
SubharmonicInfo *createSubharmonicInfo(int numHarmonicStages, int zhi);
int    calc_required_z(double harmonicFraction, double zfull);
double calc_required_r(double harmonicFraction, double rfull);
int    index_from_r(double r, double rlo);
int    index_from_z(double z, double zlo);
int    getTotalHarmonics(int harmonicStages);

/* headers/bpd_fft.cuh:14-16 */
unsigned realToComplexFFT(float *idata, long inputElements, cufftComplex **odata, int batch);
unsigned complexToComplexFFT(cufftComplex *device_idata, unsigned int inputElements,
                             cufftComplex **device_odata, int batch);
unsigned inverseComplexToComplexFFT(cufftComplex *device_idata, unsigned int inputElements,
                                    cufftComplex **device_odata, int batch);

/* headers/bpd_search.cuh:35-36 -- host helpers of the segment preparation:
 * get_fourier_amplitudes returns a malloc'd copy (caller frees) of numbins
 * bins of fft starting at loBin, zero outside [dataLoBin, dataNumbins);
 * spreadData writes the inputElements values to outputData[startIdx +
 * k * interval] and zeros between them (bpd_search.cu:16-67). */
cufftComplex *get_fourier_amplitudes(int loBin, int numbins, cufftComplex *fft, long dataNumbins,
                                     long dataLoBin);
void spreadData(cufftComplex *inputData, int inputElements, int interval, unsigned int startIdx,
                cufftComplex *outputData);

/* headers/bpd_search.cuh:37-46 */
void generate_harmonics_ffdot(unsigned short totalHarmonics, unsigned short harmonicStages,
                              SubharmonicInfo *subharmonicsInfo, double fullrlo, double fullrhi,
                              double zlo, ffdotInfo *output_ffdot,
                              unsigned short *output_binOffsetArray);
void generate_harmonic_ffdot_data(unsigned short totalHarmonics, long totalDataLength, ffdotInfo *ffdot,
                                  unsigned short *binoffsetArray, long *dataStartIdx, cufftComplex *fft,
                                  long dataNumbins, long dataLoBin, cufftComplex *output_data);
void perform_fft_harmonics(unsigned short totalHarmonics, cufftComplex *device_data, long *dataStartIdx,
                           cufftComplex *output_device_fftdata);
void perform_convolution(unsigned short totalHarmonics, cufftComplex *device_fft_data,
                         ffdotInfo *harmonicInfo, SubharmonicInfo *shi, long *dataStartIdx,
                         cufftComplex *output_deviceConvolvedSignal, long *convolutionHarmonicIdx);
void perform_inversefft(unsigned short totalHarmonics, cufftComplex *device_convolvedSignal,
                        long *convolutionHarmonicIdx, cufftComplex *output_device_ifftdata);
void generate_fundamental_powers(unsigned short totalHarmonics, cufftComplex *device_ifft_data,
                                 long *ifftHarmonicIdx, ffdotInfo *harmonicInfo, SubharmonicInfo *shi,
                                 float *output_devicePowers);
void perform_harmonic_summing(unsigned short totalHarmonics, cufftComplex *device_ifft_data,
                              long *ifftHarmonicIdx, ffdotInfo *harmonicInfo, SubharmonicInfo *shi,
                              float *output_devicePowers, int fullrlo, unsigned short *host_rinds,
                              unsigned short *device_rinds, int totalRindsBins);
void initialize_cuda_plans(unsigned short totalHarmonics, SubharmonicInfo *subharmonicInfo);
void free_cuda_plans(unsigned short totalHarmonics);

/* headers/bpd_candidates.cuh:40 (a stub in the reference; here the cells
 * above powcut of the last summed plane, as bpd_compat.h describes) */
Candidates *search_ffdot_powers(ffdotInfo *ffdot, int numharm, float powcut, long long numindep,
                                Candidates *cands);
/* headers/bpd_candidates.cuh:46-49: argument-less and empty in the
 * reference (bpd_candidates.cu:15-33); empty here too.  Sorting, harmonic
 * elimination and refinement are accel_sift_candidates and
 * accel_optimize_candidates. */
void sortCandidates();
void eliminateHarmonics();
void optimizeCandidates();
void calculateProperties();

/* headers/bpd_cudacommon.cuh:21-23 (bpd_cudacommon.cu:8-50): the caller's
 * error checks.  __checkCudaErrors exits when cudaGetLastError() reports an
 * error or the last drop-in call failed (accel_compat_status() != 0);
 * gpuAssert exits when code is not cudaSuccess; checkGPUMemory prints the
 * device's memory use. */
void __checkCudaErrors(const char *errorMessage, const char *file, const int line);
void gpuAssert(cudaError_t code, const char *file, int line);
void checkGPUMemory();

/* The reference's C headers, with the C linkage its driver gives them (it
 * includes bpd_common.h, bpd_math.h, bpd_noise.h and bpd_data.h inside
 * extern "C", AccelSearch.cu:1-7); meanings as in bpd_compat.h.  deredden is
 * also exported with C++ linkage, deredden(float2*, unsigned int), for a
 * caller that includes bpd_noise.h outside extern "C".  (Include this header
 * or bpd_compat.h, not both.) */
#ifndef BPD_COMPAT_CXX_IMPL
extern "C" {
/* headers/bpd_noise.h:16 */
void deredden(cufftComplex *fft, unsigned numOfBins);
/* headers/bpd_data.h:13 */
long readData(char *path, float **output_data);
/* headers/bpd_math.h:17-25 */
float     fast_median(float arr[], int n);
float     inverse_square_root(float x);
int       fast_log2(int n);
int       toNearestInt(double x);
long long get2PowerNGreaterThan(long long x);
/* headers/app_utilities.h:12-13 */
void logMessage(const char *message, ...);
void throwError(const char *errorMessage, ...);
}
#endif

#endif /* BPD_COMPAT_CXX_H_ */
