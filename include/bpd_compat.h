/*
 * bpd_compat.h -- the reference pipeline API of keithasr/gpu_accelsearch,
 * same function names, structs and argument meaning, implemented by
 * libaccelsearch.so on its own GB300 kernels.  A caller of the reference's
 * headers/bpd_search.cuh, bpd_subharmonics.cuh, bpd_fft.cuh, bpd_noise.h and
 * bpd_candidates.cuh includes this header instead and links
 * -laccelsearch.  Everything here has C linkage.  The reference's .cu
 * functions have C++ linkage: the same functions with that linkage (the
 * symbols an object compiled against the reference's own headers needs) are
 * declared in bpd_compat_cxx.h and exported too, so such an object links
 * against libaccelsearch.so unchanged.
 *
 * Differences kept on purpose: errors do not exit the process -- the
 * functions are void as in the reference, so check accel_compat_status()
 * (0 or a negative ACCEL_ERR_*, message in accel_last_error()); and the
 * reference's compile-time ACCEL_USELEN (32000) is a runtime setting
 * (accel_compat_set_uselen).  Device pointers are ordinary cudaMalloc
 * memory, as in the reference; the work runs on the legacy default stream.
 */
#ifndef BPD_COMPAT_H_
#define BPD_COMPAT_H_

#include "accelsearch.h"

#ifdef __cplusplus
extern "C" {
#endif

/* The structs below are shared with include/bpd_compat_cxx.h, which defines
 * BPD_COMPAT_TYPES_ONLY to take them without the C-linkage functions. */

/* headers/bpd_subharmonics.cuh:13-25 */
typedef struct SubharmonicInfo {
    unsigned short maxHarmonic;
    unsigned short currentHarmonic;
    int zmax;
    unsigned short totalKernelsTemplates;
    int kernelFFTLength;
    int *z;
    unsigned short *kernelHalfWidth;
    accel_complex *kernels_data;        /* device: FFT of the wrapped templates */
} SubharmonicInfo;

/* headers/bpd_search.cuh:15-32 */
typedef struct ffdotInfo {
    unsigned short currentHarmonic;
    unsigned short maxHarmonic;
    int numrs;
    int numzs;
    int rlo;
    int zlo;
    double rhi;
    int fftlen;
} ffdotInfo;

/* headers/bpd_candidates.cuh:15-36 */
typedef struct RDERIVS {
    double pow, phs, dpow, dphs, d2pow, d2phs, locpow;
} rderivs;

typedef struct Candidates {
    float power;
    float sigma;
    int numharm;
    double r;
    double z;
    double *pows;
    double *hirs;
    double *hizs;
    rderivs *derivs;
} Candidates;

#ifndef BPD_COMPAT_TYPES_ONLY

/* Runtime replacement of the reference's ACCEL_USELEN (bpd_common.h:24),
 * default 32000; it must be even and below 65536. */
void accel_compat_set_uselen(int uselen);
int  accel_compat_get_uselen(void);
/* Status of the last drop-in call (ACCEL_OK or ACCEL_ERR_*). */
int  accel_compat_status(void);

/* bpd_subharmonics.cuh:27-33 */
SubharmonicInfo *createSubharmonicInfo(int numHarmonicStages, int zhi);
int    calc_required_z(double harmonicFraction, double zfull);
double calc_required_r(double harmonicFraction, double rfull);
int    index_from_r(double r, double rlo);
int    index_from_z(double z, double zlo);
int    getTotalHarmonics(int harmonicStages);
/* Frees what createSubharmonicInfo allocated (the reference's caller does
 * this by hand, AccelSearch.cu:272-277). */
void   freeSubharmonicInfo(SubharmonicInfo *shi, int totalHarmonics);

/* bpd_data.h:13 (bpd_data.c:9-75): read a raw float32 time series (at most
 * 2^26 samples); *output_data points at the first sample inside a buffer
 * padded with 2000 zero samples on each side.  Returns the number of
 * samples, or 0 with accel_compat_status() set (the reference exits).
 * freeData releases the buffer (the reference never frees it). */
long readData(char *path, float **output_data);
void freeData(float *data);

/* bpd_fft.cuh:14-16: realToComplexFFT takes host samples and returns a
 * malloc'd host spectrum of n/2+1 bins (caller frees), like the reference. */
unsigned realToComplexFFT(float *idata, long inputElements, accel_complex **odata, int batch);
unsigned complexToComplexFFT(accel_complex *device_idata, unsigned int inputElements,
                             accel_complex **device_odata, int batch);
unsigned inverseComplexToComplexFFT(accel_complex *device_idata, unsigned int inputElements,
                                    accel_complex **device_odata, int batch);

/* bpd_noise.h:16 -- host spectrum, whitened on the GPU, in place. */
void deredden(accel_complex *fft, unsigned numOfBins);

/* bpd_search.cuh:37-46 */
void generate_harmonics_ffdot(unsigned short totalHarmonics, unsigned short harmonicStages,
                              SubharmonicInfo *subharmonicsInfo, double fullrlo, double fullrhi,
                              double zlo, ffdotInfo *output_ffdot,
                              unsigned short *output_binOffsetArray);
void generate_harmonic_ffdot_data(unsigned short totalHarmonics, long totalDataLength,
                                  ffdotInfo *ffdot, unsigned short *binoffsetArray,
                                  long *dataStartIdx, accel_complex *fft, long dataNumbins,
                                  long dataLoBin, accel_complex *output_data);
void perform_fft_harmonics(unsigned short totalHarmonics, accel_complex *device_data,
                           long *dataStartIdx, accel_complex *output_device_fftdata);
void perform_convolution(unsigned short totalHarmonics, accel_complex *device_fft_data,
                         ffdotInfo *harmonicInfo, SubharmonicInfo *shi, long *dataStartIdx,
                         accel_complex *output_deviceConvolvedSignal,
                         long *convolutionHarmonicIdx);
void perform_inversefft(unsigned short totalHarmonics, accel_complex *device_convolvedSignal,
                        long *convolutionHarmonicIdx, accel_complex *output_device_ifftdata);
void generate_fundamental_powers(unsigned short totalHarmonics, accel_complex *device_ifft_data,
                                 long *ifftHarmonicIdx, ffdotInfo *harmonicInfo,
                                 SubharmonicInfo *shi, float *output_devicePowers);
void perform_harmonic_summing(unsigned short totalHarmonics, accel_complex *device_ifft_data,
                              long *ifftHarmonicIdx, ffdotInfo *harmonicInfo,
                              SubharmonicInfo *shi, float *output_devicePowers, int fullrlo,
                              unsigned short *host_rinds, unsigned short *device_rinds,
                              int totalRindsBins);
void initialize_cuda_plans(unsigned short totalHarmonics, SubharmonicInfo *subharmonicInfo);
void free_cuda_plans(unsigned short totalHarmonics);

/* bpd_gpu_kernels.cuh:15-17 -- the reference's kernels as host launchers
 * with the same names and arguments (a __global__ symbol cannot cross a C
 * ABI; a caller that wrote name<<<grid, block>>>(args) calls name(args)).
 * Each covers the whole range of the reference's launch, on the legacy
 * default stream; device pointers as in the reference.  convolveSignal
 * stops at fftlen - 1 (the reference's bound also touches element fftlen);
 * addPowers takes harmonicFraction = p / 2^k, as the bank's fractions are. */
void convolveSignal(int kernelTotalNumzs, int fftlen, accel_complex *data, accel_complex *kernels,
                    int kernelTemplateLength, accel_complex *outputdata);
void generatePowers(int kernelTotalNumzs, int numrs, int fftlen, accel_complex *data, float scale,
                    float *outputdata);
void addPowers(int fundamental_numzs, int fundamental_numrs, int subharm_fftlen, int fundamental_zlo,
               int subharm_zlo, int subharm_rlo, double harmonicFraction, accel_complex *data, float scale,
               float *output_powers, int fullrlo);

/* bpd_candidates.cuh:40 (a stub in the reference).  Here: the cells of the
 * power plane left by the last perform_harmonic_summing (or, before any
 * summing, generate_fundamental_powers) whose power exceeds powcut, as a
 * malloc'd array (caller frees) of at most *ncand entries in, the number
 * found out.  ffdot is the step's harmonic info (ffdot[0] the fundamental),
 * numharm the harmonics summed in that plane; sigma uses numindep. */
Candidates *search_ffdot_powers_n(ffdotInfo *ffdot, int numharm, float powcut,
                                  long long numindep, long *ncand);
/* The reference's signature: same as above, returning the array; the
 * `cands` argument is ignored (the reference returns it unchanged). */
Candidates *search_ffdot_powers(ffdotInfo *ffdot, int numharm, float powcut, long long numindep,
                                Candidates *cands);

/* bpd_math.h:17-25 -- the reference's host helpers (C linkage, as its
 * driver includes bpd_math.h inside extern "C"): fast_median returns the
 * element of rank (n-1)/2 (the lower median) and reorders arr, like the
 * reference's quickselect; inverse_square_root is the magic-constant
 * 0x5f3759df estimate with one Newton step, rounded operation by operation;
 * fast_log2 is floor(log2(n)) for n >= 1; toNearestInt rounds half away from
 * zero; get2PowerNGreaterThan is the first power of two >= x. */
float     fast_median(float arr[], int n);
float     inverse_square_root(float x);
int       fast_log2(int n);
int       toNearestInt(double x);
long long get2PowerNGreaterThan(long long x);

/* app_utilities.h:12-13 -- printf-style logging with a newline; throwError
 * prints and exits the process, as the reference's does (it is the caller's
 * own error path; nothing in this library calls it). */
void logMessage(const char *message, ...);
void throwError(const char *errorMessage, ...);

#endif /* BPD_COMPAT_TYPES_ONLY */

#ifdef __cplusplus
}
#endif
#endif /* BPD_COMPAT_H_ */
