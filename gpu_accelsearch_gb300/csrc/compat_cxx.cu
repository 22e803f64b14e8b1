// compat_cxx.cu -- the drop-in layer under the reference's C++ linkage
// (include/bpd_compat_cxx.h): each function forwards to the C-linkage
// function of the same name in compat.cu, declared here inside a namespace
// so that both can be named in one translation unit; the two host helpers
// of the segment preparation and the caller-side error checks, which have
// no C-linkage counterpart, are written out here.
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#define BPD_COMPAT_CXX_IMPL  // the C-linkage declarations are made in cabi below
#include "../../include/bpd_compat_cxx.h"

// deredden with C++ linkage, for a caller that includes bpd_noise.h outside
// extern "C" (the reference's driver includes it inside, and gets the C one)
void deredden(cufftComplex* fft, unsigned numOfBins);

namespace cabi {
extern "C" {
SubharmonicInfo* createSubharmonicInfo(int, int);
int calc_required_z(double, double);
double calc_required_r(double, double);
int index_from_r(double, double);
int index_from_z(double, double);
int getTotalHarmonics(int);
unsigned realToComplexFFT(float*, long, accel_complex**, int);
unsigned complexToComplexFFT(accel_complex*, unsigned int, accel_complex**, int);
unsigned inverseComplexToComplexFFT(accel_complex*, unsigned int, accel_complex**, int);
void deredden(accel_complex*, unsigned);
void generate_harmonics_ffdot(unsigned short, unsigned short, SubharmonicInfo*, double, double, double,
                              ffdotInfo*, unsigned short*);
void generate_harmonic_ffdot_data(unsigned short, long, ffdotInfo*, unsigned short*, long*, accel_complex*,
                                  long, long, accel_complex*);
void perform_fft_harmonics(unsigned short, accel_complex*, long*, accel_complex*);
void perform_convolution(unsigned short, accel_complex*, ffdotInfo*, SubharmonicInfo*, long*, accel_complex*,
                         long*);
void perform_inversefft(unsigned short, accel_complex*, long*, accel_complex*);
void generate_fundamental_powers(unsigned short, accel_complex*, long*, ffdotInfo*, SubharmonicInfo*, float*);
void perform_harmonic_summing(unsigned short, accel_complex*, long*, ffdotInfo*, SubharmonicInfo*, float*, int,
                              unsigned short*, unsigned short*, int);
void initialize_cuda_plans(unsigned short, SubharmonicInfo*);
void free_cuda_plans(unsigned short);
Candidates* search_ffdot_powers(ffdotInfo*, int, float, long long, Candidates*);
int accel_compat_status(void);
const char* accel_last_error(void);
}
}  // namespace cabi

namespace {
accel_complex* ac(cufftComplex* p) { return reinterpret_cast<accel_complex*>(p); }
accel_complex** ac(cufftComplex** p) { return reinterpret_cast<accel_complex**>(p); }
}  // namespace

SubharmonicInfo* createSubharmonicInfo(int numHarmonicStages, int zhi) {
    return cabi::createSubharmonicInfo(numHarmonicStages, zhi);
}
int calc_required_z(double f, double zfull) { return cabi::calc_required_z(f, zfull); }
double calc_required_r(double f, double rfull) { return cabi::calc_required_r(f, rfull); }
int index_from_r(double r, double rlo) { return cabi::index_from_r(r, rlo); }
int index_from_z(double z, double zlo) { return cabi::index_from_z(z, zlo); }
int getTotalHarmonics(int stages) { return cabi::getTotalHarmonics(stages); }

unsigned realToComplexFFT(float* idata, long n, cufftComplex** odata, int batch) {
    return cabi::realToComplexFFT(idata, n, ac(odata), batch);
}
unsigned complexToComplexFFT(cufftComplex* din, unsigned int n, cufftComplex** dout, int batch) {
    return cabi::complexToComplexFFT(ac(din), n, ac(dout), batch);
}
unsigned inverseComplexToComplexFFT(cufftComplex* din, unsigned int n, cufftComplex** dout, int batch) {
    return cabi::inverseComplexToComplexFFT(ac(din), n, ac(dout), batch);
}

void deredden(cufftComplex* fft, unsigned numOfBins) { cabi::deredden(ac(fft), numOfBins); }

cufftComplex* get_fourier_amplitudes(int loBin, int numbins, cufftComplex* fft, long dataNumbins,
                                     long dataLoBin) {
    if (numbins <= 0) return nullptr;
    cufftComplex* out = static_cast<cufftComplex*>(malloc(sizeof(cufftComplex) * (size_t)numbins));
    if (!out) return nullptr;
    for (int k = 0; k < numbins; k++) {
        const long j = (long)loBin + k - dataLoBin;  // index into fft
        out[k] = (j >= 0 && j < dataNumbins) ? fft[j] : make_float2(0.f, 0.f);
    }
    return out;
}

void spreadData(cufftComplex* in, int inputElements, int interval, unsigned int startIdx, cufftComplex* out) {
    if (inputElements <= 0 || interval <= 0) return;
    cufftComplex* o = out + startIdx;
    std::memset(o, 0, sizeof(cufftComplex) * (size_t)inputElements * (size_t)interval);
    for (int k = 0; k < inputElements; k++) o[(size_t)k * interval] = in[k];
}

void generate_harmonics_ffdot(unsigned short totalHarmonics, unsigned short harmonicStages, SubharmonicInfo* shi,
                              double fullrlo, double fullrhi, double zlo, ffdotInfo* out,
                              unsigned short* binOffsets) {
    cabi::generate_harmonics_ffdot(totalHarmonics, harmonicStages, shi, fullrlo, fullrhi, zlo, out, binOffsets);
}
void generate_harmonic_ffdot_data(unsigned short totalHarmonics, long totalDataLength, ffdotInfo* ffdot,
                                  unsigned short* binoffsetArray, long* dataStartIdx, cufftComplex* fft,
                                  long dataNumbins, long dataLoBin, cufftComplex* output_data) {
    cabi::generate_harmonic_ffdot_data(totalHarmonics, totalDataLength, ffdot, binoffsetArray, dataStartIdx, ac(fft),
                                       dataNumbins, dataLoBin, ac(output_data));
}
void perform_fft_harmonics(unsigned short totalHarmonics, cufftComplex* device_data, long* dataStartIdx,
                           cufftComplex* out) {
    cabi::perform_fft_harmonics(totalHarmonics, ac(device_data), dataStartIdx, ac(out));
}
void perform_convolution(unsigned short totalHarmonics, cufftComplex* device_fft_data, ffdotInfo* harmonicInfo,
                         SubharmonicInfo* shi, long* dataStartIdx, cufftComplex* out, long* convIdx) {
    cabi::perform_convolution(totalHarmonics, ac(device_fft_data), harmonicInfo, shi, dataStartIdx, ac(out), convIdx);
}
void perform_inversefft(unsigned short totalHarmonics, cufftComplex* device_conv, long* convIdx, cufftComplex* out) {
    cabi::perform_inversefft(totalHarmonics, ac(device_conv), convIdx, ac(out));
}
void generate_fundamental_powers(unsigned short totalHarmonics, cufftComplex* device_ifft_data, long* idx,
                                 ffdotInfo* harmonicInfo, SubharmonicInfo* shi, float* out) {
    cabi::generate_fundamental_powers(totalHarmonics, ac(device_ifft_data), idx, harmonicInfo, shi, out);
}
void perform_harmonic_summing(unsigned short totalHarmonics, cufftComplex* device_ifft_data, long* idx,
                              ffdotInfo* harmonicInfo, SubharmonicInfo* shi, float* out, int fullrlo,
                              unsigned short* host_rinds, unsigned short* device_rinds, int totalRindsBins) {
    cabi::perform_harmonic_summing(totalHarmonics, ac(device_ifft_data), idx, harmonicInfo, shi, out, fullrlo,
                                   host_rinds, device_rinds, totalRindsBins);
}
void initialize_cuda_plans(unsigned short totalHarmonics, SubharmonicInfo* shi) {
    cabi::initialize_cuda_plans(totalHarmonics, shi);
}
void free_cuda_plans(unsigned short totalHarmonics) { cabi::free_cuda_plans(totalHarmonics); }

Candidates* search_ffdot_powers(ffdotInfo* ffdot, int numharm, float powcut, long long numindep,
                                Candidates* cands) {
    return cabi::search_ffdot_powers(ffdot, numharm, powcut, numindep, cands);
}
void sortCandidates() {}
void eliminateHarmonics() {}
void optimizeCandidates() {}
void calculateProperties() {}

void __checkCudaErrors(const char* errorMessage, const char* file, const int line) {
    const cudaError_t err = cudaGetLastError();
    const int st = cabi::accel_compat_status();
    if (err == cudaSuccess && st == 0) return;
    if (err != cudaSuccess)
        fprintf(stderr, "%s(%i): CUDA error: %s: (%d) %s.\n", file, line, errorMessage, (int)err,
                cudaGetErrorString(err));
    else
        fprintf(stderr, "%s(%i): %s: drop-in call failed (%d): %s.\n", file, line, errorMessage, st,
                cabi::accel_last_error());
    exit(EXIT_FAILURE);
}

void gpuAssert(cudaError_t code, const char* file, int line) {
    if (code == cudaSuccess) return;
    fprintf(stderr, "GPUassert: %s %s %d\n", cudaGetErrorString(code), file, line);
    exit(EXIT_FAILURE);
}

void checkGPUMemory() {
    size_t free_b = 0, total_b = 0;
    const cudaError_t e = cudaMemGetInfo(&free_b, &total_b);
    if (e != cudaSuccess) {
        printf("cudaMemGetInfo failed: %s\n", cudaGetErrorString(e));
        return;
    }
    printf("GPU memory usage: used = %f, free = %f MB, total = %f MB\n", (double)(total_b - free_b) / 1048576.0,
           (double)free_b / 1048576.0, (double)total_b / 1048576.0);
}
