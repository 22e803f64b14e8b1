// compat.cu -- the reference's pipeline API (include/bpd_compat.h) on this
// library's kernels: same names, structs and argument meaning as
// keithasr/gpu_accelsearch's headers, so its driver loop
// (AccelSearch.cu:203-247) runs unchanged against it.
//
// The stage-by-stage API materialises what the reference materialises (the
// convolved plane, the inverse-transformed plane, the fundamental power
// plane accumulated in place), using:
//   k_fft_long     forward/inverse C2C of L = R0*M points (R0 = 1, 2, 4;
//                  M <= 8192): a radix-R0 decimation-in-frequency first
//                  stage fused into the loads, then the shared-memory FFT;
//   k_conv         convolveSignal (bpd_gpu_kernels.cu:39-81) without its
//                  off-by-one bound;
//   k_powers       generatePowers (:84-116);
//   k_addpowers    addPowers (:119-170), exact integer index arithmetic.
// Host-side segment preparation (generate_harmonic_ffdot_data) is compiled
// with -ffp-contract=off and restates bpd_search.cu:16-184 operation by
// operation, so its output is bit-identical to the reference's.
#include <cufft.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <vector>

#include "../../include/bpd_compat.h"
#include "accel_internal.h"
#include "fft_smem.cuh"

namespace accel {
namespace {

struct CompatState {
    std::mutex mu;
    int uselen = 32000;
    int status = ACCEL_OK;
    float2* tw = nullptr;          // twiddle table for the shared-memory FFT
    int tw_device = -1;
    std::vector<int> fftlen, numzs;  // from initialize_cuda_plans
    std::map<long long, cufftHandle> r2c;
    const float* last_powers = nullptr;  // plane of the last powers call
    int last_numzs = 0, last_numrs = 0;
};
CompatState g_cs;

int fail(int code, const char* what, cudaError_t e = cudaSuccess) {
    g_cs.status = code;
    if (e != cudaSuccess) return set_error(code, "%s: %s", what, cudaGetErrorString(e));
    return set_error(code, "%s", what);
}

bool ensure_twiddles() {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return false;
    if (g_cs.tw && g_cs.tw_device == dev) return true;
    if (cudaMalloc(&g_cs.tw, sizeof(float2) * kTwAll) != cudaSuccess) return false;
    if (launch_twiddles(g_cs.tw, 0) != 0) return false;
    g_cs.tw_device = dev;
    return cudaStreamSynchronize(0) == cudaSuccess;
}

// ------------------------------------------------------------------ kernels
template <int M, int DIR>
__global__ void __launch_bounds__(M / 16) k_fft_long(const float2* __restrict__ in, long long ldi,
                                                     float2* __restrict__ out, long long ldo, int r0,
                                                     const float2* __restrict__ tw) {
    constexpr int T = M / 16;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int s = blockIdx.x % r0;
    const long long b = blockIdx.x / r0;
    const int t = threadIdx.x;
    const float2* x = in + b * ldi;
    const int L = r0 * M;
    float2 u[1][16];
#pragma unroll
    for (int e = 0; e < 16; e++) {
        const int idx = t + e * T;
        float2 acc = x[idx];
        for (int j = 1; j < r0; j++) {
            // W_{r0}^{DIR j s}
            float sw, cw;
            sincospif(DIR * 2.0f * (float)((j * s) % r0) / (float)r0, &sw, &cw);
            acc = cadd(acc, cmul(x[idx + j * M], make_float2(cw, sw)));
        }
        if (s) {
            float sw, cw;
            sincospif(DIR * 2.0f * (float)(idx * s) / (float)L, &sw, &cw);
            acc = cmul(acc, make_float2(cw, sw));
        }
        u[0][e] = acc;
    }
    fft_run<M, DIR, 1>(u, reinterpret_cast<float2*>(smem_raw), tw, t);
    float2* y = out + b * ldo;
#pragma unroll
    for (int e = 0; e < 16; e++) y[(long long)r0 * (t + e * T) + s] = u[0][e];
}

template <int M, int DIR>
int fft_long_m(const float2* in, long long ldi, float2* out, long long ldo, int r0, long long batch) {
    const size_t smem = sizeof(float2) * FftShape<M>::PADDED;
    if (cudaFuncSetAttribute(k_fft_long<M, DIR>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
        cudaSuccess)
        return -1;
    k_fft_long<M, DIR><<<(unsigned)(batch * r0), M / 16, smem, 0>>>(in, ldi, out, ldo, r0, g_cs.tw);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

template <int DIR>
int fft_long(const float2* in, long long ldi, float2* out, long long ldo, int L, long long batch) {
    if (L < kMinM || (L & (L - 1)) || L > 4 * kMaxM) return -2;
    const int r0 = L > kMaxM ? L / kMaxM : 1;
    const int M = L / r0;
    switch (M) {
        case 64: return fft_long_m<64, DIR>(in, ldi, out, ldo, r0, batch);
        case 128: return fft_long_m<128, DIR>(in, ldi, out, ldo, r0, batch);
        case 256: return fft_long_m<256, DIR>(in, ldi, out, ldo, r0, batch);
        case 512: return fft_long_m<512, DIR>(in, ldi, out, ldo, r0, batch);
        case 1024: return fft_long_m<1024, DIR>(in, ldi, out, ldo, r0, batch);
        case 2048: return fft_long_m<2048, DIR>(in, ldi, out, ldo, r0, batch);
        case 4096: return fft_long_m<4096, DIR>(in, ldi, out, ldo, r0, batch);
        case 8192: return fft_long_m<8192, DIR>(in, ldi, out, ldo, r0, batch);
    }
    return -2;
}

__global__ void k_conv(int numzs, int L, const float2* __restrict__ d, const float2* __restrict__ kern,
                       float2* __restrict__ out) {
    const long long n = (long long)numzs * L;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const float2 a = d[i % L], k = kern[i];
        out[i] = make_float2(a.x * k.x + a.y * k.y, a.y * k.x - a.x * k.y);
    }
}

__global__ void k_powers(int numzs, int numrs, int L, const float2* __restrict__ y, float scale,
                         float* __restrict__ p) {
    const long long n = (long long)numzs * numrs;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const int z = (int)(i / numrs), r = (int)(i - (long long)z * numrs);
        const float2 v = y[(long long)z * L + r];
        p[i] = (v.x * v.x + v.y * v.y) * scale;
    }
}

__global__ void k_addpowers(int numzs0, int numrs0, int L_h, int zlo0, int zlo_h, int rlo_h, int p, int q,
                            const float2* __restrict__ y, float scale, float* __restrict__ pw,
                            long long fullrlo) {
    const long long n = (long long)numzs0 * numrs0;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n;
         k += (long long)gridDim.x * blockDim.x) {
        const int z = (int)(k / numrs0), i = (int)(k - (long long)z * numrs0);
        const int rind = sub_rind(fullrlo, i, p, q, rlo_h);
        const int zind = sub_zind(zlo0 + kDz * z, p, q, zlo_h);
        const float2 v = y[(long long)zind * L_h + rind];
        pw[k] += (v.x * v.x + v.y * v.y) * scale;
    }
}

struct RawHit {
    int z, i;
    float power;
};
__global__ void k_threshold(int numzs, int numrs, const float* __restrict__ p, float cut, RawHit* hits,
                            unsigned long long* n, long long cap) {
    const long long tot = (long long)numzs * numrs;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < tot;
         k += (long long)gridDim.x * blockDim.x) {
        if (p[k] > cut) {
            const unsigned long long s = atomicAdd(n, 1ULL);
            if ((long long)s < cap) hits[s] = RawHit{(int)(k / numrs), (int)(k % numrs), p[k]};
        }
    }
}

unsigned grid_for(long long n) { return (unsigned)std::min<long long>((n + 255) / 256, 152LL * 32); }

// ------------------------------------------------------------- host math
int nearest_int(double x) { return (int)(x < 0 ? std::ceil(x - 0.5) : std::floor(x + 0.5)); }

float rsqrt_magic_host(float x) {
    int32_t i;
    std::memcpy(&i, &x, 4);
    i = 0x5f3759df - (i >> 1);
    float y;
    std::memcpy(&y, &i, 4);
    volatile float h = 0.5f * x;
    h = h * y;
    h = h * y;
    return y * (1.5f - h);
}

}  // namespace

}  // namespace accel

using namespace accel;

extern "C" {

void accel_compat_set_uselen(int uselen) {
    if (uselen < 2 || (uselen & 1) || uselen >= 65536) {
        fail(ACCEL_ERR_INVALID, "accel_compat_set_uselen: uselen must be even, positive and < 65536");
        return;
    }
    g_cs.uselen = uselen;
    g_cs.status = ACCEL_OK;
}
int accel_compat_get_uselen(void) { return g_cs.uselen; }
int accel_compat_status(void) { return g_cs.status; }

int calc_required_z(double f, double zfull) { return nearest_int(0.5 * zfull * f) * kDz; }
double calc_required_r(double f, double rfull) { return (int)(2 * rfull * f + 0.5) * 0.5; }
int index_from_r(double r, double rlo) { return (int)((r - rlo) * 2 + 1e-14); }
int index_from_z(double z, double zlo) { return (int)((z - zlo) * 0.5 + 1e-14); }
int getTotalHarmonics(int harmonicStages) { return 1 << (harmonicStages - 1); }

SubharmonicInfo* createSubharmonicInfo(int stages, int zhi) {
    g_cs.status = ACCEL_OK;
    if (stages < 1 || stages > kMaxStages || zhi < 0) {
        fail(ACCEL_ERR_INVALID, "createSubharmonicInfo: bad stages or zhi");
        return nullptr;
    }
    const int nh = getTotalHarmonics(stages), U = g_cs.uselen;
    SubharmonicInfo* shi = (SubharmonicInfo*)std::calloc(nh, sizeof(SubharmonicInfo));
    std::vector<BankHarmDev> hd(nh);
    std::vector<float2*> folds(nh, nullptr);
    int n = 0, tb = 0, rmax = 0;
    bool ok = true;
    for (int st = 0; st < stages && ok; st++) {
        const int maxh = st < 1 ? 1 : (1 << st);
        for (int h = 1; h <= maxh && ok; h += 2, n++) {
            SubharmonicInfo& s = shi[n];
            s.maxHarmonic = (unsigned short)maxh;
            s.currentHarmonic = (unsigned short)h;
            s.zmax = required_z(h, maxh, zhi);
            s.totalKernelsTemplates = (unsigned short)((s.zmax / kDz) * 2 + 1);
            const long long L = next_pow2((long long)(U * h) / maxh + 2 +
                                          2 * kNumBetween * z_halfwidth((double)required_z(h, maxh, zhi)));
            if (L < 2 * kMinM || L > 4 * kMaxM) {
                fail(ACCEL_ERR_UNSUPPORTED, "createSubharmonicInfo: FFT length outside 128..32768");
                ok = false;
                break;
            }
            s.kernelFFTLength = (int)L;
            s.z = (int*)std::malloc(sizeof(int) * s.totalKernelsTemplates);
            s.kernelHalfWidth = (unsigned short*)std::malloc(sizeof(unsigned short) * s.totalKernelsTemplates);
            for (int j = 0; j < s.totalKernelsTemplates; j++) {
                s.z[j] = -s.zmax + j * kDz;
                s.kernelHalfWidth[j] = (unsigned short)z_halfwidth((double)s.z[j]);
            }
            BankHarmDev& b = hd[n];
            b.harmnum = h;
            b.maxharm = maxh;
            b.zmax = s.zmax;
            b.numzs = s.totalKernelsTemplates;
            b.M = (int)(L / 2);
            b.hw0 = s.kernelHalfWidth[0];
            b.zlo = required_z(h, maxh, -zhi);
            b.tpl_base = tb;
            tb += b.numzs;
            rmax = std::max(rmax, 4 * b.hw0);
            cudaError_t e = cudaMalloc(&s.kernels_data, sizeof(float2) * L * b.numzs);
            if (e == cudaSuccess) e = cudaMalloc(&folds[n], sizeof(float2) * L * b.numzs);
            if (e != cudaSuccess) {
                fail(ACCEL_ERR_NOMEM, "createSubharmonicInfo: template bank", e);
                ok = false;
                break;
            }
            b.kstd = reinterpret_cast<float2*>(s.kernels_data);
            b.fold = folds[n];
        }
    }
    BankHarmDev* d_hd = nullptr;
    float2* resp = nullptr;
    if (ok) {
        cudaError_t e = cudaMalloc(&d_hd, sizeof(BankHarmDev) * nh);
        if (e == cudaSuccess) e = cudaMemcpy(d_hd, hd.data(), sizeof(BankHarmDev) * nh, cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaMalloc(&resp, sizeof(float2) * (size_t)tb * rmax);
        if (e == cudaSuccess) e = cudaMemset(resp, 0, sizeof(float2) * (size_t)tb * rmax);
        if (e != cudaSuccess) {
            fail(ACCEL_ERR_CUDA, "createSubharmonicInfo", e);
            ok = false;
        } else if (launch_bank_build(d_hd, hd.data(), nh, tb, resp, rmax, false, 0) != 0 ||
                   cudaStreamSynchronize(0) != cudaSuccess) {
            fail(ACCEL_ERR_CUDA, "createSubharmonicInfo: bank kernels", cudaGetLastError());
            ok = false;
        }
    }
    cudaFree(resp);
    cudaFree(d_hd);
    for (float2* f : folds) cudaFree(f);
    if (!ok) {
        freeSubharmonicInfo(shi, nh);
        return nullptr;
    }
    return shi;
}

void freeSubharmonicInfo(SubharmonicInfo* shi, int nh) {
    if (!shi) return;
    for (int h = 0; h < nh; h++) {
        std::free(shi[h].z);
        std::free(shi[h].kernelHalfWidth);
        cudaFree(shi[h].kernels_data);
    }
    std::free(shi);
}

// readData (bpd_data.c:9-75): the file's float32 samples behind
// kDatPadding zero samples, with as many zeros after them; *output_data
// points at the first sample.  The reference exits on a missing, empty or
// longer-than-2^26-sample file; here it returns 0 with the status set.
constexpr long kDatPadding = 2000;       // ACCEL_PADDING, bpd_common.h:35
constexpr long kDatMaxSamples = 1L << 26;
long readData(char* path, float** output_data) {
    g_cs.status = ACCEL_OK;
    if (!path || !output_data) {
        fail(ACCEL_ERR_INVALID, "readData: null argument");
        return 0;
    }
    *output_data = nullptr;
    FILE* f = std::fopen(path, "rb");
    if (!f) {
        fail(ACCEL_ERR_INVALID, "readData: cannot open the file");
        return 0;
    }
    long n = -1;
    if (std::fseek(f, 0, SEEK_END) == 0) {
        const long bytes = std::ftell(f);
        if (bytes >= 0) n = bytes / (long)sizeof(float);
    }
    if (n <= 0 || n > kDatMaxSamples) {
        std::fclose(f);
        fail(ACCEL_ERR_INVALID, n <= 0 ? "readData: empty or unreadable file"
                                       : "readData: the time series is longer than 2^26 samples");
        return 0;
    }
    float* buf = (float*)std::calloc((size_t)(n + 2 * kDatPadding), sizeof(float));
    if (!buf) {
        std::fclose(f);
        fail(ACCEL_ERR_NOMEM, "readData: host allocation");
        return 0;
    }
    const bool ok = std::fseek(f, 0, SEEK_SET) == 0 &&
                    std::fread(buf + kDatPadding, sizeof(float), (size_t)n, f) == (size_t)n;
    std::fclose(f);
    if (!ok) {
        std::free(buf);
        fail(ACCEL_ERR_INVALID, "readData: reading the file");
        return 0;
    }
    *output_data = buf + kDatPadding;
    return n;
}

void freeData(float* data) {
    if (data) std::free(data - kDatPadding);
}

unsigned realToComplexFFT(float* idata, long n, accel_complex** odata, int batch) {
    g_cs.status = ACCEL_OK;
    if (!idata || !odata || n < 2 || batch < 1) {
        fail(ACCEL_ERR_INVALID, "realToComplexFFT: bad argument");
        return 0;
    }
    const long nout = n / 2 + 1;
    float* d_in = nullptr;
    cufftComplex* d_out = nullptr;
    cudaError_t e = cudaMalloc(&d_in, sizeof(float) * n * batch);
    if (e == cudaSuccess) e = cudaMalloc(&d_out, sizeof(cufftComplex) * nout * batch);
    if (e == cudaSuccess) e = cudaMemcpy(d_in, idata, sizeof(float) * n * batch, cudaMemcpyHostToDevice);
    cufftHandle plan = 0;
    bool ok = e == cudaSuccess;
    if (!ok) fail(ACCEL_ERR_CUDA, "realToComplexFFT", e);
    if (ok && cufftPlan1d(&plan, (int)n, CUFFT_R2C, batch) != CUFFT_SUCCESS) ok = !fail(ACCEL_ERR_CUDA, "realToComplexFFT: plan");
    if (ok && cufftExecR2C(plan, d_in, d_out) != CUFFT_SUCCESS) ok = !fail(ACCEL_ERR_CUDA, "realToComplexFFT: exec");
    accel_complex* host = nullptr;
    if (ok) {
        host = (accel_complex*)std::malloc(sizeof(accel_complex) * nout * batch);
        e = cudaMemcpy(host, d_out, sizeof(cufftComplex) * nout * batch, cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) {
            fail(ACCEL_ERR_CUDA, "realToComplexFFT: copy", e);
            std::free(host);
            host = nullptr;
            ok = false;
        }
    }
    if (plan) cufftDestroy(plan);
    cudaFree(d_in);
    cudaFree(d_out);
    *odata = host;
    return ok ? (unsigned)nout : 0;
}

static unsigned c2c(accel_complex* din, unsigned L, accel_complex** dout, int batch, bool inverse) {
    g_cs.status = ACCEL_OK;
    if (!din || !dout || batch < 1) {
        fail(ACCEL_ERR_INVALID, "complexToComplexFFT: bad argument");
        return 0;
    }
    std::lock_guard<std::mutex> lk(g_cs.mu);
    if (!ensure_twiddles()) {
        fail(ACCEL_ERR_CUDA, "complexToComplexFFT: twiddles", cudaGetLastError());
        return 0;
    }
    float2* out = nullptr;
    cudaError_t e = cudaMalloc(&out, sizeof(float2) * (size_t)L * batch);
    if (e != cudaSuccess) {
        fail(ACCEL_ERR_NOMEM, "complexToComplexFFT", e);
        return 0;
    }
    const float2* in = reinterpret_cast<const float2*>(din);
    int rc = inverse ? fft_long<+1>(in, L, out, L, (int)L, batch) : fft_long<-1>(in, L, out, L, (int)L, batch);
    if (rc != 0 || cudaStreamSynchronize(0) != cudaSuccess) {
        fail(rc == -2 ? ACCEL_ERR_UNSUPPORTED : ACCEL_ERR_CUDA, "complexToComplexFFT: transform");
        cudaFree(out);
        return 0;
    }
    *dout = reinterpret_cast<accel_complex*>(out);
    return L;
}

unsigned complexToComplexFFT(accel_complex* din, unsigned int L, accel_complex** dout, int batch) {
    return c2c(din, L, dout, batch, false);
}
unsigned inverseComplexToComplexFFT(accel_complex* din, unsigned int L, accel_complex** dout, int batch) {
    return c2c(din, L, dout, batch, true);
}

void deredden(accel_complex* fft, unsigned numbins) {
    g_cs.status = ACCEL_OK;
    if (!fft || numbins < 8 || (long long)numbins > kMaxWhitenBins) {
        fail(ACCEL_ERR_INVALID, "deredden: bad argument (numbins must be in [8, 2^31 - 1])");
        return;
    }
    auto blocks = plan_whiten_blocks(numbins, 6, 200);  // bpd_noise.c:14 widths
    const int nb = (int)blocks.size();
    std::vector<int> s(nb), l(nb);
    int maxlen = 0;
    for (int i = 0; i < nb; i++) {
        s[i] = blocks[i].first;
        l[i] = blocks[i].second;
        maxlen = std::max(maxlen, l[i]);
    }
    float2* d = nullptr;
    int* ds = nullptr;
    int* dl = nullptr;
    double* dm = nullptr;
    cudaError_t e = cudaMalloc(&d, sizeof(float2) * numbins);
    if (e == cudaSuccess) e = cudaMalloc(&ds, sizeof(int) * nb);
    if (e == cudaSuccess) e = cudaMalloc(&dl, sizeof(int) * nb);
    if (e == cudaSuccess) e = cudaMalloc(&dm, sizeof(double) * nb);
    if (e == cudaSuccess) e = cudaMemcpy(d, fft, sizeof(float2) * numbins, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(ds, s.data(), sizeof(int) * nb, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(dl, l.data(), sizeof(int) * nb, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        fail(ACCEL_ERR_CUDA, "deredden", e);
    } else if (launch_whiten(ds, dl, nb, dm, d, numbins, maxlen, 0) != 0) {
        fail(ACCEL_ERR_CUDA, "deredden: launch", cudaGetLastError());
    } else {
        e = cudaMemcpy(fft, d, sizeof(float2) * numbins, cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) fail(ACCEL_ERR_CUDA, "deredden: copy", e);
    }
    cudaFree(d);
    cudaFree(ds);
    cudaFree(dl);
    cudaFree(dm);
}

void generate_harmonics_ffdot(unsigned short totalHarmonics, unsigned short harmonicStages,
                              SubharmonicInfo* shi, double fullrlo, double fullrhi, double zlo,
                              ffdotInfo* out, unsigned short* binOffsets) {
    // bpd_search.cu:72-127, serially (the reference's OpenMP loop races on
    // its harmonic counter)
    unsigned short counter = 0;
    for (int st = 0; st < harmonicStages; st++) {
        const int maxh = st < 1 ? 1 : (1 << st);
        for (int h = 1; h <= maxh && counter < totalHarmonics; h += 2, counter++) {
            const double f = (double)h / (double)maxh;
            const double drlo = calc_required_r(f, fullrlo);
            const double drhi = calc_required_r(f, fullrhi);
            ffdotInfo& o = out[counter];
            o.currentHarmonic = (unsigned short)h;
            o.maxHarmonic = (unsigned short)maxh;
            o.rlo = (int)std::floor(drlo);
            o.rhi = drhi;
            o.zlo = calc_required_z(f, zlo);
            if (h == 1 && maxh == 1) {
                o.numrs = g_cs.uselen;
            } else {
                o.numrs = (int)((std::ceil(drhi) - std::floor(drlo)) * 2 + 1e-14) + 1;
                if (o.numrs % 2) o.numrs = (o.numrs / 2 + 1) * 2;
            }
            o.numzs = shi[counter].totalKernelsTemplates;
            o.fftlen = shi[counter].kernelFFTLength;
            binOffsets[counter] = shi[counter].kernelHalfWidth[0];
        }
    }
}

void generate_harmonic_ffdot_data(unsigned short totalHarmonics, long totalDataLength, ffdotInfo* ffdot,
                                  unsigned short* binoffset, long* dataStartIdx, accel_complex* fft,
                                  long dataNumbins, long dataLoBin, accel_complex* output) {
    // bpd_search.cu:130-184 with get_fourier_amplitudes (:16-47) and
    // spreadData (:56-67)
    g_cs.status = ACCEL_OK;
    (void)totalDataLength;
    for (int h = 0; h < totalHarmonics; h++) {
        const int bo = binoffset[h];
        const int lobin = ffdot[h].rlo - bo;
        const int hibin = (int)std::ceil(ffdot[h].rhi) + bo;
        const int numdata = hibin - lobin + 1;
        const int nice = (int)next_pow2(numdata);
        const int half = ffdot[h].fftlen / kNumBetween;
        if (nice != half) {
            fail(ACCEL_ERR_INVALID, "generate_harmonic_ffdot_data: segment does not fit fftlen/2");
            return;
        }
        std::vector<accel_complex> amp(nice);
        for (int t = 0; t < nice; t++) {
            const long b = (long)lobin + t - dataLoBin;
            amp[t] = (b >= 0 && b < dataNumbins) ? fft[b] : accel_complex{0.f, 0.f};
        }
        std::vector<float> pw(numdata);
        for (int t = 0; t < numdata; t++) {
            volatile float a = amp[t].x * amp[t].x;
            volatile float b = amp[t].y * amp[t].y;
            pw[t] = a + b;
        }
        std::nth_element(pw.begin(), pw.begin() + (numdata - 1) / 2, pw.end());
        const double nc = rsqrt_magic_host((float)(pw[(numdata - 1) / 2] / std::log(2.0)));
        for (int t = 0; t < numdata; t++) {
            amp[t].x = (float)(amp[t].x * nc);
            amp[t].y = (float)(amp[t].y * nc);
        }
        accel_complex* o = output + dataStartIdx[h];
        std::memset(o, 0, sizeof(accel_complex) * (size_t)half * kNumBetween);
        for (int t = 0; t < half; t++) o[kNumBetween * t] = amp[t];
    }
}

void initialize_cuda_plans(unsigned short totalHarmonics, SubharmonicInfo* shi) {
    std::lock_guard<std::mutex> lk(g_cs.mu);
    g_cs.status = ACCEL_OK;
    g_cs.fftlen.assign(totalHarmonics, 0);
    g_cs.numzs.assign(totalHarmonics, 0);
    for (int h = 0; h < totalHarmonics; h++) {
        g_cs.fftlen[h] = shi[h].kernelFFTLength;
        g_cs.numzs[h] = shi[h].totalKernelsTemplates;
    }
    if (!ensure_twiddles()) fail(ACCEL_ERR_CUDA, "initialize_cuda_plans: twiddles", cudaGetLastError());
}

void free_cuda_plans(unsigned short totalHarmonics) {
    (void)totalHarmonics;
    std::lock_guard<std::mutex> lk(g_cs.mu);
    g_cs.fftlen.clear();
    g_cs.numzs.clear();
    g_cs.status = ACCEL_OK;
}

void perform_fft_harmonics(unsigned short nh, accel_complex* d_data, long* start, accel_complex* d_out) {
    g_cs.status = ACCEL_OK;
    if ((int)g_cs.fftlen.size() < nh) {
        fail(ACCEL_ERR_INVALID, "perform_fft_harmonics: initialize_cuda_plans first");
        return;
    }
    for (int h = 0; h < nh; h++) {
        const int L = g_cs.fftlen[h];
        int rc = fft_long<-1>(reinterpret_cast<const float2*>(d_data + start[h]), L,
                              reinterpret_cast<float2*>(d_out + start[h]), L, L, 1);
        if (rc) {
            fail(rc == -2 ? ACCEL_ERR_UNSUPPORTED : ACCEL_ERR_CUDA, "perform_fft_harmonics");
            return;
        }
    }
}

void perform_convolution(unsigned short nh, accel_complex* d_fft, ffdotInfo* hi, SubharmonicInfo* shi,
                         long* start, accel_complex* d_out, long* convIdx) {
    g_cs.status = ACCEL_OK;
    for (int h = 0; h < nh; h++) {
        const long long n = (long long)hi[h].numzs * hi[h].fftlen;
        k_conv<<<grid_for(n), 256>>>(hi[h].numzs, hi[h].fftlen, reinterpret_cast<const float2*>(d_fft + start[h]),
                                     reinterpret_cast<const float2*>(shi[h].kernels_data),
                                     reinterpret_cast<float2*>(d_out + convIdx[h]));
        if (cudaGetLastError() != cudaSuccess) {
            fail(ACCEL_ERR_CUDA, "perform_convolution");
            return;
        }
    }
}

void perform_inversefft(unsigned short nh, accel_complex* d_conv, long* convIdx, accel_complex* d_out) {
    g_cs.status = ACCEL_OK;
    if ((int)g_cs.fftlen.size() < nh) {
        fail(ACCEL_ERR_INVALID, "perform_inversefft: initialize_cuda_plans first");
        return;
    }
    for (int h = 0; h < nh; h++) {
        const int L = g_cs.fftlen[h];
        int rc = fft_long<+1>(reinterpret_cast<const float2*>(d_conv + convIdx[h]), L,
                              reinterpret_cast<float2*>(d_out + convIdx[h]), L, L, g_cs.numzs[h]);
        if (rc) {
            fail(rc == -2 ? ACCEL_ERR_UNSUPPORTED : ACCEL_ERR_CUDA, "perform_inversefft");
            return;
        }
    }
}

void generate_fundamental_powers(unsigned short nh, accel_complex* d_ifft, long* idx, ffdotInfo* hi,
                                 SubharmonicInfo* shi, float* d_powers) {
    (void)nh;
    g_cs.status = ACCEL_OK;
    const int off = shi[0].kernelHalfWidth[0] * kNumBetween;
    const float scale = (float)(1.0 / ((double)hi[0].fftlen * hi[0].fftlen));
    const long long n = (long long)hi[0].numzs * hi[0].numrs;
    k_powers<<<grid_for(n), 256>>>(hi[0].numzs, hi[0].numrs, hi[0].fftlen,
                                   reinterpret_cast<const float2*>(d_ifft + idx[0] + off), scale, d_powers);
    if (cudaGetLastError() != cudaSuccess) fail(ACCEL_ERR_CUDA, "generate_fundamental_powers");
    g_cs.last_powers = d_powers;
    g_cs.last_numzs = hi[0].numzs;
    g_cs.last_numrs = hi[0].numrs;
}

void perform_harmonic_summing(unsigned short nh, accel_complex* d_ifft, long* idx, ffdotInfo* hi,
                              SubharmonicInfo* shi, float* d_powers, int fullrlo, unsigned short* host_rinds,
                              unsigned short* device_rinds, int totalRindsBins) {
    (void)host_rinds;
    (void)device_rinds;
    (void)totalRindsBins;
    g_cs.status = ACCEL_OK;
    for (int h = 1; h < nh; h++) {
        const int off = shi[h].kernelHalfWidth[0] * kNumBetween;
        const float scale = (float)(1.0 / ((double)hi[h].fftlen * hi[h].fftlen));
        const long long n = (long long)hi[0].numzs * hi[0].numrs;
        k_addpowers<<<grid_for(n), 256>>>(hi[0].numzs, hi[0].numrs, hi[h].fftlen, hi[0].zlo, hi[h].zlo,
                                          hi[h].rlo, hi[h].currentHarmonic, hi[h].maxHarmonic,
                                          reinterpret_cast<const float2*>(d_ifft + idx[h] + off), scale,
                                          d_powers, (long long)fullrlo);
        if (cudaGetLastError() != cudaSuccess) {
            fail(ACCEL_ERR_CUDA, "perform_harmonic_summing");
            return;
        }
    }
    g_cs.last_powers = d_powers;
    g_cs.last_numzs = hi[0].numzs;
    g_cs.last_numrs = hi[0].numrs;
}

Candidates* search_ffdot_powers_n(ffdotInfo* ffdot, int numharm, float powcut, long long numindep,
                                  long* ncand) {
    g_cs.status = ACCEL_OK;
    if (!ffdot || !ncand || !g_cs.last_powers) {
        fail(ACCEL_ERR_INVALID, "search_ffdot_powers: no power plane yet");
        return nullptr;
    }
    const long long cap = *ncand > 0 ? *ncand : 1 << 20;
    RawHit* d_hits = nullptr;
    unsigned long long* d_n = nullptr;
    cudaError_t e = cudaMalloc(&d_hits, sizeof(RawHit) * cap);
    if (e == cudaSuccess) e = cudaMalloc(&d_n, sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMemset(d_n, 0, sizeof(unsigned long long));
    if (e != cudaSuccess) {
        fail(ACCEL_ERR_NOMEM, "search_ffdot_powers", e);
        cudaFree(d_hits);
        cudaFree(d_n);
        return nullptr;
    }
    const long long tot = (long long)g_cs.last_numzs * g_cs.last_numrs;
    k_threshold<<<grid_for(tot), 256>>>(g_cs.last_numzs, g_cs.last_numrs, g_cs.last_powers, powcut, d_hits,
                                        d_n, cap);
    unsigned long long n = 0;
    e = cudaMemcpy(&n, d_n, sizeof(n), cudaMemcpyDeviceToHost);
    const long long keep = std::min<long long>((long long)n, cap);
    std::vector<RawHit> hits(keep);
    if (e == cudaSuccess && keep > 0)
        e = cudaMemcpy(hits.data(), d_hits, sizeof(RawHit) * keep, cudaMemcpyDeviceToHost);
    cudaFree(d_hits);
    cudaFree(d_n);
    if (e != cudaSuccess) {
        fail(ACCEL_ERR_CUDA, "search_ffdot_powers", e);
        return nullptr;
    }
    std::sort(hits.begin(), hits.end(), [](const RawHit& a, const RawHit& b) {
        return a.z != b.z ? a.z < b.z : a.i < b.i;
    });
    Candidates* out = (Candidates*)std::calloc(keep > 0 ? keep : 1, sizeof(Candidates));
    for (long long k = 0; k < keep; k++) {
        Candidates& c = out[k];
        c.power = hits[k].power;
        c.numharm = numharm;
        c.r = ffdot[0].rlo + 0.5 * hits[k].i;
        c.z = ffdot[0].zlo + (double)kDz * hits[k].z;
        c.sigma = (float)accel_sigma_of_power(hits[k].power, numharm, (double)numindep);
    }
    *ncand = (long)keep;
    if ((long long)n > cap) fail(ACCEL_ERR_CAPACITY, "search_ffdot_powers: more candidates than requested");
    return out;
}

Candidates* search_ffdot_powers(ffdotInfo* ffdot, int numharm, float powcut, long long numindep,
                                Candidates* cands) {
    (void)cands;
    long n = 0;
    return search_ffdot_powers_n(ffdot, numharm, powcut, numindep, &n);
}

// ---- bpd_gpu_kernels.cuh:15-17: the reference's three kernels as host
// launchers with the same names and arguments (a __global__ symbol cannot
// cross a C ABI): each covers the whole range its reference launch covers,
// on the legacy default stream.
void convolveSignal(int kernelTotalNumzs, int fftlen, accel_complex* data, accel_complex* kernels,
                    int kernelTemplateLength, accel_complex* outputdata) {
    (void)kernelTemplateLength;  // unused by the reference kernel as well
    g_cs.status = ACCEL_OK;
    const long long n = (long long)kernelTotalNumzs * fftlen;
    if (n <= 0) return;
    k_conv<<<grid_for(n), 256>>>(kernelTotalNumzs, fftlen, reinterpret_cast<const float2*>(data),
                                 reinterpret_cast<const float2*>(kernels), reinterpret_cast<float2*>(outputdata));
    if (cudaGetLastError() != cudaSuccess) fail(ACCEL_ERR_CUDA, "convolveSignal");
}

void generatePowers(int kernelTotalNumzs, int numrs, int fftlen, accel_complex* data, float scale,
                    float* outputdata) {
    g_cs.status = ACCEL_OK;
    const long long n = (long long)kernelTotalNumzs * numrs;
    if (n <= 0) return;
    k_powers<<<grid_for(n), 256>>>(kernelTotalNumzs, numrs, fftlen, reinterpret_cast<const float2*>(data), scale,
                                   outputdata);
    if (cudaGetLastError() != cudaSuccess) fail(ACCEL_ERR_CUDA, "generatePowers");
}

void addPowers(int fundamental_numzs, int fundamental_numrs, int subharm_fftlen, int fundamental_zlo,
               int subharm_zlo, int subharm_rlo, double harmonicFraction, accel_complex* data, float scale,
               float* output_powers, int fullrlo) {
    g_cs.status = ACCEL_OK;
    // the kernel's index arithmetic is exact for harmonicFraction = p / 2^k
    // (every fraction the reference's bank uses)
    int p = -1, q = 1;
    for (int k = 0; k <= 16 && p < 0; k++, q <<= 1) {
        const double v = harmonicFraction * q;
        if (v == std::floor(v) && v >= 1.0 && v <= q) p = (int)v;
    }
    q >>= 1;
    if (p < 0) {
        fail(ACCEL_ERR_INVALID, "addPowers: harmonicFraction is not p / 2^k in (0, 1]");
        return;
    }
    const long long n = (long long)fundamental_numzs * fundamental_numrs;
    if (n <= 0) return;
    k_addpowers<<<grid_for(n), 256>>>(fundamental_numzs, fundamental_numrs, subharm_fftlen, fundamental_zlo,
                                      subharm_zlo, subharm_rlo, p, q, reinterpret_cast<const float2*>(data), scale,
                                      output_powers, (long long)fullrlo);
    if (cudaGetLastError() != cudaSuccess) fail(ACCEL_ERR_CUDA, "addPowers");
}

// ------------------------------------------ bpd_math.h, app_utilities.h
float fast_median(float arr[], int n) {
    if (!arr || n <= 0) return 0.f;
    // the order statistic of rank (n - 1) / 2, input reordered around it
    std::nth_element(arr, arr + (n - 1) / 2, arr + n);
    return arr[(n - 1) / 2];
}

float inverse_square_root(float x) { return rsqrt_magic_host(x); }

int fast_log2(int n) {
    int x = 0;
    for (; n > 1; n >>= 1) x++;
    return x;
}

int toNearestInt(double x) { return nearest_int(x); }

long long get2PowerNGreaterThan(long long x) {
    long long p = 1;
    while (p < x && p < (1LL << 62)) p <<= 1;
    return p;
}

void logMessage(const char* message, ...) {
    va_list ap;
    va_start(ap, message);
    vprintf(message, ap);
    va_end(ap);
    printf("\n");
}

void throwError(const char* errorMessage, ...) {
    va_list ap;
    va_start(ap, errorMessage);
    vprintf(errorMessage, ap);
    va_end(ap);
    printf("\n");
    exit(EXIT_FAILURE);
}

}  // extern "C"
