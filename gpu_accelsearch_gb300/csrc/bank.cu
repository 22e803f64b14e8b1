// bank.cu -- f-dot template bank, built on the GPU in double precision.
//
// Restates createSubharmonicInfo / initializeSubharmonicInfo
// (bpd_subharmonics.cu:233-354), generate_z_response (:146-226),
// generate_r_response (:78-135) and the Cephes Fresnel integrals the
// reference uses (bpd_fresnl.c:3-200).  The reference computes responses in
// double on the host, stores them as float, and FFTs them with cuFFT in
// single precision; here the responses are computed in double on the
// device, rounded to float as the reference stores them, and transformed
// by an exact-support DFT in double precision.
//
// This translation unit is compiled with -fmad=false so that double
// expressions round operation by operation like the reference's host code.
//
// Outputs per harmonic h (numzs_h templates of length L_h = 2 M_h):
//   kstd[z][0..L)   the template spectrum K = FFT_L(k) (forward, unnormalised)
//   fold[z][0..M)   A[k] / L, A[k] = conj K[k] + conj K[k+M]
//   fold[z][M..2M)  B[k] / L, B[k] = (conj K[k] - conj K[k+M]) exp(+2 pi i k / L)
// so that, for segment data repeated with period M (spread x2), the inverse
// L-point transform of D.conj(K) has even outputs IFFT_M(D.A) and odd
// outputs IFFT_M(D.B).
#include "accel_internal.h"

namespace accel {

// Cephes fresnl coefficient tables (S. L. Moshier, Cephes Math Library).
__constant__ double c_sn[6] = {-2.99181919401019853726E3, 7.08840045257738576863E5,
    -6.29741486205862506537E7, 2.54890880573376359104E9, -4.42979518059697779103E10,
    3.18016297876567817986E11};
__constant__ double c_sd[6] = {2.81376268889994315696E2, 4.55847810806532581675E4,
    5.17343888770096400730E6, 4.19320245898111231129E8, 2.24411795645340920940E10,
    6.07366389490084639049E11};
__constant__ double c_cn[6] = {-4.98843114573573548651E-8, 9.50428062829859605134E-6,
    -6.45191435683965050962E-4, 1.88843319396703850064E-2, -2.05525900955013891793E-1,
    9.99999999999999998822E-1};
__constant__ double c_cd[7] = {3.99982968972495980367E-12, 9.15439215774657478799E-10,
    1.25001862479598821474E-7, 1.22262789024179030997E-5, 8.68029542941784300606E-4,
    4.12142090722199792936E-2, 1.00000000000000000118E0};
__constant__ double c_fn[10] = {4.21543555043677546506E-1, 1.43407919780758885261E-1,
    1.15220955073585758835E-2, 3.45017939782574027900E-4, 4.63613749287867322088E-6,
    3.05568983790257605827E-8, 1.02304514164907233465E-10, 1.72010743268161828879E-13,
    1.34283276233062758925E-16, 3.76329711269987889006E-20};
__constant__ double c_fd[10] = {7.51586398353378947175E-1, 1.16888925859191382142E-1,
    6.44051526508858611005E-3, 1.55934409164153020873E-4, 1.84627567348930545870E-6,
    1.12699224763999035261E-8, 3.60140029589371370404E-11, 5.88754533621578410010E-14,
    4.52001434074129701496E-17, 1.25443237090011264384E-20};
__constant__ double c_gn[11] = {5.04442073643383265887E-1, 1.97102833525523411709E-1,
    1.87648584092575249293E-2, 6.84079380915393090172E-4, 1.15138826111884280931E-5,
    9.82852443688422223854E-8, 4.45344415861750144738E-10, 1.08268041139020870318E-12,
    1.37555460633261799868E-15, 8.36354435630677421531E-19, 1.86958710162783235106E-22};
__constant__ double c_gd[11] = {1.47495759925128324529E0, 3.37748989120019970451E-1,
    2.53603741420338795122E-2, 8.14679107184306179049E-4, 1.27545075667729118702E-5,
    1.04314589657571990585E-7, 4.60680728146520428211E-10, 1.10273215066240270757E-12,
    1.38796531259578871258E-15, 8.39158816283118707363E-19, 1.86958710162783236342E-22};

constexpr double kPi = 3.14159265358979323846264338327950288;
constexpr double kSqrt2 = 1.41421356237309504880168872420969808;
constexpr double kPiBy2 = 1.57079632679489661923132169163975144;

__device__ double horner(double x, const double* c, int deg) {
    double acc = c[0];
    for (int k = 1; k <= deg; ++k) acc = acc * x + c[k];
    return acc;
}
__device__ double horner1(double x, const double* c, int deg) {
    double acc = x + c[0];
    for (int k = 1; k < deg; ++k) acc = acc * x + c[k];
    return acc;
}

__device__ void fresnel(double xa, double* ss, double* cc) {
    double x = fabs(xa), x2 = x * x, s, c;
    if (x2 < 2.5625) {
        double t = x2 * x2;
        s = x * x2 * horner(t, c_sn, 5) / horner1(t, c_sd, 6);
        c = x * horner(t, c_cn, 5) / horner(t, c_cd, 6);
    } else if (x > 36974.0) {
        c = 0.5;
        s = 0.5;
    } else {
        x2 = x * x;
        double t = kPi * x2;
        double u = 1.0 / (t * t);
        t = 1.0 / t;
        double f = 1.0 - u * horner(u, c_fn, 9) / horner1(u, c_fd, 10);
        double g = t * horner(u, c_gn, 10) / horner1(u, c_gd, 11);
        t = kPiBy2 * x2;
        double ct = cos(t), st = sin(t);
        t = kPi * x;
        c = 0.5 + (f * st - g * ct) / t;
        s = 0.5 - (f * ct + g * st) / t;
    }
    if (xa < 0.0) { c = -c; s = -s; }
    *cc = c;
    *ss = s;
}

// One CTA per template.  Writes the 4*hw response points (float, as the
// reference stores them) into resp[tpl * rstride ...].
__global__ void k_template_response(const BankHarmDev* __restrict__ hd, int nh, float2* resp,
                                    int rstride) {
    int tpl = blockIdx.x;
    int h = 0;
    while (h + 1 < nh && tpl >= hd[h + 1].tpl_base) h++;
    int j = tpl - hd[h].tpl_base;
    int z = -hd[h].zmax + j * kDz;
    int hw = z_halfwidth((double)z);
    int numkern = 2 * kNumBetween * hw;
    float2* out = resp + (size_t)tpl * rstride;
    if (z == 0) {
        // generate_r_response(0, 2, numkern): a serial recurrence; one thread.
        if (threadIdx.x == 0) {
            double startr = kPi * (numkern / (double)(2 * kNumBetween));
            double delta = -kPi / kNumBetween;
            double tmp = sin(0.5 * delta);
            double alpha = -2.0 * tmp * tmp;
            double beta = sin(delta);
            double c = cos(startr), s = sin(startr), r = startr;
            for (int i = 0; i < numkern; i++, r += delta) {
                double sinc = (r == 0.0) ? 1.0 : s / r;
                out[i] = make_float2((float)(c * sinc), (float)(s * sinc));
                tmp = c;
                c = alpha * tmp - beta * s + c;
                s = alpha * s + beta * tmp + s;
            }
            out[numkern / 2] = make_float2(1.0f, 0.0f);  // roffset = 0 correction
        }
        return;
    }
    double absz = fabs((double)z);
    double startr = -(0.5 * z);
    int signz = (z < 0) ? -1 : 1;
    double zd = signz * kSqrt2 / sqrt(absz);
    double cons = zd / 2.0;
    double pibyz = kPi / z;
    startr += numkern / (double)(2 * kNumBetween);
    // r advances by -1/numbetween per point; startr is an integer here, so
    // the reference's running sum is exact and r_i = startr - i/2.
    for (int i = threadIdx.x; i < numkern; i += blockDim.x) {
        double r = startr - 0.5 * i;
        double yy = r * zd;
        double zz = yy + z * zd;
        double xx = pibyz * r * r;
        double c = cos(xx), s = sin(xx);
        double fsy, fcy, fsz, fcz;
        fresnel(yy, &fsy, &fcy);
        fresnel(zz, &fsz, &fcz);
        double tre = signz * (fcz - fcy);
        double tim = fsy - fsz;
        out[i] = make_float2((float)((tre * c - tim * s) * cons), (float)(-(tre * s + tim * c) * cons));
    }
}

// Exact-support DFT.  The wrapped template of length L has the upper half
// of the response at [0, 2hw) and the lower half at [L-2hw, L).  For
// k < M:  Se = sum_{t even} k_t w^t,  So = sum_{t odd} k_t w^t,
// w = exp(-2 pi i k / L);  K[k] = Se + So, K[k+M] = Se - So,
// A[k] = 2 conj(Se), B[k] = 2 conj(So w).
__global__ void k_template_dft(const BankHarmDev* __restrict__ hd, int nh, const float2* resp,
                               int rstride) {
    int tpl = blockIdx.y;
    int h = 0;
    while (h + 1 < nh && tpl >= hd[h + 1].tpl_base) h++;
    const BankHarmDev H = hd[h];
    int j = tpl - H.tpl_base;
    int z = -H.zmax + j * kDz;
    int hw2 = 2 * z_halfwidth((double)z);  // points per half
    const int L = 2 * H.M;
    extern __shared__ double2 s_k[];        // [2*hw2]: index = wrapped position order
    const float2* rr = resp + (size_t)tpl * rstride;
    for (int i = threadIdx.x; i < 2 * hw2; i += blockDim.x) {
        // wrapped t in [0, hw2) <- resp[hw2 + t];  t in [L-hw2, L) <- resp[t - (L-hw2)]
        float2 v = (i < hw2) ? rr[hw2 + i] : rr[i - hw2];
        s_k[i] = make_double2((double)v.x, (double)v.y);
    }
    __syncthreads();
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= H.M) return;
    double sw, cw;
    sincospi(-2.0 * k / L, &sw, &cw);  // w = exp(-2 pi i k / L)
    double ser = 0, sei = 0, sor = 0, soi = 0;
    // first run: t = 0 .. hw2-1 (even t first element)
    double pr = 1.0, pi = 0.0;
    for (int t = 0; t < hw2; t++) {
        double2 v = s_k[t];
        double xr = v.x * pr - v.y * pi, xi = v.x * pi + v.y * pr;
        if (t & 1) { sor += xr; soi += xi; } else { ser += xr; sei += xi; }
        double npr = pr * cw - pi * sw;
        pi = pr * sw + pi * cw;
        pr = npr;
    }
    // second run: t = L-hw2 .. L-1; w^(L-hw2) = exp(+2 pi i k hw2 / L)
    sincospi(2.0 * (double)((long long)k * hw2 % L) / L, &pi, &pr);
    for (int t = 0; t < hw2; t++) {
        double2 v = s_k[hw2 + t];
        double xr = v.x * pr - v.y * pi, xi = v.x * pi + v.y * pr;
        if ((L - hw2 + t) & 1) { sor += xr; soi += xi; } else { ser += xr; sei += xi; }
        double npr = pr * cw - pi * sw;
        pi = pr * sw + pi * cw;
        pr = npr;
    }
    float2* kstd = H.kstd + (size_t)j * L;
    kstd[k] = make_float2((float)(ser + sor), (float)(sei + soi));
    kstd[k + H.M] = make_float2((float)(ser - sor), (float)(sei - soi));
    // folded spectra scaled by 1/L (exact for a power of two), so that the
    // plane kernels' |y|^2 is already the normalised power |y / L|^2; a
    // short transform's fold is stored in decimated order
    const double inv_l = 1.0 / L;
    float2* fold = H.fold + (size_t)j * 2 * H.M;
    const int pk = decimated_pos(k, H.M, mixed_radix(H.M));
    fold[pk] = make_float2((float)(2.0 * ser * inv_l), (float)(-2.0 * sei * inv_l));
    // So * w, then conjugate, times 2
    double qr = sor * cw - soi * sw, qi = sor * sw + soi * cw;
    fold[H.M + pk] = make_float2((float)(2.0 * qr * inv_l), (float)(-2.0 * qi * inv_l));
}

// FP16 copy of the folded bank, scaled per template by its largest
// component so that every stored value lies in [-1, 1].
__global__ void k_fold_to_half(const BankHarmDev* __restrict__ hd, int nh) {
    int tpl = blockIdx.x;
    int h = 0;
    while (h + 1 < nh && tpl >= hd[h + 1].tpl_base) h++;
    const BankHarmDev H = hd[h];
    int j = tpl - H.tpl_base;
    const float2* f = H.fold + (size_t)j * 2 * H.M;
    __shared__ float s_max[32];
    float m = 0.f;
    for (int i = threadIdx.x; i < 2 * H.M; i += blockDim.x) {
        float2 v = f[i];
        m = fmaxf(m, fmaxf(fabsf(v.x), fabsf(v.y)));
    }
    for (int off = 16; off > 0; off >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, off));
    if ((threadIdx.x & 31) == 0) s_max[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x < 32) {
        int nw = blockDim.x >> 5;
        m = threadIdx.x < nw ? s_max[threadIdx.x] : 0.f;
        for (int off = 16; off > 0; off >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, off));
        if (threadIdx.x == 0) s_max[0] = m > 0.f ? m : 1.f;
    }
    __syncthreads();
    float sc = s_max[0], inv = 1.0f / sc;
    if (threadIdx.x == 0) H.fold16_scale[j] = sc;
    __half2* o = H.fold16 + (size_t)j * 2 * H.M;
    for (int i = threadIdx.x; i < 2 * H.M; i += blockDim.x) {
        float2 v = f[i];
        o[i] = __floats2half2_rn(v.x * inv, v.y * inv);
    }
}

// Entry i of the twiddle buffer: the table W^m (m < kTwN), then the packed
// per-pass sections (accel_common.cuh), each a copy of table entry m, then
// the radix-R sections of the short transforms.
__global__ void k_twiddles(float2* tw) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kTwAll) return;
    if (i >= kTwTotal) {  // the radix-R sections: exp(2 pi i g b / (R N2))
        int R = 5, n2 = kMixedMinN2;
        for (int r = 5; r <= 7; r++)
            for (int n = kMixedMinN2; n <= kMixedMaxN2; n *= 2)
                if (i >= tw_form_off(r, n)) R = r, n2 = n;
        const int j = i - tw_form_off(R, n2), g = j / n2 + 1, b = j % n2;
        double s, c;
        sincospi(2.0 * (double)(g * b) / (double)(R * n2), &s, &c);
        tw[i] = make_float2((float)c, (float)s);
        return;
    }
    int m = i;
    if (i >= kTwN + kTwFull256) {
        const int q = i - kTwN - kTwFull256, j = q / 16 + 1, k = q % 16;
        m = (j * k * (kTwN / 256)) & (kTwN - 1);
    } else if (i >= kTwN) {
        const int p = i - kTwN;
        const int nrs[7] = {64, 128, 256, 512, 1024, 2048, 4096};
        int NR = 64;
        for (int j = 0; j < 7; j++)
            if (p >= tw_pack_off(nrs[j])) NR = nrs[j];
        const int q = p - tw_pack_off(NR), k = q >> 2, slot = q & 3;
        m = ((1 << slot) * k * (kTwN / NR)) & (kTwN - 1);
    }
    double s, c;
    sincospi(2.0 * m / kTwN, &s, &c);
    tw[i] = make_float2((float)c, (float)s);
}

int launch_twiddles(float2* tw, cudaStream_t st) {
    k_twiddles<<<(kTwAll + 255) / 256, 256, 0, st>>>(tw);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int launch_bank_build(const BankHarmDev* hd_dev, const BankHarmDev* hd_host, int nh, int ntpl,
                      float2* resp, int rstride, bool fp16, cudaStream_t st) {
    k_template_response<<<ntpl, 128, 0, st>>>(hd_dev, nh, resp, rstride);
    if (cudaGetLastError() != cudaSuccess) return -1;
    int maxM = 0;
    for (int h = 0; h < nh; h++) maxM = hd_host[h].M > maxM ? hd_host[h].M : maxM;
    dim3 grid((maxM + 127) / 128, ntpl);
    size_t smem = sizeof(double2) * (size_t)rstride;
    if (smem > 48 * 1024) {
        if (cudaFuncSetAttribute(k_template_dft, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem) != cudaSuccess)
            return -1;
    }
    k_template_dft<<<grid, 128, smem, st>>>(hd_dev, nh, resp, rstride);
    if (cudaGetLastError() != cudaSuccess) return -1;
    if (fp16) {
        k_fold_to_half<<<ntpl, 256, 0, st>>>(hd_dev, nh);
        if (cudaGetLastError() != cudaSuccess) return -1;
    }
    return 0;
}


// --------------------------------------------------------------------------
// Candidate refinement (the reference's optimizeCandidates stub,
// bpd_candidates.cu:24-27).
//
// The power the plane kernels compute at fundamental-plane position
// (r, z) is |sum_j X[j] conj(F(r - j - z/2; z))|^2 over the 2 hw(z) bins
// j in [ceil(r - hw), ceil(r + hw)), where F is the response that
// generate_z_response samples (bpd_subharmonics.cu:146-226; its loop
// variable is the argument x) and X the whitened spectrum: the planes are
// this expression on the grid r = rlo + i/2, z even.  Here it is evaluated
// at any (r, z), for every harmonic k r / H, k z / H (k = 1..H) of a
// candidate, and the summed power is maximised on three nested 5 x 5 grids
// (steps 1/4, 1/16, 1/64 in r and 1, 1/4, 1/16 in z around the best point
// so far).
// F(x; z), evaluated directly (the reference's small-offset series
// corrections are expansions of the same function).
__device__ double2 response_at(double x, double z) {
    if (fabs(z) < 1e-4) {  // generate_r_response: e^{i pi x} sin(pi x) / (pi x)
        const double px = kPi * x;
        double s, c;
        sincos(px, &s, &c);
        const double sinc = (x == 0.0) ? 1.0 : s / px;
        return make_double2(c * sinc, s * sinc);
    }
    const double absz = fabs(z);
    const int signz = (z < 0) ? -1 : 1;
    const double zd = signz * kSqrt2 / sqrt(absz);
    const double cons = zd / 2.0;
    const double yy = x * zd;
    const double zz = yy + z * zd;
    const double xx = kPi / z * x * x;
    const double c = cos(xx), s = sin(xx);
    double fsy, fcy, fsz, fcz;
    fresnel(yy, &fsy, &fcy);
    fresnel(zz, &fsz, &fcz);
    const double tre = signz * (fcz - fcy);
    const double tim = fsy - fsz;
    return make_double2((tre * c - tim * s) * cons, -(tre * s + tim * c) * cons);
}

// Power of one harmonic at (r, z), summed by one warp.
__device__ double warp_power(const float2* __restrict__ X, long long nb, double r, double z, int lane) {
    const int hw = z_halfwidth(z);
    const long long j0 = (long long)ceil(r - hw);
    const double base = r - 0.5 * z;
    double re = 0.0, im = 0.0;
    for (int i = lane; i < 2 * hw; i += 32) {
        const long long j = j0 + i;
        if (j < 0 || j >= nb) continue;
        const double2 w = response_at(base - (double)j, z);
        const float2 v = X[j];
        // X[j] * conj(w)
        re += (double)v.x * w.x + (double)v.y * w.y;
        im += (double)v.y * w.x - (double)v.x * w.y;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        re += __shfl_xor_sync(0xffffffffu, re, o);
        im += __shfl_xor_sync(0xffffffffu, im, o);
    }
    return re * re + im * im;
}

constexpr int kOptWarps = 4;

__global__ void __launch_bounds__(32 * kOptWarps) k_optimize(const OptArgs a) {
    extern __shared__ uint32_t okeys[];  // a.maxdata keys
    const int ci = blockIdx.x;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const OptCand& cand = a.in[ci];
    const float2* __restrict__ X = a.spec[cand.trial];
    const long long nb = a.numbins[cand.trial];
    const int H = cand.numharm;
    __shared__ double s_pow[25];
    __shared__ double s_best[3];  // r, z, power
    __shared__ double s_n2[kMaxHarm];
    __shared__ int hist[256];
    __shared__ int bc[2];
    // every harmonic's power normalisation, as the search applies it to the
    // candidate's step: the squared magic rsqrt of the segment's median
    // power / ln 2 (bpd_search.cu:144-181)
    for (int k = 0; k < H; k++) {
        const int nd = cand.numdata[k];
        const long long lo = cand.lobin[k];
        for (int i = threadIdx.x; i < nd; i += blockDim.x) {
            const long long b = lo + i;
            const float2 v = (b >= 0 && b < nb) ? X[b] : make_float2(0.f, 0.f);
            okeys[i] = __float_as_uint(power_exact(v));
        }
        __syncthreads();
        const uint32_t mk = block_select_u32(okeys, nd, (nd - 1) / 2, hist, bc);
        if (threadIdx.x == 0) {
            const double nrm = (double)rsqrt_norm((float)((double)__uint_as_float(mk) / kLn2), a.exact_rsqrt);
            s_n2[k] = nrm * nrm;
        }
        __syncthreads();
    }
    // summed power of every harmonic at (r, z)
    auto summed = [&](double r, double z) {
        double p = 0.0;
        for (int k = 1; k <= H; k++) p += s_n2[k - 1] * warp_power(X, nb, r * k / H, z * k / H, lane);
        return p;
    };
    if (threadIdx.x == 0) {
        s_best[0] = cand.r;
        s_best[1] = cand.z;
    }
    __syncthreads();
    if (a.refine) {
        const double dr[3] = {0.25, 1.0 / 16, 1.0 / 64}, dz[3] = {1.0, 0.25, 1.0 / 16};
        for (int lv = 0; lv < 3; lv++) {
            const double r0 = s_best[0], z0 = s_best[1];
            for (int g = warp; g < 25; g += kOptWarps) {
                const double p = summed(r0 + (g / 5 - 2) * dr[lv], z0 + (g % 5 - 2) * dz[lv]);
                if (lane == 0) s_pow[g] = p;
            }
            __syncthreads();
            if (threadIdx.x == 0) {
                int bg = 12;  // the centre unless something is strictly larger
                for (int g = 0; g < 25; g++)
                    if (s_pow[g] > s_pow[bg]) bg = g;
                s_best[0] = r0 + (bg / 5 - 2) * dr[lv];
                s_best[1] = z0 + (bg % 5 - 2) * dz[lv];
            }
            __syncthreads();
        }
    }
    // the harmonics' powers at the final position (warp k % warps)
    const double r = s_best[0], z = s_best[1];
    __shared__ double s_h[kMaxHarm];
    for (int k = 1 + warp; k <= H; k += kOptWarps) {
        const double p = s_n2[k - 1] * warp_power(X, nb, r * k / H, z * k / H, lane);
        if (lane == 0) s_h[k - 1] = p;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        OptOut o;
        o.r = r;
        o.z = z;
        double sum = 0.0;
        for (int k = 0; k < kMaxHarm; k++) {
            o.harm[k] = k < H ? (float)s_h[k] : 0.f;
            if (k < H) sum += s_h[k];
        }
        o.power = sum;
        a.out[ci] = o;
    }
}

int launch_optimize(const OptArgs& a, cudaStream_t st) {
    if (a.n <= 0) return 0;
    const size_t smem = sizeof(uint32_t) * (size_t)a.maxdata;
    if (smem > 48 * 1024 &&
        cudaFuncSetAttribute(k_optimize, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return -1;
    k_optimize<<<a.n, 32 * kOptWarps, smem, st>>>(a);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace accel
