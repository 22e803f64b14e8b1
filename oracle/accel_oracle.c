/*
 * accel_oracle.c -- CPU oracle (TEST INFRASTRUCTURE ONLY; see accel_oracle.h).
 *
 * Every function below names the reference file:line it restates.  Paths are
 * relative to the keithasr/gpu_accelsearch project root.
 */
#include "accel_oracle.h"

#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define O_PI      3.14159265358979323846264338327950288
#define O_SQRT2   1.41421356237309504880168872420969808
#define O_PIBY2   1.57079632679489661923132169163975144
#define O_NUMFINTBINS 16   /* bpd_common.h:45 */
#define O_DR   0.5         /* bpd_common.h:31 */
#define O_RDR  2
#define O_DZ   2
#define O_RDZ  0.5
#define O_NUMBETWEEN 2
#define O_DBLCORRECT 1e-14

/* ------------------------------------------------------------------ */
/* bpd_math.c:94-105 -- magic-constant inverse square root plus one   */
/* Newton step, evaluated left to right in single precision.          */
float orc_rsqrt_magic(float x)
{
    union { float f; int32_t i; } t;
    t.f = x;
    t.i = 0x5f3759df - (t.i >> 1);
    float y = t.f;
    float h = 0.5f * x;
    h = h * y;
    h = h * y;
    return y * (1.5f - h);
}

/* Normalisation mode: 0 = the magic-constant rsqrt above (the reference's
 * arithmetic), 1 = IEEE single-precision 1/sqrt(x) (correctly rounded sqrt,
 * then a correctly rounded divide) -- the GPU build's exact option. */
static int orc_exact_rsqrt = 0;
void orc_set_exact_rsqrt(int on) { orc_exact_rsqrt = on != 0; }
float orc_rsqrt_norm(float x)
{
    if (orc_exact_rsqrt) return 1.0f / sqrtf(x);
    return orc_rsqrt_magic(x);
}

static int cmp_float(const void *a, const void *b)
{
    float x = *(const float *)a, y = *(const float *)b;
    return (x > y) - (x < y);
}

/* bpd_math.c:20-91 -- quickselect returns the element of rank (n-1)/2
 * (lower median).  The value is an order statistic, so sorting a copy
 * gives the same float. */
float orc_select_lower_median(const float *a, int n)
{
    if (n <= 0) return 0.0f;
    float *t = (float *)malloc(sizeof(float) * (size_t)n);
    memcpy(t, a, sizeof(float) * (size_t)n);
    qsort(t, (size_t)n, sizeof(float), cmp_float);
    float m = t[(n - 1) / 2];
    free(t);
    return m;
}

/* bpd_math.c:113-122 */
long long orc_next_pow2(long long x)
{
    long long i = 1;
    while (i < x) i <<= 1;
    return i;
}

/* ------------------------------------------------------------------ */
/* Fresnel integrals S(x), C(x): the Cephes rational approximations   */
/* (S. L. Moshier, Cephes Math Library, fresnl.c), as used by the      */
/* reference at bpd_fresnl.c:3-200.  Coefficients are Cephes' tables.  */
static const double FS_N[6] = { -2.99181919401019853726E3, 7.08840045257738576863E5,
    -6.29741486205862506537E7, 2.54890880573376359104E9, -4.42979518059697779103E10,
    3.18016297876567817986E11 };
static const double FS_D[6] = { 2.81376268889994315696E2, 4.55847810806532581675E4,
    5.17343888770096400730E6, 4.19320245898111231129E8, 2.24411795645340920940E10,
    6.07366389490084639049E11 };
static const double FC_N[6] = { -4.98843114573573548651E-8, 9.50428062829859605134E-6,
    -6.45191435683965050962E-4, 1.88843319396703850064E-2, -2.05525900955013891793E-1,
    9.99999999999999998822E-1 };
static const double FC_D[7] = { 3.99982968972495980367E-12, 9.15439215774657478799E-10,
    1.25001862479598821474E-7, 1.22262789024179030997E-5, 8.68029542941784300606E-4,
    4.12142090722199792936E-2, 1.00000000000000000118E0 };
static const double FF_N[10] = { 4.21543555043677546506E-1, 1.43407919780758885261E-1,
    1.15220955073585758835E-2, 3.45017939782574027900E-4, 4.63613749287867322088E-6,
    3.05568983790257605827E-8, 1.02304514164907233465E-10, 1.72010743268161828879E-13,
    1.34283276233062758925E-16, 3.76329711269987889006E-20 };
static const double FF_D[10] = { 7.51586398353378947175E-1, 1.16888925859191382142E-1,
    6.44051526508858611005E-3, 1.55934409164153020873E-4, 1.84627567348930545870E-6,
    1.12699224763999035261E-8, 3.60140029589371370404E-11, 5.88754533621578410010E-14,
    4.52001434074129701496E-17, 1.25443237090011264384E-20 };
static const double FG_N[11] = { 5.04442073643383265887E-1, 1.97102833525523411709E-1,
    1.87648584092575249293E-2, 6.84079380915393090172E-4, 1.15138826111884280931E-5,
    9.82852443688422223854E-8, 4.45344415861750144738E-10, 1.08268041139020870318E-12,
    1.37555460633261799868E-15, 8.36354435630677421531E-19, 1.86958710162783235106E-22 };
static const double FG_D[11] = { 1.47495759925128324529E0, 3.37748989120019970451E-1,
    2.53603741420338795122E-2, 8.14679107184306179049E-4, 1.27545075667729118702E-5,
    1.04314589657571990585E-7, 4.60680728146520428211E-10, 1.10273215066240270757E-12,
    1.38796531259578871258E-15, 8.39158816283118707363E-19, 1.86958710162783236342E-22 };

/* Horner with an explicit leading coefficient: c[0] x^deg + ... + c[deg] */
static double horner(double x, const double *c, int deg)
{
    double acc = c[0];
    for (int k = 1; k <= deg; ++k) acc = acc * x + c[k];
    return acc;
}
/* Horner with an implied leading 1: x^deg + c[0] x^(deg-1) + ... + c[deg-1] */
static double horner1(double x, const double *c, int deg)
{
    double acc = x + c[0];
    for (int k = 1; k < deg; ++k) acc = acc * x + c[k];
    return acc;
}

int orc_fresnl(double xa, double *ssa, double *cca)
{
    double x = fabs(xa), x2 = x * x, ss, cc;
    if (x2 < 2.5625) {
        double t = x2 * x2;
        ss = x * x2 * horner(t, FS_N, 5) / horner1(t, FS_D, 6);
        cc = x * horner(t, FC_N, 5) / horner(t, FC_D, 6);
    } else if (x > 36974.0) {
        cc = 0.5;
        ss = 0.5;
    } else {
        x2 = x * x;
        double t = O_PI * x2;
        double u = 1.0 / (t * t);
        t = 1.0 / t;
        double f = 1.0 - u * horner(u, FF_N, 9) / horner1(u, FF_D, 10);
        double g = t * horner(u, FG_N, 10) / horner1(u, FG_D, 11);
        t = O_PIBY2 * x2;
        double c = cos(t), s = sin(t);
        t = O_PI * x;
        cc = 0.5 + (f * s - g * c) / t;
        ss = 0.5 - (f * c + g * s) / t;
    }
    if (xa < 0.0) { cc = -cc; ss = -ss; }
    *cca = cc;
    *ssa = ss;
    return 0;
}

/* ------------------------------------------------------------------ */
/* bpd_subharmonics.cu:31-45 */
int orc_z_halfwidth(double z)
{
    z = fabs(z);
    int m = (int)(z * (0.00089 * z + 0.3131) + O_NUMFINTBINS);
    m = (m < O_NUMFINTBINS) ? O_NUMFINTBINS : m;
    if (z > 100 && m > 0.6 * z) m = (int)(0.6 * z);
    return m;
}

static int nearest_int(double x) { return (int)(x < 0 ? ceil(x - 0.5) : floor(x + 0.5)); }

/* bpd_subharmonics.cu:10-13 */
int orc_calc_required_z(double f, double zfull)
{
    return nearest_int(O_RDZ * zfull * f) * O_DZ;
}

/* bpd_subharmonics.cu:16-19 */
double orc_calc_required_r(double f, double rfull)
{
    return (int)(O_RDR * rfull * f + 0.5) * O_DR;
}

/* bpd_subharmonics.cu:60-67 with ACCEL_USELEN as a parameter */
int orc_fft_length(int numharm, int harmnum, int zmax, int uselen)
{
    double f = (double)harmnum / (double)numharm;
    int bins_needed = ((uselen * harmnum) / numharm) + 2;
    int end_effects = 2 * O_NUMBETWEEN * orc_z_halfwidth(orc_calc_required_z(f, zmax));
    return (int)orc_next_pow2(bins_needed + end_effects);
}

/* bpd_subharmonics.cu:78-135 -- sinc interpolation kernel via a
 * trigonometric recurrence; argument accumulated by repeated addition. */
void orc_r_response(double roffset, int numbetween, int numkern, float *out)
{
    double startr = O_PI * (numkern / (double)(2 * numbetween) + roffset);
    double delta = -O_PI / numbetween;
    double tmp = sin(0.5 * delta);
    double alpha = -2.0 * tmp * tmp;
    double beta = sin(delta);
    double c = cos(startr), s = sin(startr);
    double r = startr, sinc;
    for (int i = 0; i < numkern; i++, r += delta) {
        sinc = (r == 0.0) ? 1.0 : s / r;
        out[2 * i] = (float)(c * sinc);
        out[2 * i + 1] = (float)(s * sinc);
        tmp = c;
        c = alpha * tmp - beta * s + c;
        s = alpha * s + beta * tmp + s;
    }
    if (roffset < 1E-3) {
        tmp = roffset * roffset;
        out[numkern] = (float)(1 - 6.579736267392905746 * tmp);
        out[numkern + 1] = (float)(roffset * (O_PI - 10.335425560099940058 * tmp));
    }
}

/* bpd_subharmonics.cu:146-226 -- constant-f-dot correlation response from
 * Fresnel integrals, sampled every 1/numbetween bins. */
void orc_z_response(double roffset, int numbetween, double z, int numkern, float *out)
{
    double absz = fabs(z);
    if (absz < 1E-4) { orc_r_response(roffset, numbetween, numkern, out); return; }
    double startr = roffset - (0.5 * z), ip;
    double startroffset = (startr < 0) ? 1.0 + modf(startr, &ip) : modf(startr, &ip);
    int signz = (z < 0.0) ? -1 : 1;
    double zd = signz * O_SQRT2 / sqrt(absz);
    double cons = zd / 2.0;
    double pibyz = O_PI / z;
    startr += numkern / (double)(2 * numbetween);
    double delta = -1.0 / numbetween;
    double r = startr;
    for (int i = 0; i < numkern; i++, r += delta) {
        double yy = r * zd;
        double zz = yy + z * zd;
        double xx = pibyz * r * r;
        double c = cos(xx), s = sin(xx);
        double fsy, fcy, fsz, fcz;
        orc_fresnl(yy, &fsy, &fcy);
        orc_fresnl(zz, &fsz, &fcz);
        double tre = signz * (fcz - fcy);
        double tim = fsy - fsz;
        out[2 * i] = (float)((tre * c - tim * s) * cons);
        out[2 * i + 1] = (float)(-(tre * s + tim * c) * cons);
    }
    if (startroffset < 1E-3 && absz < 1E-3) {
        double zz = z * z, xx = startroffset * startroffset;
        int h = numkern / 2;
        double re = 1.0 - 0.16449340668482264365 * zz;
        double im = -0.5235987755982988731 * z;
        re = (float)re; im = (float)im;
        re += startroffset * 1.6449340668482264365 * z;
        re = (float)re;
        im += startroffset * (O_PI - 0.5167712780049970029 * zz);
        im = (float)im;
        re += xx * (-6.579736267392905746 + 0.9277056288952613070 * zz);
        im += xx * (3.1006276680299820175 * z);
        out[2 * h] = (float)re;
        out[2 * h + 1] = (float)im;
    }
}

/* bpd_subharmonics.cu:253-267 -- upper half of the response at [0,2hw),
 * lower half at [L-2hw, L), zeros between. */
void orc_wrapped_template(int fftlen, int z, float *out)
{
    int hw = orc_z_halfwidth((double)z);
    int numkern = 2 * O_NUMBETWEEN * hw;
    int half = numkern / 2;
    float *resp = (float *)malloc(sizeof(float) * 2 * (size_t)numkern);
    orc_z_response(0.0, O_NUMBETWEEN, (double)z, numkern, resp);
    memset(out, 0, sizeof(float) * 2 * (size_t)fftlen);
    memcpy(out, resp + 2 * half, sizeof(float) * 2 * (size_t)half);
    memcpy(out + 2 * (size_t)(fftlen - half), resp, sizeof(float) * 2 * (size_t)half);
    free(resp);
}

/* ------------------------------------------------------------------ */
/* bpd_noise.c:12-92 with the block widths (6, 200 in the reference) as */
/* parameters.  Interleaved float complex, in place.                   */
void orc_deredden(float *c, unsigned numbins, int initialbuflen, int maxbuflen)
{
    int ind, lastbuflen, binnum = 1, numwrote = 1;
    long k;
    float dslope = 1.0f, norm;
    c[0] = 1.0f;
    c[1] = 0.0f;
    float *pb = (float *)malloc(sizeof(float) * (size_t)numbins);
    for (k = 0; k < (long)numbins; k++) {
        float a = c[2 * k] * c[2 * k];
        float b = c[2 * k + 1] * c[2 * k + 1];
        pb[k] = a + b;
    }
    int buflen = initialbuflen;
    float mean_old = (float)(orc_select_lower_median(pb + binnum, buflen) / log(2.0));
    norm = orc_rsqrt_norm(mean_old);
    for (ind = numwrote; ind < binnum + buflen / 2; ind++) {
        c[2 * ind] *= norm;
        c[2 * ind + 1] *= norm;
    }
    numwrote += buflen / 2;
    binnum += buflen;
    lastbuflen = buflen;
    buflen = (int)(initialbuflen * log(binnum));
    if (buflen > maxbuflen) buflen = maxbuflen;
    while ((unsigned)(binnum + buflen) < numbins) {
        double mean_new = orc_select_lower_median(pb + binnum, buflen) / log(2.0);
        dslope = (float)((mean_new - mean_old) / (0.5 * (lastbuflen + buflen)));
        for (k = 0, ind = numwrote; ind < binnum + buflen / 2; k++, ind++) {
            float lv = dslope * (float)k;
            lv = mean_old + lv;
            norm = orc_rsqrt_norm(lv);
            c[2 * ind] *= norm;
            c[2 * ind + 1] *= norm;
        }
        numwrote += (int)k;
        binnum += buflen;
        lastbuflen = buflen;
        mean_old = (float)mean_new;
        buflen = (int)(initialbuflen * log(binnum));
        if (buflen > maxbuflen) buflen = maxbuflen;
    }
    for (k = 0, ind = numwrote; ind < (long)numbins; k++, ind++) {
        float lv = dslope * (float)k;
        lv = mean_old + lv;
        norm = orc_rsqrt_norm(lv);
        c[2 * ind] *= norm;
        c[2 * ind + 1] *= norm;
    }
    free(pb);
}

/* ------------------------------------------------------------------ */
/* Bank geometry: createSubharmonicInfo / initializeSubharmonicInfo     */
/* (bpd_subharmonics.cu:233-279, 319-354) without the template data.   */
int orc_bank_geometry(int zmax, int numharm, int uselen, int *info)
{
    int stages = 0;
    while ((1 << stages) < numharm) stages++;
    stages += 1;                                   /* fast_log2(numharm)+1 */
    int n = 0;
    for (int st = 0; st < stages; st++) {
        int maxh = (st < 1) ? 1 : (1 << st);
        for (int h = 1; h <= maxh; h += 2) {
            double f = (double)h / (double)maxh;
            int zm = orc_calc_required_z(f, zmax);
            int *o = info + n * ORC_HINFO;
            o[0] = h;
            o[1] = maxh;
            o[2] = zm;
            o[3] = (zm / O_DZ) * 2 + 1;
            o[4] = orc_fft_length(maxh, h, zmax, uselen);
            o[5] = orc_z_halfwidth((double)(-zm));
            o[6] = orc_calc_required_z(f, -zmax);
            n++;
        }
    }
    return n;
}

/* bpd_search.cu:72-127, one harmonic. */
void orc_step_ffdot(int harmnum, int maxharm, int zmax, int uselen, double startr, double lastr,
                    int *rlo, double *rhi, int *zlo, int *numrs)
{
    double f = (double)harmnum / (double)maxharm;
    double drlo = orc_calc_required_r(f, startr);
    double drhi = orc_calc_required_r(f, lastr);
    *rlo = (int)floor(drlo);
    *rhi = drhi;
    *zlo = orc_calc_required_z(f, -zmax);
    if (harmnum == 1 && maxharm == 1) {
        *numrs = uselen;
    } else {
        int n = (int)((ceil(drhi) - floor(drlo)) * O_RDR + O_DBLCORRECT) + 1;
        if (n % O_RDR) n = (n / O_RDR + 1) * O_RDR;
        *numrs = n;
    }
}

/* bpd_search.cu:130-184 (+ get_fourier_amplitudes :16-47, spreadData
 * :56-67).  Only the first numdata bins are median normalised; the rest
 * of the fftlen/2 copied bins keep their whitened values.  Returns 0, or
 * -1 when next_pow2(numdata) != fftlen/2. */
int orc_segment_data(const float *wspec, long numbins, int rlo, double rhi, int hw0, int fftlen,
                     float *out)
{
    int lobin = rlo - hw0;
    int hibin = (int)ceil(rhi) + hw0;
    int numdata = hibin - lobin + 1;
    int nice = (int)orc_next_pow2(numdata);
    if (nice != fftlen / O_NUMBETWEEN) return -1;
    float *amp = (float *)malloc(sizeof(float) * 2 * (size_t)nice);
    for (int t = 0; t < nice; t++) {
        long b = (long)lobin + t;
        if (b >= 0 && b < numbins) {
            amp[2 * t] = wspec[2 * b];
            amp[2 * t + 1] = wspec[2 * b + 1];
        } else {
            amp[2 * t] = 0.0f;
            amp[2 * t + 1] = 0.0f;
        }
    }
    float *pw = (float *)malloc(sizeof(float) * (size_t)numdata);
    for (int t = 0; t < numdata; t++) {
        float a = amp[2 * t] * amp[2 * t];
        float b = amp[2 * t + 1] * amp[2 * t + 1];
        pw[t] = a + b;
    }
    double nc = orc_rsqrt_norm((float)(orc_select_lower_median(pw, numdata) / log(2.0)));
    for (int t = 0; t < numdata; t++) {
        amp[2 * t] = (float)(amp[2 * t] * nc);
        amp[2 * t + 1] = (float)(amp[2 * t + 1] * nc);
    }
    memset(out, 0, sizeof(float) * 2 * (size_t)fftlen);
    for (int t = 0; t < fftlen / O_NUMBETWEEN; t++) {
        out[2 * (O_NUMBETWEEN * t)] = amp[2 * t];
        out[2 * (O_NUMBETWEEN * t) + 1] = amp[2 * t + 1];
    }
    free(pw);
    free(amp);
    return 0;
}

/* AccelSearch.cu:203-245: startr advances by uselen/2 while
 * startr + uselen/2 < highestBin. */
long orc_step_count(long highest_bin, long rlo, int uselen)
{
    long n = 0;
    long half = (unsigned short)(uselen * O_DR);
    for (long s = rlo; s + half < highest_bin; s += half) n++;
    return n;
}

/* ------------------------------------------------------------------ */
/* FP64 radix-2 FFT (in place, unnormalised).                          */
void orc_fft(double *x, int n, int sign)
{
    for (int i = 1, j = 0; i < n; i++) {
        int bit = n >> 1;
        for (; j & bit; bit >>= 1) j ^= bit;
        j ^= bit;
        if (i < j) {
            double t0 = x[2 * i], t1 = x[2 * i + 1];
            x[2 * i] = x[2 * j]; x[2 * i + 1] = x[2 * j + 1];
            x[2 * j] = t0; x[2 * j + 1] = t1;
        }
    }
    for (int len = 2; len <= n; len <<= 1) {
        int half = len >> 1;
        double ang = sign * 2.0 * O_PI / len;
        for (int k = 0; k < half; k++) {
            double wr = cos(ang * k), wi = sin(ang * k);
            for (int i = k; i < n; i += len) {
                int j = i + half;
                double ur = x[2 * i], ui = x[2 * i + 1];
                double vr = x[2 * j] * wr - x[2 * j + 1] * wi;
                double vi = x[2 * j] * wi + x[2 * j + 1] * wr;
                x[2 * i] = ur + vr; x[2 * i + 1] = ui + vi;
                x[2 * j] = ur - vr; x[2 * j + 1] = ui - vi;
            }
        }
    }
}

/* ------------------------------------------------------------------ */
struct orc_ctx {
    int zmax, numharm, uselen, nh;
    int info[16 * ORC_HINFO];
    double *kspec[16];   /* conj-free FFT of wrapped float templates */
};

orc_ctx *orc_create(int zmax, int numharm, int uselen)
{
    orc_ctx *c = (orc_ctx *)calloc(1, sizeof(orc_ctx));
    c->zmax = zmax;
    c->numharm = numharm;
    c->uselen = uselen;
    c->nh = orc_bank_geometry(zmax, numharm, uselen, c->info);
    for (int h = 0; h < c->nh; h++) {
        int *o = c->info + h * ORC_HINFO;
        int numzs = o[3], L = o[4], zm = o[2];
        c->kspec[h] = (double *)malloc(sizeof(double) * 2 * (size_t)L * numzs);
        float *tmp = (float *)malloc(sizeof(float) * 2 * (size_t)L);
        for (int j = 0; j < numzs; j++) {
            int z = -zm + j * O_DZ;
            orc_wrapped_template(L, z, tmp);
            double *d = c->kspec[h] + 2 * (size_t)L * j;
            for (int t = 0; t < 2 * L; t++) d[t] = tmp[t];
            orc_fft(d, L, -1);
        }
        free(tmp);
    }
    return c;
}

void orc_destroy(orc_ctx *c)
{
    if (!c) return;
    for (int h = 0; h < c->nh; h++) free(c->kspec[h]);
    free(c);
}

int orc_num_harmonics(const orc_ctx *c) { return c->nh; }
int orc_uselen(const orc_ctx *c) { return c->uselen; }

/* One harmonic of one step: P_h[z][i] = |IFFT(D . conj K_z)[2 hw0 + i]|^2 / L^2
 * (bpd_search.cu:228-307, bpd_gpu_kernels.cu:39-116) in FP64. */
static int harmonic_plane(orc_ctx *c, const float *wspec, long numbins, double startr, int h,
                          double *plane, int wcap, int nthreads)
{
    int *o = c->info + h * ORC_HINFO;
    int L = o[4], numzs = o[3], hw0 = o[5];
    double lastr = startr + (unsigned short)(c->uselen * O_DR) - O_DR;
    int rlo, zlo, numrs;
    double rhi;
    orc_step_ffdot(o[0], o[1], c->zmax, c->uselen, startr, lastr, &rlo, &rhi, &zlo, &numrs);
    float *seg = (float *)malloc(sizeof(float) * 2 * (size_t)L);
    if (orc_segment_data(wspec, numbins, rlo, rhi, hw0, L, seg) != 0) { free(seg); return -1; }
    double *dd = (double *)malloc(sizeof(double) * 2 * (size_t)L);
    for (int t = 0; t < 2 * L; t++) dd[t] = seg[t];
    orc_fft(dd, L, -1);
    free(seg);
    double scale = 1.0 / ((double)L * (double)L);
    int off = hw0 * O_NUMBETWEEN;
    int ncopy = numrs < wcap ? numrs : wcap;
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic) num_threads(nthreads)
#endif
    for (int j = 0; j < numzs; j++) {
        double *y = (double *)malloc(sizeof(double) * 2 * (size_t)L);
        const double *k = c->kspec[h] + 2 * (size_t)L * j;
        for (int t = 0; t < L; t++) {
            double dr = dd[2 * t], di = dd[2 * t + 1], kr = k[2 * t], ki = k[2 * t + 1];
            y[2 * t] = dr * kr + di * ki;
            y[2 * t + 1] = di * kr - dr * ki;
        }
        orc_fft(y, L, +1);
        double *row = plane + (size_t)j * wcap;
        for (int i = 0; i < ncopy; i++) {
            double re = y[2 * (off + i)], im = y[2 * (off + i) + 1];
            row[i] = (re * re + im * im) * scale;
        }
        free(y);
    }
    free(dd);
    (void)nthreads;
    return numrs;
}

int orc_harmonic_plane(orc_ctx *c, const float *wspec, long numbins, double startr, int h,
                       double *plane, int wcap)
{
    return harmonic_plane(c, wspec, numbins, startr, h, plane, wcap, 1);
}

/* Harmonic summing (bpd_search.cu:310-360, bpd_gpu_kernels.cu:119-170)
 * with the reference's index arithmetic, plus the candidate threshold
 * that the reference leaves as a stub (bpd_candidates.cu:4-9). */
long orc_run_steps(orc_ctx *c, const float *wspec, long numbins, long rlo, long step0,
                   long nsteps, const double *powcut, double *stage_planes, orc_cand *cands,
                   long cap, int nthreads)
{
    int nh = c->nh, U = c->uselen;
    int *o0 = c->info;
    int numzs0 = o0[3];
    int zlo0 = o0[6];
    int nstages = 0;
    for (int h = 0; h < nh; h++) if (((h + 1) & h) == 0) nstages++;
    long half = (unsigned short)(U * O_DR);
    long ncand = 0;
    double *planes[16];
    int wcap[16];
    for (int h = 0; h < nh; h++) {
        int *o = c->info + h * ORC_HINFO;
        wcap[h] = o[4];
        planes[h] = (double *)malloc(sizeof(double) * (size_t)o[3] * (size_t)wcap[h]);
    }
    double *sum = (double *)malloc(sizeof(double) * (size_t)numzs0 * U);
    for (long s = 0; s < nsteps; s++) {
        long step = step0 + s;
        double startr = (double)(rlo + step * half);
        int fullrlo = (int)startr;
        for (int h = 0; h < nh; h++)
            harmonic_plane(c, wspec, numbins, startr, h, planes[h], wcap[h], nthreads);
        double lastr = startr + half - O_DR;
        for (int z = 0; z < numzs0; z++)
            for (int i = 0; i < U; i++) sum[(size_t)z * U + i] = planes[0][(size_t)z * wcap[0] + i];
        int stage = 0;
        for (int h = 0; h < nh; h++) {
            if (h > 0) {
                int *o = c->info + h * ORC_HINFO;
                double f = (double)o[0] / (double)o[1];
                int hrlo, hzlo, hnumrs;
                double hrhi;
                orc_step_ffdot(o[0], o[1], c->zmax, U, startr, lastr, &hrlo, &hrhi, &hzlo, &hnumrs);
#ifdef _OPENMP
#pragma omp parallel for schedule(static) num_threads(nthreads)
#endif
                for (int z = 0; z < numzs0; z++) {
                    int zz = zlo0 + z * O_DZ;
                    int subz = (int)(zz * f);
                    int zind = (int)((subz - hzlo) * O_RDZ);
                    const double *prow = planes[h] + (size_t)zind * wcap[h];
                    double *srow = sum + (size_t)z * U;
                    for (int i = 0; i < U; i++) {
                        double rr = fullrlo + i * O_DR;
                        double subr = (int)(O_RDR * rr * f + 0.5) * O_DR;
                        unsigned short rind = (unsigned short)(int)((subr - hrlo) * O_RDR);
                        srow[i] += prow[rind];
                    }
                }
            }
            if (((h + 1) & h) == 0) {
                if (stage_planes) {
                    double *dst = stage_planes + ((size_t)s * nstages + stage) * (size_t)numzs0 * U;
                    memcpy(dst, sum, sizeof(double) * (size_t)numzs0 * U);
                }
                if (powcut) {
                    double cut = powcut[stage];
                    for (int z = 0; z < numzs0; z++)
                        for (int i = 0; i < U; i++) {
                            double p = sum[(size_t)z * U + i];
                            if (p > cut) {
                                if (ncand < cap && cands) {
                                    cands[ncand].step = (int)step;
                                    cands[ncand].ridx = i;
                                    cands[ncand].zidx = z;
                                    cands[ncand].numharm = h + 1;
                                    cands[ncand].power = p;
                                }
                                ncand++;
                            }
                        }
                }
                stage++;
            }
        }
    }
    free(sum);
    for (int h = 0; h < nh; h++) free(planes[h]);
    return ncand;
}

/* ------------------------------------------------------------------ */
/* log of the Gamma(n,1) upper tail: -x + log(sum_{k<n} x^k / k!)     */
static double log_gamma_q(int n, double x)
{
    double term = 1.0, s = 1.0;
    for (int k = 1; k < n; k++) { term *= x / k; s += term; }
    return -x + log(s);
}

double orc_power_cut(double sigma, int numharm, double numindep)
{
    double logp = log(0.5 * erfc(sigma / O_SQRT2)) - log(numindep > 1.0 ? numindep : 1.0);
    double lo = 0.0, hi = 4096.0;
    for (int it = 0; it < 200; it++) {
        double mid = 0.5 * (lo + hi);
        if (log_gamma_q(numharm, mid) > logp) lo = mid; else hi = mid;
    }
    return 0.5 * (lo + hi);
}
