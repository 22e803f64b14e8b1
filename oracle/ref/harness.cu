/*
 * harness.cu -- extern "C" entry points over the reference's own host code,
 * used only to pin the oracle (tests/golden/make_golden.py).  Built by
 * oracle/ref/Makefile together with the reference's sources, which stay
 * where they lie; nothing here is part of the product.
 */
extern "C" {
#include "bpd_math.h"
#include "bpd_noise.h"
#include "bpd_fresnl.h"
}
#include "bpd_subharmonics.cuh"
#include "bpd_search.cuh"

/* Defined in bpd_subharmonics.cu without a header declaration. */
int calculateFFTLength(unsigned short numharm, unsigned short harmnum, int max_zfull);
int z_response_halfwidth(double z);
cufftComplex *generate_r_response(double roffset, int numbetween, int numkern);
cufftComplex *generate_z_response(double roffset, int numbetween, double z, int numkern);

cudaError_t refshim_malloc(void **p, size_t n) { *p = malloc(n); return cudaSuccess; }
cudaError_t refshim_memcpy(void *d, const void *s, size_t n, cudaMemcpyKind) { memcpy(d, s, n); return cudaSuccess; }
cudaError_t refshim_free(void *p) { free(p); return cudaSuccess; }

/* Stand-in for bpd_fft.cu:80: returns the wrapped time-domain templates
 * unchanged, so createSubharmonicInfo yields them for the golden files. */
unsigned complexToComplexFFT(cufftComplex *idata, unsigned int n, cufftComplex **odata, int batch)
{
    *odata = idata;
    (void)batch;
    return n;
}

extern "C" {
int ref_uselen(void) { return ACCEL_USELEN; }
float ref_rsqrt(float x) { return inverse_square_root(x); }
float ref_fast_median(float *a, int n) { return fast_median(a, n); }
int ref_fresnl(double x, double *s, double *c) { return fresnl(x, s, c); }
int ref_z_halfwidth(double z) { return z_response_halfwidth(z); }
int ref_calc_required_z(double f, double z) { return calc_required_z(f, z); }
double ref_calc_required_r(double f, double r) { return calc_required_r(f, r); }
int ref_fft_length(int numharm, int harmnum, int zmax) { return calculateFFTLength(numharm, harmnum, zmax); }
void ref_deredden(float *c, unsigned n) { deredden((cufftComplex *)c, n); }

void ref_r_response(double roffset, int nb, int numkern, float *out)
{
    cufftComplex *r = generate_r_response(roffset, nb, numkern);
    memcpy(out, r, sizeof(cufftComplex) * numkern);
    free(r);
}
void ref_z_response(double roffset, int nb, double z, int numkern, float *out)
{
    cufftComplex *r = generate_z_response(roffset, nb, z, numkern);
    memcpy(out, r, sizeof(cufftComplex) * numkern);
    free(r);
}

/* createSubharmonicInfo (templates left in the time domain, see above). */
void *ref_create_bank(int stages, int zhi) { return createSubharmonicInfo(stages, zhi); }
/* harmnum, maxharm, zmax, numzs, fftlen, hw0 */
void ref_bank_info(void *bank, int h, int *o)
{
    SubharmonicInfo *s = (SubharmonicInfo *)bank + h;
    o[0] = s->currentHarmonic; o[1] = s->maxHarmonic; o[2] = s->zmax;
    o[3] = s->totalKernelsTemplates; o[4] = s->kernelFFTLength; o[5] = s->kernelHalfWidth[0];
}
const float *ref_bank_templates(void *bank, int h) { return (const float *)((SubharmonicInfo *)bank)[h].kernels_data; }

/* generate_harmonics_ffdot for one step: per harmonic rlo, numrs, numzs,
 * fftlen, zlo, binoffset (ints) and rhi (double). */
void ref_step_ffdot(void *bank, int stages, double startr, double lastr, double zlo, int *oi, double *orhi)
{
    int nh = getTotalHarmonics(stages);
    ffdotInfo *fi = (ffdotInfo *)malloc(sizeof(ffdotInfo) * nh);
    unsigned short *bo = (unsigned short *)malloc(sizeof(unsigned short) * nh);
    generate_harmonics_ffdot(nh, stages, (SubharmonicInfo *)bank, startr, lastr, zlo, fi, bo);
    for (int h = 0; h < nh; h++) {
        oi[6 * h + 0] = fi[h].rlo; oi[6 * h + 1] = fi[h].numrs; oi[6 * h + 2] = fi[h].numzs;
        oi[6 * h + 3] = fi[h].fftlen; oi[6 * h + 4] = fi[h].zlo; oi[6 * h + 5] = bo[h];
        orhi[h] = fi[h].rhi;
    }
    free(fi);
    free(bo);
}

/* generate_harmonic_ffdot_data for one step: all harmonics' spread
 * segments, concatenated as in AccelSearch.cu:142-154. */
void ref_step_data(void *bank, int stages, double startr, double lastr, double zlo,
                   const float *wspec, long numbins, float *out)
{
    int nh = getTotalHarmonics(stages);
    SubharmonicInfo *shi = (SubharmonicInfo *)bank;
    ffdotInfo *fi = (ffdotInfo *)malloc(sizeof(ffdotInfo) * nh);
    unsigned short *bo = (unsigned short *)malloc(sizeof(unsigned short) * nh);
    long *start = (long *)malloc(sizeof(long) * nh);
    long total = 0;
    for (int h = 0; h < nh; h++) { start[h] = total; total += shi[h].kernelFFTLength; }
    generate_harmonics_ffdot(nh, stages, shi, startr, lastr, zlo, fi, bo);
    generate_harmonic_ffdot_data(nh, total, fi, bo, start, (cufftComplex *)wspec, numbins, 0,
                                 (cufftComplex *)out);
    free(fi); free(bo); free(start);
}
}
