/*
 * accel_oracle.h -- CPU oracle for the Fourier-domain acceleration search.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product library links, loads or
 * calls this code.  It is imported by tests/, by __graft_entry__.smoke() (as
 * the checker) and by bench.py's cpu_baseline / --impl reference leg.
 *
 * It restates the reference algorithm (keithasr/gpu_accelsearch) in plain C:
 * the host numerics bit-for-bit (whitening, median normalisation, template
 * responses, geometry), and the cuFFT / kernel stages in FP64.  The
 * restatement is pinned against the reference's own host code, compiled from
 * its sources by oracle/ref/Makefile into oracle/_ref/, through the golden
 * fixtures in tests/golden/ (see tests/golden/make_golden.py).
 *
 * Compile with -ffp-contract=off so that no multiply-add is fused: the
 * reference's host arithmetic is plain IEEE single/double operations.
 */
#ifndef ACCEL_ORACLE_H_
#define ACCEL_ORACLE_H_

#ifdef __cplusplus
extern "C" {
#endif

/* ---- reference host math (bpd_math.c, bpd_fresnl.c) ------------------- */
float  orc_rsqrt_magic(float x);                       /* bpd_math.c:94-105  */
void   orc_set_exact_rsqrt(int on);                   /* GPU build's exact-rsqrt option */
float  orc_rsqrt_norm(float x);                        /* the normalisation in force  */
float  orc_select_lower_median(const float *a, int n); /* bpd_math.c:20-91   */
long long orc_next_pow2(long long x);                  /* bpd_math.c:113-122 */
int    orc_fresnl(double x, double *s, double *c);     /* bpd_fresnl.c:160-200 */

/* ---- template geometry and responses (bpd_subharmonics.cu) ------------ */
int    orc_z_halfwidth(double z);                       /* :31-45  */
int    orc_calc_required_z(double f, double zfull);     /* :10-13  */
double orc_calc_required_r(double f, double rfull);     /* :16-19  */
int    orc_fft_length(int numharm, int harmnum, int zmax, int uselen); /* :60-67 */
void   orc_r_response(double roffset, int numbetween, int numkern, float *out);          /* :78-135  */
void   orc_z_response(double roffset, int numbetween, double z, int numkern, float *out); /* :146-226 */
/* Wrapped, zero-filled time-domain template of length fftlen (:253-267). */
void   orc_wrapped_template(int fftlen, int z, float *out);

/* ---- whitening (bpd_noise.c:12-92), parameterised block widths -------- */
void   orc_deredden(float *cplx, unsigned numbins, int initialbuflen, int maxbuflen);

/* ---- per-step geometry and segment data (bpd_search.cu) --------------- */
/* Per harmonic of a bank: harmnum, maxharm, zmax_h, numzs, fftlen, hw0, zlo */
#define ORC_HINFO 7
int    orc_bank_geometry(int zmax, int numharm, int uselen, int *info /* 16*ORC_HINFO */);
/* ffdotInfo for one step (bpd_search.cu:72-127): rlo, numrs, zlo; rhi double */
void   orc_step_ffdot(int harmnum, int maxharm, int zmax, int uselen,
                      double startr, double lastr, int *rlo, double *rhi, int *zlo, int *numrs);
/* generate_harmonic_ffdot_data for one harmonic (bpd_search.cu:130-184):
 * spread segment of fftlen complex (interleaved re,im) */
int    orc_segment_data(const float *wspec, long numbins, int rlo, double rhi,
                        int hw0, int fftlen, float *out);
/* Number of overlap-save steps of the main loop (AccelSearch.cu:209) */
long   orc_step_count(long highest_bin, long rlo, int uselen);

/* ---- FP64 pipeline --------------------------------------------------- */
typedef struct orc_ctx orc_ctx;
typedef struct {
    int step;      /* step index within the trial            */
    int ridx;      /* fundamental r index (r = startr + ridx/2) */
    int zidx;      /* fundamental z index (z = -zmax + 2 zidx)  */
    int numharm;   /* harmonics summed: 1, 2, 4, 8, ...         */
    double power;  /* summed normalised power                   */
} orc_cand;

orc_ctx *orc_create(int zmax, int numharm, int uselen);
void     orc_destroy(orc_ctx *c);
int      orc_num_harmonics(const orc_ctx *c);
int      orc_uselen(const orc_ctx *c);
/* Runs steps [step0, step0+nsteps) of a trial whose whitened spectrum holds
 * numbins complex bins, first step at rlo.  stage_planes (nullable) receives,
 * per step and stage, the cumulative power plane [numzs0][uselen].  Cands
 * above powcut[stage] are written up to cap; returns the total count. */
long     orc_run_steps(orc_ctx *c, const float *wspec, long numbins, long rlo,
                       long step0, long nsteps, const double *powcut,
                       double *stage_planes, orc_cand *cands, long cap, int nthreads);
/* Single-harmonic power plane of one step (P_h[z][i], i < numrs_h) for
 * checking the plane kernel directly.  Returns numrs_h. */
int      orc_harmonic_plane(orc_ctx *c, const float *wspec, long numbins, double startr,
                            int h, double *plane /* numzs_h * wcap */, int wcap);

/* Power cut for an n-harmonic sum: Gamma(n,1) upper tail equal to the
 * one-sided Gaussian tail at sigma, divided by numindep. */
double   orc_power_cut(double sigma, int numharm, double numindep);

/* Double-precision complex FFT, in place, unnormalised; sign -1 forward
 * (e^{-2 pi i}), +1 inverse.  n a power of two. */
void     orc_fft(double *x, int n, int sign);

#ifdef __cplusplus
}
#endif
#endif
