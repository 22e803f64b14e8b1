/*
 * accelsearch.h -- C ABI of libaccelsearch.so, a GB300 (sm_103a)
 * Fourier-domain acceleration search.
 *
 * Two layers:
 *
 *  1. The context API (accel_*).  Every call returns an int status
 *     (ACCEL_OK or a negative ACCEL_ERR_*), never exits, and leaves a
 *     message for accel_last_error() (per host thread).  All device work of a
 *     context is issued on its stream; one context per host thread.
 *
 *  2. Drop-in entry points with the reference's names and argument meaning
 *     (keithasr/gpu_accelsearch, headers/bpd_*.h / *.cuh), for callers of
 *     that pipeline API.  They run on a process-wide default context, as the
 *     reference keeps its plans and streams in process globals
 *     (bpd_search.cu:10-13).  accel_complex is layout-compatible with
 *     cufftComplex.  Each declaration cites the reference interface it
 *     replaces.
 *
 * All pointers named *_dev are device pointers; all others are host memory.
 */
#ifndef ACCELSEARCH_H_
#define ACCELSEARCH_H_

#ifdef __cplusplus
extern "C" {
#endif

#define ACCEL_OK               0
#define ACCEL_ERR_INVALID     -1   /* bad argument or configuration        */
#define ACCEL_ERR_CUDA        -2   /* a CUDA runtime or launch error        */
#define ACCEL_ERR_NOMEM       -3   /* device or host allocation failed      */
#define ACCEL_ERR_CAPACITY    -4   /* candidate buffer overflowed           */
#define ACCEL_ERR_UNSUPPORTED -5   /* outside the built kernel shapes       */
#define ACCEL_ERR_BUDGET      -6   /* request exceeds the HBM budget        */

typedef struct { float x, y; } accel_complex;   /* == cufftComplex */

typedef struct accel_config {
    int zmax;               /* largest |f-dot| (bins), even; reference zhi       */
    int numharm;            /* harmonics summed: 1, 2, 4, 8 or 16                */
    int fftlen;             /* fundamental segment length L (power of two)       */
    int uselen;             /* 0: derived, L - 2 - 4*halfwidth(zmax), even       */
    int whiten_initbuf;     /* first whitening block (reference: 6)              */
    int whiten_maxbuf;      /* largest whitening block (reference: 200)          */
    double sigma;           /* candidate threshold in Gaussian sigma (6)         */
    double numindep;        /* trial-count divisor of the tail probability (1)   */
    int template_fp16;      /* 1: FP16 folded templates, scaled per template     */
    int chunk_segments;     /* segments per launch group (0: automatic)          */
    long long cand_capacity;/* raw candidates kept per search (0: automatic)     */
    int device;             /* CUDA device ordinal                               */
    int exact_rsqrt;        /* 1: whitening and segment normalisation use an IEEE */
                            /* 1/sqrt instead of the reference's magic-constant  */
                            /* approximation (bpd_math.c:94-105; ~1.75e-3 error) */
    int short_transforms;   /* 1: each harmonic's segment transform has the      */
                            /* shortest length R*2^k (R = 1, 5, 6, 7) that holds */
                            /* its data instead of the reference's power of two  */
                            /* (bpd_subharmonics.cu:60-67); the powers kept are   */
                            /* the same up to FP32 rounding.  Such a harmonic's  */
                            /* segment spectra (accel_prepare_segments) and      */
                            /* folded templates (accel_bank_spectra) are stored  */
                            /* in decimated order: position (k mod R)*(M/R)+k/R  */
                            /* holds point k (M = fftlen/2 of accel_harmonic)    */
    int reserved[5];
} accel_config;

typedef struct accel_harmonic {
    int harmnum, maxharm;   /* harmonic fraction harmnum/maxharm                 */
    int zmax, numzs;        /* templates z = -zmax .. zmax step 2                */
    int fftlen;             /* segment length L_h transformed (short_transforms: */
                            /* may be R*2^k instead of the reference's 2^k)     */
    int halfwidth;          /* halfwidth of the widest template (binOffset)      */
    int zlo;                /* lowest f-dot of the harmonic's plane              */
    int plane_width;        /* powers per f-dot row kept on the device           */
} accel_harmonic;

typedef struct accel_candidate {
    int trial;              /* index of the time series in the search call       */
    int step;               /* overlap-save step within the trial                */
    double r;               /* Fourier frequency of the fundamental (bins)       */
    double z;               /* f-dot of the fundamental (bins)                   */
    int numharm;            /* harmonics summed                                  */
    float power;            /* summed normalised power                           */
    float sigma;            /* equivalent Gaussian significance                  */
} accel_candidate;

/* Kernel accounting of a context (accel_get_stats).  Kinds: 0 segment
 * preparation, 1 power planes, 2 harmonic sum, 3 whitening, 4 R2C FFT
 * (cuFFT; not counted in `launches`), 5 fundamental plane fused with the
 * harmonic sum, 6 power planes and harmonic sums of a launch group in one
 * persistent launch (accel_tuning.persistent). */
#define ACCEL_KINDS 7
typedef struct accel_stats {
    long long launches;                 /* kernels of this library launched   */
    long long kind_launches[ACCEL_KINDS];
    double kind_ms[ACCEL_KINDS];        /* CUDA-event time when profiling      */
    long long segments;                 /* overlap-save steps searched         */
    long long cells;                    /* fundamental f-fdot cells searched   */
    double search_ms;                   /* CUDA-event time of the accel_search* */
                                        /* calls, first copy to last read-back */
    long long searches;
    long long graph_launches;           /* searches launched as a CUDA graph   */
    long long graph_builds;             /* of which the graph was instantiated */
                                        /* anew (the others updated it)        */
} accel_stats;

/* Launch shape of a context's search (accel_get_tuning/accel_set_tuning). */
typedef struct accel_tuning {
    int chunk_segments;     /* overlap-save steps per launch group            */
    int plane_split;        /* plane kernel: 0 one thread carries the even and */
                            /* the odd transform at once, 1 it runs them one  */
                            /* after the other (fewer registers, more CTAs    */
                            /* per SM); the fused sum always uses 0           */
    int fused_sum;          /* 1: sum harmonics inside the fundamental's plane */
                            /* kernel; 0: store all planes, tiled sum kernel  */
    int hsum_rowwise;       /* 1: row-wise harmonic-sum kernel instead of the  */
                            /* shared-memory tiled one                        */
    int serial_sum;         /* 1: no overlap of a group's harmonic sum (second */
                            /* stream) with the next group's transforms       */
    int hsum_pipelined;     /* 1: tiled sum from persistent CTAs that overlap */
                            /* the next tiles' copies with the current sums   */
                            /* (producer warps); 0: one CTA per tile          */
    int graph;              /* 1 (default): a search from device-resident     */
                            /* data records its launch groups into a CUDA     */
                            /* graph and launches that (the executable graph  */
                            /* is kept and updated in place while the launch  */
                            /* sequence keeps its shape); 0: direct launches. */
                            /* Searches that copy series from host memory     */
                            /* always launch directly                         */
    int hsum_tile_rows;     /* f-dot rows per tile of the tiled harmonic sum: */
                            /* 8, 16 (default; 0 reads as 16) or 32           */
    int persistent;         /* 1: a launch group's plane rows and harmonic-sum */
                            /* tiles run in one persistent launch from one    */
                            /* work queue, each segment summed as soon as its */
                            /* rows are written (still in L2); segment lengths*/
                            /* other than 8192 and plans it cannot take fall  */
                            /* back to the separate kernels                   */
    int hsum_row_copies;    /* 1: the tiled sum brings each rectangle in by   */
                            /* one bulk copy per row; 0 (default): one 3-D   */
                            /* tensor-map copy (TMA box) per harmonic where  */
                            /* the plan's boxes fit                           */
    int wait_test;          /* failure-detection test, 0 in normal use: each  */
                            /* tile of the tiled harmonic sum expects 16      */
                            /* bytes that never arrive, so its bounded copy   */
                            /* wait (about 33 ms) runs out, the tile sets the */
                            /* error word and returns, and the search fails   */
                            /* with ACCEL_ERR_CUDA; no GPU fault, the context */
                            /* stays usable                                   */
} accel_tuning;

typedef struct accel_ctx accel_ctx;

/* ---------------------------------------------------------------- context */
const char *accel_version(void);
const char *accel_last_error(void);
void accel_config_init(accel_config *cfg);
int  accel_create(const accel_config *cfg, accel_ctx **out);
int  accel_destroy(accel_ctx *ctx);
/* Run all further work of ctx on this cudaStream_t (NULL: the context's own,
 * a blocking stream ordered with the legacy default stream).  Waits for the
 * work already issued on the previous stream. */
int  accel_set_stream(accel_ctx *ctx, void *cuda_stream);
int  accel_synchronize(accel_ctx *ctx);
/* Time every kernel with CUDA events on the context's stream (1) or not (0). */
int  accel_profile(accel_ctx *ctx, int enable);
int  accel_get_stats(accel_ctx *ctx, accel_stats *out);
int  accel_reset_stats(accel_ctx *ctx);

int  accel_get_tuning(const accel_ctx *ctx, accel_tuning *out);
/* Changing chunk_segments reallocates the per-group work buffers. */
int  accel_set_tuning(accel_ctx *ctx, const accel_tuning *t);

int  accel_num_harmonics(const accel_ctx *ctx);
int  accel_num_stages(const accel_ctx *ctx);
int  accel_uselen(const accel_ctx *ctx);
int  accel_harmonic_info(const accel_ctx *ctx, int h, accel_harmonic *out);
/* Power cuts per stage (1, 2, 4, ... harmonics), float[num_stages]. */
int  accel_get_power_cuts(const accel_ctx *ctx, float *cuts);
int  accel_set_power_cuts(accel_ctx *ctx, const float *cuts);
/* Search geometry of a series of n samples at dt seconds (host only):
 * first bin rlo = floor(n*dt) (AccelSearch.cu:101) and the number of
 * overlap-save steps (AccelSearch.cu:209). */
long long accel_first_bin(long long nsamples, double dt);
/* Power of an n-harmonic sum whose Gamma(n,1) tail equals the one-sided
 * Gaussian tail at sigma divided by numindep (the stage cut), and the
 * inverse (a candidate's significance). */
double accel_power_cut(double sigma, int numharm, double numindep);
double accel_sigma_of_power(double power, int numharm, double numindep);
long long accel_step_count(const accel_ctx *ctx, long long nsamples, double dt);
/* Geometry of one harmonic (harmnum/maxharm, widest halfwidth hw0) for the
 * step starting at startr (generate_harmonics_ffdot, bpd_search.cu:72-127,
 * and the segment bounds of :138-144), host only.  out[0..4] = rlo,
 * ceil(rhi), numrs, lobin, numdata. */
int  accel_step_harmonic(long long startr, int uselen, int harmnum, int maxharm, int hw0,
                         long long *out);
/* addPowers index arithmetic (bpd_gpu_kernels.cu:139-153), host only: the
 * sub-harmonic column rind[i] of fundamental column i < nr and the
 * sub-harmonic row zind[z] of fundamental row z < nz (fundamental zlo0,
 * sub-harmonic zlo_h). */
int  accel_harmonic_indices(long long startr, int uselen, int harmnum, int maxharm, int hw0,
                            int zlo0, int zlo_h, int nr, int nz, int *rind, int *zind);

/* Autotuner: for each segment length fftlens[i] (others from *base) build a
 * context, whiten a seeded synthetic spectrum on the device and time a
 * search of `steps` overlap-save steps for every launch shape; the fastest
 * (fundamental f-fdot cells per second) is returned in best_cfg (with its
 * chunk_segments) and best_tuning, its rate in *best_rate. */
int  accel_autotune(const accel_config *base, const int *fftlens, int nlens, int steps,
                    accel_config *best_cfg, accel_tuning *best_tuning, double *best_rate);

/* ------------------------------------------------------------ whole search */
/* Search ntrials time series: R2C FFT, whitening, every overlap-save step,
 * harmonic summing and thresholding.  series[i] holds nsamples[i] float32
 * samples (host memory, or device memory when series_on_device).  Returns
 * the number of candidates in *ncand; fetch them with accel_candidates. */
int  accel_search(accel_ctx *ctx, int ntrials, const float *const *series,
                  const long long *nsamples, const double *dt, int series_on_device,
                  long long *ncand);
/* The same from whitened spectra already on the device (bins [0, numbins)). */
int  accel_search_spectra(accel_ctx *ctx, int ntrials, const accel_complex *const *wspec_dev,
                          const long long *numbins, const long long *rlo, long long *ncand);
/* Candidates of the last search, sorted by (trial, step, numharm, z, r). */
int  accel_candidates(accel_ctx *ctx, accel_candidate *out, long long cap, long long *n);
/* Candidate sifting, host only (the reference's sortCandidates and
 * eliminateHarmonics stubs, bpd_candidates.cu:15-33, AccelSearch.cu:290-305).
 * Per trial: order by sigma (descending; ties by power, then r, z,
 * numharm); keep a candidate only if no kept one is strictly closer than
 * min_dr bins in r (any z or harmonic count); then, when maxharm > 1, drop
 * a kept candidate whose r is within harm_dr bins of (a/b) times a stronger
 * kept candidate's r, 1 <= a, b <= maxharm, a != b.  Output ordered by
 * trial, then sigma; *nout = survivors (at most cap written). */
int  accel_sift_candidates(const accel_candidate *in, long long n, double min_dr, int maxharm,
                           double harm_dr, accel_candidate *out, long long cap, long long *nout);

/* A refined candidate with the properties of its fundamental. */
typedef struct accel_optimized {
    accel_candidate cand;   /* r, z, power and sigma at the refined position  */
    double r_grid, z_grid;  /* the position it started from                   */
    float harm_power[16];   /* power of harmonic k r/numharm, k z/numharm     */
    double f, fdot;         /* r / T (Hz) and z / T^2 (Hz/s), T = tobs        */
    double period, pdot;    /* 1 / f (s) and -fdot / f^2                      */
} accel_optimized;

/* Candidate refinement and properties (the reference's optimizeCandidates
 * and calculateProperties stubs, bpd_candidates.cu:24-33).  For each
 * candidate, on the whitened spectrum of its trial: the summed power of its
 * numharm harmonics (k r/numharm, k z/numharm; each the plane kernels'
 * correlation |sum_j X[j] conj(F(r - j - z/2; z))|^2 over 2 hw(z) bins,
 * F the response of generate_z_response, bpd_subharmonics.cu:146-226,
 * scaled by the segment normalisation the search applied to that harmonic
 * in the candidate's step) is maximised over three nested 5 x 5 grids
 * (steps 1/4, 1/16, 1/64 bins in r and 1, 1/4, 1/16 in z); refine = 0 only
 * evaluates at the given position.  wspec_dev[t], numbins[t], rlo[t] (the
 * first bin searched) and tobs[t] (seconds) describe trial t.  numharm of
 * every candidate must be one of this context's stages. */
int  accel_optimize_candidates(accel_ctx *ctx, int ntrials, const accel_complex *const *wspec_dev,
                               const long long *numbins, const long long *rlo, const double *tobs,
                               const accel_candidate *in, long long n, int refine,
                               accel_optimized *out);
/* The whitened spectrum of trial t of the last accel_search, resident on the
 * device until the next search (for accel_optimize_candidates). */
int  accel_trial_spectrum(accel_ctx *ctx, int trial, const accel_complex **spec_dev,
                          long long *numbins);

/* ------------------------------------------------------------ stage calls */
/* Whitening in place (deredden, bpd_noise.c:12-92), numbins <= 2^31 - 1. */
int  accel_whiten(accel_ctx *ctx, accel_complex *spec_dev, long long numbins);
/* Host only: the whitening block plan of deredden's recurrence
 * (bpd_noise.c:33-79) -- block k holds bins [start[k], start[k] + len[k]).
 * Writes the first min(*nblocks, cap) blocks and sets *nblocks to the full
 * count; ACCEL_ERR_INVALID when numbins is not in [initbuf + 2, 2^31 - 1] or
 * a width is below 1. */
int  accel_whiten_blocks(long long numbins, int initbuf, int maxbuf, int *start, int *len,
                         long long cap, long long *nblocks);
/* Whitening in place, like accel_whiten, for callers that cannot allocate
 * device memory.  No counterpart in the reference.  Some hosts forbid
 * cudaMalloc on the data path: a real-time pipeline that sizes all memory at
 * start-up (cudaMalloc synchronises the device and can fail under memory
 * pressure mid-observation), or a plugin running inside another
 * application's memory pool or under a hard device-memory limit.  This entry
 * point needs no context and calls no cudaMalloc, cudaFree or other
 * allocating routine: its scratch is a static 2 MiB device array that every
 * GPU loading the library holds until exit, enough for 131072 whitening
 * blocks (about 1.2e7 bins with the default widths 6/200); larger spectra
 * are rejected with ACCEL_ERR_INVALID, as are more than 2^31 - 1 bins.  The
 * first call on a device looks up the array's device address
 * (cudaGetSymbolAddress).  The block table reaches the device by a copy from
 * host arrays that every call rewrites, so the call must not be made while
 * its stream is being captured into a CUDA graph: it then returns
 * ACCEL_ERR_UNSUPPORTED.  All calls share the array: calls whose GPU work
 * overlaps race, so serialise them (one stream, or synchronise).
 * cuda_stream may be NULL (the legacy default stream). */
int  accel_whiten_noalloc(accel_complex *spec_dev, long long numbins, int initbuf, int maxbuf,
                          void *cuda_stream);
/* Real-to-complex FFT of a device series into spec_dev (n/2+1 bins), n
 * even.  Computed from power-of-two cuFFT plans only (the n/2 complex pairs
 * by one C2C transform when n/2 is a power of two, else by Bluestein's
 * chirp-z form), so that trials of many lengths make no plan per length. */
int  accel_rfft(accel_ctx *ctx, const float *series_dev, long long n, accel_complex *spec_dev);
/* Segment spectra of nseg steps (first bins startr[]): per step and
 * harmonic the M_h = L_h/2 point spectrum of the normalised segment, packed
 * at dhalf_dev + s*segment_stride + offset_h (see accel_layout). */
int  accel_prepare_segments(accel_ctx *ctx, const accel_complex *wspec_dev, long long numbins,
                            const long long *startr, int nseg, accel_complex *dhalf_dev);
/* Power planes of nseg steps from prepared segment spectra: per step and
 * harmonic numzs_h rows of plane_width_h powers (row stride plane_stride_h). */
int  accel_power_planes(accel_ctx *ctx, const accel_complex *dhalf_dev, int nseg, float *planes_dev);
/* Harmonic sums of nseg steps from power planes; optional stage planes
 * [nseg][nstages][numzs0][uselen]; candidates appended to the context. */
int  accel_sum_harmonics(accel_ctx *ctx, const float *planes_dev, const long long *startr,
                         int nseg, float *stage_dev, long long *ncand);
/* Layout of the per-step buffers used above (elements, not bytes):
 * dhalf: segment_stride, offsets[h];  planes: plane_stride, offsets[h],
 * row strides[h]. */
int  accel_layout(const accel_ctx *ctx, long long *dhalf_stride, long long *dhalf_off,
                  long long *plane_stride, long long *plane_off, int *row_stride);
/* Copy of the template bank: kstd [numzs][L_h] and fold [numzs][L_h]. */
int  accel_bank_spectra(const accel_ctx *ctx, int h, accel_complex *kstd, accel_complex *fold);

/* ------------------------------------------------------------------ serving */
/* A request server with continuous batching (no counterpart in the
 * reference, whose driver searches one trial per process run).  An
 * admission thread admits requests in arrival order while their device
 * memory (series and spectrum, 12 bytes per sample) fits
 * hbm_budget_bytes, and copies, transforms and whitens them on its own
 * stream; a scheduler thread fills each launch group from one template
 * bank (one bank per zmax, built on first use), shortest remaining work
 * first -- a request admitted while others are in flight joins the next
 * group with room, and a short request overtakes a long one -- except that
 * while requests have waited longer than max_wait_s, every other group
 * serves them, oldest first, so that none starves while arrivals
 * continue.  Further groups are launched before the oldest one's
 * candidates are read back.  A request's candidates do not depend on what
 * it was batched with. */
typedef struct accel_server accel_server;

typedef struct accel_server_config {
    double hbm_budget_bytes;  /* device memory for admitted requests (150e9)  */
    int max_active;           /* requests searched at once (0: no limit)       */
    int fftlen;               /* fundamental segment length of every bank      */
    int numharm;              /* harmonics summed                              */
    double sigma;             /* candidate threshold                           */
    int chunk_segments;       /* steps per launch group (0: 128)               */
    int device;
    double max_wait_s;        /* requests waiting longer than this since their */
                              /* submission get every other launch group,     */
                              /* oldest first (0: 1.0 s)                       */
    int max_chunk_segments;   /* > chunk_segments: a launch group grows with   */
                              /* its bank's backlog of prepared steps (a third */
                              /* of it, as groups are kept three deep) up to   */
                              /* this many steps; 0: groups of chunk_segments  */
    int reserved[5];
} accel_server_config;

typedef struct accel_server_stats {
    long long submitted, admitted, completed, queued, active;
    double bytes_in_use;      /* budgeted bytes of the admitted requests       */
    long long cells;          /* fundamental f-fdot cells searched             */
    double gpu_ms;            /* CUDA-event time of the launch groups          */
    double admit_ms;          /* admission-thread time (copy, R2C, whitening)  */
    double group_ms;          /* scheduler time launching and completing groups */
                              /* (includes waiting for the GPU)               */
    double gap_ms;            /* GPU time between consecutive launch groups    */
                              /* while later groups were already queued: the  */
                              /* group stream waiting on the host (or on a    */
                              /* new request's transform and whitening)       */
    double idle_ms;           /* the same after the queue had drained: no step */
                              /* was left to launch (waiting for arrivals)    */
    double wait_ms;           /* part of group_ms blocked on groups' completion */
    double launch_ms;         /* part of group_ms building and launching groups */
    double prep_gpu_ms;       /* CUDA-event time of the requests' transforms and */
                              /* whitening (admission stream)                */
    long long groups;         /* launch groups read back                       */
    long long group_segments; /* their overlap-save segments                   */
} accel_server_stats;

void accel_server_config_init(accel_server_config *cfg);
int  accel_server_create(const accel_server_config *cfg, accel_server **out);
/* Finishes every submitted request, then frees the server. */
int  accel_server_destroy(accel_server *srv);
/* Queue one trial of nsamples float32 samples (host memory, read when the
 * request is admitted: keep it valid until the request completes).  A
 * request larger than the whole budget fails with ACCEL_ERR_BUDGET. */
int  accel_server_submit(accel_server *srv, const float *series, long long nsamples, double dt,
                         int zmax, long long *id);
/* Wait up to timeout_s (< 0: forever); *done = 1 once the request finished. */
int  accel_server_wait(accel_server *srv, long long id, double timeout_s, int *done);
/* Candidates of a finished request (sorted by step, numharm, z, r) and its
 * latency from submission to completion. */
int  accel_server_result(accel_server *srv, long long id, accel_candidate *out, long long cap,
                         long long *n, double *latency_ms);
int  accel_server_release(accel_server *srv, long long id);
/* Latency breakdown of a completed request, milliseconds: [0] submission to
 * admission (HBM budget, admission queue), [1] admission's host
 * work (copy from the caller's memory, transform and whitening launches),
 * [2] prepared to its first launch group, [3] first launch group to
 * completion.  The four add up to the latency accel_server_result reports. */
int  accel_server_timing(accel_server *srv, long long id, double out_ms[4]);
int  accel_server_get_stats(accel_server *srv, accel_server_stats *out);

/* ------------------------------------------------------- dedispersion */
/* Incoherent dedispersion, the step upstream of the search that produces
 * its DM-trial time series (the reference starts from dedispersed series:
 * README.md names dedispersion as the step before it; no function of the
 * reference is replaced).  Direct method:
 *   out[d][t] = sum over channels c, in order, of in[c][t + delay[d][c]].
 * accel_dedisperse_delays (host only): delay[d][c] = floor(4.148808e3 *
 * dms[d] * (f_c^-2 - f_ref^-2) / tsamp + 1/2) samples, f_c = f_top_mhz +
 * c * chan_bw_mhz (chan_bw_mhz < 0 for channels in descending frequency),
 * f_ref the highest channel frequency; delays is int[ndm][nchan], the
 * largest delay in *max_delay. */
int  accel_dedisperse_delays(int nchan, double f_top_mhz, double chan_bw_mhz, double tsamp,
                             const float *dms, int ndm, int *delays, int *max_delay);
/* filterbank_dev: float[nchan][nsamp] (time contiguous) on the device;
 * delays: int[ndm][nchan] in host memory; out_dev: float[ndm][nout] on the
 * device, nout <= nsamp - max delay.  Runs on cuda_stream (NULL: the legacy
 * default stream); each DM trial row of out_dev is a series accel_search
 * takes with series_on_device = 1. */
int  accel_dedisperse(const float *filterbank_dev, int nchan, long long nsamp, const int *delays,
                      int ndm, float *out_dev, long long nout, void *cuda_stream);

/* SIGPROC filterbank reader (host only; the reference reads dedispersed
 * .dat series only, bpd_data.c:9-75, and no function of it is replaced):
 * the header keywords, then nifs = 1 time-major samples of 8 bits (unsigned,
 * or two's-complement when the one-byte "signed" keyword is nonzero), 16 bits
 * (unsigned) or 32 bits (float).  *data is a malloc'd float32
 * [nchans][nsamples], channel-major as accel_dedisperse takes it (channel c
 * at fch1 + c * foff MHz); free it with accel_free_host. */
typedef struct accel_filterbank_info {
    int nchans, nbits, nifs;
    long long nsamples;
    double tsamp;           /* seconds                                        */
    double fch1, foff;      /* MHz: first channel, channel step               */
    double tstart;          /* MJD                                            */
    char source_name[80];
    int header_bytes;
    int is_signed;          /* "signed" keyword: 8-bit samples are int8      */
} accel_filterbank_info;
int  accel_read_filterbank(const char *path, accel_filterbank_info *info, float **data);
void accel_free_host(void *p);

#ifdef __cplusplus
}
#endif
#endif /* ACCELSEARCH_H_ */
