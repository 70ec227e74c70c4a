/*
 * grtm_gb300.h -- C ABI of the GB300 layered-medium Green's-function library
 * (generalized reflection-transmission method).
 *
 * Drop-in for the reference project cangyeone/grtm_cuda: the library exports
 * the reference's entry point `green` with its signature and file formats,
 * plus a status-returning, array-based interface for many receivers.
 * Plain C types only; every call reports errors through its return value.
 */
#ifndef GRTM_GB300_H_
#define GRTM_GB300_H_

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define GRT_API __attribute__((visibility("default")))
#else
#define GRT_API
#endif

/* status codes */
#define GRT_OK 0
#define GRT_ERR_ARG 1          /* bad argument */
#define GRT_ERR_IO 2           /* file could not be opened or written */
#define GRT_ERR_PARSE 3        /* malformed input file */
#define GRT_ERR_MODEL 4        /* layered model the method cannot take */
#define GRT_ERR_CUDA 5         /* CUDA runtime error (message in grt_last_error) */
#define GRT_ERR_NOMEM 6        /* device or host allocation failed */
#define GRT_ERR_TIMEOUT 7      /* a bounded device wait gave up */
#define GRT_ERR_UNSUPPORTED 8  /* size beyond what this library handles */

/* wavenumber grids */
#define GRT_K_REFERENCE 0      /* per-frequency k_max rule of the reference, dk = 2 pi / L */
#define GRT_K_FIXED 1          /* nk_fixed points k_j = j dk at every frequency */
#define GRT_K_CUSTOM 2         /* opts.nk_custom[iw] points k_j = j dk at frequency iw */

/* working precision of the per-(w,k) kernel and the wavenumber sum */
#define GRT_FP32 0
#define GRT_FP64 1

/* corrections of reference quirks; 0 reproduces the reference */
#define GRT_FIX_RLAYER 1       /* receiver layer located with the receiver depth */
#define GRT_FIX_REXUT 2        /* d/dz terms use the local vertical wavenumber */
#define GRT_FIX_DZ 4           /* d/dz terms without the doubled factor / reused product */
#define GRT_FIX_COLS 8         /* corrected output columns: moment tensor 30 defined columns (0-9
                                * displacement, 10-19 d/dz, 20-29 d/dr; the m = 1 transverse terms
                                * with b1; the m = 0 radial terms 2, 3 with the radial coefficients
                                * where green.cu:1652-1653 take the vertical ones), single force d/dr
                                * column 10 with its 1/r, Bessel second derivatives from Bessel's
                                * equation.  The 30-column layout runs the SIMT wavenumber sum. */
#define GRT_FIX_SHSRC 16       /* moment-tensor SH source terms: the reference (get_src_tensor,
                                * green.cu:1409-1412) gives the m = 1 and m = 2 SH terms one
                                * reflection factor; with this bit m = 1 (a jump of the SH
                                * displacement) takes 1 - e Rdu e above the source and m = 2 (a jump
                                * of the SH traction) 1 + e Rud e below it, and the moment-tensor
                                * solution satisfies reciprocity with the single-force one. */
#define GRT_FIX_COLS20 32      /* corrected moment-tensor columns in the reference's 20-column layout, the one
                                * the tensor-core sum takes: displacement 0-9 and d/dr 10-19 as GRT_FIX_COLS
                                * gives them in its columns 0-9 and 20-29 (the m = 0 radial columns 2, 3 and
                                * d/dr 12, 13 with the radial coefficients a20, a00; the m = 1 transverse
                                * column 5 and d/dr 15 with b1), no d/dz columns; Bessel second derivatives from
                                * Bessel's equation; single forces as GRT_FIX_COLS.  Ignored with GRT_FIX_COLS. */

/* A layered model: n_layer layers given by the depth of their top (ztop[0] = 0),
 * the last one being the half-space.  Units: km, km/s, g/cm^3. */
typedef struct grt_model {
    int n_layer;
    const double *ztop, *vp, *vs, *rho, *qp, *qs;
    double hs;      /* source depth */
    double hr;      /* receiver depth */
    int src_type;   /* 0 single force, otherwise moment tensor */
} grt_model;

typedef struct grt_opts {
    double dt;            /* sampling interval, s */
    int log2n;            /* N = 2^log2n samples (2..15) */
    double t0;            /* reduction time, s */
    double taper;         /* fraction of the band tapered at the top */
    double sigma_factor;  /* imaginary frequency sigma = sigma_factor / (N dt); reference: 2 */
    int k_mode;           /* GRT_K_REFERENCE or GRT_K_FIXED */
    int nk_fixed;         /* points of the fixed grid */
    double dk;            /* > 0 overrides the wavenumber step */
    int precision;        /* GRT_FP32 or GRT_FP64 */
    int fix;              /* GRT_FIX_* bits */
    const int *nk_custom; /* GRT_K_CUSTOM: points per frequency, N/2 entries (e.g. a learned grid) */
    const int *k_stride;  /* GRT_K_CUSTOM, optional: per-frequency stride m in 1..64, k_j = j m dk
                           * (N/2 entries; NULL = 1).  FP32 plans (tensor-core sum) need one stride
                           * per aligned block of 64 frequencies. */
    int n_freq_sel;       /* > 0: evaluate only these positive frequencies (a spectra-only plan: */
    const int *freq_sel;  /* distinct indices in 0..N/2-1, any order; grt_plan_fetch_freqs reads them,
                           * traces, synthesis and files are GRT_ERR_UNSUPPORTED).  0 / NULL: all. */
    int k_slice;          /* FP32 tensor-core sum: wavenumbers per split-K slice, a multiple of 8 (16 for
                           * 3xBF16; 0: chosen to fill the GPU).  Plans with one k_slice add each frequency's
                           * wavenumbers in the same order: their sums agree bit for bit on a common k range. */
    int tc_split;         /* FP32 tensor-core sum: GRT_TC_3XTF32 (hi*hi + hi*lo + lo*hi of TF32 halves, about
                           * 2^-21 per product) or GRT_TC_3XBF16 (the same with BF16 halves, about 2^-16 per
                           * product, half the operand bytes and twice the MMA rate) */
} grt_opts;

#define GRT_TC_3XTF32 0
#define GRT_TC_3XBF16 1

typedef struct grt_report {
    int n_layer;          /* after source-interface insertion */
    int s_layer, r_layer;
    double zs, zr;
    int nw;               /* positive frequencies evaluated (N/2, or n_freq_sel) */
    int n_samples;        /* N */
    int n_cols;           /* defined output columns: 15 single force, 20 moment tensor (30 with GRT_FIX_COLS) */
    long long n_wk;       /* (w,k) points evaluated */
    int nk_max;
    double dk, df, sigma;
    float ms_grt, ms_bessel, ms_ksum, ms_spectral, ms_total;  /* device time of the last execute */
    int kernel_launches;  /* kernels launched by the last execute */
    long long h2d_bytes;  /* bytes the plan uploads (layer tables, grids, receivers) */
    long long d2h_bytes;  /* bytes one fetch of the traces downloads */
    int ksum_impl;        /* wavenumber sum: 0 SIMT FP32/FP64, 1 tensor cores 3xTF32, 2 FP32 SGEMMs (cuBLAS),
                           * 3 tensor cores 3xBF16 */
    int k_slice;          /* tensor-core sum: wavenumbers per split-K slice (0 for the SIMT sum) */
    long long n_layer_evals;  /* layers the GRT kernel evaluated over all (w,k) points (below n_wk x n_layer
                               * where depth truncation starts the recursion above the half-space) */
} grt_report;

typedef struct grt_ctx grt_ctx;
typedef struct grt_plan grt_plan;

/* Contexts own a CUDA stream on one device and a cache of the device memory
 * their plans and batches release (reused by the next ones, up to half the
 * device memory).  A context (with its plans and batches) is used from one
 * host thread at a time; different contexts may run on different threads at
 * once (their work then shares the GPU).  Destroy plans and batches first. */
GRT_API int grt_create(grt_ctx **ctx, int device);
GRT_API void grt_destroy(grt_ctx *ctx);
/* Return the context's cached device memory to the driver. */
GRT_API void grt_trim(grt_ctx *ctx);
/* high != 0: the context's streams (its own and those of the batches made on
 * it afterwards) take the device's greatest stream priority, so its kernels'
 * blocks are scheduled ahead of other contexts' pending blocks (a small job
 * beside a long batch on another context); 0: the default priority.  Only
 * while the context holds no plan or batch (GRT_ERR_ARG otherwise). */
GRT_API int grt_set_priority(grt_ctx *ctx, int high);
/* Wait for all work the process queued on a device (every context's streams):
 * cudaDeviceSynchronize, for callers that hold no CUDA runtime of their own. */
GRT_API int grt_device_synchronize(int device);
GRT_API const char *grt_last_error(const grt_ctx *ctx);
GRT_API const char *grt_status_string(int status);

/* A plan holds one model, its grids, its receivers and all device buffers.
 * Creating it uploads the inputs; executing it runs the kernels, leaving the
 * results in device memory; fetching copies them to the host. */
GRT_API int grt_plan_create(grt_ctx *ctx, const grt_model *model, const grt_opts *opts, int n_dist,
                    const double *dist, grt_plan **plan);
GRT_API int grt_plan_execute(grt_plan *plan, grt_report *report);
/* traces: [n_dist][n_cols][N] doubles; spectra: [n_dist][n_cols][N] complex as
 * (re, im) doubles (after taper and Hermitian fill).  Either may be NULL. */
GRT_API int grt_plan_fetch(grt_plan *plan, double *traces, double *spectra);
/* traces as float32 [n_dist][n_cols][N] (FP32 plans: their working precision) */
GRT_API int grt_plan_fetch_f32(grt_plan *plan, float *traces);
/* Page-locked host memory (cudaHostAlloc) for fetch destinations: copies into
 * it run at the host link's full rate instead of through a staging buffer.
 * Allocate once and reuse: pinning is slow.  No counterpart in the reference. */
GRT_API int grt_host_alloc(size_t bytes, void **ptr);
GRT_API void grt_host_free(void *ptr);
/* spectra at selected frequency indices (0..N-1) only: [n_dist][n_cols][n_freq]
 * complex as (re, im) doubles.  A plan made with opts.freq_sel answers for
 * its selected frequencies only (others: GRT_ERR_ARG). */
GRT_API int grt_plan_fetch_freqs(grt_plan *plan, int n_freq, const int *freq_idx, double *spectra);
GRT_API int grt_plan_info(const grt_plan *plan, grt_report *report);
GRT_API void grt_plan_destroy(grt_plan *plan);
/* Grid of a model and options without a plan or a device: fills the layer,
 * frequency and wavenumber fields of report (n_wk, nk_max, dk, ...), the
 * timing fields zero.  Errors as grt_plan_create, message on stderr. */
GRT_API int grt_grid(const grt_model *model, const grt_opts *opts, grt_report *report);

/* Convergence sweep of the plain method (training data and judge of the
 * learned wavenumber sampler).  For the frequencies freq_idx[0..n_freq) it
 * evaluates the per-(w,k) kernel on the grid of opts (unit stride) and, for
 * each frequency and distance r_b, forms the weighted integrand envelope
 * g(k) = max_q |K_q(w,k)| (1+k)^2 min(1, (k r_b)^-1/2).  Outputs, all
 * [n_freq][n_band] (alias_out [n_freq][n_band][6]); all but kmax_out optional:
 *   kmax_out   smallest k_c whose envelope tail beyond k_c is at most tol times
 *              the envelope total, or at most tol_abs[i] when tol_abs is given;
 *   tail_out   envelope fraction beyond k_judge[i] (needs k_judge);
 *   env_out    envelope total;
 *   alias_out  with S_q^(s) = s dk sum_{j = 0 mod s, j dk < k_c} K_q J0(k r_b):
 *              [0] = max_q |S_q^(1)|, [s] = max_q |S_q^(2^s) - S_q^(1)| (s = 1..5),
 *              the spatial aliasing of a 2^s times coarser step at r_b.
 * FP32 kernel; layer tables for the listed frequencies only (opts.freq_sel
 * must be empty).  No counterpart in the reference (its k_max is the fixed
 * rule of cal_kmax, green.cu:108-162). */
GRT_API int grt_sweep_kmax(grt_ctx *ctx, const grt_model *model, const grt_opts *opts, int n_freq,
                           const int *freq_idx, int n_band, const double *band_r, double tol,
                           const double *tol_abs, const double *k_judge, double *kmax_out, double *tail_out,
                           double *env_out, double *alias_out);

/* The learned sampler's network: n_in -> 64 -> 64 -> 64 -> n_out with SiLU
 * hidden activations, FP32, trained by the library's own CUDA kernels
 * (forward, backward, Adam) on mean squared error.  Host arrays in and out,
 * row-major [n][n_in] / [n][n_out].  No counterpart in the reference. */
typedef struct grt_mlp grt_mlp;
GRT_API int grt_mlp_create(grt_ctx *ctx, int n_in, int n_out, unsigned long long seed, grt_mlp **mlp);
GRT_API void grt_mlp_destroy(grt_mlp *mlp);
GRT_API int grt_mlp_n_params(const grt_mlp *mlp);
GRT_API int grt_mlp_get_params(grt_mlp *mlp, float *params);
GRT_API int grt_mlp_set_params(grt_mlp *mlp, const float *params);
GRT_API int grt_mlp_forward(grt_mlp *mlp, int n, const float *x, float *y);
/* loss and its gradient with respect to the parameters (for checks) */
GRT_API int grt_mlp_loss_grad(grt_mlp *mlp, int n, const float *x, const float *t, float *loss, float *grad);
/* epochs of shuffled mini-batch Adam; loss of the last batch */
GRT_API int grt_mlp_train(grt_mlp *mlp, int n, const float *x, const float *t, int epochs, int batch, float lr,
                          unsigned long long seed, float *loss);

/* Batches: many jobs -- layered models with any layer count, source depth,
 * receiver set, grid and length -- executed together.  The per-(w,k) kernel
 * runs as one persistent launch over the wavenumber tiles of every job; each
 * job's Bessel table, wavenumber sum and spectral stage follow on side
 * streams; the whole execution is captured once into a CUDA graph, so each
 * grt_batch_execute is a single graph launch.  With autotune != 0 the GRT
 * launch shape (wavenumbers per tile = threads per block; one block per tile
 * or a persistent grid of a multiple of the resident blocks) is picked by
 * timing the candidates on a sample of the batch's tiles; otherwise one block
 * per tile of 128.  All jobs share one precision.  No counterpart in the
 * reference (one model per call). */
typedef struct grt_job {
    const grt_model *model;
    const grt_opts *opts;
    int n_dist;
    const double *dist;
    float *out_f32;   /* optional (FP32 batches): page-locked memory (grt_host_alloc) for the job's
                       * float32 traces [n_dist][n_cols][N]; every execute copies them there as soon
                       * as the job's stages finish, beside the later jobs' work.  NULL: fetch them. */
} grt_job;

#define GRT_TUNE_MAX 16
typedef struct grt_tune {
    int tuned;                     /* 1: picked by timing; 2: reused from an earlier batch of the
                                    * same precision and deepest model on this device (any context of
                                    * the process); 0: default */
    int grt_shape;                 /* chosen GRT launch: 0-2 one block per tile of 64/128/256
                                    * wavenumbers, 3-4 persistent with 128/256 threads */
    int grt_threads, grt_blocks;   /* its threads per block; persistent grid (0: one per tile) */
    int n_cand;                    /* candidates tried */
    int cand_threads[GRT_TUNE_MAX], cand_blocks[GRT_TUNE_MAX];
    float cand_ms[GRT_TUNE_MAX];   /* their times on the sample */
    double sample_fraction;        /* fraction of the tiles timed */
    /* the tensor-core wavenumber sums' split of the k range (FP32 batches; jobs without opts.k_slice):
     * candidate splits of the largest job timed, the best one's ratio to the wave-filling default
     * applied to every job */
    int tc_tuned;                  /* 1 timed, 2 reused from an earlier batch of the same kind, 0 default */
    int tc_nsplit;                 /* the largest job's k slices */
    int tc_n_cand;
    int tc_cand_split[4];
    float tc_cand_ms[4];
} grt_tune;

typedef struct grt_batch grt_batch;
GRT_API int grt_batch_create(grt_ctx *ctx, int n_jobs, const grt_job *jobs, int autotune, grt_batch **batch);
/* report: aggregate (n_wk, bytes, launches; ms_grt and ms_total of the graph) */
GRT_API int grt_batch_execute(grt_batch *batch, grt_report *report);
/* grt_batch_execute in three steps, for callers that overlap consecutive
 * batches: grt_batch_launch starts the graph and returns; grt_batch_wait_stages
 * returns once every job's device stages are done (the traces of all jobs but
 * the last one already downloaded into their out_f32 destinations; the last
 * job's download is started on the batch's copy stream), so that the caller
 * can launch its next batch while that download drains; grt_batch_finish
 * waits for it, checks the device error word and fills the report.  Call
 * them in this order, once each per execution. */
GRT_API int grt_batch_launch(grt_batch *batch);
GRT_API int grt_batch_wait_stages(grt_batch *batch);
GRT_API int grt_batch_finish(grt_batch *batch, grt_report *report);
GRT_API int grt_batch_fetch(grt_batch *batch, int job, double *traces, double *spectra);
GRT_API int grt_batch_fetch_f32(grt_batch *batch, int job, float *traces);
/* The same without waiting (FP32 batches): the copy of the last execute's
 * traces into `traces` (page-locked memory from grt_host_alloc, left
 * untouched until grt_batch_wait returns) runs on the batch's own copy stream
 * beside later work on the context, such as the sampler's judge.
 * grt_batch_wait waits for every copy started; grt_batch_execute and
 * grt_batch_destroy wait for them first. */
GRT_API int grt_batch_fetch_f32_async(grt_batch *batch, int job, float *traces);
GRT_API int grt_batch_wait(grt_batch *batch);
GRT_API int grt_batch_fetch_freqs(grt_batch *batch, int job, int n_freq, const int *freq_idx, double *spectra);
/* job = -1: the batch's aggregate report */
GRT_API int grt_batch_info(const grt_batch *batch, int job, grt_report *report, grt_tune *tune);
/* Forget the autotuner's choices (kept per device for the process, shared by
 * its contexts): the next autotuned batch of each kind times its candidates
 * again. */
GRT_API void grt_tune_clear(void);
GRT_API void grt_batch_destroy(grt_batch *batch);

/* Binary output of a plan's traces (beside the reference's %.18e text,
 * green.cu:2242-2258, which dominates wall time at many receivers):
 * "GRTMBIN1", int32 version (1), n_dist, n_cols, N, float64 dt, t0, sigma,
 * float64 dist[n_dist], float32 traces [n_dist][n_cols][N], little-endian.
 * No counterpart in the reference. */
GRT_API int grt_plan_write(grt_plan *plan, const char *path);

/* Earth-flattening transform of a spherical model (the reference's caller-side
 * preprocessing, greent.py:13-47 and 65-67, moved into the library): a layer
 * of thickness h whose bottom lies at radius r is stretched by R / (r + h/2),
 * and so are its Vp and Vs; the flat tops are the running sum of the
 * stretched thicknesses; source and receiver depths map by R ln(R / (R - z)).
 * Density and Q are unchanged.  Host only (no device). */
GRT_API int grt_flatten(int n_layer, const double *ztop, const double *vp, const double *vs, double hs, double hr,
                        double r_earth, double *ztop_f, double *vp_f, double *vs_f, double *hs_f, double *hr_f);

/* Seismograms from a moment-tensor job (a single-force job: its displacement
 * columns weighted by grt_sf_weights for the force src->f, below): after
 * grt_plan_execute (or grt_batch_execute), the receivers' Green's-function
 * columns are combined
 * for a source mechanism and azimuth, convolved with a source-time function,
 * and brought to the time domain in one fused kernel (combination, source
 * spectrum, phase/taper/scale, Hermitian fill, inverse DFT, e^{sigma t}).
 * Combination, in the azimuthal families of the displacement columns 0-9
 * (m = 2: columns 0, 4, 6; m = 1: 1, 5, 7; m = 0: 3, 8; the isotropic
 * horizontal part of the m = 2 family: 2, 9), phi = the receiver's azimuth
 * from the source:
 *   Z = c2 G6 - c1 G7 + Mzz G8 - h G9,  R = c2 G0 - c1 G1 + Mzz G3 - h G2,
 *   T = s2 G4 - s1 G5,
 *   c2 = (Mxx-Myy)/2 cos 2phi + Mxy sin 2phi, s2 = -(Mxx-Myy)/2 sin 2phi + Mxy cos 2phi,
 *   c1 = Mxz cos phi + Myz sin phi,            s1 = -Mxz sin phi + Myz cos phi,
 *   h = (Mxx+Myy)/2,
 * giving displacement Z up, R away from the source, T clockwise (azimuth
 * increasing): by reciprocity every term equals the moment tensor contracted
 * with the gradient, at the source, of the single-force solution for a unit
 * force at the receiver.  A corrected layout (GRT_FIX_COLS or GRT_FIX_COLS20) and
 * GRT_FIX_SHSRC are needed for that; with the reference's columns R of Mzz
 * and h, and the SH parts, keep the reference's errors.
 * The source-time function s_n (at opts.dt) enters as dt sum_n s_n e^{-i (w - i sigma) n dt},
 * so the seismogram is dt sum_m s_m G(t - m dt) (circularly, with the damped
 * wrap-around of the method).  No counterpart in the reference, which stops
 * at the columns. */
typedef struct grt_source {
    double m[6];          /* Mxx, Myy, Mzz, Mxy, Mxz, Myz; x north, y east, z down (moment-tensor jobs) */
    int n_stf;            /* source-time samples (0: impulse) */
    const double *stf;
    double f[3];          /* Fx, Fy, Fz; x north, y east, z down (single-force jobs) */
} grt_source;
/* double couple: strike, dip, rake in degrees, scalar moment m0 -> m[6] (Aki & Richards, Box 4.4) */
GRT_API void grt_dc_moment(double strike, double dip, double rake, double m0, double *m);
/* The combination above as weights: w[3 (Z, R, T)][30] of the moment-tensor
 * columns for moment tensor m[6] at one azimuth (degrees), for callers that
 * combine fetched or written columns themselves.  Host only (no device).  No
 * counterpart in the reference. */
GRT_API void grt_mt_weights(const double *m, double azimuth, double *w);
/* Single force: w[3 (Z up, R away, T clockwise)][15] of the single-force
 * columns for force f[3] = (Fx, Fy, Fz; x north, y east, z down) at the
 * receiver's azimuth from the source (degrees clockwise from north):
 *   Z = Fr G3 + Fz G4,  R = Fr G0 + Fz G1,  T = Ft G2,
 *   Fr = Fx cos phi + Fy sin phi, Ft = -Fx sin phi + Fy cos phi.
 * The displacement columns 0-4 are the reference's in both layouts.  Host
 * only (no device); grt_plan_synth applies them to single-force jobs (with
 * src->f).  No counterpart in the reference. */
GRT_API void grt_sf_weights(const double *f, double azimuth, double *w);
/* azimuth: degrees clockwise from north, one per receiver; seis: [n_dist][3 (Z, R, T)][N] */
GRT_API int grt_plan_synth(grt_plan *plan, const grt_source *src, const double *azimuth, double *seis);
GRT_API int grt_batch_synth(grt_batch *batch, int job, const grt_source *src, const double *azimuth, double *seis);

/* Predicted error of a plan's traces (the judge of the FP32 path): for each
 * receiver, the relative L2 error its traces [n_cols][N] are expected to have
 * against the FP64 path of the same method.  The per-(w,k) coefficients carry
 * relative rounding noise eps(w), independent from one wavenumber to the
 * next; the wavenumber sum adds it up, the spectral stage carries it to the
 * trace (taper, inverse DFT, e^{sigma t} de-damping), and it is compared with
 * the trace's own norm; the sum's own rounding is a floor under it.  eps > 0
 * gives eps(w) = eps; eps = 0 measures it: an FP64 evaluation of the plan's
 * (w,k) points at 16 spot frequencies (about 16 / (N/2) of an FP64 plan's GRT
 * work) against the plan's FP32 coefficients (FP64 plans: GRT_EPS_FP64).
 * The estimate follows the measured error over five orders of magnitude,
 * including the far receivers of short windows where the wavenumber sum
 * cancels by a factor 10^6 and FP32 cannot reach 1e-3; a caller recomputes
 * the receivers above its tolerance in FP64.  After grt_plan_execute /
 * grt_batch_execute; est: n_dist doubles.  Full plans only (a frequency
 * selection has no traces: GRT_ERR_UNSUPPORTED).  No counterpart in the
 * reference (FP64 only). */
#define GRT_EPS_FP64 1e-15
GRT_API int grt_plan_error_estimate(grt_plan *plan, double eps, double *est);
GRT_API int grt_batch_error_estimate(grt_batch *batch, int job, double eps, double *est);

/* create + execute + fetch + destroy */
GRT_API int grt_run(grt_ctx *ctx, const grt_model *model, const grt_opts *opts, int n_dist,
            const double *dist, double *traces, double *spectra, grt_report *report);

/* For callers that cannot allocate device memory -- a process whose GPU memory
 * is reserved by another runtime (a framework's caching allocator, a service
 * with a fixed device budget) or code running where cudaMalloc is not
 * permitted.  The traces grt_run gives in FP32, to FP32 rounding (it runs
 * the generic GRT form and the SIMT wavenumber sum), for small jobs,
 * allocating nothing on the device: all intermediates live in one library-owned device
 * array of 32 MiB per GPU and the job tables in a 4 MiB host array.  A GPU
 * takes the device array when the library's kernels are first loaded on it
 * (with CUDA's default lazy module loading, at the first grt_run_noalloc call
 * there; with CUDA_MODULE_LOADING=EAGER, when its context is created) and
 * holds it until the process exits.  Jobs that need more return
 * GRT_ERR_UNSUPPORTED with the sizes on stderr.  Every call looks up the
 * array's address on `device` (cudaGetSymbolAddress, no allocation), copies
 * synchronously and waits for its kernels: do not call it inside a stream
 * capture.  Calls share the arrays: calls that overlap on the GPU, or come
 * from several host threads at once, race.  Runs on the default stream of
 * `device`; traces: host [n_dist][n_cols][N] doubles (n_cols 15 for a single
 * force, 20 for a moment tensor).
 * Reference-rule and fixed grids of all frequencies only (GRT_K_CUSTOM or a
 * frequency selection: GRT_ERR_UNSUPPORTED).
 * No counterpart in the reference. */
GRT_API int grt_run_noalloc(int device, const grt_model *model, const grt_opts *opts, int n_dist,
                            const double *dist, double *traces);

/* The reference's file-to-file call with a status: reads the positional input
 * file, writes oname_w (N rows x 30 "re,im," pairs) and oname_t (N rows x 30
 * values), each "%.18e,", exactly as the reference does.  Runs in FP32 unless
 * the environment variable GRT_PRECISION=fp64. */
GRT_API int grt_green(const char *iname, const char *oname_w, const char *oname_t);

/* Replaces: extern "C" void green(char *iname, char *oname_w, char *oname_t);
 * cusrc/popm/popm.h:159-161, defined at cusrc/popm/func/green.cu:1975.
 * Same signature and files; errors go to stderr (the reference has no
 * status).  Callers: cusrc/main.cu:8, greent.py:94-98 (ctypes). */
GRT_API void green(char *iname, char *oname_w, char *oname_t);

#ifdef __cplusplus
}
#endif
#endif
