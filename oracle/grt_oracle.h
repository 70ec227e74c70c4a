/*
 * grt_oracle.h -- FP64 CPU oracle of the layered-medium Green's-function
 * pipeline (generalized reflection-transmission method).
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the CUDA
 * product in grtm_cuda_gb300/.  Only tests/, __graft_entry__.smoke() and the
 * cpu_baseline / reference arm of bench.py may load it.  The product never
 * links it and never falls back to it.
 *
 * It restates, step by step and in plain FP64 C, what the reference
 * (cangyeone/grtm_cuda, cusrc/popm/func/green.cu) computes, including the
 * reference's known quirks (they are switchable, see GRTO_FIX_*), so that the
 * reference's own golden vectors demo/oname_{t,w}.txt can be reproduced.
 *
 * Pinned: to those golden vectors (single force, surface receiver), and with
 * the quirks corrected, to first principles the tests check per (w, k) and
 * per trace -- source-receiver reciprocity, the traction-free surface,
 * continuity across interfaces, the source's jump conditions and the
 * moment-tensor displacement obtained by reciprocity.  Those checks found the
 * quirks GRTO_FIX_SHSRC and the m = 0 radial columns of GRTO_FIX_COLS.
 */
#ifndef GRT_ORACLE_H_
#define GRT_ORACLE_H_

#ifdef __cplusplus
extern "C" {
#endif

#define GRTO_MAXL 256      /* layers after source-interface insertion */

/* status codes */
#define GRTO_OK 0
#define GRTO_ERR_IO 1
#define GRTO_ERR_PARSE 2
#define GRTO_ERR_MODEL 3
#define GRTO_ERR_ARG 4
#define GRTO_ERR_NOMEM 5

/* k-grid modes */
#define GRTO_K_REFERENCE 0 /* ragged per-frequency k_max (green.cu:2145-2194) */
#define GRTO_K_FIXED 1     /* nk_fixed points k_j = j*dk for every frequency */

/* Corrections of reference quirks.  0 = bug-compatible with the reference. */
#define GRTO_FIX_RLAYER 1  /* receiver layer searched with hr, not hs (green.cu:2092-2101) */
#define GRTO_FIX_REXUT 2   /* d/dz terms use this (w,k) point's nu, not slot 0's (green.cu:674-675) */
#define GRTO_FIX_DZ 4      /* d/dz vertical factors without the double nu / reuse quirks
                              (green.cu:720, 842, 902) */
/* Not a correction: evaluate the same recursion in the well-conditioned
 * basis (see grt_oracle.c).  Same results where the reference's 4x4 solve is
 * well conditioned; accurate also at w -> 0 where the reference loses digits. */
#define GRTO_STABLE 8
/* Corrected output columns (not the reference's layout): moment tensor with
 * 30 defined columns -- displacement 0-9 (the m = 1 transverse term with b1
 * where green.cu:1657 has b2), d/dz 10-19 from the z-derivative coefficients
 * (the block green.cu:1666-1677 writes and then overwrites), d/dr 20-29
 * (green.cu:1680-1691, column 25 with b1); single force: the d/dr column 10
 * with the 1/r of its b1 k J1' term; second Bessel derivatives from Bessel's
 * equation instead of dd_besselj (green.cu:1540-1554); the m = 0 radial
 * moment-tensor columns 2, 3 (and their d/dz 12, 13, d/dr 22, 23) from the
 * radial coefficients a2[0], a0[0] where green.cu:1652-1653 use the vertical
 * ones a2[1], a0[1]. */
#define GRTO_FIX_COLS 16
/* SH source terms of the moment tensor (get_src_tensor, green.cu:1409-1412):
 * the reference gives the m = 1 and m = 2 SH terms one reflection factor,
 * 1 + e Rdu e up and e Rud e - 1 down.  m = 1 (a vertical couple: a jump of
 * the SH displacement) needs opposite signs up and down, 1 - e Rdu e up;
 * m = 2 (a jump of the SH traction) the same sign, 1 + e Rud e down -- as the
 * P-SV terms beside them have (wru0/wrd0 for m = 1, wru1/wrd1 for m = 0, 2).
 * With this bit the moment-tensor SH coefficients satisfy reciprocity with
 * the single-force solution. */
#define GRTO_FIX_SHSRC 32
/* Not a correction of a quirk but of a convention, in the oracle only: the
 * reference's stress terms take the real mu0 = b0^2 rho with attenuated
 * velocities -- the viscoelastic medium of density rho (b0 / beta(w))^2.
 * With this bit they take mu = rho beta(w)^2, the standard viscoelastic
 * medium of density rho. */
#define GRTO_ATTEN_MU 64

typedef struct grto_job {
    /* model after source-interface insertion (green.cu:1995-2049) */
    int n_layer;
    double h[GRTO_MAXL];   /* thickness; last entry keeps the half-space top depth */
    double a0[GRTO_MAXL], b0[GRTO_MAXL], rho[GRTO_MAXL], qp[GRTO_MAXL], qs[GRTO_MAXL];
    double mu[GRTO_MAXL];  /* b0^2 * rho (real, unattenuated) */
    int inserted;          /* 1 if a source interface was inserted */
    double hs, hr;         /* source / receiver depth as given, km */
    int s_layer, r_layer;
    double zs, zr;         /* depth of source / receiver below the top of its layer */
    int src_type;          /* 0 single force, otherwise moment tensor */
    /* time / frequency grid (green.cu:2051-2080) */
    double dt, t0, taper, twin;
    int nf1, nf2, n_ptam, log2n;
    int nw;                /* number of positive frequencies, N/2 */
    double df, sigma, dk, vmax, vmin;
    /* wavenumber grid */
    int k_mode, nk_fixed;
    int fix;               /* GRTO_FIX_* bits */
    /* receivers */
    int n_dist;
    const double *dist;
    double dist0;          /* the single distance of an input file */
} grto_job;

/* Parse a reference input file (format of green.cu:1995-2060). */
int grto_parse(const char *path, grto_job *job);

/* Build a job from arrays: n_in layers given by depth-to-top ztop (ztop[0] = 0). */
int grto_model(grto_job *job, int n_in, const double *ztop, const double *vp,
               const double *vs, const double *rho, const double *qp,
               const double *qs, double hs, double hr, int src_type);

/* Grid and layer location (green.cu:2065-2101).  sigma_factor: sigma = f / T
 * (the reference uses 2).  dk_override > 0 replaces the reference's dk. */
int grto_setup(grto_job *job, double dt, int log2n, double t0, double taper,
               double sigma_factor, int k_mode, int nk_fixed, double dk_override,
               int fix);

/* Number of wavenumbers used at frequency index iw. */
int grto_nk(const grto_job *job, int iw);

/* Total number of (w,k) points. */
long long grto_nkw(const grto_job *job);

/* Full pipeline for job->n_dist receivers (job->dist).
 *   spec: n_dist x N x 30 complex (re,im interleaved) after taper and
 *         Hermitian fill, or NULL;
 *   sig:  n_dist x N x 30 real time series after the inverse DFT and
 *         de-damping, or NULL.  N = 2*nw. */
int grto_run(const grto_job *job, double *spec, double *sig, int nthreads);

/* k-sums (before taper) of frequencies iw0 <= iw < iw1 for all receivers:
 * sums [iw1-iw0][n_dist][30] complex.  Used to time a bounded sample. */
int grto_run_band(const grto_job *job, int iw0, int iw1, double *sums, int nthreads);

/* Per-(w,k) receiver coefficients, for kernel-level comparisons.
 *   out: 16 complex (re,im) = a0[2], a1[2], a2[2], b1, b2, a0t[2], a1t[2],
 *   a2t[2], b1t, b2t (a2/b2 are zero for a single force). */
int grto_point(const grto_job *job, int iw, double k, double *out);

/* Integrand values (15 or 30 columns) at (iw, k) for distance r. */
int grto_integrand(const grto_job *job, int iw, double k, double r, double *out);

/* Whole reference call: read iname, write oname_w / oname_t like green(). */
int grto_green(const char *iname, const char *oname_w, const char *oname_t,
               int nthreads);

/* Bessel functions exactly as the reference evaluates them. */
double grto_besselj(double x, int n);
double grto_d_besselj(double x, int n);
double grto_dd_besselj(double x, int n);
double grto_dd_besselj_exact(double x, int n);

#ifdef __cplusplus
}
#endif
#endif
