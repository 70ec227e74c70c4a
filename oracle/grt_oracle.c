/*
 * grt_oracle.c -- FP64 CPU oracle of the GRT Green's-function pipeline.
 *
 * TEST INFRASTRUCTURE ONLY (the checker): tests/, __graft_entry__.smoke() and
 * bench.py's cpu_baseline / reference arm load this; the product never does.
 *
 * Every function names the reference lines it restates (paths relative to the
 * reference project).  The reference has no CPU implementation of the GRT path
 * (its CPU file cusrc/popm/func/grtc.c is never compiled and is incomplete),
 * so this is a restatement of the CUDA kernels in cusrc/popm/func/green.cu in
 * sequential FP64 C, one (w,k) point at a time.  Library calls of the
 * reference are replaced by their mathematical definitions:
 *   cublasZmatinvBatched + cublasZgemmBatched (green.cu:1813,1816): the 4x4
 *       interface solve T = E1^-1 E2, here Gauss-Jordan with partial pivoting;
 *   cufftExecZ2Z(INVERSE) (green.cu:2233): x_n = sum_j X_j exp(+2 pi i jn/N),
 *       here an iterative radix-2 FFT.
 * Complex elementary functions follow the reference's vendored complex type
 * (cusrc/scilib/cucomplex.hpp:925 log, :945 sqrt = polar(sqrt|z|, arg z / 2),
 * :963 exp), i.e. principal branches.
 */
#include "grt_oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifdef GRTO_COUNT
/* op_count.cpp builds this file as C++ with an operation-counting complex type */
#include "grt_count.hpp"
thread_local grto_tally grto_cnt;
#else
#include <complex.h>
typedef double _Complex cplx;
#define GRTO_COUNT_PAUSE ((void)0)
#define GRTO_COUNT_RESUME ((void)0)
#define GRTO_COUNT_FN(n) ((void)0)
#endif

#define PI 3.1415926535897932384626433
#define PI2 (3.1415926535897932384626433 * 2)

/* ------------------------------------------------------------------ */
/* complex helpers (cucomplex.hpp semantics)                           */
/* ------------------------------------------------------------------ */
static inline cplx mkc(double re, double im) { return re + im * I; }
/* (the operation count takes 20 for each of these three) */
static inline cplx c_log(cplx z)
{
    GRTO_COUNT_FN(20);
    GRTO_COUNT_PAUSE;
    cplx r = mkc(log(hypot(creal(z), cimag(z))), atan2(cimag(z), creal(z)));
    GRTO_COUNT_RESUME;
    return r;
}
static inline cplx c_sqrt(cplx z)
{
    GRTO_COUNT_FN(20);
    GRTO_COUNT_PAUSE;
    double m = sqrt(hypot(creal(z), cimag(z)));
    double t = atan2(cimag(z), creal(z)) / 2.0;
    cplx r = mkc(m * cos(t), m * sin(t));
    GRTO_COUNT_RESUME;
    return r;
}
static inline cplx c_exp(cplx z)
{
    GRTO_COUNT_FN(20);
    GRTO_COUNT_PAUSE;
    double e = exp(creal(z));
    cplx r = mkc(e * cos(cimag(z)), e * sin(cimag(z)));
    GRTO_COUNT_RESUME;
    return r;
}

/* 2x2 inverse in place, green.cu:388-400 (mat_inv_2) */
static void inv2(cplx a[2][2])
{
    cplx b00 = a[0][0], b01 = a[0][1], b10 = a[1][0], b11 = a[1][1];
    cplx d = a[0][0] * a[1][1] - a[0][1] * a[1][0];
    a[0][0] = b11 / d;
    a[1][1] = b00 / d;
    a[0][1] = -b01 / d;
    a[1][0] = -b10 / d;
}

/* c = a b (2x2) */
static void mm2(const cplx a[2][2], const cplx b[2][2], cplx c[2][2])
{
    for (int i = 0; i < 2; i++)
        for (int j = 0; j < 2; j++) c[i][j] = a[i][0] * b[0][j] + a[i][1] * b[1][j];
}

/* Solve E1 X = E2 for 4x4 complex X (replaces cublasZmatinvBatched + Zgemm,
 * green.cu:1811-1817).  Gauss-Jordan with partial pivoting. */
static int solve4(cplx A[4][4], cplx B[4][4])
{
    for (int c = 0; c < 4; c++) {
        int p = c;
        double best = cabs(A[c][c]);
        for (int r = c + 1; r < 4; r++) {
            double v = cabs(A[r][c]);
            if (v > best) { best = v; p = r; }
        }
        if (best == 0.0) return -1;
        if (p != c) {
            for (int j = 0; j < 4; j++) {
                cplx t = A[c][j]; A[c][j] = A[p][j]; A[p][j] = t;
                t = B[c][j]; B[c][j] = B[p][j]; B[p][j] = t;
            }
        }
        cplx inv = 1.0 / A[c][c];
        for (int j = 0; j < 4; j++) { A[c][j] *= inv; B[c][j] *= inv; }
        for (int r = 0; r < 4; r++) {
            if (r == c) continue;
            cplx f = A[r][c];
            if (f == 0) continue;
            for (int j = 0; j < 4; j++) { A[r][j] -= f * A[c][j]; B[r][j] -= f * B[c][j]; }
        }
    }
    return 0;
}

/* ------------------------------------------------------------------ */
/* Bessel functions, green.cu:1418-1554.  J0/J1 are the polynomial       */
/* approximations of Abramowitz & Stegun 9.4.1-9.4.6; J_n (n>=2) by      */
/* upward recurrence for x > n and Miller's downward recurrence          */
/* otherwise (Numerical Recipes bessj).                                  */
/* ------------------------------------------------------------------ */
static double bj0(double x)
{
    static const double a[7] = {1.00000000, -2.24999970, 1.26562080, -0.31638660, 0.04444790, -0.00394440, 0.00021000};
    static const double b[7] = {0.79788456, -0.00000077, -0.00552740, -0.00009512, 0.00137237, -0.00072805, 0.00014476};
    static const double c[7] = {-0.78539816, -0.04166397, -0.00003954, 0.00262573, -0.00054125, -0.00029333, 0.00013558};
    double ax = fabs(x);
    if (ax <= 3) {
        double x2 = (ax / 3.0) * (ax / 3.0);
        return a[0] + x2 * (a[1] + x2 * (a[2] + x2 * (a[3] + x2 * (a[4] + x2 * (a[5] + x2 * a[6])))));
    }
    double x1 = 3.0 / ax;
    double fct = b[0] + x1 * (b[1] + x1 * (b[2] + x1 * (b[3] + x1 * (b[4] + x1 * (b[5] + x1 * b[6])))));
    double th = ax + c[0] + x1 * (c[1] + x1 * (c[2] + x1 * (c[3] + x1 * (c[4] + x1 * (c[5] + x1 * c[6])))));
    return fct * cos(th) / sqrt(ax);
}

static double bj1(double x)
{
    static const double a[7] = {0.50000000, -0.56249985, 0.21093573, -0.03954289, 0.00443319, -0.00031761, 0.00001109};
    static const double b[7] = {0.79788456, 0.00000156, 0.01659667, 0.00017105, -0.00249511, 0.00113653, -0.00020033};
    static const double c[7] = {-2.35619449, 0.12499612, 0.00005650, -0.00637879, 0.00074348, 0.00079824, -0.00029166};
    double ax = fabs(x);
    if (ax <= 3.0) {
        double x2 = (ax / 3.0) * (ax / 3.0);
        return x * (a[0] + x2 * (a[1] + x2 * (a[2] + x2 * (a[3] + x2 * (a[4] + x2 * (a[5] + x2 * a[6]))))));
    }
    double x1 = 3.0 / ax;
    double fct = b[0] + x1 * (b[1] + x1 * (b[2] + x1 * (b[3] + x1 * (b[4] + x1 * (b[5] + x1 * b[6])))));
    double th = ax + c[0] + x1 * (c[1] + x1 * (c[2] + x1 * (c[3] + x1 * (c[4] + x1 * (c[5] + x1 * c[6])))));
    double sign = x >= 0 ? 1.0 : -1.0;
    return sign * fct * cos(th) / sqrt(ax);
}

double grto_besselj(double x, int n)
{
    const int iacc = 40;
    const double bigno = 1e10, bigni = 1e-10;
    int nn = n;
    double res;
    if (n == 0) return bj0(x);
    if (n == 1) return bj1(x);
    if (n < 0) n = -n;
    double ax = fabs(x);
    if (ax == 0) res = 0.0;
    else if (ax > n) {
        double tox = 2.0 / ax, bjm = bj0(ax), bj = bj1(ax);
        for (int j = 0; j < n - 1; j++) {
            double bjp = (double)(j + 1) * tox * bj - bjm;
            bjm = bj;
            bj = bjp;
        }
        res = bj;
    } else {
        double tox = 2.0 / ax;
        int m = 2 * ((n + (int)(sqrt((double)(iacc * n)))) / 2);
        int jsum = 0;
        double sum = 0.0, bjp = 0.0, bj = 1.0;
        res = 0.0;
        for (int j = m; j >= 1; j--) {
            double bjm = (double)j * tox * bj - bjp;
            bjp = bj;
            bj = bjm;
            if (fabs(bj) > bigno) {
                bj *= bigni; bjp *= bigni; res *= bigni; sum *= bigni;
            }
            if (jsum != 0) sum += bj;
            jsum = 1 - jsum;
            if (j == n) res = bjp;
        }
        sum = 2.0 * sum - bj;
        res = res / sum;
    }
    if (x < 0.0 && (n % 2) == 1) res = -res;
    if (nn < 0 && (n % 2) == 1) res = -res;
    return res;
}

double grto_d_besselj(double x, int n)
{
    const double bigni = 1e-10;
    if (fabs(x) < bigni) return (grto_besselj(bigni, n) - grto_besselj(0, n)) / bigni;
    return (double)n * grto_besselj(x, n) / x - grto_besselj(x, n + 1);
}

double grto_dd_besselj(double x, int n)
{
    const double bigni = 1e-10;
    if (fabs(x) < bigni) return (grto_d_besselj(bigni, n) - grto_d_besselj(0, n)) / bigni;
    return (double)n * grto_besselj(x, n - 1) / x - grto_besselj(x, n) * (n + n * n + x * x) / x / x;
}

/* J_n''(x) from Bessel's equation, -J_{n-1}/x + ((n^2 + n)/x^2 - 1) J_n (series near 0) */
double grto_dd_besselj_exact(double x, int n)
{
    if (fabs(x) < 1e-3) {
        double x2 = x * x;
        return n == 0 ? -0.5 + 3.0 * x2 / 16.0 : n == 1 ? -0.375 * x : 0.25 - x2 / 8.0;
    }
    double jm = n == 0 ? -grto_besselj(x, 1) : grto_besselj(x, n - 1);
    return -jm / x + ((double)(n * n + n) / (x * x) - 1.0) * grto_besselj(x, n);
}

/* ------------------------------------------------------------------ */
/* input parsing, green.cu:1989-2060                                    */
/* ------------------------------------------------------------------ */
static int finish_model(grto_job *J, int n_in, const double *zt, const double *vp,
                        const double *vs, const double *rh, const double *qpa,
                        const double *qsa)
{
    /* source-interface insertion, green.cu:2001-2030: a copy of the layer
     * holding the source starts at hs when ztop[i-1] < hs < ztop[i]. */
    int t = 0;
    J->inserted = 0;
    if (n_in < 2 || n_in + 1 > GRTO_MAXL) return GRTO_ERR_MODEL;
    for (int i = 0; i < n_in; i++) {
        if (i > 0 && zt[i - 1] < J->hs && zt[i] > J->hs) {
            J->h[t] = J->hs; J->a0[t] = vp[i - 1]; J->b0[t] = vs[i - 1];
            J->rho[t] = rh[i - 1]; J->qp[t] = qpa[i - 1]; J->qs[t] = qsa[i - 1];
            t++;
            J->inserted = 1;
        }
        J->h[t] = zt[i]; J->a0[t] = vp[i]; J->b0[t] = vs[i];
        J->rho[t] = rh[i]; J->qp[t] = qpa[i]; J->qs[t] = qsa[i];
        t++;
    }
    /* The reference always adds one layer (green.cu:2030).  When nothing was
     * inserted (source exactly on an interface, in the half-space or at the
     * surface) its extra layer is uninitialised memory; here the layer count
     * is kept instead.  A source in the half-space is rejected. */
    if (!J->inserted && J->hs > zt[n_in - 1]) return GRTO_ERR_MODEL;
    J->n_layer = t;
    J->vmax = 0;
    J->vmin = 100000;
    for (int i = 0; i < t; i++) {                     /* green.cu:2034-2037 */
        if (J->a0[i] > J->vmax) J->vmax = J->a0[i];
        if (J->b0[i] < J->vmin) J->vmin = J->b0[i];
    }
    for (int i = 0; i < t - 1; i++) J->h[i] = J->h[i + 1] - J->h[i];  /* 2044-2046 */
    for (int i = 0; i < t; i++) J->mu[i] = J->b0[i] * J->b0[i] * J->rho[i];  /* 2047-2049 */
    return GRTO_OK;
}

int grto_model(grto_job *J, int n_in, const double *ztop, const double *vp,
               const double *vs, const double *rho, const double *qp,
               const double *qs, double hs, double hr, int src_type)
{
    memset(J, 0, sizeof(*J));
    J->hs = hs;
    J->hr = hr;
    J->src_type = src_type;
    return finish_model(J, n_in, ztop, vp, vs, rho, qp, qs);
}

int grto_parse(const char *path, grto_job *J)
{
    FILE *f = fopen(path, "r");
    if (!f) return GRTO_ERR_IO;
    memset(J, 0, sizeof(*J));
    int n = 0;
    double zt[GRTO_MAXL], vp[GRTO_MAXL], vs[GRTO_MAXL], rh[GRTO_MAXL], qp[GRTO_MAXL], qs[GRTO_MAXL];
    int ok = fscanf(f, "%lf %lf %d", &J->hs, &J->hr, &n) == 3;
    if (!ok || n < 2 || n + 1 > GRTO_MAXL) { fclose(f); return GRTO_ERR_PARSE; }
    for (int i = 0; i < n && ok; i++)
        ok = fscanf(f, " %lf , %lf , %lf , %lf , %lf , %lf", &zt[i], &vp[i], &vs[i], &rh[i], &qp[i], &qs[i]) == 6;
    ok = ok && fscanf(f, "%lf %lf %d %d %lf %d %lf %lf %d %d", &J->dt, &J->dist0, &J->nf1,
                      &J->nf2, &J->twin, &J->log2n, &J->t0, &J->taper, &J->n_ptam,
                      &J->src_type) == 10;
    fclose(f);
    if (!ok) return GRTO_ERR_PARSE;
    double hs = J->hs, hr = J->hr, dt = J->dt, dist0 = J->dist0, t0 = J->t0, taper = J->taper, twin = J->twin;
    int nf1 = J->nf1, nf2 = J->nf2, log2n = J->log2n, n_ptam = J->n_ptam, st = J->src_type;
    int rc = grto_model(J, n, zt, vp, vs, rh, qp, qs, hs, hr, st);
    J->dt = dt; J->dist0 = dist0; J->t0 = t0; J->taper = taper; J->twin = twin;
    J->nf1 = nf1; J->nf2 = nf2; J->log2n = log2n; J->n_ptam = n_ptam;
    return rc;
}

/* layer velocities at complex frequency w (green.cu:177-180 / 2148-2153) */
static void attenuate(const grto_job *J, cplx w, cplx *alpha, cplx *beta)
{
    cplx lw = c_log(w / PI2);
    for (int i = 0; i < J->n_layer; i++) {
        cplx cs = 1.0 + lw / (PI * J->qs[i]) + I / (2.0 * J->qs[i]);
        cplx cp = 1.0 + lw / (PI * J->qp[i]) + I / (2.0 * J->qp[i]);
        alpha[i] = J->a0[i] * cp;
        beta[i] = J->b0[i] * cs;
    }
}

static inline cplx omega(const grto_job *J, int iw) { return mkc(PI2 * J->df * iw, -J->sigma); }

/* cal_kmax, green.cu:108-162 */
static double cal_kmax(const grto_job *J, cplx w, const cplx *b, int nf)
{
    double pmin = 0, dzmax = 0, kmax;
    int s = J->s_layer, r = J->r_layer;
    if (r == s - 1) {
        pmin = fmax(cabs(w / b[s]), cabs(w / b[s - 1]));
        dzmax = fmin(J->zs, J->h[r] - J->zr);
    } else if (r < s - 1) {
        pmin = fmax(cabs(w / b[s]), cabs(w / b[s - 1]));
        dzmax = fmin(J->zs, J->hs - J->hr);
        for (int lay = r; lay <= s - 2; lay++) {
            if (pmin < cabs(w / b[lay + 1])) pmin = cabs(w / b[lay + 1]);
            if (dzmax > J->h[lay]) dzmax = J->h[lay];
        }
    } else if (r == s) {
        pmin = cabs(w / b[s]);
        dzmax = fabs(J->hr - J->hs);
    } else if (r == s + 1) {
        pmin = fmax(cabs(w / b[s]), cabs(w / b[s + 1]));
        dzmax = fmin(J->h[s] - J->zs, J->zr);
    } else {
        pmin = fmax(cabs(w / b[s]), cabs(w / b[s + 1]));
        dzmax = fmin(J->h[s] - J->zs, fabs(J->hr - J->hs));
        for (int lay = s + 1; lay < r - 1; lay++) {
            if (pmin < cabs(w / b[lay])) pmin = cabs(w / b[lay]);
            if (dzmax > J->h[lay]) dzmax = J->h[lay];
        }
    }
    if (dzmax < 0.2) {
        if (nf < 10) kmax = fmin(pmin + 2.0, 20. * pmin);
        else kmax = fmin(pmin + 2.0, 2.0 * pmin);
    } else {
        kmax = sqrt((3.0 / dzmax) * (3.0 / dzmax) + pmin * pmin);
    }
    if ((kmax - pmin) < 0.5) kmax = pmin + 0.5;
    return kmax;
}

int grto_setup(grto_job *J, double dt, int log2n, double t0, double taper,
               double sigma_factor, int k_mode, int nk_fixed, double dk_override, int fix)
{
    if (dt <= 0 || log2n < 2 || log2n > 24) return GRTO_ERR_ARG;
    J->dt = dt; J->log2n = log2n; J->t0 = t0; J->taper = taper;
    J->k_mode = k_mode; J->nk_fixed = nk_fixed; J->fix = fix;
    if (k_mode == GRTO_K_FIXED && nk_fixed < 2) return GRTO_ERR_ARG;
    /* green.cu:2065-2080 */
    J->nw = (int)pow(2, log2n - 1);
    int n = 2 * J->nw;
    double twin = n * dt;
    J->df = 1 / (n * dt);
    J->sigma = sigma_factor / twin;
    double vavg = (J->vmax + J->vmin) * 0.5;
    double L = (J->vmax * twin + 0 + J->vmax / vavg * sqrt(0 + (J->hs - J->hr) * (J->hs - J->hr)) + 100);
    L = L * 2;
    J->dk = dk_override > 0 ? dk_override : 2 * PI / L;
    /* source layer, green.cu:2081-2090 */
    double hs = J->hs, hr = J->hr;
    J->s_layer = -1;
    for (int i = 0; i < J->n_layer; i++) {
        if (hs <= J->h[i]) { J->s_layer = i; J->zs = hs; break; }
        hs -= J->h[i];
    }
    /* receiver layer, green.cu:2092-2101.  The reference tests the reduced
     * source depth hs instead of hr; GRTO_FIX_RLAYER tests hr. */
    J->r_layer = -1;
    for (int i = 0; i < J->n_layer; i++) {
        double probe = (fix & GRTO_FIX_RLAYER) ? hr : hs;
        if (probe <= J->h[i]) { J->r_layer = i; J->zr = hr; break; }
        hr -= J->h[i];
    }
    if (J->s_layer < 0 || J->s_layer > J->n_layer - 2) return GRTO_ERR_MODEL;
    if (J->r_layer < 0) return GRTO_ERR_MODEL;
    return GRTO_OK;
}

int grto_nk(const grto_job *J, int iw)
{
    if (J->k_mode == GRTO_K_FIXED) return J->nk_fixed;
    /* green.cu:2145-2165 */
    cplx a[GRTO_MAXL], b[GRTO_MAXL];
    cplx w = omega(J, iw);
    attenuate(J, w, a, b);
    double kmax;
    if (iw < 3) kmax = cal_kmax(J, mkc(PI2 * J->df * 3.0, -J->sigma), b, iw);
    else kmax = cal_kmax(J, w, b, iw);
    kmax = 1.1 * kmax;
    return (int)(kmax / J->dk) + 2;
}

long long grto_nkw(const grto_job *J)
{
    long long s = 0;
    for (int iw = 0; iw < J->nw; iw++) s += grto_nk(J, iw);
    return s;
}

/* ------------------------------------------------------------------ */
/* per-(w,k) GRT                                                       */
/* ------------------------------------------------------------------ */
typedef struct {
    cplx a0[2], a1[2], a2[2], b1, b2;
    cplx a0t[2], a1t[2], a2t[2], b1t, b2t;
} ypar_t;

typedef struct {
    cplx tdd1[2][2], tuu1[2][2], rdu1[2][2], rud1[2][2];
    cplx tdd0, tuu0, rdu0, rud0;
} mrt_t;

typedef struct {
    cplx rud1[2][2], rdu1[2][2], tu1[2][2], td1[2][2];
    cplx rud0, rdu0, tu0, td0;
} grt_t;

/* vertical wavenumbers and E matrix of one layer: set_pars green.cu:184-194,
 * mat_PSV_E green.cu:196-214 */
static void layer_pars(double k, cplx w, cplx a, cplx b, cplx u, cplx *r, cplx *v, cplx E[4][4])
{
    cplx wa = w / a, wb = w / b;
    *r = c_sqrt(k * k - wa * wa);
    *v = c_sqrt(k * k - wb * wb);
    if (creal(*r) < 0) *r = -*r;
    if (creal(*v) < 0) *v = -*v;
    cplx x = k * k + (*v) * (*v);
    E[0][0] = a * k / w;
    E[0][1] = b * (*v) / w;
    E[0][2] = E[0][0];
    E[0][3] = E[0][1];
    E[1][0] = a * (*r) / w;
    E[1][1] = b * k / w;
    E[1][2] = -E[1][0];
    E[1][3] = -E[1][1];
    E[2][0] = -2.0 * a * u * k * (*r) / w;
    E[2][1] = -b * u * x / w;
    E[2][2] = -E[2][0];
    E[2][3] = -E[2][1];
    E[3][0] = -a * u * x / w;
    E[3][1] = -2.0 * b * u * k * (*v) / w;
    E[3][2] = E[3][0];
    E[3][3] = E[3][1];
}

/* shear modulus of each layer at this frequency: the reference's real
 * mu0 = b0^2 rho (green.cu:182, 2048), or with GRTO_ATTEN_MU the standard
 * viscoelastic rho beta(w)^2 from the attenuated S velocity */
static void shear_moduli(const grto_job *J, const cplx *beta, cplx *mue)
{
    for (int i = 0; i < J->n_layer; i++)
        mue[i] = (J->fix & GRTO_ATTEN_MU) ? J->rho[i] * beta[i] * beta[i] : (cplx)J->mu[i];
}

static void point_eval(const grto_job *J, const cplx *alpha, const cplx *beta, double k,
                       cplx w, const cplx slot0[2], ypar_t *Y)
{
    const int L = J->n_layer, s = J->s_layer, rl = J->r_layer;
    const double zs = J->zs, zr = J->zr;
    cplx rr[GRTO_MAXL], vv[GRTO_MAXL];
    static __thread cplx E[GRTO_MAXL][4][4];
    static __thread mrt_t M[GRTO_MAXL];
    static __thread grt_t G[GRTO_MAXL + 1];
    memset(G, 0, sizeof(grt_t) * (L + 1));

    cplx mue[GRTO_MAXL];
    shear_moduli(J, beta, mue);
    for (int i = 0; i < L; i++) layer_pars(k, w, alpha[i], beta[i], mue[i], &rr[i], &vv[i], E[i]);

    /* interface R/T: get_emat_e1e2 green.cu:235-262, cuBLAS solve, get_mrt_psv
     * green.cu:359-387; SH closed form get_mrt_sh green.cu:339-353 */
    for (int j = 0; j < L - 1; j++) {
        cplx E1[4][4], E2[4][4];
        for (int i = 0; i < 2; i++)
            for (int c = 0; c < 2; c++) {
                E1[i][c] = E[j + 1][i][c];
                E1[i + 2][c] = E[j + 1][i + 2][c];
                E1[i][c + 2] = -E[j][i][c + 2];
                E1[i + 2][c + 2] = -E[j][i + 2][c + 2];
                E2[i][c] = E[j][i][c];
                E2[i + 2][c] = E[j][i + 2][c];
                E2[i][c + 2] = -E[j + 1][i][c + 2];
                E2[i + 2][c + 2] = -E[j + 1][i + 2][c + 2];
            }
        solve4(E1, E2);
        for (int i = 0; i < 2; i++)
            for (int c = 0; c < 2; c++) {
                M[j].tdd1[i][c] = E2[i][c];
                M[j].tuu1[i][c] = E2[i + 2][c + 2];
                M[j].rdu1[i][c] = E2[i + 2][c];
                M[j].rud1[i][c] = E2[i][c + 2];
            }
        cplx wa = vv[j] * mue[j], wb = vv[j + 1] * mue[j + 1];
        M[j].tdd0 = 2. * wa / (wa + wb);
        M[j].rdu0 = (wa - wb) / (wa + wb);
        M[j].rud0 = -M[j].rdu0;
        M[j].tuu0 = 2. * wb / (wa + wb);
    }

    /* generalized coefficients, get_grt green.cu:424-613 */
    {
        cplx a[2][2], b[2][2];
        for (int i = 0; i < 2; i++)
            for (int c = 0; c < 2; c++) { a[i][c] = E[0][i + 2][c]; b[i][c] = E[0][i + 2][c + 2]; }
        inv2(a);
        for (int i = 0; i < 2; i++)
            for (int c = 0; c < 2; c++) G[0].rud1[i][c] = -(a[i][0] * b[0][c] + a[i][1] * b[1][c]);
        G[0].rud0 = 1.0;
        for (int lay = 0; lay < s; lay++) {
            cplx exu[2] = {c_exp(-rr[lay] * J->h[lay]), c_exp(-vv[lay] * J->h[lay])};
            const mrt_t *m = &M[lay];
            cplx tem1 = G[lay].rud0 * exu[1], tem2 = m->rdu0 * exu[1], tem3 = m->tdd0 * exu[1];
            G[lay + 1].tu0 = m->tuu0 / (1. - tem1 * tem2);
            G[lay + 1].rud0 = m->rud0 + tem3 * tem1 * G[lay + 1].tu0;
            for (int i = 0; i < 2; i++) {
                for (int c = 0; c < 2; c++) {
                    a[i][c] = -(m->rdu1[i][0] * exu[0] * G[lay].rud1[0][c] + m->rdu1[i][1] * exu[1] * G[lay].rud1[1][c]) * exu[c];
                    b[i][c] = (m->tdd1[i][0] * exu[0] * G[lay].rud1[0][c] + m->tdd1[i][1] * exu[1] * G[lay].rud1[1][c]) * exu[c];
                }
                a[i][i] = 1.0 + a[i][i];
            }
            inv2(a);
            mm2(a, m->tuu1, G[lay + 1].tu1);
            for (int i = 0; i < 2; i++)
                for (int c = 0; c < 2; c++)
                    G[lay + 1].rud1[i][c] = m->rud1[i][c] + b[i][0] * G[lay + 1].tu1[0][c] + b[i][1] * G[lay + 1].tu1[1][c];
        }
        const mrt_t *mh = &M[L - 2];
        G[L - 1].rdu0 = mh->rdu0;
        G[L - 1].td0 = mh->tdd0;
        memcpy(G[L - 1].td1, mh->tdd1, sizeof(mh->tdd1));
        memcpy(G[L - 1].rdu1, mh->rdu1, sizeof(mh->rdu1));
        for (int lay = L - 3; lay >= s; lay--) {
            cplx exu[2] = {c_exp(-rr[lay + 1] * J->h[lay + 1]), c_exp(-vv[lay + 1] * J->h[lay + 1])};
            const mrt_t *m = &M[lay];
            cplx tem1 = m->rud0 * exu[1], tem2 = G[lay + 2].rdu0 * exu[1], tem3 = m->tuu0 * exu[1];
            G[lay + 1].td0 = m->tdd0 / (1.0 - tem1 * tem2);
            G[lay + 1].rdu0 = m->rdu0 + tem3 * tem2 * G[lay + 1].td0;
            for (int i = 0; i < 2; i++) {
                for (int c = 0; c < 2; c++) {
                    a[i][c] = -(m->rud1[i][0] * exu[0] * G[lay + 2].rdu1[0][c] + m->rud1[i][1] * exu[1] * G[lay + 2].rdu1[1][c]) * exu[c];
                    b[i][c] = (m->tuu1[i][0] * exu[0] * G[lay + 2].rdu1[0][c] + m->tuu1[i][1] * exu[1] * G[lay + 2].rdu1[1][c]) * exu[c];
                }
                a[i][i] = 1. + a[i][i];
            }
            inv2(a);
            mm2(a, m->tdd1, G[lay + 1].td1);
            for (int i = 0; i < 2; i++)
                for (int c = 0; c < 2; c++)
                    G[lay + 1].rdu1[i][c] = m->rdu1[i][c] + b[i][0] * G[lay + 1].td1[0][c] + b[i][1] * G[lay + 1].td1[1][c];
        }
    }

    /* source terms: get_src_single green.cu:1271-1332, get_src_tensor 1334-1413 */
    const cplx sr = rr[s], sv = vv[s], sa = alpha[s], sb = beta[s];
    const cplx su = mue[s];
    const double sh = J->h[s];
    cplx sexd[2] = {c_exp(-sr * (sh - zs)), c_exp(-sv * (sh - zs))};
    cplx sexu[2] = {c_exp(-sr * zs), c_exp(-sv * zs)};
    const cplx (*RD)[2] = (const cplx (*)[2])G[s + 1].rdu1;
    const cplx (*RU)[2] = (const cplx (*)[2])G[s].rud1;
    cplx wru0[2][2], wrd0[2][2], wru1[2][2], wrd1[2][2];
    for (int i = 0; i < 2; i++)
        for (int c = 0; c < 2; c++) {
            double id = (i == c) ? 1.0 : 0.0;
            cplx ed = sexd[i] * RD[i][c] * sexd[c];
            cplx eu = sexu[i] * RU[i][c] * sexu[c];
            wru0[i][c] = ed - id;
            wrd0[i][c] = id - eu;
            wru1[i][c] = ed + id;
            wrd1[i][c] = id + eu;
        }
    cplx ssh = 1. / (2. * su * sv);
    cplx gu0[2], gd0[2], gu1[2], gd1[2], gshu = 0, gshd = 0;
    cplx su0[2], sd0[2], su1[2], sd1[2], su2[2], sd2[2], shu1 = 0, shd1 = 0, shu2 = 0, shd2 = 0;
    cplx shu_fac = 1. + sexd[1] * G[s + 1].rdu0 * sexd[1];
    if (J->src_type == 0) {
        cplx tmp1 = sb / (2.0 * su * sa * w * sr * sv);
        cplx f00 = sb * sv * sr * tmp1, f01 = -sa * k * sr * tmp1;
        cplx f10 = k * sb * sv * tmp1, f11 = -sa * sr * sv * tmp1;
        for (int i = 0; i < 2; i++) {
            gu0[i] = wru0[i][0] * f00 + wru0[i][1] * f01;
            gd0[i] = wrd0[i][0] * f00 + wrd0[i][1] * f01;
            gu1[i] = wru1[i][0] * f10 + wru1[i][1] * f11;
            gd1[i] = wrd1[i][0] * f10 + wrd1[i][1] * f11;
        }
        gshu = shu_fac * ssh;
        gshd = (sexu[1] * G[s].rud0 * sexu[1] + 1.) * ssh;
    } else {
        cplx tmp1 = sb / (2.0 * su * sa * w);
        cplx s2[2] = {tmp1 * k / sr * k * sb, -k * tmp1 / sr * sa * sr};
        cplx s1[2] = {tmp1 / sv * (-2.0) * k * sv * sb, tmp1 / sv * (k * k + sv * sv) * sa};
        cplx s0[2] = {tmp1 * sr * sb, tmp1 * sa * (-k)};
        for (int i = 0; i < 2; i++) {
            su0[i] = wru1[i][0] * s0[0] + wru1[i][1] * s0[1];
            sd0[i] = wrd1[i][0] * s0[0] + wrd1[i][1] * s0[1];
            su1[i] = wru0[i][0] * s1[0] + wru0[i][1] * s1[1];
            sd1[i] = wrd0[i][0] * s1[0] + wrd0[i][1] * s1[1];
            su2[i] = wru1[i][0] * s2[0] + wru1[i][1] * s2[1];
            sd2[i] = wrd1[i][0] * s2[0] + wrd1[i][1] * s2[1];
        }
        cplx shd_fac = sexu[1] * G[s].rud0 * sexu[1] - 1.;
        /* green.cu:1409-1412 give m = 1 and m = 2 one factor; GRTO_FIX_SHSRC
         * gives m = 1 a displacement jump's (1 - e R e up) and m = 2 a
         * traction jump's (e R e + 1 down) */
        int fsh = (J->fix & GRTO_FIX_SHSRC) != 0;
        shu1 = (fsh ? 2. - shu_fac : shu_fac) * sv * ssh;
        shd1 = shd_fac * sv * ssh;
        shu2 = shu_fac * k * ssh;
        shd2 = (fsh ? shd_fac + 2. : shd_fac) * k * ssh;
    }

    /* receiver side: get_ypars_a_single green.cu:615-939 and
     * get_ypars_a_tensor green.cu:942-1267 (identical propagation) */
    const cplx rr_r = rr[rl], rv_r = vv[rl];
    const double rh = J->h[rl];
    cplx rexd[2] = {c_exp(-rr_r * zr), c_exp(-rv_r * zr)};
    cplx rexdt[2] = {-rr_r * c_exp(-rr_r * zr), -rv_r * c_exp(-rv_r * zr)};
    cplx rexu[2], rexut[2];
    if (L - 1 == rl) {
        rexu[0] = rexu[1] = rexut[0] = rexut[1] = 0;
    } else {
        rexu[0] = c_exp(-rr_r * (rh - zr));
        rexu[1] = c_exp(-rv_r * (rh - zr));
        /* green.cu:674-675 multiply by slot 0's nu (F12); fixed: this point's */
        cplx fr = (J->fix & GRTO_FIX_REXUT) ? rr_r : slot0[0];
        cplx fv = (J->fix & GRTO_FIX_REXUT) ? rv_r : slot0[1];
        rexut[0] = c_exp(-rr_r * (rh - zr)) * fr;
        rexut[1] = c_exp(-rv_r * (rh - zr)) * fv;
    }
    cplx tmp1[2][2], tmp2[2][2], yu_psv[2][2], yd_psv[2][2];
    for (int i = 0; i < 2; i++)
        for (int c = 0; c < 2; c++) {
            tmp1[i][c] = sexd[i] * RD[i][c] * sexd[c];
            tmp2[i][c] = sexu[i] * RU[i][c] * sexu[c];
        }
    mm2(tmp1, tmp2, yu_psv);
    mm2(tmp2, tmp1, yd_psv);
    for (int i = 0; i < 2; i++)
        for (int c = 0; c < 2; c++) {
            double id = (i == c) ? 1.0 : 0.0;
            yu_psv[i][c] = id - yu_psv[i][c];
            yd_psv[i][c] = id - yd_psv[i][c];
        }
    inv2(yu_psv);
    inv2(yd_psv);
    cplx y_sh = 1. / (1. - sexd[1] * G[s + 1].rdu0 * sexd[1] * sexu[1] * G[s].rud0 * sexu[1]);
    const cplx (*Er)[4] = (const cplx (*)[4])E[rl];
    const int fixdz = (J->fix & GRTO_FIX_DZ) != 0;

    cplx yu0 = 0, yu0t = 0, yd0 = 0, yd0t = 0;
    cplx yu1[2][2] = {{0}}, yu1t[2][2] = {{0}}, yd1[2][2] = {{0}}, yd1t[2][2] = {{0}};
    int up;
    if (s == rl && zr <= zs) {
        rexd[0] = c_exp(-rr_r * zr);
        rexd[1] = c_exp(-rv_r * zr);
        rexu[0] = c_exp(-rr_r * (zs - zr));
        rexu[1] = c_exp(-rv_r * (zs - zr));
        rexdt[0] = -rr_r * c_exp(-rr_r * zr);
        rexdt[1] = -rv_r * c_exp(-rv_r * zr);
        rexut[0] = rr_r * c_exp(-rr_r * (zs - zr));
        rexut[1] = rv_r * c_exp(-rv_r * (zs - zr));
        cplx u0 = rexd[1] * G[s].rud0 * sexu[1] + rexu[1];
        /* green.cu:720 multiplies rexut[1] (which already holds nu) by nu again */
        cplx u0t = rexdt[1] * G[s].rud0 * sexu[1] + (fixdz ? rexut[1] : rexut[1] * rv_r);
        cplx u[2][2], ut[2][2];
        for (int i = 0; i < 2; i++)
            for (int c = 0; c < 2; c++) {
                u[i][c] = Er[i][0] * rexd[0] * RU[0][c] * sexu[c] + Er[i][1] * rexd[1] * RU[1][c] * sexu[c] + Er[i][c + 2] * rexu[c];
                ut[i][c] = Er[i][0] * rexdt[0] * RU[0][c] * sexu[c] + Er[i][1] * rexdt[1] * RU[1][c] * sexu[c] + Er[i][c + 2] * rexut[c];
            }
        yu0 = u0 * y_sh;
        yu0t = u0t * y_sh;
        mm2(u, yu_psv, yu1);
        mm2(ut, yu_psv, yu1t);
        up = 1;  /* zr == zs: the reference writes nothing; the upper branch is used */
    } else if (s == rl && zr > zs) {
        rexd[0] = c_exp(-rr[s] * (zr - zs));
        rexd[1] = c_exp(-vv[s] * (zr - zs));
        rexu[0] = c_exp(-rr[s] * (J->h[s] - zr));
        rexu[1] = c_exp(-vv[s] * (J->h[s] - zr));
        rexdt[0] = -rr_r * rexd[0];
        rexdt[1] = -rv_r * rexd[1];
        rexut[0] = rr_r * rexu[0];
        rexut[1] = rv_r * rexu[1];
        cplx d0 = rexd[1] + rexu[1] * G[s + 1].rdu0 * sexd[1];
        cplx d0t = rexdt[1] + rexut[1] * G[s + 1].rdu0 * sexd[1];
        cplx d[2][2], dt[2][2];
        for (int i = 0; i < 2; i++)
            for (int c = 0; c < 2; c++) {
                d[i][c] = Er[i][c] * rexd[c] + Er[i][2] * rexu[0] * RD[0][c] * sexd[c] + Er[i][3] * rexu[1] * RD[1][c] * sexd[c];
                dt[i][c] = Er[i][c] * rexdt[c] + Er[i][2] * rexut[0] * RD[0][c] * sexd[c] + Er[i][3] * rexut[1] * RD[1][c] * sexd[c];
            }
        yd0 = d0 * y_sh;
        yd0t = d0t * y_sh;
        mm2(d, yd_psv, yd1);
        mm2(dt, yd_psv, yd1t);
        up = 0;
    } else if (rl < s) {
        cplx ex[2] = {c_exp(-rr_r * rh), c_exp(-rv_r * rh)};
        cplx u0 = rexd[1] * G[rl].rud0 * ex[1] + rexu[1];
        cplx u0t = rexdt[1] * G[rl].rud0 * ex[1] + rexut[1];
        cplx u[2][2], ut[2][2];
        for (int i = 0; i < 2; i++)
            for (int c = 0; c < 2; c++) {
                u[i][c] = Er[i][0] * rexd[0] * G[rl].rud1[0][c] * ex[c] + Er[i][1] * rexd[1] * G[rl].rud1[1][c] * ex[c] + Er[i][c + 2] * rexu[c];
                ut[i][c] = Er[i][0] * rexdt[0] * G[rl].rud1[0][c] * ex[c] + Er[i][1] * rexdt[1] * G[rl].rud1[1][c] * ex[c] + Er[i][c + 2] * rexut[c];
            }
        for (int lay = s - 1; lay >= rl; lay--) {
            if (lay == s - 1) {
                yu0 = G[lay + 1].tu0 * sexu[1] * y_sh;
                for (int i = 0; i < 2; i++)
                    for (int c = 0; c < 2; c++)
                        yu1[i][c] = G[lay + 1].tu1[i][0] * sexu[0] * yu_psv[0][c] + G[lay + 1].tu1[i][1] * sexu[1] * yu_psv[1][c];
            } else {
                cplx e2[2] = {c_exp(-rr[lay + 1] * J->h[lay + 1]), c_exp(-vv[lay + 1] * J->h[lay + 1])};
                yu0 = G[lay + 1].tu0 * e2[1] * yu0;
                cplx t[2][2];
                for (int i = 0; i < 2; i++)
                    for (int c = 0; c < 2; c++)
                        t[i][c] = G[lay + 1].tu1[i][0] * e2[0] * yu1[0][c] + G[lay + 1].tu1[i][1] * e2[1] * yu1[1][c];
                memcpy(yu1, t, sizeof(t));
            }
        }
        cplx yprop = yu0;
        yu0 = u0 * yprop;
        /* green.cu:842 multiplies by the already-updated yu0 */
        yu0t = fixdz ? u0t * yprop : u0t * yu0;
        cplx t[2][2], tt[2][2];
        mm2(u, yu1, t);
        mm2(ut, yu1, tt);
        memcpy(yu1, t, sizeof(t));
        memcpy(yu1t, tt, sizeof(tt));
        up = 1;
    } else {
        /* r_layer > s_layer.  The reference's loop (green.cu:858-915) takes the
         * transmission of the wrong interfaces, the phase of layer lay-2 and the
         * upper reverberation matrix.  This is the physically consistent form:
         * down-going from the source through interfaces s+1..rl. */
        cplx ex[2] = {c_exp(-rr_r * rh), c_exp(-rv_r * rh)};
        cplx R0 = (rl + 1 <= L - 1) ? G[rl + 1].rdu0 : 0;
        cplx d0 = rexu[1] * R0 * ex[1] + rexd[1];
        cplx d0t = rexut[1] * R0 * ex[1] + rexdt[1];
        cplx d[2][2], dt[2][2];
        for (int i = 0; i < 2; i++)
            for (int c = 0; c < 2; c++) {
                cplx g0 = (rl + 1 <= L - 1) ? G[rl + 1].rdu1[0][c] : 0;
                cplx g1 = (rl + 1 <= L - 1) ? G[rl + 1].rdu1[1][c] : 0;
                d[i][c] = Er[i][c] * rexd[c] + Er[i][2] * rexu[0] * g0 * ex[c] + Er[i][3] * rexu[1] * g1 * ex[c];
                dt[i][c] = Er[i][c] * rexdt[c] + Er[i][2] * rexut[0] * g0 * ex[c] + Er[i][3] * rexut[1] * g1 * ex[c];
            }
        for (int lay = s + 1; lay <= rl; lay++) {
            if (lay == s + 1) {
                yd0 = G[lay].td0 * sexd[1] * y_sh;
                for (int i = 0; i < 2; i++)
                    for (int c = 0; c < 2; c++)
                        yd1[i][c] = G[lay].td1[i][0] * sexd[0] * yd_psv[0][c] + G[lay].td1[i][1] * sexd[1] * yd_psv[1][c];
            } else {
                cplx e2[2] = {c_exp(-rr[lay - 1] * J->h[lay - 1]), c_exp(-vv[lay - 1] * J->h[lay - 1])};
                yd0 = G[lay].td0 * e2[1] * yd0;
                cplx t[2][2];
                for (int i = 0; i < 2; i++)
                    for (int c = 0; c < 2; c++)
                        t[i][c] = G[lay].td1[i][0] * e2[0] * yd1[0][c] + G[lay].td1[i][1] * e2[1] * yd1[1][c];
                memcpy(yd1, t, sizeof(t));
            }
        }
        cplx yprop = yd0;
        yd0 = d0 * yprop;
        yd0t = d0t * yprop;
        cplx t[2][2], tt[2][2];
        mm2(d, yd1, t);
        mm2(dt, yd1, tt);
        memcpy(yd1, t, sizeof(t));
        memcpy(yd1t, tt, sizeof(tt));
        up = 0;
    }

    memset(Y, 0, sizeof(*Y));
    if (J->src_type == 0) {
        const cplx *g0 = up ? gu0 : gd0, *g1 = up ? gu1 : gd1;
        cplx gsh = up ? gshu : gshd;
        cplx (*y1)[2] = up ? yu1 : yd1, (*y1t)[2] = up ? yu1t : yd1t;
        cplx y0 = up ? yu0 : yd0, y0t = up ? yu0t : yd0t;
        Y->b1 = y0 * gsh;
        Y->b1t = y0t * gsh;
        for (int i = 0; i < 2; i++) {
            Y->a0[i] = y1[i][0] * g0[0] + y1[i][1] * g0[1];
            Y->a1[i] = y1[i][0] * g1[0] + y1[i][1] * g1[1];
            Y->a0t[i] = y1t[i][0] * g0[0] + y1t[i][1] * g0[1];
            Y->a1t[i] = y1t[i][0] * g1[0] + y1t[i][1] * g1[1];
        }
    } else {
        const cplx *s0 = up ? su0 : sd0, *s1 = up ? su1 : sd1, *s2 = up ? su2 : sd2;
        cplx h1 = up ? shu1 : shd1, h2 = up ? shu2 : shd2;
        cplx (*y1)[2] = up ? yu1 : yd1, (*y1t)[2] = up ? yu1t : yd1t;
        cplx y0 = up ? yu0 : yd0, y0t = up ? yu0t : yd0t;
        Y->b1 = y0 * h1;
        Y->b2 = y0 * h2;
        Y->b1t = y0t * h1;
        Y->b2t = y0t * h2;
        for (int i = 0; i < 2; i++) {
            Y->a0[i] = y1[i][0] * s0[0] + y1[i][1] * s0[1];
            Y->a1[i] = y1[i][0] * s1[0] + y1[i][1] * s1[1];
            Y->a2[i] = y1[i][0] * s2[0] + y1[i][1] * s2[1];
            Y->a0t[i] = y1t[i][0] * s0[0] + y1t[i][1] * s0[1];
            Y->a1t[i] = y1t[i][0] * s1[0] + y1t[i][1] * s1[1];
            Y->a2t[i] = y1t[i][0] * s2[0] + y1t[i][1] * s2[1];
        }
    }
}

/* ------------------------------------------------------------------ */
/* Well-conditioned formulation of the same recursion (GRTO_STABLE).    */
/*                                                                     */
/* The reference's eigenvector matrix E (mat_PSV_E, green.cu:196-214)  */
/* has P and SV columns that become parallel as w -> 0 (both tend to    */
/* e^{-kz}(1,1,-2uk,-2uk)); its 4x4 interface solve then loses up to    */
/* 13 digits in FP64.  This mode uses, in every layer, the basis        */
/*   p = w/a E_P = (k, r, -2ukr, -ux),  d = (w/a E_P - w/b E_SV)/(r-v)   */
/* i.e. E_d = [p d] S^{-1} with S = w [[1/a, 1/(a(r-v))], [0, -1/(b(r-v))]] */
/* and writes every entry without cancellation (k-v = wb^2/(k+v),      */
/* r-v = (wb^2-wa^2)/(r+v), ...).  Phase factors become upper-triangular */
/* S^{-1} diag(e^{-rz}, e^{-vz}) S = [[e_r, (e_r-e_v)/(r-v)], [0, e_v]]. */
/* The generalized R/T recursion, source and receiver formulas are the   */
/* reference's, with every matrix expressed in this basis.  Outputs are  */
/* the same physical coefficients (basis independent).                   */
/* ------------------------------------------------------------------ */
typedef struct { cplx m[2][2]; } m2_t;

static m2_t M2(cplx a, cplx b, cplx c, cplx d) { m2_t r = {{{a, b}, {c, d}}}; return r; }
static m2_t m2mul(m2_t a, m2_t b)
{
    return M2(a.m[0][0] * b.m[0][0] + a.m[0][1] * b.m[1][0], a.m[0][0] * b.m[0][1] + a.m[0][1] * b.m[1][1],
              a.m[1][0] * b.m[0][0] + a.m[1][1] * b.m[1][0], a.m[1][0] * b.m[0][1] + a.m[1][1] * b.m[1][1]);
}
static m2_t m2add(m2_t a, m2_t b, double s)
{
    return M2(a.m[0][0] + s * b.m[0][0], a.m[0][1] + s * b.m[0][1], a.m[1][0] + s * b.m[1][0], a.m[1][1] + s * b.m[1][1]);
}
static m2_t m2scale(m2_t a, cplx s) { return M2(a.m[0][0] * s, a.m[0][1] * s, a.m[1][0] * s, a.m[1][1] * s); }
static m2_t m2inv_det(m2_t a, cplx det) { return M2(a.m[1][1] / det, -a.m[0][1] / det, -a.m[1][0] / det, a.m[0][0] / det); }
static m2_t m2inv(m2_t a) { return m2inv_det(a, a.m[0][0] * a.m[1][1] - a.m[0][1] * a.m[1][0]); }
static m2_t m2eye(void) { return M2(1, 0, 0, 1); }
static m2_t m2zero(void) { return M2(0, 0, 0, 0); }
static void m2vec(m2_t a, const cplx x[2], cplx y[2])
{
    y[0] = a.m[0][0] * x[0] + a.m[0][1] * x[1];
    y[1] = a.m[1][0] * x[0] + a.m[1][1] * x[1];
}

typedef struct {
    cplx a, b, r, v, x, rmv, wa2, wb2;
    cplx mu;
    cplx p[4], d[4];
    cplx detG, detH, detT;
} slay_t;

static void slayer(double k, cplx w, cplx a, cplx b, cplx mu, slay_t *L)
{
    /* (w/a)^2, (w/b)^2 and their difference depend on the frequency only:
     * not counted as per-(w,k) work */
    GRTO_COUNT_PAUSE;
    cplx wa = w / a, wb = w / b;
    L->a = a; L->b = b; L->mu = mu;
    L->wa2 = wa * wa;
    L->wb2 = wb * wb;
    cplx W = L->wb2 - L->wa2;          /* v^2 - r^2 with sign: r^2 - v^2 = W */
    GRTO_COUNT_RESUME;
    L->r = c_sqrt(k * k - L->wa2);
    L->v = c_sqrt(k * k - L->wb2);
    if (creal(L->r) < 0) L->r = -L->r;
    if (creal(L->v) < 0) L->v = -L->v;
    L->x = k * k + L->v * L->v;
    cplx rpv = L->r + L->v;
    L->rmv = W / rpv;                    /* r - v */
    cplx dv = L->wb2 / (k + L->v);       /* k - v */
    cplx dr = L->wa2 / (k + L->r);       /* k - r */
    L->p[0] = k; L->p[1] = L->r; L->p[2] = -2 * mu * k * L->r; L->p[3] = -mu * L->x;
    L->d[0] = dv / L->rmv;
    L->d[1] = -dr / L->rmv;
    L->d[2] = mu * (dr * dr - W) / L->rmv;
    L->d[3] = -mu * dv * dv / L->rmv;
    L->detG = mu * L->v * L->wb2 / L->rmv;
    L->detH = -mu * L->r * L->wb2 / L->rmv;
    cplx ray = L->x * (dr * dr - W) + 2 * k * L->r * dv * dv;   /* x^2 - 4k^2 r v */
    L->detT = mu * mu * ray / L->rmv;
}

/* (exp(y) - 1) / y */
static cplx expm1_over(cplx y)
{
    if (cabs(y) < 0.5) {
        cplx s = 1, t = 1;
        for (int n = 2; n < 18; n++) { t = t * y / n; s += t; }
        return s;
    }
    return (c_exp(y) - 1.0) / y;
}

/* S^{-1} diag(e^{-rz}, e^{-vz}) S */
static m2_t sphase(const slay_t *L, double z)
{
    cplx er = c_exp(-L->r * z), ev = c_exp(-L->v * z);
    cplx y = -L->rmv * z;
    cplx dd = (cabs(y) < 0.5) ? -z * ev * expm1_over(y) : (er - ev) / L->rmv;
    return M2(er, dd, 0, ev);
}

/* S^{-1} diag(sg r0 e^{-rz}, sg v0 e^{-vz}) S, r0/v0 = own nu unless nu0 */
static m2_t sdphase(const slay_t *L, double z, double sg, const cplx *nu0)
{
    cplx er = c_exp(-L->r * z), ev = c_exp(-L->v * z);
    cplx y = -L->rmv * z;
    cplx dd = (cabs(y) < 0.5) ? -z * ev * expm1_over(y) : (er - ev) / L->rmv;
    cplx r0, v0, off;
    if (!nu0) { r0 = L->r; v0 = L->v; off = er + L->v * dd; }
    else { r0 = nu0[0]; v0 = nu0[1]; off = r0 * dd + ev * (r0 - v0) / L->rmv; }
    return M2(sg * r0 * er, sg * off, 0, sg * v0 * ev);
}

typedef struct { m2_t td, tu, rd, ru; cplx tdd0, tuu0, rdu0, rud0; } smrt_t;

/* interface between U (layer j) and D (layer j+1): F = E_D^{-1} E_U with
 * E = Pi^T [[G, G], [H, -H]], P = G_D^{-1} G_U, Q = H_D^{-1} H_U */
static void sinterface(const slay_t *U, const slay_t *D, smrt_t *m)
{
    m2_t GU = M2(U->p[0], U->d[0], U->p[3], U->d[3]), HU = M2(U->p[1], U->d[1], U->p[2], U->d[2]);
    m2_t GD = M2(D->p[0], D->d[0], D->p[3], D->d[3]), HD = M2(D->p[1], D->d[1], D->p[2], D->d[2]);
    m2_t P = m2mul(m2inv_det(GD, D->detG), GU);
    m2_t Q = m2mul(m2inv_det(HD, D->detH), HU);
    m2_t S = m2add(P, Q, 1), Dm = m2add(P, Q, -1);
    m2_t Si = m2inv(S);
    m->rd = m2scale(m2mul(Si, Dm), -1);
    m->tu = m2scale(Si, 2);
    m->td = m2scale(m2mul(Q, m2mul(Si, P)), 2);
    m->ru = m2mul(Dm, Si);
    cplx wa = U->v * U->mu, wb = D->v * D->mu;
    m->tdd0 = 2. * wa / (wa + wb);
    m->rdu0 = (wa - wb) / (wa + wb);
    m->rud0 = -m->rdu0;
    m->tuu0 = 2. * wb / (wa + wb);
}

static void point_eval_stable(const grto_job *J, const cplx *alpha, const cplx *beta, double k,
                              cplx w, const cplx slot0[2], ypar_t *Y)
{
    const int L = J->n_layer, s = J->s_layer, rl = J->r_layer;
    const double zs = J->zs, zr = J->zr;
    static __thread slay_t Ls[GRTO_MAXL];
    static __thread smrt_t M[GRTO_MAXL];
    static __thread m2_t Rud[GRTO_MAXL + 1], Rdu[GRTO_MAXL + 1], Tu[GRTO_MAXL + 1], Td[GRTO_MAXL + 1];
    static __thread cplx rud0[GRTO_MAXL + 1], rdu0[GRTO_MAXL + 1], tu0[GRTO_MAXL + 1], td0[GRTO_MAXL + 1];
    cplx mue[GRTO_MAXL];
    GRTO_COUNT_PAUSE;
    shear_moduli(J, beta, mue);
    GRTO_COUNT_RESUME;
    for (int i = 0; i < L; i++) slayer(k, w, alpha[i], beta[i], mue[i], &Ls[i]);
    for (int j = 0; j < L - 1; j++) sinterface(&Ls[j], &Ls[j + 1], &M[j]);

    /* free surface: R = T^{-1} diag(1,-1) T with T = stress rows of E_d */
    {
        const slay_t *l0 = &Ls[0];
        m2_t T = M2(l0->p[2], l0->d[2], l0->p[3], l0->d[3]);
        m2_t adj = M2(T.m[1][1], -T.m[0][1], -T.m[1][0], T.m[0][0]);
        m2_t DT = M2(T.m[0][0], T.m[0][1], -T.m[1][0], -T.m[1][1]);
        Rud[0] = m2scale(m2mul(adj, DT), 1.0 / l0->detT);
        rud0[0] = 1.0;
    }
    for (int lay = 0; lay < s; lay++) {      /* get_grt top-down, green.cu:471-520 */
        m2_t Lam = sphase(&Ls[lay], J->h[lay]);
        cplx ev = Lam.m[1][1];
        const smrt_t *m = &M[lay];
        cplx tem1 = rud0[lay] * ev, tem2 = m->rdu0 * ev, tem3 = m->tdd0 * ev;
        tu0[lay + 1] = m->tuu0 / (1. - tem1 * tem2);
        rud0[lay + 1] = m->rud0 + tem3 * tem1 * tu0[lay + 1];
        m2_t X = m2mul(Lam, m2mul(Rud[lay], Lam));
        m2_t A = m2add(m2eye(), m2mul(m->rd, X), -1);
        m2_t Bm = m2mul(m->td, X);
        Tu[lay + 1] = m2mul(m2inv(A), m->tu);
        Rud[lay + 1] = m2add(m->ru, m2mul(Bm, Tu[lay + 1]), 1);
    }
    {                                          /* half space, green.cu:522-531 */
        const smrt_t *mh = &M[L - 2];
        rdu0[L - 1] = mh->rdu0; td0[L - 1] = mh->tdd0;
        Td[L - 1] = mh->td; Rdu[L - 1] = mh->rd;
    }
    for (int lay = L - 3; lay >= s; lay--) {  /* bottom-up, green.cu:532-594 */
        m2_t Lam = sphase(&Ls[lay + 1], J->h[lay + 1]);
        cplx ev = Lam.m[1][1];
        const smrt_t *m = &M[lay];
        cplx tem1 = m->rud0 * ev, tem2 = rdu0[lay + 2] * ev, tem3 = m->tuu0 * ev;
        td0[lay + 1] = m->tdd0 / (1.0 - tem1 * tem2);
        rdu0[lay + 1] = m->rdu0 + tem3 * tem2 * td0[lay + 1];
        m2_t X = m2mul(Lam, m2mul(Rdu[lay + 2], Lam));
        m2_t A = m2add(m2eye(), m2mul(m->ru, X), -1);
        m2_t Bm = m2mul(m->tu, X);
        Td[lay + 1] = m2mul(m2inv(A), m->td);
        Rdu[lay + 1] = m2add(m->rd, m2mul(Bm, Td[lay + 1]), 1);
    }

    /* source (get_src_single / get_src_tensor) */
    const slay_t *S = &Ls[s];
    m2_t Ldn = sphase(S, J->h[s] - zs), Lup = sphase(S, zs);
    cplx sexd1 = Ldn.m[1][1], sexu1 = Lup.m[1][1];
    m2_t RD = Rdu[s + 1], RU = Rud[s];
    m2_t ED = m2mul(Ldn, m2mul(RD, Ldn)), EU = m2mul(Lup, m2mul(RU, Lup));
    m2_t wru0 = m2add(ED, m2eye(), -1), wrd0 = m2add(m2eye(), EU, -1);
    m2_t wru1 = m2add(ED, m2eye(), 1), wrd1 = m2add(m2eye(), EU, 1);
    const cplx su = S->mu;
    cplx ssh = 1. / (2. * su * S->v);
    cplx gu0[2], gd0[2], gu1[2], gd1[2], gshu = 0, gshd = 0;
    cplx su0[2], sd0[2], su1[2], sd1[2], su2[2], sd2[2], shu1 = 0, shd1 = 0, shu2 = 0, shd2 = 0;
    cplx shu_fac = 1. + sexd1 * rdu0[s + 1] * sexd1;
    cplx f1[2] = {S->d[1] / (2. * S->detH), -S->r / (2. * S->detH)};  /* -1/2 H^{-1} e_2 */
    if (J->src_type == 0) {
        cplx f0[2] = {-S->d[0] / (2. * S->detG), k / (2. * S->detG)};  /* 1/2 G^{-1} e_3 */
        m2vec(wru0, f0, gu0); m2vec(wrd0, f0, gd0);
        m2vec(wru1, f1, gu1); m2vec(wrd1, f1, gd1);
        gshu = shu_fac * ssh;
        gshd = (sexu1 * rud0[s] * sexu1 + 1.) * ssh;
    } else {
        cplx s2[2] = {k * f1[0], k * f1[1]};
        cplx s1[2] = {-S->d[3] / (2. * su * S->detG), -(su * S->x) / (2. * su * S->detG)};
        cplx al = -S->b * S->b / (2. * su * S->a * S->a);
        cplx be = (k / 2.) * (2. * S->b * S->b / (S->a * S->a) - 1.);
        cplx s0[2] = {(S->d[2] * al - S->d[1] * be) / S->detH, (-S->p[2] * al + S->p[1] * be) / S->detH};
        m2vec(wru1, s0, su0); m2vec(wrd1, s0, sd0);
        m2vec(wru0, s1, su1); m2vec(wrd0, s1, sd1);
        m2vec(wru1, s2, su2); m2vec(wrd1, s2, sd2);
        cplx shd_fac = sexu1 * rud0[s] * sexu1 - 1.;
        int fsh = (J->fix & GRTO_FIX_SHSRC) != 0;   /* as in point_eval */
        shu1 = (fsh ? 2. - shu_fac : shu_fac) * S->v * ssh; shd1 = shd_fac * S->v * ssh;
        shu2 = shu_fac * k * ssh; shd2 = (fsh ? shd_fac + 2. : shd_fac) * k * ssh;
    }
    m2_t yu_psv = m2inv(m2add(m2eye(), m2mul(ED, EU), -1));
    m2_t yd_psv = m2inv(m2add(m2eye(), m2mul(EU, ED), -1));
    cplx y_sh = 1. / (1. - sexd1 * rdu0[s + 1] * sexd1 * sexu1 * rud0[s] * sexu1);

    /* receiver (get_ypars_a_*) */
    const slay_t *R = &Ls[rl];
    const double rh = J->h[rl];
    m2_t Edsp = M2(R->p[0], R->d[0], R->p[1], R->d[1]);
    m2_t Eusp = M2(R->p[0], R->d[0], -R->p[1], -R->d[1]);
    const int fixdz = (J->fix & GRTO_FIX_DZ) != 0;
    const cplx *nu0 = (J->fix & GRTO_FIX_REXUT) ? NULL : slot0;
    cplx y0, y0t;
    m2_t y1, y1t;
    int up;
    if (s == rl && zr <= zs) {
        m2_t L1 = sphase(R, zr), L2 = sphase(R, zs - zr);
        m2_t L1t = sdphase(R, zr, -1, NULL), L2t = sdphase(R, zs - zr, +1, NULL);
        cplx e1v = L1.m[1][1], e2v = L2.m[1][1];
        cplx u0 = e1v * rud0[s] * sexu1 + e2v;
        cplx u0t = -R->v * e1v * rud0[s] * sexu1 + (fixdz ? R->v * e2v : R->v * e2v * R->v);
        m2_t U = m2add(m2mul(Edsp, m2mul(L1, m2mul(RU, Lup))), m2mul(Eusp, L2), 1);
        m2_t Ut = m2add(m2mul(Edsp, m2mul(L1t, m2mul(RU, Lup))), m2mul(Eusp, L2t), 1);
        y0 = u0 * y_sh; y0t = u0t * y_sh;
        y1 = m2mul(U, yu_psv); y1t = m2mul(Ut, yu_psv);
        up = 1;
    } else if (s == rl) {
        m2_t L1 = sphase(R, zr - zs), L2 = sphase(R, J->h[s] - zr);
        m2_t L1t = sdphase(R, zr - zs, -1, NULL), L2t = sdphase(R, J->h[s] - zr, +1, NULL);
        cplx e1v = L1.m[1][1], e2v = L2.m[1][1];
        cplx d0 = e1v + e2v * rdu0[s + 1] * sexd1;
        cplx d0t = -R->v * e1v + R->v * e2v * rdu0[s + 1] * sexd1;
        m2_t Dm = m2add(m2mul(Edsp, L1), m2mul(Eusp, m2mul(L2, m2mul(RD, Ldn))), 1);
        m2_t Dt = m2add(m2mul(Edsp, L1t), m2mul(Eusp, m2mul(L2t, m2mul(RD, Ldn))), 1);
        y0 = d0 * y_sh; y0t = d0t * y_sh;
        y1 = m2mul(Dm, yd_psv); y1t = m2mul(Dt, yd_psv);
        up = 0;
    } else if (rl < s) {
        int last = rl == L - 1;
        m2_t Ld_ = sphase(R, zr), Ldt = sdphase(R, zr, -1, NULL);
        m2_t Lu_ = last ? m2zero() : sphase(R, rh - zr);
        m2_t Lut = last ? m2zero() : sdphase(R, rh - zr, +1, nu0);
        m2_t Ex = sphase(R, rh);
        cplx u0 = Ld_.m[1][1] * rud0[rl] * Ex.m[1][1] + Lu_.m[1][1];
        cplx u0t = -R->v * Ld_.m[1][1] * rud0[rl] * Ex.m[1][1] + Lut.m[1][1];
        m2_t U = m2add(m2mul(Edsp, m2mul(Ld_, m2mul(Rud[rl], Ex))), m2mul(Eusp, Lu_), 1);
        m2_t Ut = m2add(m2mul(Edsp, m2mul(Ldt, m2mul(Rud[rl], Ex))), m2mul(Eusp, Lut), 1);
        cplx yu0 = tu0[s] * sexu1 * y_sh;
        m2_t yu1 = m2mul(Tu[s], m2mul(Lup, yu_psv));
        for (int lay = s - 2; lay >= rl; lay--) {
            m2_t Lm = sphase(&Ls[lay + 1], J->h[lay + 1]);
            yu0 = tu0[lay + 1] * Lm.m[1][1] * yu0;
            yu1 = m2mul(Tu[lay + 1], m2mul(Lm, yu1));
        }
        y0 = u0 * yu0;
        y0t = fixdz ? u0t * yu0 : u0t * y0;
        y1 = m2mul(U, yu1); y1t = m2mul(Ut, yu1);
        up = 1;
    } else {
        int last = rl == L - 1;
        m2_t Ld_ = sphase(R, zr), Ldt = sdphase(R, zr, -1, NULL);
        m2_t Lu_ = last ? m2zero() : sphase(R, rh - zr);
        m2_t Lut = last ? m2zero() : sdphase(R, rh - zr, +1, nu0);
        m2_t Rb = last ? m2zero() : Rdu[rl + 1];
        cplx Rb0 = last ? 0 : rdu0[rl + 1];
        m2_t Ex = sphase(R, rh);
        cplx d0 = Lu_.m[1][1] * Rb0 * Ex.m[1][1] + Ld_.m[1][1];
        cplx d0t = Lut.m[1][1] * Rb0 * Ex.m[1][1] - R->v * Ld_.m[1][1];
        m2_t Dm = m2add(m2mul(Edsp, Ld_), m2mul(Eusp, m2mul(Lu_, m2mul(Rb, Ex))), 1);
        m2_t Dt = m2add(m2mul(Edsp, Ldt), m2mul(Eusp, m2mul(Lut, m2mul(Rb, Ex))), 1);
        cplx yd0 = td0[s + 1] * sexd1 * y_sh;
        m2_t yd1 = m2mul(Td[s + 1], m2mul(Ldn, yd_psv));
        for (int lay = s + 2; lay <= rl; lay++) {
            m2_t Lm = sphase(&Ls[lay - 1], J->h[lay - 1]);
            yd0 = td0[lay] * Lm.m[1][1] * yd0;
            yd1 = m2mul(Td[lay], m2mul(Lm, yd1));
        }
        y0 = d0 * yd0; y0t = d0t * yd0;
        y1 = m2mul(Dm, yd1); y1t = m2mul(Dt, yd1);
        up = 0;
    }

    memset(Y, 0, sizeof(*Y));
    if (J->src_type == 0) {
        const cplx *g0 = up ? gu0 : gd0, *g1 = up ? gu1 : gd1;
        cplx gsh = up ? gshu : gshd;
        Y->b1 = y0 * gsh;
        Y->b1t = y0t * gsh;
        m2vec(y1, g0, Y->a0); m2vec(y1, g1, Y->a1);
        m2vec(y1t, g0, Y->a0t); m2vec(y1t, g1, Y->a1t);
    } else {
        const cplx *q0 = up ? su0 : sd0, *q1 = up ? su1 : sd1, *q2 = up ? su2 : sd2;
        cplx h1 = up ? shu1 : shd1, h2 = up ? shu2 : shd2;
        Y->b1 = y0 * h1; Y->b2 = y0 * h2; Y->b1t = y0t * h1; Y->b2t = y0t * h2;
        m2vec(y1, q0, Y->a0); m2vec(y1, q1, Y->a1); m2vec(y1, q2, Y->a2);
        m2vec(y1t, q0, Y->a0t); m2vec(y1t, q1, Y->a1t); m2vec(y1t, q2, Y->a2t);
    }
}

/* dispatch between the reference restatement and the stable formulation */
static void point_any(const grto_job *J, const cplx *alpha, const cplx *beta, double k,
                      cplx w, const cplx slot0[2], ypar_t *Y)
{
    if (J->fix & GRTO_STABLE) point_eval_stable(J, alpha, beta, k, w, slot0, Y);
    else point_eval(J, alpha, beta, k, w, slot0, Y);
}

/* integrands at one distance: get_int_val_single green.cu:1558-1621,
 * get_int_val_tensor green.cu:1626-1716 (columns 10-19 overwritten there by
 * the d/dr terms; 20-29 are never written and are zero here) */
static void integrand(int src_type, int fix, const ypar_t *p, double k, double dist, cplx out[30])
{
    double x = dist * k;
    int cf = (fix & GRTO_FIX_COLS) != 0;
    double j0 = grto_besselj(x, 0), j1 = grto_besselj(x, 1), j2 = grto_besselj(x, 2);
    double j0d = grto_d_besselj(x, 0), j1d = grto_d_besselj(x, 1), j2d = grto_d_besselj(x, 2);
    double j0dd = cf ? grto_dd_besselj_exact(x, 0) : grto_dd_besselj(x, 0);
    double j1dd = cf ? grto_dd_besselj_exact(x, 1) : grto_dd_besselj(x, 1);
    double j2dd = cf ? grto_dd_besselj_exact(x, 2) : grto_dd_besselj(x, 2);
    for (int i = 0; i < 30; i++) out[i] = 0;
    if (src_type == 0) {
        out[0] = p->b1 * j1 / dist + p->a1[0] * k * j1d;
        out[1] = p->a0[0] * k * j0d;
        out[2] = p->a1[0] * j1 / dist + p->b1 * k * j1d;
        out[3] = p->a1[1] * k * j1;
        out[4] = p->a0[1] * k * j0;
        out[5] = p->b1t * j1 / dist + p->a1t[0] * k * j1d;
        out[6] = p->a0t[0] * k * j0d;
        out[7] = p->a1t[0] * j1 / dist + p->b1t * k * j1d;
        out[8] = p->a1t[1] * k * j1;
        out[9] = p->a0t[1] * k * j0;
        /* green.cu:1596 writes b1 j1d k without the 1/r of d/dr (b1 J1(kr)/r) */
        out[10] = -p->b1 * j1 / dist / dist + p->b1 * j1d * k / (cf ? dist : 1.0) + p->a1[0] * k * j1dd * k;
        out[11] = p->a0[0] * k * j0dd * k;
        out[12] = -p->a1[0] * j1 / dist / dist + p->a1[0] * j1d * k / dist + p->b1 * k * j1dd * k;
        out[13] = p->a1[1] * k * j1d * k;
        out[14] = p->a0[1] * k * j0d * k;
    } else {
        cplx b1u = cf ? p->b1 : p->b2, b1tu = cf ? p->b1t : p->b2t;   /* green.cu:1657, 1672, 1686 use b2 */
        out[0] = p->b2 * 2.0 * j2 / dist + p->a2[0] * k * j2d;
        out[1] = p->b1 * j1 / dist + p->a1[0] * k * j1d;
        /* green.cu:1652-1653 build the m = 0 radial terms from the vertical
         * coefficients (a2[1], a0[1]); GRTO_FIX_COLS takes the radial ones, as
         * every other radial column does (the free surface's zero shear
         * traction, d/dz a[0] = k a[1] at z = 0, shows a[0] radial) */
        const cplx *a2h = cf ? &p->a2[0] : &p->a2[1], *a0h = cf ? &p->a0[0] : &p->a0[1];
        out[2] = *a2h * k * j0d;
        out[3] = *a0h * k * j0d;
        out[4] = p->b2 * k * j2d + 2.0 * p->a2[0] * j2 / dist;
        out[5] = b1u * k * j1d + p->a1[0] * j1 / dist;
        out[6] = p->a2[1] * k * j2;
        out[7] = p->a1[1] * k * j1;
        out[8] = p->a0[1] * k * j0;
        out[9] = p->a2[1] * k * j0;
        int o = cf ? 20 : 10;   /* d/dr block: 20-29 corrected, 10-19 (over d/dz) in the reference */
        if (cf) {
            out[10] = p->b2t * 2.0 * j2 / dist + p->a2t[0] * k * j2d;
            out[11] = p->b1t * j1 / dist + p->a1t[0] * k * j1d;
            out[12] = p->a2t[0] * k * j0d;
            out[13] = p->a0t[0] * k * j0d;
            out[14] = p->b2t * k * j2d + 2.0 * p->a2t[0] * j2 / dist;
            out[15] = b1tu * k * j1d + p->a1t[0] * j1 / dist;
            out[16] = p->a2t[1] * k * j2;
            out[17] = p->a1t[1] * k * j1;
            out[18] = p->a0t[1] * k * j0;
            out[19] = p->a2t[1] * k * j0;
        }
        out[o + 0] = -p->b2 * 2.0 * j2 / dist / dist + p->b2 * 2.0 * j2d * k / dist + p->a2[0] * k * j2dd * k;
        out[o + 1] = -p->b1 * j1 / dist / dist + p->b1 * j1d * k / dist + p->a1[0] * k * j1dd * k;
        out[o + 2] = *a2h * k * j0dd * k;
        out[o + 3] = *a0h * k * j0dd * k;
        out[o + 4] = p->b2 * k * j2dd * k - 2.0 * p->a2[0] * j2 / dist / dist + 2.0 * p->a2[0] * j2d * k / dist;
        out[o + 5] = b1u * k * j1dd * k - p->a1[0] * j1 / dist / dist + p->a1[0] * j1d * k / dist;
        out[o + 6] = p->a2[1] * k * j2d * k;
        out[o + 7] = p->a1[1] * k * j1d * k;
        out[o + 8] = p->a0[1] * k * j0d * k;
        out[o + 9] = p->a2[1] * k * j0d * k;
    }
}

/* nu of layer r_layer at the first (w,k) point of the reference's list
 * (w = -i sigma, k = 0), which green.cu:674-675 reads as par[r_layer]. */
static void slot0_nu(const grto_job *J, cplx out[2])
{
    cplx a[GRTO_MAXL], b[GRTO_MAXL], E[4][4];
    cplx w = omega(J, 0);
    attenuate(J, w, a, b);
    layer_pars(0.0, w, a[J->r_layer], b[J->r_layer], J->mu[J->r_layer], &out[0], &out[1], E);
}

int grto_point(const grto_job *J, int iw, double k, double *out)
{
    cplx a[GRTO_MAXL], b[GRTO_MAXL], slot0[2];
    ypar_t Y;
    if (iw < 0 || iw >= J->nw) return GRTO_ERR_ARG;
    cplx w = omega(J, iw);
    attenuate(J, w, a, b);
    slot0_nu(J, slot0);
    point_any(J, a, b, k, w, slot0, &Y);
    const cplx *v = (const cplx *)&Y;
    for (int i = 0; i < 16; i++) { out[2 * i] = creal(v[i]); out[2 * i + 1] = cimag(v[i]); }
    return GRTO_OK;
}

#ifdef GRTO_COUNT
/* Complex operations of one per-(w,k) evaluation (point_any), the
 * per-frequency attenuation and slot-0 wavenumbers excluded. */
extern "C" long long grto_count_point(const grto_job *J, int iw, double k)
{
    cplx a[GRTO_MAXL], b[GRTO_MAXL], slot0[2];
    ypar_t Y;
    cplx w = omega(J, iw);
    attenuate(J, w, a, b);
    slot0_nu(J, slot0);
    grto_cnt.flops = 0;
    grto_cnt.paused = 0;
    point_any(J, a, b, k, w, slot0, &Y);
    return grto_cnt.flops;
}
#endif

int grto_integrand(const grto_job *J, int iw, double k, double r, double *out)
{
    cplx a[GRTO_MAXL], b[GRTO_MAXL], slot0[2], v[30];
    ypar_t Y;
    if (iw < 0 || iw >= J->nw) return GRTO_ERR_ARG;
    cplx w = omega(J, iw);
    attenuate(J, w, a, b);
    slot0_nu(J, slot0);
    point_any(J, a, b, k, w, slot0, &Y);
    integrand(J->src_type, J->fix, &Y, k, r, v);
    for (int i = 0; i < 30; i++) { out[2 * i] = creal(v[i]); out[2 * i + 1] = cimag(v[i]); }
    return GRTO_OK;
}

/* in-place radix-2 FFT with exp(+2 pi i jn/N) (unnormalised inverse) */
static void ifft_inplace(cplx *x, int n)
{
    for (int i = 1, j = 0; i < n; i++) {
        int bit = n >> 1;
        for (; j & bit; bit >>= 1) j ^= bit;
        j ^= bit;
        if (i < j) { cplx t = x[i]; x[i] = x[j]; x[j] = t; }
    }
    for (int len = 2; len <= n; len <<= 1) {
        double ang = 2 * PI / len;
        for (int i = 0; i < n; i += len) {
            for (int j = 0; j < len / 2; j++) {
                cplx wj = mkc(cos(ang * j), sin(ang * j));
                cplx u = x[i + j], v = x[i + j + len / 2] * wj;
                x[i + j] = u + v;
                x[i + j + len / 2] = u - v;
            }
        }
    }
}

int grto_run(const grto_job *J, double *spec, double *sig, int nthreads)
{
    const int nw = J->nw, N = 2 * nw, nd = J->n_dist;
    const double *dist = J->dist;
    if (nd < 1 || !dist) return GRTO_ERR_ARG;
    const int ncol = 30;
    cplx *out = (cplx *)calloc((size_t)nd * N * ncol, sizeof(cplx));
    if (!out) return GRTO_ERR_NOMEM;
    cplx slot0[2];
    slot0_nu(J, slot0);
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 1)
#endif
    for (int iw = 0; iw < nw; iw++) {
        cplx a[GRTO_MAXL], b[GRTO_MAXL], v[30];
        cplx w = omega(J, iw);
        attenuate(J, w, a, b);
        int nk = grto_nk(J, iw);
        /* k-sum of integrate(), green.cu:1873-1903: weight dk, dk/2 at k = 0 */
        for (int ik = 0; ik < nk; ik++) {
            double k = J->dk * ik;
            ypar_t Y;
            point_any(J, a, b, k, w, slot0, &Y);
            for (int d = 0; d < nd; d++) {
                integrand(J->src_type, J->fix, &Y, k, dist[d], v);
                cplx *o = out + ((size_t)d * N + iw) * ncol;
                if (ik == 0) for (int c = 0; c < ncol; c++) o[c] = v[c] * J->dk / 2.0;
                else for (int c = 0; c < ncol; c++) o[c] += v[c] * J->dk;
            }
        }
    }
    /* phase, taper and scale: green.cu:1905-1921 */
    int wc = (int)((double)nw * (1 - J->taper));
    double ifftcoef = J->df * nw / PI;
    for (int d = 0; d < nd; d++) {
        cplx *o = out + (size_t)d * N * ncol;
        for (int iw = 0; iw < nw; iw++) {
            double phi = PI2 * J->df * iw * J->t0;
            double st0 = 1;
            if (iw > wc) st0 = 0.5 * (1. + cos((iw - wc + 1) * PI / (nw - wc + 1)));
            for (int c = 0; c < ncol; c++) o[iw * ncol + c] = st0 * (o[iw * ncol + c] * mkc(cos(phi), sin(phi))) * ifftcoef;
        }
        /* Hermitian fill: green.cu:1925-1938 */
        for (int iw = 0; iw < nw; iw++)
            for (int c = 0; c < ncol; c++) o[(nw + iw) * ncol + c] = iw == 0 ? 0 : conj(o[(nw - iw) * ncol + c]);
    }
    if (spec) {
        for (size_t i = 0; i < (size_t)nd * N * ncol; i++) { spec[2 * i] = creal(out[i]); spec[2 * i + 1] = cimag(out[i]); }
    }
    if (sig) {
        /* inverse DFT and de-damping: green.cu:2227-2239 */
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 1)
#endif
        for (int dc = 0; dc < nd * ncol; dc++) {
            int d = dc / ncol, c = dc % ncol;
            cplx *x = (cplx *)malloc(sizeof(cplx) * N);
            for (int i = 0; i < N; i++) x[i] = out[((size_t)d * N + i) * ncol + c];
            ifft_inplace(x, N);
            for (int j = 0; j < N; j++) {
                double s = creal(x[j]) / ((double)nw) / 2.0;
                s = s * exp(((double)j) * J->dt * J->sigma) * exp(J->t0 * J->sigma);
                sig[((size_t)d * N + j) * ncol + c] = s;
            }
            free(x);
        }
    }
    free(out);
    return GRTO_OK;
}

int grto_run_band(const grto_job *J, int iw0, int iw1, double *sums, int nthreads)
{
    const int nd = J->n_dist, ncol = 30;
    if (nd < 1 || !J->dist || iw0 < 0 || iw1 > J->nw || iw1 <= iw0) return GRTO_ERR_ARG;
    cplx slot0[2];
    slot0_nu(J, slot0);
    cplx *out = (cplx *)calloc((size_t)(iw1 - iw0) * nd * ncol, sizeof(cplx));
    if (!out) return GRTO_ERR_NOMEM;
    /* parallel over (frequency, k-block) so that a few frequencies still use all cores */
    const int kb = 256;
    int nblk = 0;
    for (int iw = iw0; iw < iw1; iw++) nblk += (grto_nk(J, iw) + kb - 1) / kb;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel
#endif
    {
        cplx *loc = (cplx *)calloc((size_t)(iw1 - iw0) * nd * ncol, sizeof(cplx));
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 1)
#endif
        for (int b = 0; b < nblk; b++) {
            int iw = iw0, rem = b;
            for (;; iw++) {
                int n = (grto_nk(J, iw) + kb - 1) / kb;
                if (rem < n) break;
                rem -= n;
            }
            int nk = grto_nk(J, iw);
            cplx a[GRTO_MAXL], bb[GRTO_MAXL], v[30];
            cplx w = omega(J, iw);
            attenuate(J, w, a, bb);
            for (int ik = rem * kb; ik < nk && ik < (rem + 1) * kb; ik++) {
                double k = J->dk * ik;
                ypar_t Y;
                point_any(J, a, bb, k, w, slot0, &Y);
                double wk = ik == 0 ? J->dk / 2.0 : J->dk;
                for (int d = 0; d < nd; d++) {
                    integrand(J->src_type, J->fix, &Y, k, J->dist[d], v);
                    cplx *o = loc + ((size_t)(iw - iw0) * nd + d) * ncol;
                    for (int c = 0; c < ncol; c++) o[c] += v[c] * wk;
                }
            }
        }
#ifdef _OPENMP
#pragma omp critical
#endif
        for (size_t i = 0; i < (size_t)(iw1 - iw0) * nd * ncol; i++) out[i] += loc[i];
        free(loc);
    }
    if (sums)
        for (size_t i = 0; i < (size_t)(iw1 - iw0) * nd * ncol; i++) {
            sums[2 * i] = creal(out[i]);
            sums[2 * i + 1] = cimag(out[i]);
        }
    free(out);
    return GRTO_OK;
}

int grto_green(const char *iname, const char *oname_w, const char *oname_t, int nthreads)
{
    grto_job J;
    int rc = grto_parse(iname, &J);
    if (rc) return rc;
    rc = grto_setup(&J, J.dt, J.log2n, J.t0, J.taper, 2.0, GRTO_K_REFERENCE, 0, 0.0, 0);
    if (rc) return rc;
    J.n_dist = 1;
    J.dist = &J.dist0;
    const int N = 2 * J.nw;
    double *spec = (double *)malloc(sizeof(double) * N * 60);
    double *sig = (double *)malloc(sizeof(double) * N * 30);
    if (!spec || !sig) { free(spec); free(sig); return GRTO_ERR_NOMEM; }
    rc = grto_run(&J, spec, sig, nthreads);
    if (!rc) {
        /* writers: green.cu:2242-2258 */
        FILE *f = fopen(oname_t, "w");
        if (!f) rc = GRTO_ERR_IO;
        else {
            for (int j = 0; j < N; j++) {
                for (int c = 0; c < 30; c++) fprintf(f, "%.18e,", sig[j * 30 + c]);
                fprintf(f, "\n");
            }
            fclose(f);
        }
        f = rc ? NULL : fopen(oname_w, "w");
        if (!rc && !f) rc = GRTO_ERR_IO;
        if (f) {
            for (int j = 0; j < N; j++) {
                for (int c = 0; c < 30; c++) fprintf(f, "%.18e,%.18e,", spec[(j * 30 + c) * 2], spec[(j * 30 + c) * 2 + 1]);
                fprintf(f, "\n");
            }
            fclose(f);
        }
    }
    free(spec);
    free(sig);
    return rc;
}
