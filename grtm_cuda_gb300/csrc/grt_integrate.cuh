// grt_integrate.cuh -- wavenumber integration and the spectral stage.
//
//  bessel_table_kernel  B[j][b][r]: the nine Bessel functions of k_j r the
//                       integrands use, evaluated once per (k grid, receiver
//                       set) in FP64 with the reference's own formulas
//                       (green.cu:1418-1554) -- including the k r argument
//                       reduction -- and stored in the working precision.
//  ksum_kernel          S[r][c][iw] = sum_j w_j (integrand c)(w_iw, k_j, r):
//                       the k-sum of integrate() (green.cu:1873-1903) for all
//                       receivers at once, driven by the column tables below
//                       (get_int_val_single / _tensor, green.cu:1558-1716).
//  spectral_kernel      phase e^{i w t0}, cosine taper and scale
//                       (green.cu:1905-1921), Hermitian fill (1925-1938),
//                       inverse DFT and e^{sigma t} de-damping (2227-2239),
//                       one trace per block, FFT in shared memory: the FP64
//                       plans' form (FP32 plans run fft::c2r_kernel,
//                       grt_fft.cuh).
#pragma once
#include "grt_cplx.cuh"
#include "grt_types.h"

namespace grt {

// ---------------------------------------------------------------- Bessel
__device__ __forceinline__ double bj0_ref(double x)
{
    // Abramowitz & Stegun 9.4.1 / 9.4.3 (as evaluated by the reference)
    double ax = fabs(x);
    if (ax <= 3.0) {
        double y = (ax / 3.0) * (ax / 3.0);
        return 1.0 + y * (-2.2499997 + y * (1.2656208 + y * (-0.3163866 + y * (0.0444479 + y * (-0.0039444 + y * 0.00021)))));
    }
    double t = 3.0 / ax;
    double f = 0.79788456 + t * (-0.00000077 + t * (-0.0055274 + t * (-0.00009512 + t * (0.00137237 + t * (-0.00072805 + t * 0.00014476)))));
    double th = ax - 0.78539816 + t * (-0.04166397 + t * (-0.00003954 + t * (0.00262573 + t * (-0.00054125 + t * (-0.00029333 + t * 0.00013558)))));
    return f * cos(th) / sqrt(ax);
}

__device__ __forceinline__ double bj1_ref(double x)
{
    // Abramowitz & Stegun 9.4.4 / 9.4.6
    double ax = fabs(x);
    if (ax <= 3.0) {
        double y = (ax / 3.0) * (ax / 3.0);
        return x * (0.5 + y * (-0.56249985 + y * (0.21093573 + y * (-0.03954289 + y * (0.00443319 + y * (-0.00031761 + y * 0.00001109))))));
    }
    double t = 3.0 / ax;
    double f = 0.79788456 + t * (0.00000156 + t * (0.01659667 + t * (0.00017105 + t * (-0.00249511 + t * (0.00113653 + t * (-0.00020033))))));
    double th = ax - 2.35619449 + t * (0.12499612 + t * (0.0000565 + t * (-0.00637879 + t * (0.00074348 + t * (0.00079824 + t * (-0.00029166))))));
    return (x >= 0 ? 1.0 : -1.0) * f * cos(th) / sqrt(ax);
}

// J_n for n >= 0: upward recurrence above n, Miller's downward recurrence
// below (normalised by J0 + 2 sum J_2m), as green.cu:1467-1529 does
__device__ __forceinline__ double bjn_ref(double x, int n)
{
    if (n == 0) return bj0_ref(x);
    if (n == 1) return bj1_ref(x);
    double ax = fabs(x), res;
    if (ax == 0.0) return 0.0;
    if (ax > n) {
        double tox = 2.0 / ax, bjm = bj0_ref(ax), bj = bj1_ref(ax);
        for (int j = 1; j < n; j++) {
            double bjp = j * tox * bj - bjm;
            bjm = bj;
            bj = bjp;
        }
        res = bj;
    } else {
        double tox = 2.0 / ax;
        int m = 2 * ((n + (int)sqrt((double)(40 * n))) / 2);
        bool acc = false;
        double sum = 0.0, bjp = 0.0, bj = 1.0;
        res = 0.0;
        for (int j = m; j >= 1; j--) {
            double bjm = j * tox * bj - bjp;
            bjp = bj;
            bj = bjm;
            if (fabs(bj) > 1e10) { bj *= 1e-10; bjp *= 1e-10; res *= 1e-10; sum *= 1e-10; }
            if (acc) sum += bj;
            acc = !acc;
            if (j == n) res = bjp;
        }
        sum = 2.0 * sum - bj;
        res /= sum;
    }
    if (x < 0.0 && (n & 1)) res = -res;
    return res;
}

__device__ __forceinline__ double dbj_ref(double x, int n)
{
    if (fabs(x) < 1e-10) return (bjn_ref(1e-10, n) - bjn_ref(0.0, n)) / 1e-10;
    return n * bjn_ref(x, n) / x - bjn_ref(x, n + 1);
}

// the reference's second derivative expression (green.cu:1543-1554)
// J_n''(x) from Bessel's equation: -J_{n-1}/x + ((n^2 + n)/x^2 - 1) J_n
// (series near 0), the corrected-columns form
__device__ __forceinline__ double ddbj_exact(double x, int n)
{
    if (fabs(x) < 1e-3) {
        const double x2 = x * x;
        return n == 0 ? -0.5 + 3.0 * x2 / 16.0 : n == 1 ? -0.375 * x : 0.25 - x2 / 8.0;
    }
    const double jm = n == 0 ? -bjn_ref(x, 1) : bjn_ref(x, n - 1);
    return -jm / x + ((double)(n * n + n) / (x * x) - 1.0) * bjn_ref(x, n);
}

__device__ __forceinline__ double ddbj_ref(double x, int n)
{
    if (fabs(x) < 1e-10) return (dbj_ref(1e-10, n) - dbj_ref(0.0, n)) / 1e-10;
    return n * bjn_ref(x, n - 1) / x - bjn_ref(x, n) * (n + n * n + x * x) / x / x;
}

// FP32 evaluation of the same formulas for x > 3 (the asymptotic branch of
// A&S 9.4.3 / 9.4.6, where x = k r reaches 10^4): x is reduced modulo 2 pi in
// FP64 (two-constant Cody-Waite split), the phase polynomial and amplitude
// are FP32.  J2, J3 by the reference's upward recurrence (used for x > n).
__device__ __forceinline__ void bessel_big_x(double x, float v[NBASIS], bool exact)
{
    const double TWO_PI_HI = 6.28318530717958623200e+00;   // 2 pi rounded to double
    const double TWO_PI_LO = 2.44929359829470635445e-16;   // 2 pi - TWO_PI_HI
    double n = rint(x * 0.15915494309189533577);
    float xr = (float)fma(-n, TWO_PI_LO, fma(-n, TWO_PI_HI, x));   // x mod 2 pi in [-pi, pi]
    float xf = (float)x;
    float t = 3.0f / xf;
    float f0 = 0.79788456f + t * (-0.00000077f + t * (-0.0055274f + t * (-0.00009512f + t * (0.00137237f + t * (-0.00072805f + t * 0.00014476f)))));
    float p0 = -0.78539816f + t * (-0.04166397f + t * (-0.00003954f + t * (0.00262573f + t * (-0.00054125f + t * (-0.00029333f + t * 0.00013558f)))));
    float f1 = 0.79788456f + t * (0.00000156f + t * (0.01659667f + t * (0.00017105f + t * (-0.00249511f + t * (0.00113653f + t * (-0.00020033f))))));
    float p1 = -2.35619449f + t * (0.12499612f + t * (0.0000565f + t * (-0.00637879f + t * (0.00074348f + t * (0.00079824f + t * (-0.00029166f))))));
    float is = rsqrtf(xf);
    float j0 = f0 * cosf(xr + p0) * is;
    float j1 = f1 * cosf(xr + p1) * is;
    float ix = 1.0f / xf;
    float j2 = 2.0f * ix * j1 - j0;                  // x > 3 > n: upward recurrence
    float j3 = 4.0f * ix * j2 - j1;
    v[BJ0] = j0;
    v[BJ1] = j1;
    v[BJ2] = j2;
    v[BJ0D] = -j1;                                   // 0 J0 / x - J1
    v[BJ1D] = ix * j1 - j2;
    v[BJ2D] = 2.0f * ix * j2 - j3;
    if (exact) {                                     // Bessel's equation
        v[BJ0DD] = j1 * ix - j0;
        v[BJ1DD] = -j0 * ix + (2.0f * ix * ix - 1.0f) * j1;
        v[BJ2DD] = -j1 * ix + (6.0f * ix * ix - 1.0f) * j2;
    } else {                                         // reference second-derivative expression
        v[BJ0DD] = -j0;
        v[BJ1DD] = ix * j0 - j1 * (2.0f + xf * xf) * ix * ix;
        v[BJ2DD] = 2.0f * ix * j1 - j2 * (6.0f + xf * xf) * ix * ix;
    }
}

// tile_rows = 0: layout B[j][b][r]; tile_rows > 0: receiver tiles of 16,
// B[r / 16][j][b][r % 16] with tile_rows rows per tile (a stage of the
// tensor-core sum then reads 8 consecutive rows as one contiguous block)
// Bessel table layouts: [row][basis][receiver], or tiled for the tensor-core
// sum, [receiver / 32][row][basis][32] with the receivers of row j permuted by
// r ^ 8 (j & 3) (so that a warp's reads of 8 receivers x 4 rows hit 32 banks)
constexpr int kBesselTile = 32;
__device__ __forceinline__ long long btab_index(int j, int b, int r, int nr, int tile_rows)
{
    if (tile_rows > 0)
        return (((long long)(r >> 5) * tile_rows + j) * NBASIS + b) * kBesselTile + ((r & 31) ^ ((j & 3) << 3));
    return ((long long)j * NBASIS + b) * nr + r;
}

template <typename R>
__global__ void bessel_table_kernel(R *B, int nk, int nr, double dk, const double *dist, int tile_rows, int exact_dd)
{
    long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= (long long)nk * nr) return;
    int r = (int)(t % nr);
    int j = (int)(t / nr);
    double x = dist[r] * (dk * j);
    if (sizeof(R) == 4 && x > 3.0) {
        float vf[NBASIS];
        bessel_big_x(x, vf, exact_dd != 0);
#pragma unroll
        for (int b = 0; b < NBASIS; b++) B[btab_index(j, b, r, nr, tile_rows)] = (R)vf[b];
        return;
    }
    double v[NBASIS];
    v[BJ0] = bjn_ref(x, 0);
    v[BJ1] = bjn_ref(x, 1);
    v[BJ2] = bjn_ref(x, 2);
    v[BJ0D] = dbj_ref(x, 0);
    v[BJ1D] = dbj_ref(x, 1);
    v[BJ2D] = dbj_ref(x, 2);
    v[BJ0DD] = exact_dd ? ddbj_exact(x, 0) : ddbj_ref(x, 0);
    v[BJ1DD] = exact_dd ? ddbj_exact(x, 1) : ddbj_ref(x, 1);
    v[BJ2DD] = exact_dd ? ddbj_exact(x, 2) : ddbj_ref(x, 2);
#pragma unroll
    for (int b = 0; b < NBASIS; b++) B[btab_index(j, b, r, nr, tile_rows)] = (R)v[b];
}

// ---------------------------------------------------------------- column tables
// An integrand column is a sum of terms coef * r^-rpow * (K_q k^kp) J_b(k r).
struct Pair { int q, kp, b; };
struct Term { int pair, rpow; double coef; };

// single force, green.cu:1582-1600
constexpr __device__ Pair kSinglePairs[] = {
    {QS_B1, 0, BJ1},   {QS_A10, 1, BJ1D},  {QS_A00, 1, BJ0D},  {QS_A10, 0, BJ1},   {QS_B1, 1, BJ1D},
    {QS_A11, 1, BJ1},  {QS_A01, 1, BJ0},   {QS_B1T, 0, BJ1},   {QS_A1T0, 1, BJ1D}, {QS_A0T0, 1, BJ0D},
    {QS_A1T0, 0, BJ1}, {QS_B1T, 1, BJ1D},  {QS_A1T1, 1, BJ1},  {QS_A0T1, 1, BJ0},  {QS_A10, 2, BJ1DD},
    {QS_A00, 2, BJ0DD}, {QS_B1, 2, BJ1DD}, {QS_A11, 2, BJ1D},  {QS_A01, 2, BJ0D},
};
constexpr int kSingleNP = sizeof(kSinglePairs) / sizeof(Pair);
constexpr __device__ Term kSingleTerms[] = {
    // col 0..4: displacement
    {0, 1, 1.0}, {1, 0, 1.0},
    {2, 0, 1.0},
    {3, 1, 1.0}, {4, 0, 1.0},
    {5, 0, 1.0},
    {6, 0, 1.0},
    // col 5..9: d/dz
    {7, 1, 1.0}, {8, 0, 1.0},
    {9, 0, 1.0},
    {10, 1, 1.0}, {11, 0, 1.0},
    {12, 0, 1.0},
    {13, 0, 1.0},
    // col 10..14: d/dr
    {0, 2, -1.0}, {4, 0, 1.0}, {14, 0, 1.0},
    {15, 0, 1.0},
    {3, 2, -1.0}, {1, 1, 1.0}, {16, 0, 1.0},
    {17, 0, 1.0},
    {18, 0, 1.0},
};
constexpr __device__ int kSingleCol[16] = {0, 2, 3, 5, 6, 7, 9, 10, 12, 13, 14, 17, 18, 21, 22, 23};  // term ranges
constexpr int kSingleNC = 15;

// moment tensor, green.cu:1650-1691 (the d/dz block 10-19 is overwritten there)
constexpr __device__ Pair kTensorPairs[] = {
    {QT_B2, 0, BJ2},   {QT_A20, 1, BJ2D},  {QT_B1, 0, BJ1},    {QT_A10, 1, BJ1D},  {QT_A21, 1, BJ0D},
    {QT_A01, 1, BJ0D}, {QT_B2, 1, BJ2D},   {QT_A20, 0, BJ2},   {QT_B2, 1, BJ1D},   {QT_A10, 0, BJ1},
    {QT_A21, 1, BJ2},  {QT_A11, 1, BJ1},   {QT_A01, 1, BJ0},   {QT_A21, 1, BJ0},   {QT_A20, 2, BJ2DD},
    {QT_B1, 1, BJ1D},  {QT_A10, 2, BJ1DD}, {QT_A21, 2, BJ0DD}, {QT_A01, 2, BJ0DD}, {QT_B2, 2, BJ2DD},
    {QT_B2, 2, BJ1DD}, {QT_A21, 2, BJ2D},  {QT_A11, 2, BJ1D},  {QT_A01, 2, BJ0D},  {QT_A21, 2, BJ0D},
};
constexpr int kTensorNP = sizeof(kTensorPairs) / sizeof(Pair);
constexpr __device__ Term kTensorTerms[] = {
    {0, 1, 2.0}, {1, 0, 1.0},                    // 0
    {2, 1, 1.0}, {3, 0, 1.0},                    // 1
    {4, 0, 1.0},                                 // 2
    {5, 0, 1.0},                                 // 3
    {6, 0, 1.0}, {7, 1, 2.0},                    // 4
    {8, 0, 1.0}, {9, 1, 1.0},                    // 5
    {10, 0, 1.0},                                // 6
    {11, 0, 1.0},                                // 7
    {12, 0, 1.0},                                // 8
    {13, 0, 1.0},                                // 9
    {0, 2, -2.0}, {6, 1, 2.0}, {14, 0, 1.0},     // 10
    {2, 2, -1.0}, {15, 1, 1.0}, {16, 0, 1.0},    // 11
    {17, 0, 1.0},                                // 12
    {18, 0, 1.0},                                // 13
    {19, 0, 1.0}, {7, 2, -2.0}, {1, 1, 2.0},     // 14
    {20, 0, 1.0}, {9, 2, -1.0}, {3, 1, 1.0},     // 15
    {21, 0, 1.0},                                // 16
    {22, 0, 1.0},                                // 17
    {23, 0, 1.0},                                // 18
    {24, 0, 1.0},                                // 19
};
constexpr __device__ int kTensorCol[21] = {0, 2, 4, 5, 6, 8, 10, 11, 12, 13, 14, 17, 20, 21, 22, 25, 28, 29, 30, 31, 32};
constexpr int kTensorNC = 20;

// corrected single force: the d/dr column 10 term b1 k J1'(kr) carries 1/r
constexpr __device__ Term kSingleFixTerms[] = {
    {0, 1, 1.0}, {1, 0, 1.0},
    {2, 0, 1.0},
    {3, 1, 1.0}, {4, 0, 1.0},
    {5, 0, 1.0},
    {6, 0, 1.0},
    {7, 1, 1.0}, {8, 0, 1.0},
    {9, 0, 1.0},
    {10, 1, 1.0}, {11, 0, 1.0},
    {12, 0, 1.0},
    {13, 0, 1.0},
    {0, 2, -1.0}, {4, 1, 1.0}, {14, 0, 1.0},
    {15, 0, 1.0},
    {3, 2, -1.0}, {1, 1, 1.0}, {16, 0, 1.0},
    {17, 0, 1.0},
    {18, 0, 1.0},
};

// corrected moment tensor: 30 columns -- displacement 0-9 (column 5, the m = 1
// transverse term, with b1 where green.cu:1657 has b2; the m = 0 radial
// columns 2, 3 with the radial coefficients a20, a00 where green.cu:1652-1653
// have the vertical a21, a01), d/dz 10-19 from the z-derivative coefficients
// (the block green.cu:1666-1677 writes and then overwrites), d/dr 20-29
// (green.cu:1680-1691, column 25 with b1, 22 and 23 radial)
constexpr int QTT = QT_N;   // offset of the z-derivative coefficient columns
constexpr __device__ Pair kTensorFixPairs[] = {
    {QT_B2, 0, BJ2},   {QT_A20, 1, BJ2D},  {QT_B1, 0, BJ1},    {QT_A10, 1, BJ1D},  {QT_A20, 1, BJ0D},
    {QT_A00, 1, BJ0D}, {QT_B2, 1, BJ2D},   {QT_A20, 0, BJ2},   {QT_B2, 1, BJ1D},   {QT_A10, 0, BJ1},
    {QT_A21, 1, BJ2},  {QT_A11, 1, BJ1},   {QT_A01, 1, BJ0},   {QT_A21, 1, BJ0},   {QT_A20, 2, BJ2DD},
    {QT_B1, 1, BJ1D},  {QT_A10, 2, BJ1DD}, {QT_A20, 2, BJ0DD}, {QT_A00, 2, BJ0DD}, {QT_B2, 2, BJ2DD},
    {QT_B2, 2, BJ1DD}, {QT_A21, 2, BJ2D},  {QT_A11, 2, BJ1D},  {QT_A01, 2, BJ0D},  {QT_A21, 2, BJ0D},
    // 25..38: z-derivative coefficients
    {QTT + QT_B2, 0, BJ2},   {QTT + QT_A20, 1, BJ2D}, {QTT + QT_B1, 0, BJ1},  {QTT + QT_A10, 1, BJ1D},
    {QTT + QT_A20, 1, BJ0D}, {QTT + QT_A00, 1, BJ0D}, {QTT + QT_B2, 1, BJ2D}, {QTT + QT_A20, 0, BJ2},
    {QTT + QT_B1, 1, BJ1D},  {QTT + QT_A10, 0, BJ1},  {QTT + QT_A21, 1, BJ2}, {QTT + QT_A11, 1, BJ1},
    {QTT + QT_A01, 1, BJ0},  {QTT + QT_A21, 1, BJ0},
    // 39: b1 k^2 J1''
    {QT_B1, 2, BJ1DD},
};
constexpr int kTensorFixNP = sizeof(kTensorFixPairs) / sizeof(Pair);
constexpr __device__ Term kTensorFixTerms[] = {
    {0, 1, 2.0}, {1, 0, 1.0},                    // 0
    {2, 1, 1.0}, {3, 0, 1.0},                    // 1
    {4, 0, 1.0},                                 // 2
    {5, 0, 1.0},                                 // 3
    {6, 0, 1.0}, {7, 1, 2.0},                    // 4
    {15, 0, 1.0}, {9, 1, 1.0},                   // 5
    {10, 0, 1.0},                                // 6
    {11, 0, 1.0},                                // 7
    {12, 0, 1.0},                                // 8
    {13, 0, 1.0},                                // 9
    {25, 1, 2.0}, {26, 0, 1.0},                  // 10: d/dz
    {27, 1, 1.0}, {28, 0, 1.0},                  // 11
    {29, 0, 1.0},                                // 12
    {30, 0, 1.0},                                // 13
    {31, 0, 1.0}, {32, 1, 2.0},                  // 14
    {33, 0, 1.0}, {34, 1, 1.0},                  // 15
    {35, 0, 1.0},                                // 16
    {36, 0, 1.0},                                // 17
    {37, 0, 1.0},                                // 18
    {38, 0, 1.0},                                // 19
    {0, 2, -2.0}, {6, 1, 2.0}, {14, 0, 1.0},     // 20: d/dr
    {2, 2, -1.0}, {15, 1, 1.0}, {16, 0, 1.0},    // 21
    {17, 0, 1.0},                                // 22
    {18, 0, 1.0},                                // 23
    {19, 0, 1.0}, {7, 2, -2.0}, {1, 1, 2.0},     // 24
    {39, 0, 1.0}, {9, 2, -1.0}, {3, 1, 1.0},     // 25
    {21, 0, 1.0},                                // 26
    {22, 0, 1.0},                                // 27
    {23, 0, 1.0},                                // 28
    {24, 0, 1.0},                                // 29
};
constexpr __device__ int kTensorFixCol[31] = {0,  2,  4,  5,  6,  8,  10, 11, 12, 13, 14, 16, 18, 19, 20, 22,
                                              24, 25, 26, 27, 28, 31, 34, 35, 36, 39, 42, 43, 44, 45, 46};
constexpr int kTensorFixNC = 30;

// corrected moment tensor in the 20-column layout of the tensor-core sum:
// displacement 0-9 and d/dr 10-19 as in the 30-column corrected layout (its
// columns 0-9 and 20-29) -- the m = 0 radial columns 2, 3 (d/dr 12, 13) with
// the radial coefficients a20, a00 where green.cu:1652-1653 take a21, a01,
// the m = 1 transverse column 5 (d/dr 15) with b1 where green.cu:1657, 1686
// have b2 -- without the d/dz block the reference overwrites
constexpr __device__ Pair kTensorFix20Pairs[] = {
    {QT_B2, 0, BJ2},   {QT_A20, 1, BJ2D},  {QT_B1, 0, BJ1},    {QT_A10, 1, BJ1D},  {QT_A20, 1, BJ0D},
    {QT_A00, 1, BJ0D}, {QT_B2, 1, BJ2D},   {QT_A20, 0, BJ2},   {QT_B1, 2, BJ1DD},  {QT_A10, 0, BJ1},
    {QT_A21, 1, BJ2},  {QT_A11, 1, BJ1},   {QT_A01, 1, BJ0},   {QT_A21, 1, BJ0},   {QT_A20, 2, BJ2DD},
    {QT_B1, 1, BJ1D},  {QT_A10, 2, BJ1DD}, {QT_A20, 2, BJ0DD}, {QT_A00, 2, BJ0DD}, {QT_B2, 2, BJ2DD},
    {QT_A21, 2, BJ2D}, {QT_A11, 2, BJ1D},  {QT_A01, 2, BJ0D},  {QT_A21, 2, BJ0D},
};
constexpr int kTensorFix20NP = sizeof(kTensorFix20Pairs) / sizeof(Pair);
constexpr __device__ Term kTensorFix20Terms[] = {
    {0, 1, 2.0}, {1, 0, 1.0},                    // 0
    {2, 1, 1.0}, {3, 0, 1.0},                    // 1
    {4, 0, 1.0},                                 // 2
    {5, 0, 1.0},                                 // 3
    {6, 0, 1.0}, {7, 1, 2.0},                    // 4
    {15, 0, 1.0}, {9, 1, 1.0},                   // 5
    {10, 0, 1.0},                                // 6
    {11, 0, 1.0},                                // 7
    {12, 0, 1.0},                                // 8
    {13, 0, 1.0},                                // 9
    {0, 2, -2.0}, {6, 1, 2.0}, {14, 0, 1.0},     // 10: d/dr
    {2, 2, -1.0}, {15, 1, 1.0}, {16, 0, 1.0},    // 11
    {17, 0, 1.0},                                // 12
    {18, 0, 1.0},                                // 13
    {19, 0, 1.0}, {7, 2, -2.0}, {1, 1, 2.0},     // 14
    {8, 0, 1.0}, {9, 2, -1.0}, {3, 1, 1.0},      // 15
    {20, 0, 1.0},                                // 16
    {21, 0, 1.0},                                // 17
    {22, 0, 1.0},                                // 18
    {23, 0, 1.0},                                // 19
};
constexpr __device__ int kTensorFix20Col[21] = {0, 2, 4, 5, 6, 8, 10, 11, 12, 13, 14, 17, 20, 21, 22, 25, 28, 29, 30, 31, 32};

template <int SRC> struct Cols;
template <> struct Cols<kSingle> {
    static constexpr int NP = kSingleNP, NC = kSingleNC, NQ = QS_N, NT = sizeof(kSingleTerms) / sizeof(Term);
    __device__ static constexpr Pair pair(int i) { return kSinglePairs[i]; }
    __device__ static constexpr Term term(int i) { return kSingleTerms[i]; }
    __device__ static constexpr int col(int i) { return kSingleCol[i]; }
};
template <> struct Cols<kTensor> {
    static constexpr int NP = kTensorNP, NC = kTensorNC, NQ = QT_N, NT = sizeof(kTensorTerms) / sizeof(Term);
    __device__ static constexpr Pair pair(int i) { return kTensorPairs[i]; }
    __device__ static constexpr Term term(int i) { return kTensorTerms[i]; }
    __device__ static constexpr int col(int i) { return kTensorCol[i]; }
};
template <> struct Cols<kColSingleFix> {
    static constexpr int NP = kSingleNP, NC = kSingleNC, NQ = QS_N, NT = sizeof(kSingleFixTerms) / sizeof(Term);
    __device__ static constexpr Pair pair(int i) { return kSinglePairs[i]; }
    __device__ static constexpr Term term(int i) { return kSingleFixTerms[i]; }
    __device__ static constexpr int col(int i) { return kSingleCol[i]; }
};
template <> struct Cols<kColTensorFix20> {
    static constexpr int NP = kTensorFix20NP, NC = kTensorNC, NQ = QT_N, NT = sizeof(kTensorFix20Terms) / sizeof(Term);
    __device__ static constexpr Pair pair(int i) { return kTensorFix20Pairs[i]; }
    __device__ static constexpr Term term(int i) { return kTensorFix20Terms[i]; }
    __device__ static constexpr int col(int i) { return kTensorFix20Col[i]; }
};
template <> struct Cols<kColTensorFix> {
    static constexpr int NP = kTensorFixNP, NC = kTensorFixNC, NQ = 2 * QT_N, NT = sizeof(kTensorFixTerms) / sizeof(Term);
    __device__ static constexpr Pair pair(int i) { return kTensorFixPairs[i]; }
    __device__ static constexpr Term term(int i) { return kTensorFixTerms[i]; }
    __device__ static constexpr int col(int i) { return kTensorFixCol[i]; }
};

// ---------------------------------------------------------------- tensor-core plan
// How the tensor-core wavenumber sum divides a column layout: the coefficient
// columns q that feed some pair (the others are neither stored for it nor
// read), dealt into two groups of about equal pair counts, largest first (one
// CTA per group: the accumulators of half of the pairs for 32 receivers fit
// in tensor memory), and the operand tiles of a stage block ordered group by
// group, q by q, so that a group's tiles are one contiguous copy.
struct TcPlan {
    int nqu;                    // coefficient columns stored for the tensor cores
    int qslot[16];              // operand tile of column q in a stage block (-1: not stored)
    int gq0[2], gnq[2];         // first tile and number of tiles of each group
    int gnp[2];                 // pairs of each group
    int gpair[2][32];           // group-local slot -> pair (slots in tile order)
    int pslot[40], pgrp[40];    // pair -> group-local slot, group
    int tfirst[16], tcount[16]; // per tile: first group-local slot and number of its pairs
};

#pragma nv_diagnostic push
#pragma nv_diag_suppress 20091
template <int SRC>
__host__ __device__ constexpr TcPlan make_tcplan()
{
    static_assert(SRC == kColSingle || SRC == kColTensor || SRC == kColSingleFix || SRC == kColTensorFix20,
                  "tensor-core layouts only");
    constexpr int NQ = Cols<SRC>::NQ, NP = Cols<SRC>::NP;
    auto pair_q = [](int p) { return Cols<SRC>::pair(p).q; };
    TcPlan t{};
    int cnt[16] = {}, grp[16] = {};
    for (int q = 0; q < 16; q++) {
        grp[q] = -1;
        t.qslot[q] = -1;
    }
    for (int p = 0; p < NP; p++) cnt[pair_q(p)]++;
    int load[2] = {0, 0};
    for (int it = 0; it < NQ; it++) {
        int best = -1;
        for (int q = 0; q < NQ; q++)
            if (grp[q] < 0 && cnt[q] > 0 && (best < 0 || cnt[q] > cnt[best])) best = q;
        if (best < 0) break;
        const int g = load[1] < load[0] ? 1 : 0;
        grp[best] = g;
        load[g] += cnt[best];
    }
    int pos = 0;
    for (int g = 0; g < 2; g++) {
        t.gq0[g] = pos;
        for (int q = 0; q < NQ; q++) {
            if (grp[q] != g) continue;
            t.qslot[q] = pos;
            t.tfirst[pos] = t.gnp[g];
            t.tcount[pos] = cnt[q];
            for (int p = 0; p < NP; p++)
                if (pair_q(p) == q) {
                    t.gpair[g][t.gnp[g]] = p;
                    t.pslot[p] = t.gnp[g];
                    t.pgrp[p] = g;
                    t.gnp[g]++;
                }
            pos++;
            t.gnq[g]++;
        }
    }
    t.nqu = pos;
    return t;
}
#pragma nv_diagnostic pop

// error-free sum s + x = hi + lo (Knuth TwoSum)
template <typename R> __device__ __forceinline__ void two_sum_acc(R &hi, R &lo, R x)
{
    R s = hi + x;
    R bp = s - hi;
    R e = (hi - (s - bp)) + (x - bp);
    hi = s;
    lo += e;
}

constexpr int kSumThreads = 128;
constexpr int kSumChunk = 16;   // k-steps accumulated plainly before a compensated fold

template <typename R>
struct KsumArgs {
    const R *K;            // [nq][nkw] complex
    const R *B;            // [nbrow][NBASIS][nr], row i at k = i dk
    const int *nk;         // [nw]
    const int *ks;         // [nw] k stride m: frequency iw sums k_j = j m dk (null: 1)
    const long long *koff; // [nw]
    const double *dist;    // [nr]
    R *S;                  // [nr][nc][nw] complex
    long long nkw;
    double dk;
    int nw, nr, rt, jt;    // receivers per block, k-lanes per receiver (rt * jt = 128)
};

// One thread per (w, receiver, k-lane); k-lanes of a receiver reduce at the end.
// Each thread accumulates the output columns directly:
//   col_c += (coef_t r^-rpow_t) (w_k k^kp_t J_bt(k r)) K_qt(w, k)
// over the terms t of column c.  coef_t and rpow_t are compile-time constants
// of the column tables, so a thread holds 1/r and 1/r^2 and its 2 NC
// accumulators; k-chunks are summed plainly and folded with TwoSum.
template <typename R, int SRC>
__global__ void __launch_bounds__(kSumThreads) ksum_kernel(KsumArgs<R> A)
{
    using CT = Cols<SRC>;
    constexpr int NC = CT::NC, NQ = CT::NQ;
    __shared__ R red[kSumThreads * 2];
    const int ntile = (A.nr + A.rt - 1) / A.rt;
    const int iw = blockIdx.x / ntile;
    const int r0 = (blockIdx.x % ntile) * A.rt;
    const int rloc = threadIdx.x % A.rt, lane = threadIdx.x / A.rt;
    const int r = r0 + rloc;
    const bool rvalid = r < A.nr;
    const int rr = rvalid ? r : 0;
    const int nk = A.nk[iw];
    const long long off = A.koff[iw];
    const C<R> *K = reinterpret_cast<const C<R> *>(A.K) + off;
    const double drr = A.dist[rr];
    const R ir = (R)(1.0 / drr), ir2 = (R)(1.0 / (drr * drr));

    R hi[NC][2], lo[NC][2];
#pragma unroll
    for (int c = 0; c < NC; c++) hi[c][0] = hi[c][1] = lo[c][0] = lo[c][1] = R(0);
    const int m = A.ks ? A.ks[iw] : 1;
    const R dk = (R)(A.dk * m), dk_half = (R)(0.5 * A.dk * m);

    for (int jb = lane * kSumChunk; jb < nk; jb += A.jt * kSumChunk) {
        R acc[NC][2];
#pragma unroll
        for (int c = 0; c < NC; c++) acc[c][0] = acc[c][1] = R(0);
        const int je = min(jb + kSumChunk, nk);
        for (int j = jb; j < je; j++) {
            // k^p weights only scale the coefficients: working precision suffices
            const R k = dk * (R)j;
            const R w = (j == 0) ? dk_half : dk;
            const R wk[3] = {w, w * k, w * k * k};
            const R *Bj = A.B + (long long)j * m * NBASIS * A.nr + rr;
            R bv[NBASIS];
#pragma unroll
            for (int b = 0; b < NBASIS; b++) bv[b] = Bj[(long long)b * A.nr];
            C<R> kq[NQ];
#pragma unroll
            for (int q = 0; q < NQ; q++) kq[q] = K[(long long)q * A.nkw + j];
#pragma unroll
            for (int c = 0; c < NC; c++) {
#pragma unroll
                for (int t = CT::col(c); t < CT::col(c + 1); t++) {
                    const Term T = CT::term(t);
                    const Pair P = CT::pair(T.pair);
                    R f = wk[P.kp] * bv[P.b];
                    if (T.rpow == 1) f *= ir;
                    else if (T.rpow == 2) f *= ir2;
                    f *= (R)T.coef;
                    acc[c][0] += kq[P.q].x * f;
                    acc[c][1] += kq[P.q].y * f;
                }
            }
        }
#pragma unroll
        for (int c = 0; c < NC; c++) {
            two_sum_acc(hi[c][0], lo[c][0], acc[c][0]);
            two_sum_acc(hi[c][1], lo[c][1], acc[c][1]);
        }
    }
    // reduce the k-lanes of each receiver, column by column
    C<R> *S = reinterpret_cast<C<R> *>(A.S);
#pragma unroll
    for (int c = 0; c < NC; c++) {
        R v0 = hi[c][0] + lo[c][0], v1 = hi[c][1] + lo[c][1];
        if (A.jt > 1) {
            __syncthreads();
            red[2 * threadIdx.x] = v0;
            red[2 * threadIdx.x + 1] = v1;
            __syncthreads();
            if (lane == 0) {
                R s0 = 0, s1 = 0, c0 = 0, c1 = 0;
                for (int l = 0; l < A.jt; l++) {
                    two_sum_acc(s0, c0, red[2 * (l * A.rt + rloc)]);
                    two_sum_acc(s1, c1, red[2 * (l * A.rt + rloc) + 1]);
                }
                v0 = s0 + c0;
                v1 = s1 + c1;
            }
        }
        if (lane == 0 && rvalid) S[((long long)r * NC + c) * A.nw + iw] = C<R>{v0, v1};
    }
}

// ---------------------------------------------------------------- error estimate
// Terms of a column layout flattened for host code: term t adds
// coef[t] r^-rpow[t] w_k k^kp[t] J_b[t](k r) K_q[t](w, k) to column c for
// col[c] <= t < col[c + 1].
struct ColTerms {
    int nc, nt, np;
    int col[32], q[48], kp[48], b[48], rpow[48], pair[48];
    double coef[48];
    int pq[48], pkp[48], pb[48];   // pair p = (coefficient column, power of k, Bessel function)
};
#pragma nv_diagnostic push
#pragma nv_diag_suppress 20091
template <int SRC> __host__ __device__ constexpr ColTerms make_colterms()
{
    ColTerms o{};
    o.nc = Cols<SRC>::NC;
    o.nt = Cols<SRC>::NT;
    for (int c = 0; c <= o.nc; c++) o.col[c] = Cols<SRC>::col(c);
    for (int t = 0; t < o.nt; t++) {
        const Term T = Cols<SRC>::term(t);
        const Pair P = Cols<SRC>::pair(T.pair);
        o.q[t] = P.q;
        o.kp[t] = P.kp;
        o.b[t] = P.b;
        o.rpow[t] = T.rpow;
        o.coef[t] = T.coef;
        o.pair[t] = T.pair;
    }
    o.np = Cols<SRC>::NP;
    for (int i = 0; i < o.np; i++) {
        const Pair P = Cols<SRC>::pair(i);
        o.pq[i] = P.q;
        o.pkp[i] = P.kp;
        o.pb[i] = P.b;
    }
    return o;
}
#pragma nv_diagnostic pop

// Noise-floor estimate of the wavenumber sums (the judge of the FP32 path).
// With relative rounding noise eps on every coefficient K_q(w, k),
// independent from one wavenumber to the next, a column's k-sum at distance r
// has the variance eps^2 sum_t coef_t^2 r^-2rpow_t sum_k w_k^2 k^2kp_t
// |K_q_t(w, k)|^2 J_b_t(k r)^2; J^2 is replaced by its mean 1 / (1 + pi k r).
// This kernel forms, per frequency, class c = (q, kp) and distance band b,
//   H[iw][c][b] = sum_k w_k^2 k^(2 kp_c) |K_qc(w, k)|^2 / (1 + pi k r_b),
// reading the coefficients from the flat columns or from the tensor-core
// operand tiles (hi + lo words).  One block per (frequency, class).
constexpr int kNoiseBands = 16;
constexpr int kNoiseThreads = 128;
template <typename R>
struct NoiseArgs {
    const R *K;              // [nq][nkw] complex, or null
    const float *Kt;         // tensor-core operand tiles (FP32 plans), or null
    const long long *kt_base;
    int nqt, kt_bf16;        // tiles per stage block; the 3xBF16 form
    int qslot[16];           // tile of coefficient column q (tensor-core layout)
    const int *nk, *ks;
    const long long *koff;
    long long nkw;
    double dk;
    int nw, ncls;
    int cls_q[32], cls_p[32];
    float rb[kNoiseBands];   // band distances, km
    float *H;                // [nw][ncls][kNoiseBands]
};

// coefficient K_q(w_iw, k_j) read back from the tensor-core operand tiles (hi + lo)
template <typename R>
__device__ __forceinline__ void tile_coef(const NoiseArgs<R> &A, int iw, int q, int j, float &re, float &im)
{
    const int wl = iw % (kTileRows / 2), tk = A.kt_bf16 ? kTileK16 : kTileK;
    const float *t = A.Kt + A.kt_base[iw / (kTileRows / 2)] +
                     ((long long)(j / tk) * A.nqt + A.qslot[q]) * 2 * (kTileRows * kTileK);
    if (A.kt_bf16) {
        const unsigned short *u = reinterpret_cast<const unsigned short *>(t);
        const unsigned ore = kt_tile_off16(wl, j % tk) / 2, oim = kt_tile_off16(kTileRows / 2 + wl, j % tk) / 2;
        re = bf16_val(u[ore]) + bf16_val(u[2 * kTileRows * kTileK + ore]);
        im = bf16_val(u[oim]) + bf16_val(u[2 * kTileRows * kTileK + oim]);
        return;
    }
    const unsigned ore = kt_tile_off(wl, j % tk) / 4, oim = kt_tile_off(kTileRows / 2 + wl, j % tk) / 4;
    re = t[ore] + t[kTileRows * kTileK + ore];
    im = t[oim] + t[kTileRows * kTileK + oim];
}

template <typename R>
__global__ void __launch_bounds__(kNoiseThreads) noise_kernel(NoiseArgs<R> A)
{
    __shared__ float red[kNoiseThreads][kNoiseBands + 1];
    const int iw = blockIdx.x / A.ncls, c = blockIdx.x % A.ncls;
    const int q = A.cls_q[c], kp = A.cls_p[c];
    const int nk = A.nk[iw], m = A.ks ? A.ks[iw] : 1;
    const double dkm = A.dk * m;
    float acc[kNoiseBands];
#pragma unroll
    for (int b = 0; b < kNoiseBands; b++) acc[b] = 0.f;
    for (int j = threadIdx.x; j < nk; j += blockDim.x) {
        float re, im;
        if (A.Kt) {
            tile_coef(A, iw, q, j, re, im);
        } else {
            const C<R> v = reinterpret_cast<const C<R> *>(A.K)[(long long)q * A.nkw + A.koff[iw] + j];
            re = (float)v.x;
            im = (float)v.y;
        }
        const float k = (float)(dkm * j), w = (float)(j == 0 ? 0.5 * dkm : dkm);
        float a = w * w * (re * re + im * im);
        for (int e = 0; e < kp; e++) a *= k * k;
#pragma unroll
        for (int b = 0; b < kNoiseBands; b++) acc[b] += a / (1.f + 3.14159265f * k * A.rb[b]);
    }
#pragma unroll
    for (int b = 0; b < kNoiseBands; b++) red[threadIdx.x][b] = acc[b];
    __syncthreads();
    if (threadIdx.x < kNoiseBands) {
        float s = 0.f;
        for (int t = 0; t < (int)blockDim.x; t++) s += red[t][threadIdx.x];
        A.H[((long long)iw * A.ncls + c) * kNoiseBands + threadIdx.x] = s;
    }
}

// The coefficients' actual FP32 noise at a few spot frequencies, against an
// FP64 evaluation of the same (w, k) points: per spot frequency s, class c and
// distance band b,
//   num[s][c][b] = sum_k w_k^2 k^(2 kp) |K32_q - K64_q|^2 / (1 + pi k r_b),
//   den[s][c][b] = sum_k w_k^2 k^(2 kp) |K64_q|^2 / (1 + pi k r_b),
// weighted as the wavenumber sum at band distance r_b weights them (the
// relative error of the coefficients varies with k, and a far receiver
// weighs the small wavenumbers more).  K64: flat [nq][nkw64] complex of a
// spectra-only FP64 plan over the spot frequencies (koff64).
template <typename R>
__global__ void __launch_bounds__(kNoiseThreads) spot_noise_kernel(NoiseArgs<R> A, const double *K64,
                                                                   const long long *koff64, long long nkw64,
                                                                   const int *rows, double *out)
{
    __shared__ float red[kNoiseThreads][2 * kNoiseBands + 1];
    const int s = blockIdx.x / A.ncls, c = blockIdx.x % A.ncls;
    const int iw = rows[s], q = A.cls_q[c], kp = A.cls_p[c];
    const int nk = A.nk[iw], m = A.ks ? A.ks[iw] : 1;
    const double dkm = A.dk * m;
    float num[kNoiseBands], den[kNoiseBands];
#pragma unroll
    for (int b = 0; b < kNoiseBands; b++) num[b] = den[b] = 0.f;
    for (int j = threadIdx.x; j < nk; j += blockDim.x) {
        double re, im;
        if (A.Kt) {
            float fr, fi;
            tile_coef(A, iw, q, j, fr, fi);
            re = fr;
            im = fi;
        } else {
            const C<R> v = reinterpret_cast<const C<R> *>(A.K)[(long long)q * A.nkw + A.koff[iw] + j];
            re = (double)v.x;
            im = (double)v.y;
        }
        const C<double> v64 = reinterpret_cast<const C<double> *>(K64)[(long long)q * nkw64 + koff64[s] + j];
        const double k = dkm * j, w = (j == 0 ? 0.5 * dkm : dkm);
        double f = w * w;
        for (int e = 0; e < kp; e++) f *= k * k;
        const float dn = (float)(f * ((re - v64.x) * (re - v64.x) + (im - v64.y) * (im - v64.y)));
        const float dd = (float)(f * (v64.x * v64.x + v64.y * v64.y));
#pragma unroll
        for (int b = 0; b < kNoiseBands; b++) {
            const float wr = 1.f / (1.f + 3.14159265f * (float)k * A.rb[b]);
            num[b] += dn * wr;
            den[b] += dd * wr;
        }
    }
#pragma unroll
    for (int b = 0; b < kNoiseBands; b++) {
        red[threadIdx.x][b] = num[b];
        red[threadIdx.x][kNoiseBands + b] = den[b];
    }
    __syncthreads();
    if (threadIdx.x < 2 * kNoiseBands) {
        double t = 0.0;
        for (int i = 0; i < (int)blockDim.x; i++) t += red[i][threadIdx.x];
        out[(long long)blockIdx.x * 2 * kNoiseBands + threadIdx.x] = t;   // [s][c][num b..., den b...]
    }
}

// sum of squares of each receiver's traces [nr][nc][N] (one block per receiver)
template <typename R>
__global__ void trace_norm_kernel(const R *sig, long long per_rcv, double *out)
{
    __shared__ double red[256];
    const R *x = sig + blockIdx.x * per_rcv;
    double s = 0.0;
    for (long long i = threadIdx.x; i < per_rcv; i += blockDim.x) s += (double)x[i] * (double)x[i];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int h = blockDim.x / 2; h > 0; h >>= 1) {
        if ((int)threadIdx.x < h) red[threadIdx.x] += red[threadIdx.x + h];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[blockIdx.x] = red[0];
}

// ---------------------------------------------------------------- plain sum as GEMMs
// The plain FP32 wavenumber sum written as real matrix products, one per
// pair p = (q, kp, b) of the integrand tables (green.cu:1582-1600 /
// 1650-1691):
//   D_p[part][w][r] = sum_k A_q[part][w][k] Bc_(kp,b)[k][r],
//   A_q = Re / Im K_q(w, k) (planar rows), Bc = w_k k^kp J_b(k r),
// then S_c(w, r) = sum_(t in c) coef_t r^-rpow_t D_p(t)(w, r).  The products
// run as cuBLAS SGEMM in FP32 (a plain library GEMM), k split in slices whose
// partial products the combination adds with TwoSum.
// A[q][part][w][j], zero beyond the frequency's nk (grid-stride, j fastest)
static __global__ void gemm_a_kernel(const float *K, const int *nk, const long long *koff, long long nkw, int nw, int nkp,
                              int nq, float *A)
{
    const long long n = (long long)nq * nw * nkp;
    const float2 *Kc = reinterpret_cast<const float2 *>(K);
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        const int j = (int)(e % nkp);
        const long long qw = e / nkp;
        const int iw = (int)(qw % nw), q = (int)(qw / nw);
        float2 v = make_float2(0.f, 0.f);
        if (j < nk[iw]) v = Kc[(long long)q * nkw + koff[iw] + j];
        A[(((long long)q * 2) * nw + iw) * nkp + j] = v.x;
        A[(((long long)q * 2 + 1) * nw + iw) * nkp + j] = v.y;
    }
}

// Bc[j][r] = w_j k_j^kp J_b(k_j r) from the Bessel table B[j][b][r] (zero beyond its rows)
static __global__ void gemm_b_kernel(const float *B, int nbrow, int nr, int nkp, double dk, int kp, int b, float *Bc)
{
    const long long n = (long long)nkp * nr;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        const int r = (int)(e % nr), j = (int)(e / nr);
        float v = 0.f;
        if (j < nbrow) {
            const double k = dk * j;
            double f = (j == 0) ? 0.5 * dk : dk;
            for (int i = 0; i < kp; i++) f *= k;
            v = (float)f * B[((long long)j * NBASIS + b) * nr + r];
        }
        Bc[e] = v;
    }
}

// S[r][c][w] = sum over the column's terms and the k slices of
// coef_t r^-rpow_t D[s][p_t][part][w][r], with TwoSum; one thread per (w, r)
template <int SRC>
__global__ void gemm_combine_kernel(const float *D, int ns, int nw, int nr, const double *dist, float *S)
{
    using CT = Cols<SRC>;
    const long long n = (long long)nw * nr;
    const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (e >= n) return;
    const int r = (int)(e % nr), w = (int)(e / nr);
    const double dr = dist[r];
    const float ir = (float)(1.0 / dr), ir2 = (float)(1.0 / (dr * dr));
    const long long pstride = 2LL * nw * nr, sstride = (long long)CT::NP * pstride;
    C<float> *So = reinterpret_cast<C<float> *>(S);
#pragma unroll 1
    for (int c = 0; c < CT::NC; c++) {
        float hr = 0.f, lr = 0.f, hi = 0.f, li = 0.f;
        for (int t = CT::col(c); t < CT::col(c + 1); t++) {
            const Term T = CT::term(t);
            const float f = (float)T.coef * (T.rpow == 1 ? ir : T.rpow == 2 ? ir2 : 1.f);
            const float *Dp = D + T.pair * pstride + (long long)w * nr + r;
            for (int s = 0; s < ns; s++) {
                two_sum_acc(hr, lr, f * Dp[s * sstride]);
                two_sum_acc(hi, li, f * Dp[s * sstride + (long long)nw * nr]);
            }
        }
        So[((long long)r * CT::NC + c) * nw + w] = C<float>{hr + lr, hi + li};
    }
}

// ---------------------------------------------------------------- spectral stage
template <typename R>
struct SpecArgs {
    const R *S;            // [ntr][nw] complex  (ntr = nr * nc traces)
    const R *post;         // [nw] complex: e^{i w t0} * taper * df nw / pi
    const R *tw;           // [N/2] complex: e^{+2 pi i m / N}
    const double *damp;    // [N]: e^{sigma (n dt + t0)} / N
    R *spec_out;           // [ntr][N] complex or null
    R *sig_out;            // [ntr][N] or null (working precision)
    int nw, logn;
};

// In-place radix-2 decimation-in-time inverse DFT (exp(+2 pi i) kernel) of
// the bit-reversed spectrum in x (the block's shared memory).  Three
// consecutive stages run fused: a thread takes the 8 elements
// base + m half (m = 0..7) of one group through stages s, s+1, s+2 in
// registers -- the same butterflies and twiddles as three separate stages
// (pairs (m, m+1), then (m, m+2) for m = 0, 1, 4, 5, then (m, m+4)), so one
// barrier per three stages; the remaining one or two stages run unfused.
template <typename R>
__device__ __forceinline__ void ifft_inplace(C<R> *x, const C<R> *tw, int logn)
{
    const int N = 1 << logn;
    int s = 1;
    for (; s + 2 <= logn; s += 3) {
        const int half = 1 << (s - 1);
        for (int t = threadIdx.x; t < N / 8; t += blockDim.x) {
            const int pos = t & (half - 1), base = (t >> (s - 1)) * 8 * half + pos;
            C<R> v[8];
#pragma unroll
            for (int m = 0; m < 8; m++) v[m] = x[base + m * half];
            {
                const C<R> w = tw[pos * (N >> s)];
#pragma unroll
                for (int m = 0; m < 8; m += 2) {
                    const C<R> u = v[m], q = v[m + 1] * w;
                    v[m] = u + q;
                    v[m + 1] = u - q;
                }
            }
#pragma unroll
            for (int i = 0; i < 4; i++) {
                const int m = (i & 1) + (i >> 1) * 4;   // 0, 1, 4, 5
                const C<R> w = tw[(pos + (m & 1) * half) * (N >> (s + 1))];
                const C<R> u = v[m], q = v[m + 2] * w;
                v[m] = u + q;
                v[m + 2] = u - q;
            }
#pragma unroll
            for (int m = 0; m < 4; m++) {
                const C<R> w = tw[(pos + m * half) * (N >> (s + 2))];
                const C<R> u = v[m], q = v[m + 4] * w;
                v[m] = u + q;
                v[m + 4] = u - q;
            }
#pragma unroll
            for (int m = 0; m < 8; m++) x[base + m * half] = v[m];
        }
        __syncthreads();
    }
    for (; s <= logn; s++) {
        const int half = 1 << (s - 1);
        const int tstride = N >> s;
        for (int b = threadIdx.x; b < N / 2; b += blockDim.x) {
            const int grp = b >> (s - 1), pos = b & (half - 1);
            const int i0 = grp * (half << 1) + pos, i1 = i0 + half;
            const C<R> w = tw[pos * tstride];
            const C<R> u = x[i0], v = x[i1] * w;
            x[i0] = u + v;
            x[i1] = u - v;
        }
        __syncthreads();
    }
}

// the inverse DFT above, then Re(x) e^{sigma t} / N into out
template <typename R>
__device__ __forceinline__ void ifft_dedamp(C<R> *x, const C<R> *tw, const double *damp, int logn, R *out)
{
    ifft_inplace(x, tw, logn);
    const int N = 1 << logn;
    if (out)
        for (int n = threadIdx.x; n < N; n += blockDim.x) out[n] = (R)((double)x[n].x * damp[n]);
}

// Seismograms: per (receiver, component) block, the Green's-function columns'
// spectra combined with real weights W[trace][col] (azimuth and moment
// tensor), times the source-time spectrum stf[w] (null: impulse), then the
// same phase/taper/scale, Hermitian fill, inverse DFT and de-damping as the
// spectral stage.
template <typename R>
struct SynthArgs {
    const R *S;            // [nr][nc][nw] complex wavenumber sums
    const R *W;            // [nr * nout][nc] combination weights
    const R *stf;          // [nw] complex source-time spectrum, or null
    const R *post, *tw;
    const double *damp;
    R *out;                // [nr * nout][N]
    int nw, logn, nc, nout;
};

template <typename R>
__global__ void __launch_bounds__(512) synth_kernel(SynthArgs<R> A)
{
    extern __shared__ __align__(16) unsigned char smem_syn[];
    C<R> *x = reinterpret_cast<C<R> *>(smem_syn);
    const int N = 1 << A.logn, nw = A.nw;
    const long long tr = blockIdx.x;
    const long long r = tr / A.nout;
    const C<R> *S = reinterpret_cast<const C<R> *>(A.S) + r * A.nc * nw;
    const R *W = A.W + tr * A.nc;
    const C<R> *post = reinterpret_cast<const C<R> *>(A.post);
    const C<R> *stf = reinterpret_cast<const C<R> *>(A.stf);
    for (int n = threadIdx.x; n <= nw; n += blockDim.x) {
        C<R> y = {R(0), R(0)};
        if (n < nw) {
            for (int c = 0; c < A.nc; c++) {
                const R wc = W[c];
                if (wc != R(0)) y = y + S[(long long)c * nw + n] * wc;
            }
            y = y * post[n];
            if (stf) y = y * stf[n];
        }
        x[__brev((unsigned)n) >> (32 - A.logn)] = y;                       // n = nw: 0 (Nyquist)
        if (n > 0 && n < nw) x[__brev((unsigned)(N - n)) >> (32 - A.logn)] = conj(y);
    }
    __syncthreads();
    ifft_dedamp(x, reinterpret_cast<const C<R> *>(A.tw), A.damp, A.logn, A.out + tr * N);
}

// Spectra-only plans (a frequency selection): Y[tr][row] = S[tr][row] post[row],
// the phase, taper and scale of the spectral stage without fill or transform.
template <typename R>
__global__ void select_kernel(const R *S, const R *post, R *out, long long n, int nw)
{
    const C<R> *s = reinterpret_cast<const C<R> *>(S), *q = reinterpret_cast<const C<R> *>(post);
    C<R> *y = reinterpret_cast<C<R> *>(out);
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x)
        y[e] = s[e] * q[e % nw];
}

// Spectra of every trace at nf chosen frequencies, gathered on the device
// (the fetch of a few frequencies without filling the full spectra):
// Y[f][tr] = S[tr][n] post[n] for n = idx[f] < nw, 0 at nw, conj(Y at N - n)
// above; with sel (a spectra-only plan) the already-scaled spec[tr][sel[f]].
template <typename R>
__global__ void gather_freqs_kernel(const R *S_, const R *post_, const R *spec_, const int *idx, const int *sel,
                                    long long ntr, int nw, int nf, R *out_)
{
    const C<R> *S = reinterpret_cast<const C<R> *>(S_), *post = reinterpret_cast<const C<R> *>(post_);
    const C<R> *spec = reinterpret_cast<const C<R> *>(spec_);
    C<R> *out = reinterpret_cast<C<R> *>(out_);
    const long long n_all = ntr * nf;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n_all;
         e += (long long)gridDim.x * blockDim.x) {
        const int f = (int)(e / ntr);
        const long long tr = e % ntr;
        C<R> y;
        if (sel) {
            y = spec[tr * nw + sel[f]];
        } else {
            const int n = idx[f], N = 2 * nw;
            if (n < nw) y = S[tr * nw + n] * post[n];
            else if (n == nw) y = C<R>{R(0), R(0)};
            else y = conj(S[tr * nw + N - n] * post[N - n]);
        }
        out[e] = y;
    }
}

// The full spectrum of every trace (the reference's `out` after taper and
// Hermitian fill), written only when a caller fetches spectra: Y[tr][n] =
// S[tr][n] post[n] for n < nw, 0 at nw, conj(Y[N - n]) above.
template <typename R>
__global__ void spec_fill_kernel(const R *S_, const R *post_, R *spec, long long ntr, int nw)
{
    const int N = 2 * nw;
    const C<R> *S = reinterpret_cast<const C<R> *>(S_), *post = reinterpret_cast<const C<R> *>(post_);
    C<R> *Y = reinterpret_cast<C<R> *>(spec);
    const long long n_all = ntr * N;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n_all;
         e += (long long)gridDim.x * blockDim.x) {
        const long long tr = e / N;
        const int n = (int)(e % N);
        C<R> y;
        if (n < nw) y = S[tr * nw + n] * post[n];
        else if (n == nw) y = C<R>{R(0), R(0)};
        else y = conj(S[tr * nw + N - n] * post[N - n]);
        Y[e] = y;
    }
}

template <typename R>
__global__ void __launch_bounds__(512) spectral_kernel(SpecArgs<R> A)
{
    extern __shared__ __align__(16) unsigned char smem_spec[];
    C<R> *x = reinterpret_cast<C<R> *>(smem_spec);
    const int N = 1 << A.logn, nw = A.nw;
    const long long tr = blockIdx.x;
    const C<R> *S = reinterpret_cast<const C<R> *>(A.S) + tr * nw;
    const C<R> *post = reinterpret_cast<const C<R> *>(A.post);
    const C<R> *tw = reinterpret_cast<const C<R> *>(A.tw);
    // full spectrum Y (reference's `out` after Hermitian fill), loaded bit-reversed
    for (int n = threadIdx.x; n < N; n += blockDim.x) {
        C<R> y;
        if (n < nw) y = S[n] * post[n];
        else if (n == nw) y = C<R>{R(0), R(0)};
        else y = conj(S[N - n] * post[N - n]);
        if (A.spec_out) reinterpret_cast<C<R> *>(A.spec_out)[tr * N + n] = y;
        unsigned rev = __brev((unsigned)n) >> (32 - A.logn);
        x[rev] = y;
    }
    __syncthreads();
    ifft_inplace(x, tw, A.logn);
    if (A.sig_out) {
        for (int n = threadIdx.x; n < N; n += blockDim.x)
            A.sig_out[tr * N + n] = (R)((double)x[n].x * A.damp[n]);
    }
}

}  // namespace grt
