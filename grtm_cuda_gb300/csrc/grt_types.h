// grt_types.h -- data layouts shared by the host driver and the kernels.
#pragma once
#include <stdint.h>

namespace grt {

constexpr int kMaxLayers = 256;     // after source-interface insertion
constexpr int kGrtThreads = 128;    // one (w,k) point per thread, 128 k per tile
constexpr int kNlevSlots = 64;      // counters of layers evaluated, spread to keep their atomics apart

// Per (frequency, layer) record, built on the host in FP64 once per
// frequency (the reference rebuilds these per (w,k): set_pars, green.cu:164-195).
// The FP64 squares feed the only FP64 step of the FP32 path: the real part
// of k^2 - (w/alpha)^2, where the vertical slowness branch is selected.
template <typename R>
struct alignas(16) LayerW {
    double wa2x, wa2y, wb2x, wb2y;  // (w/alpha)^2, (w/beta)^2
    R wa2[2], wb2[2];               // the same, rounded
    R W[2];                         // (w/beta)^2 - (w/alpha)^2  (= r^2 - v^2)
    R iW[2];                        // 1 / W
    R a[2], b[2];                   // attenuated velocities alpha(w), beta(w)
    R mu, h;                        // b0^2 rho, thickness (half-space: top depth)
    float wa2lo, wb2lo;             // Re(wa^2) - (float)Re(wa^2), same for wb^2 (double-float low words)
    float wa2ylo, wb2ylo, hlo;      // low words of Im(wa^2), Im(wb^2) and of the thickness
    float pad_;
};
static_assert(sizeof(LayerW<float>) % 16 == 0, "TMA bulk copies need 16-byte multiples");
static_assert(sizeof(LayerW<double>) % 16 == 0, "TMA bulk copies need 16-byte multiples");

// column sets of the per-(w,k) receiver coefficients written by the GRT kernel
enum SrcKind { kSingle = 0, kTensor = 1 };
// output column layouts: the reference's (bug-compatible) ones, and the
// corrected ones selected by GRT_FIX_COLS (single force: the d/dr column 10
// with its 1/r; moment tensor: 30 defined columns, d/dz in 10-19, d/dr in 20-29)
// kColTensorFix20: the moment tensor's corrected columns in the 20-column
// layout of the tensor-core sum (displacement 0-9 and d/dr 10-19, no d/dz)
enum ColKind { kColSingle = 0, kColTensor = 1, kColSingleFix = 2, kColTensorFix = 3, kColTensorFix20 = 4 };
// single force: b1, a0[0], a0[1], a1[0], a1[1] and their d/dz versions
enum QSingle { QS_B1 = 0, QS_A00, QS_A01, QS_A10, QS_A11, QS_B1T, QS_A0T0, QS_A0T1, QS_A1T0, QS_A1T1, QS_N };
// moment tensor: b1, b2, a0[0..1], a1[0..1], a2[0..1]
enum QTensor { QT_B1 = 0, QT_B2, QT_A00, QT_A01, QT_A10, QT_A11, QT_A20, QT_A21, QT_N };

// compiled forms of the per-(w,k) GRT evaluation (see grt_point)
enum GrtSpec { kSpecGeneric = 0, kSpecAboveTensor = 1 };

// reference-quirk switches (0 = reproduce the reference)
enum Fix { kFixRLayer = 1, kFixRexut = 2, kFixDz = 4, kFixCols = 8, kFixShsrc = 16, kFixCols20 = 32 };

template <typename R>
struct GrtArgs {
    const LayerW<R> *tab;      // [nw][L]
    const int2 *tiles;         // (iw, j0) per block
    const int *nk;             // [nw]
    const int *ks;             // [nw] k stride m: k_j = j m dk (null: 1)
    const long long *koff;     // [nw] offset of frequency iw in the flattened (w,k) list
    R *K;                      // [nq][nkw] complex (re, im)
    long long nkw;
    double dk;
    double zs, zr;
    double hs_layer, hr_layer; // thickness of source / receiver layer
    int L, s, rl, src, fix, nq;
    R slot0[4];                // nu_alpha, nu_beta of layer rl at (w = -i sigma, k = 0)
    unsigned int *err;         // device error word (bounded waits that gave up)
    unsigned long long *nlev;  // kNlevSlots counters of layers evaluated (depth truncation), or null
    // tensor-core layout of the coefficients (FP32 plans): when Kt is set the
    // kernel writes, instead of K, TF32 hi/lo words straight into the operand
    // tiles of the wavenumber GEMM: block (frequency tile of 64, k stage of 8)
    // at Kt + kt_base[tile] + stage * nqt * 2048 floats, inside it [tile][hi|lo]
    // K-major core-matrix tiles of 128 rows (re rows 0-63, im rows 64-127),
    // one tile per coefficient column the sum reads (make_tcplan)
    float *Kt;
    const long long *kt_base;
    int nqt;
    int kt_bf16;               // tiles in the 3xBF16 form (16 k per stage, bf16 hi/lo words)
    signed char qslot[16];     // tile of coefficient column q in a stage block (-1: not stored)
    // two-pass evaluation (specialised FP32 form): the bottom-up pass leaves
    // R^du and its SH term at the source here, [kRduPlanes][nkw], for the
    // pass that follows (null: one pass)
    R *rdu;
};
constexpr int kRduPlanes = 10;   // R^du (2 x 2 complex) and R^du_0 (complex)

// Bessel basis functions of k r, in the order the integrand formulas use them
enum Basis { BJ0 = 0, BJ1, BJ2, BJ0D, BJ1D, BJ2D, BJ0DD, BJ1DD, BJ2DD, NBASIS };

}  // namespace grt
