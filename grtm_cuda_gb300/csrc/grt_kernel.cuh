// grt_kernel.cuh -- the per-(w,k) generalized reflection/transmission kernel.
//
// One thread evaluates one (w,k) point for one layered model: interface
// coefficients, the bottom-up and top-down generalized R/T recursions, the
// source terms and the receiver coefficients, and writes the receiver
// coefficients (b1, a0, a1, ... of get_ypars_a_single / _tensor,
// green.cu:615-1267) for the wavenumber integration.
//
// The reference materialises every stage in HBM (about 2.6 KB per
// (w,k,layer)) and solves each interface with batched cuBLAS 4x4 inverses and
// GEMMs, (L-1) times over (green.cu:1810-1818).  Here everything stays in
// registers, the interface solve is closed form, and the recursion is written
// in a basis in which every quantity stays O(1) as w -> 0, so that FP32 is
// accurate at all frequencies:
//   layer eigenvectors   p = (k, r, -2 mu k r, -mu x),
//                        d = (w/a E_P - w/b E_SV) / (r - v)
//   with r - v = (wb^2 - wa^2)/(r + v), k - v = wb^2/(k + v), k - r = wa^2/(k + r)
//   phase matrices       [[e^{-rz}, (e^{-rz} - e^{-vz})/(r - v)], [0, e^{-vz}]]
//   interface            P = G_D^-1 G_U, Q = H_D^-1 H_U (G, H: even/odd rows of E_d)
//                        Rd = -(P+Q)^-1 (P-Q), Tu = 2 (P+Q)^-1,
//                        Td = 2 Q (P+Q)^-1 P,  Ru = (P-Q)(P+Q)^-1
// The layer table of the block's frequency is staged in shared memory with a
// TMA bulk copy (cp.async.bulk) completing on an mbarrier.
#pragma once
#include "grt_cplx.cuh"
#include "grt_integrate.cuh"
#include "grt_types.h"

namespace grt {

// Inlining policy of the large helpers.  Fully inlined, the per-point body
// outgrows the instruction cache (a dozen call sites of the complex
// exponential alone, each with the slow path of sincosf); one out-of-line
// copy of the chosen helpers keeps the hot loop resident.
#ifndef GRT_INLINE_EXP
#define GRT_INLINE_EXP __noinline__
#endif
#ifndef GRT_INLINE_LAYER
#define GRT_INLINE_LAYER __forceinline__
#endif
#ifndef GRT_INLINE_IF
#define GRT_INLINE_IF __forceinline__
#endif
#ifndef GRT_INLINE_PHASE
#define GRT_INLINE_PHASE __forceinline__
#endif

// ---------------------------------------------------------------- layer data
template <typename R>
struct SL {
    C<R> r, v, rmv, irmv;       // vertical wavenumbers, r - v, 1/(r - v)
    C<R> rlo, vlo;              // FP32 kernel: low words of r and v (double-float); FP64: zero
    C<R> p1, p2, p3;            // p0 = k
    C<R> d0, d1, d2, d3;
    C<R> detG, detH;
    C<R> x;
    R mu;
};

// k^2 carried as an unevaluated sum of two words: FP64 for the FP64 kernel,
// double-float (hi + lo, about 48 bits) for the FP32 kernel
template <typename R> struct K2 { double v; };
template <> struct K2<float> { float hi, lo; };
__device__ __forceinline__ void make_k2(double k2, K2<double> &o) { o.v = k2; }
__device__ __forceinline__ void make_k2(double k2, K2<float> &o)
{
    o.hi = (float)k2;
    o.lo = (float)(k2 - (double)o.hi);
}
// Re(c k^2 - w2): the subtraction that selects the vertical-slowness branch.
// Near the branch point it cancels; the high words cancel exactly (Sterbenz)
// and the low words supply the digits FP32 alone would lose.
__device__ __forceinline__ double re_minus(const K2<double> &k2, double c, double w2, float, float)
{
    return c * k2.v - w2;
}
__device__ __forceinline__ float re_minus(const K2<float> &k2, float c, double, float w2hi, float w2lo)
{
    return (c * k2.hi - w2hi) + (c * k2.lo - w2lo);
}

// ---------------------------------------------------------------- double-float
// Error-free transformations (Knuth's two-sum, FMA two-product).  The FP32
// kernel uses them where a rounding error would be multiplied by a large
// factor: the vertical wavenumbers r, v enter the layer phases e^{-r h} as
// r h, which reaches hundreds of radians at high frequency in thick stacks,
// so an FP32 rounding of r (relative 6e-8, different at every k) becomes a
// phase noise of ~1e-5 that the oscillatory wavenumber sum at large distance
// does not average out.  r, v and the exponents r h, v h are therefore
// carried as hi + lo pairs (about 44 bits); the R/T algebra stays FP32.
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e)
{
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}
__device__ __forceinline__ void two_prod(float a, float b, float &p, float &e)
{
    p = __fmul_rn(a, b);
    e = fmaf(a, b, -p);
}
// k^2 - w2 with w2 = w2hi + w2lo, as hi + lo
__device__ __forceinline__ void df_minus(const K2<float> &k2, float w2hi, float w2lo, float &hi, float &lo)
{
    float s, e;
    two_sum(k2.hi, -w2hi, s, e);
    e = __fadd_rn(e, __fsub_rn(k2.lo, w2lo));
    two_sum(s, e, hi, lo);
}
// low word of sqrt(z + zlo) given r0 = fl(sqrt(z)): one Newton step
// (z + zlo - r0^2) / (2 r0), with r0^2 formed exactly so the residual keeps
// its digits
__device__ __forceinline__ C<float> sqrt_lo(C<float> z, C<float> zlo, C<float> r0)
{
    if (r0.x == 0.f && r0.y == 0.f) return {0.f, 0.f};
    float ah, al, bh, bl, ch, cl, th, tl;
    two_prod(r0.x, r0.x, ah, al);
    two_prod(r0.y, r0.y, bh, bl);
    two_prod(r0.x, r0.y, ch, cl);
    two_sum(ah, -bh, th, tl);
    const C<float> d = {__fsub_rn(z.x, th) + (((zlo.x - tl) - al) + bl),
                        __fsub_rn(z.y, 2.f * ch) + (zlo.y - 2.f * cl)};
    return d * rcp(r0) * 0.5f;
}

// a depth or thickness as hi + lo (lo = 0 in the FP64 kernel)
template <typename R> struct Zd { R hi, lo; };
template <typename R> __device__ __forceinline__ Zd<R> zd(double d)
{
    Zd<R> o;
    o.hi = (R)d;
    o.lo = (R)(d - (double)o.hi);
    return o;
}

// e^{-(nu + nulo)(z + zlo)}, the exponent formed in double-float
template <typename R>
__device__ GRT_INLINE_EXP C<R> exp_nz(C<R> nu, C<R> nulo, Zd<R> z)
{
    if constexpr (sizeof(R) == 4) {
        float px, ex, py, ey;
        two_prod(nu.x, z.hi, px, ex);
        two_prod(nu.y, z.hi, py, ey);
        const C<float> lo = {ex + nulo.x * z.hi + nu.x * z.lo, ey + nulo.y * z.hi + nu.y * z.lo};
        const C<float> e = cexp_(C<float>{-px, -py});
        return e - e * lo;   // e^{hi} (1 - lo), |lo| < 1e-4
    } else {
        return cexp_(nu * (-z.hi));
    }
}

template <typename R>
__device__ GRT_INLINE_LAYER void make_layer(const LayerW<R> &T, const K2<R> &k2, R k, SL<R> &L)
{
    if constexpr (sizeof(R) == 4) {
        C<R> zr, zrl, zv, zvl;
        df_minus(k2, T.wa2[0], T.wa2lo, zr.x, zrl.x);
        df_minus(k2, T.wb2[0], T.wb2lo, zv.x, zvl.x);
        zr.y = -T.wa2[1];
        zrl.y = -T.wa2ylo;
        zv.y = -T.wb2[1];
        zvl.y = -T.wb2ylo;
        L.r = csqrt_(zr);
        L.v = csqrt_(zv);
        L.rlo = sqrt_lo(zr, zrl, L.r);
        L.vlo = sqrt_lo(zv, zvl, L.v);
    } else {
        C<R> zr = {re_minus(k2, R(1), T.wa2x, 0.f, 0.f), -T.wa2[1]};
        C<R> zv = {re_minus(k2, R(1), T.wb2x, 0.f, 0.f), -T.wb2[1]};
        L.r = csqrt_(zr);
        L.v = csqrt_(zv);
        L.rlo = L.vlo = C<R>{R(0), R(0)};
    }
    L.x = C<R>{re_minus(k2, R(2), T.wb2x, (float)T.wb2[0], T.wb2lo), -T.wb2[1]};  // k^2 + v^2 = 2k^2 - wb^2
    const C<R> wa2 = {T.wa2[0], T.wa2[1]}, wb2 = {T.wb2[0], T.wb2[1]};
    const C<R> W = {T.W[0], T.W[1]}, iW = {T.iW[0], T.iW[1]};
    C<R> rpv = L.r + L.v;
    L.irmv = rpv * iW;                 // 1/(r - v)
    L.rmv = W * rcp(rpv);              // r - v
    C<R> dv = wb2 * rcp(k + L.v);      // k - v
    C<R> dr = wa2 * rcp(k + L.r);      // k - r
    const R mu = T.mu;
    L.mu = mu;
    L.p1 = L.r;
    L.p2 = L.r * (R(-2) * mu * k);
    L.p3 = L.x * (-mu);
    L.d0 = dv * L.irmv;
    L.d1 = -(dr * L.irmv);
    L.d2 = (dr * dr - W) * L.irmv * mu;
    L.d3 = dv * dv * L.irmv * (-mu);
    C<R> m = wb2 * rpv * iW * mu;      // mu wb^2 / (r - v)
    L.detG = L.v * m;
    L.detH = -(L.r * m);
}

// S^-1 diag(e^{-rz}, e^{-vz}) S  (upper triangular)
template <typename R>
__device__ GRT_INLINE_PHASE M2<R> phase(const SL<R> &L, Zd<R> zz, C<R> *ev_out = nullptr)
{
    const R z = zz.hi;
    C<R> er = exp_nz(L.r, L.rlo, zz), ev = exp_nz(L.v, L.vlo, zz);
    C<R> y = L.rmv * (-z);
    C<R> dd;
    if (abs2(y) < R(0.25)) dd = ev * expm1_over_small(y) * (-z);
    else dd = (er - ev) * L.irmv;
    if (ev_out) *ev_out = ev;
    return {er, dd, {R(0), R(0)}, ev};
}

// S^-1 diag(sg r0 e^{-rz}, sg v0 e^{-vz}) S; r0, v0 = own nu unless given
template <typename R>
__device__ GRT_INLINE_PHASE M2<R> dphase(const SL<R> &L, Zd<R> zz, R sg, const C<R> *nu0)
{
    const R z = zz.hi;
    C<R> er = exp_nz(L.r, L.rlo, zz), ev = exp_nz(L.v, L.vlo, zz);
    C<R> y = L.rmv * (-z);
    C<R> dd;
    if (abs2(y) < R(0.25)) dd = ev * expm1_over_small(y) * (-z);
    else dd = (er - ev) * L.irmv;
    C<R> r0, v0, off;
    if (!nu0) {
        r0 = L.r; v0 = L.v;
        off = er + L.v * dd;                       // (r e_r - v e_v)/(r - v)
    } else {
        r0 = nu0[0]; v0 = nu0[1];
        off = r0 * dd + ev * (r0 - v0) * L.irmv;   // (r0 e_r - v0 e_v)/(r - v)
    }
    return {r0 * er * sg, off * sg, {R(0), R(0)}, v0 * ev * sg};
}

template <typename R>
struct IF {
    M2<R> td, tu, rd, ru;
    C<R> tdd0, tuu0, rdu0;  // rud0 = -rdu0
};

// interface between U (upper layer) and D (lower layer)
template <typename R>
__device__ GRT_INLINE_IF void interface_rt(const SL<R> &U, const SL<R> &D, R k, IF<R> &m)
{
    const C<R> kk = {k, R(0)};
    M2<R> GU = {kk, U.d0, U.p3, U.d3}, HU = {U.p1, U.d1, U.p2, U.d2};
    M2<R> GDi = inv_det(M2<R>{kk, D.d0, D.p3, D.d3}, D.detG);
    M2<R> HDi = inv_det(M2<R>{D.p1, D.d1, D.p2, D.d2}, D.detH);
    M2<R> P = GDi * GU, Q = HDi * HU;
    M2<R> S = P + Q, Dm = P - Q;
    M2<R> Si = inv(S);
    m.rd = (Si * Dm) * R(-1);
    m.tu = Si * R(2);
    m.td = (Q * (Si * P)) * R(2);
    m.ru = Dm * Si;
    // SH (get_mrt_sh, green.cu:339-353)
    C<R> wa = U.v * U.mu, wb = D.v * D.mu;
    C<R> is = rcp(wa + wb);
    m.tdd0 = wa * is * R(2);
    m.rdu0 = (wa - wb) * is;
    m.tuu0 = wb * is * R(2);
}

// where this thread's coefficients go: the flat column K[q][koff + j], or the
// tensor-core operand block of its (frequency tile, k stage)
struct KOut {
    long long idx;        // koff[iw] + j
    float *blk;           // operand block, or null
    unsigned ore, oim;    // offsets of the re / im rows inside a q tile (floats; bf16 words in the BF16 form)
    int bf16;             // the 3xBF16 form
};

template <typename R>
__device__ __forceinline__ KOut make_kout(const GrtArgs<R> &A, int iw, int j)
{
    KOut o{A.koff[iw] + j, nullptr, 0u, 0u, 0};
    if (sizeof(R) == 4 && A.Kt) {
        const int wl = iw % (kTileRows / 2);
        // a stage block is nqt x (hi, lo) tiles of 4 KB in both forms
        const int tk = A.kt_bf16 ? kTileK16 : kTileK;
        o.blk = A.Kt + A.kt_base[iw / (kTileRows / 2)] + (long long)(j / tk) * A.nqt * 2 * (kTileRows * kTileK);
        if (A.kt_bf16) {
            o.bf16 = 1;
            o.ore = kt_tile_off16(wl, j % tk) / 2;
            o.oim = kt_tile_off16(kTileRows / 2 + wl, j % tk) / 2;
        } else {
            o.ore = kt_tile_off(wl, j % tk) / 4;
            o.oim = kt_tile_off(kTileRows / 2 + wl, j % tk) / 4;
        }
    }
    return o;
}

// the tensor-core tile of each coefficient column comes with the job
// (make_tcplan of its column layout; columns no pair reads are not stored)
template <int SRCK, typename R>
__device__ __forceinline__ void store_q(const GrtArgs<R> &A, int q, const KOut &o, C<R> v)
{
    if (sizeof(R) == 4 && o.blk) {
        const int slot = q < 16 ? A.qslot[q] : -1;
        if (slot < 0) return;
        float *t = o.blk + slot * 2 * (kTileRows * kTileK);
        const float x = (float)v.x, y = (float)v.y;
        if (o.bf16) {
            // BF16 hi / lo words of the 3xBF16 product, [tile][hi|lo] tiles of 2048 bf16
            unsigned short *u = reinterpret_cast<unsigned short *>(t), xh, xl, yh, yl;
            bf16_split(x, xh, xl);
            bf16_split(y, yh, yl);
            u[o.ore] = xh;
            u[2 * kTileRows * kTileK + o.ore] = xl;
            u[o.oim] = yh;
            u[2 * kTileRows * kTileK + o.oim] = yl;
            return;
        }
        // TF32 hi / lo words of the 3xTF32 product, [tile][hi|lo] tiles of 1024 floats
        const float xh = tf32_rna(x), yh = tf32_rna(y);
        t[o.ore] = xh;
        t[kTileRows * kTileK + o.ore] = tf32_rna(x - xh);
        t[o.oim] = yh;
        t[kTileRows * kTileK + o.oim] = tf32_rna(y - yh);
        return;
    }
    reinterpret_cast<C<R> *>(A.K)[(long long)q * A.nkw + o.idx] = v;
}

// bounded wait on an mbarrier phase; gives up (error word) instead of hanging
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, unsigned int *err)
{
    uint32_t done = 0;
    for (int it = 0; it < (1 << 22); it++) {
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}\n"
            : "=r"(done)
            : "r"(bar), "r"(parity)
            : "memory");
        if (done) return true;
    }
    if (err) atomicOr(err, 1u);
    return false;
}

// The per-(w,k) evaluation of one thread: job A, its layer table for
// frequency iw already staged in T, wavenumber index j (< nk[iw]).
// SPEC: kSpecGeneric handles every job; kSpecAboveTensor only moment-tensor
// jobs with the receiver in a layer above the source's and the eight
// coefficient columns of the reference layout (the usual surface receivers).
// Its code is a third shorter (the other receiver cases and source kinds
// compiled out), which the instruction cache repays: a 40-layer job's GRT
// went from 174 to 159 ms.
// Returns the layers it evaluated: every layer without depth truncation (the
// roofline's L), fewer where the recursion starts above the half-space.
// PASS: 0 the whole evaluation; 1 the bottom-up pass alone, which leaves
// R^du and R^du_0 at the source in A.rdu; 2 the rest, which takes them from
// there.  Two passes keep one layer loop per kernel: run as one, warps at
// different depths of the truncated bottom-up loop and of the top-down loop
// share the instruction cache (instruction-fetch stalls were the top stall).
template <typename R, int SPEC, int PASS = 0>
__device__ __forceinline__ int grt_point(const GrtArgs<R> &A, const LayerW<R> *T, int iw, int j)
{
    const int L = A.L, s = A.s, rl = A.rl;
    constexpr bool kAboveTensor = SPEC == kSpecAboveTensor;
    const bool below = !kAboveTensor && rl > s, same = !kAboveTensor && rl == s;
    const bool above = kAboveTensor || rl < s;
    const bool single = !kAboveTensor && A.src == kSingle, fullq = !kAboveTensor && A.nq > QT_N;
    const int jj = j;
    const double kd = A.dk * (A.ks ? A.ks[iw] : 1) * jj;
    K2<R> k2;
    make_k2(kd * kd, k2);
    const R k = (R)kd;
    const C<R> zero = {R(0), R(0)};

    // ---------------- bottom-up pass: R^du and T^d from the half-space to s+1
    SL<R> D, U;
    M2<R> Rdu = zero2<R>();
    C<R> rdu0 = zero;
    M2<R> PD = eye2<R>();      // r_layer > s: Td(rl) Lam(rl-1) ... Td(s+1)
    C<R> pd0 = {R(1), R(0)};
    // receiver coefficients (u0, u0t, U, Ut) -- filled by the pass that sees rl
    M2<R> Urec = zero2<R>(), Utrec = zero2<R>();
    C<R> u0 = zero, u0t = zero;
    const C<R> slot0[2] = {{A.slot0[0], A.slot0[1]}, {A.slot0[2], A.slot0[3]}};
    const C<R> *nu0 = (A.fix & kFixRexut) ? nullptr : slot0;
    const R zr = (R)A.zr;
    const Zd<R> Zr = zd<R>(A.zr), Zhr = zd<R>(A.hr_layer), Zhr_r = zd<R>(A.hr_layer - A.zr);

    int jlow = L - 2;
    if constexpr (PASS != 2) {
    make_layer(T[L - 1], k2, k, D);
    // Depth truncation: below the source (below the receiver when it lies
    // deeper), a wave reflected from beneath the layer where the slower, S,
    // vertical wavenumber has accumulated sum Re(v) h > lim comes back damped
    // by e^{-2 lim}: 1.5e-8 with lim = 9 in FP32 (under half an FP32 ulp,
    // 3e-8), 4e-18 with lim = 20 in FP64, under the working precision; the
    // recursion starts there with the layer beneath as the half-space.  At
    // wavenumbers where S is evanescent this skips most of the deep stack.
    {
        const R lim = sizeof(R) == 4 ? R(9) : R(20);
        const int j0 = below ? rl + 1 : s + 1;
        R e = R(0);
        for (int jl = j0; jl <= L - 3; jl++) {
            const C<R> zv = {k * k - T[jl].wb2[0], -T[jl].wb2[1]};
            e += csqrt_(zv).x * T[jl].h;
            if (e > lim) {
                jlow = jl;
                break;
            }
        }
    }
    if (jlow < L - 2) make_layer(T[jlow + 1], k2, k, D);

    for (int jf = jlow; jf >= s; jf--) {
        make_layer(T[jf], k2, k, U);
        IF<R> m;
        interface_rt(U, D, k, m);
        M2<R> Tdn;
        C<R> td0n;
        if (jf == jlow) {
            Rdu = m.rd;
            rdu0 = m.rdu0;
            Tdn = m.td;
            td0n = m.tdd0;
        } else {
            C<R> ev;
            M2<R> Lam = phase(D, Zd<R>{T[jf + 1].h, (R)T[jf + 1].hlo}, &ev);
            // SH, green.cu:537-548
            C<R> tem1 = (-m.rdu0) * ev, tem2 = rdu0 * ev, tem3 = m.tuu0 * ev;
            td0n = m.tdd0 * rcp(R(1) - tem1 * tem2);
            rdu0 = m.rdu0 + tem3 * tem2 * td0n;
            // P-SV, green.cu:556-587
            M2<R> X = ut_mul_right(ut_mul_left(Lam, Rdu), Lam);
            M2<R> Am = eye_minus(m.ru * X);
            M2<R> Bm = m.tu * X;
            Tdn = inv(Am) * m.td;
            Rdu = m.rd + Bm * Tdn;
            if (below && jf + 1 < rl) {
                PD = ut_mul_right(PD, Lam) * Tdn;
                pd0 = pd0 * ev * td0n;
            }
        }
        if (below && jf + 1 == rl) {
            PD = Tdn;
            pd0 = td0n;
        }
        if (below && jf == rl) {
            // receiver below the source, inside layer rl (corrected form)
            C<R> exv, ldv, luv;
            M2<R> Ld = phase(U, Zr, &ldv), Lu = phase(U, Zhr_r, &luv);
            M2<R> Ldt = dphase(U, Zr, R(-1), (const C<R> *)nullptr);
            M2<R> Lut = dphase(U, Zhr_r, R(1), nu0);
            M2<R> Ex = phase(U, Zhr, &exv);
            M2<R> Ed = {{k, R(0)}, U.d0, U.p1, U.d1}, Eu = {{k, R(0)}, U.d0, -U.p1, -U.d1};
            M2<R> RE = Rdu * Ex;
            Urec = Ed * Ld + Eu * ut_mul_left(Lu, RE);
            Utrec = Ed * Ldt + Eu * ut_mul_left(Lut, RE);
            u0 = luv * rdu0 * exv + ldv;
            u0t = Lut.d * rdu0 * exv - U.v * ldv;
        }
        D = U;
    }
    if (below && rl == L - 1) {
        // receiver in the half-space: only the down-going field
        make_layer(T[L - 1], k2, k, U);
        C<R> ldv;
        M2<R> Ld = phase(U, Zr, &ldv);
        M2<R> Ldt = dphase(U, Zr, R(-1), (const C<R> *)nullptr);
        M2<R> Ed = {{k, R(0)}, U.d0, U.p1, U.d1};
        Urec = Ed * Ld;
        Utrec = Ed * Ldt;
        u0 = ldv;
        u0t = -(U.v * ldv);
    }
    }   // PASS != 2
    const long long fi = A.koff[iw] + j;   // this point in the flattened (w,k) list
    if constexpr (PASS == 1) {
        R *o = A.rdu + fi;
        const R v[kRduPlanes] = {Rdu.a.x, Rdu.a.y, Rdu.b.x, Rdu.b.y, Rdu.c.x, Rdu.c.y, Rdu.d.x, Rdu.d.y,
                                 rdu0.x, rdu0.y};
#pragma unroll
        for (int c = 0; c < kRduPlanes; c++) o[(long long)c * A.nkw] = v[c];
        return jlow + 2 - s;
    }
    if constexpr (PASS == 2) {
        const R *o = A.rdu + fi;
        R v[kRduPlanes];
#pragma unroll
        for (int c = 0; c < kRduPlanes; c++) v[c] = o[(long long)c * A.nkw];
        Rdu = M2<R>{{v[0], v[1]}, {v[2], v[3]}, {v[4], v[5]}, {v[6], v[7]}};
        rdu0 = C<R>{v[8], v[9]};
    }
    const M2<R> RD = Rdu;      // R^du at the bottom of the source layer
    const C<R> RD0 = rdu0;

    // ---------------- top-down pass: R^ud and T^u from the free surface to s
    make_layer(T[0], k2, k, U);
    M2<R> Rud;
    {
        // free surface: R = T^-1 diag(1,-1) T, T = stress rows of E_d,
        // det T = mu^2 (x^2 - 4 k^2 r v)/(r - v) without cancellation
        C<R> dv = C<R>{T[0].wb2[0], T[0].wb2[1]} * rcp(k + U.v);
        C<R> dr = C<R>{T[0].wa2[0], T[0].wa2[1]} * rcp(k + U.r);
        C<R> W = {T[0].W[0], T[0].W[1]};
        C<R> ray = U.x * (dr * dr - W) + U.r * dv * dv * (R(2) * k);
        C<R> detT = ray * U.irmv * (U.mu * U.mu);
        M2<R> Tm = {U.p2, U.d2, U.p3, U.d3};
        M2<R> adj = {Tm.d, -Tm.b, -Tm.c, Tm.a};
        M2<R> DT = {Tm.a, Tm.b, -Tm.c, -Tm.d};
        Rud = (adj * DT) * rcp(detT);
    }
    C<R> rud0 = {R(1), R(0)};
    M2<R> PC = eye2<R>();      // r_layer < s: Tu(rl+1) Lam(rl+1) ... Tu(s)
    C<R> pc0 = {R(1), R(0)};
    for (int jf = 0; jf < s; jf++) {
        if (jf == rl) {
            // receiver above the source, inside layer rl (green.cu:775-857)
            C<R> exv, ldv, luv = zero;
            const bool last = false;
            (void)last;
            M2<R> Ld = phase(U, Zr, &ldv), Lu = phase(U, Zhr_r, &luv);
            M2<R> Ldt = dphase(U, Zr, R(-1), (const C<R> *)nullptr);
            M2<R> Lut = dphase(U, Zhr_r, R(1), nu0);
            M2<R> Ex = phase(U, Zhr, &exv);
            M2<R> Ed = {{k, R(0)}, U.d0, U.p1, U.d1}, Eu = {{k, R(0)}, U.d0, -U.p1, -U.d1};
            M2<R> RE = Rud * Ex;
            Urec = Ed * ut_mul_left(Ld, RE) + Eu * Lu;
            Utrec = Ed * ut_mul_left(Ldt, RE) + Eu * Lut;
            u0 = ldv * rud0 * exv + luv;
            u0t = -(U.v * ldv * rud0 * exv) + Lut.d;
        }
        make_layer(T[jf + 1], k2, k, D);
        IF<R> m;
        interface_rt(U, D, k, m);
        C<R> ev;
        M2<R> Lam = phase(U, Zd<R>{T[jf].h, (R)T[jf].hlo}, &ev);
        // SH, green.cu:476-482
        C<R> tem1 = rud0 * ev, tem2 = m.rdu0 * ev, tem3 = m.tdd0 * ev;
        C<R> tu0n = m.tuu0 * rcp(R(1) - tem1 * tem2);
        rud0 = (-m.rdu0) + tem3 * tem1 * tu0n;
        // P-SV, green.cu:486-519
        M2<R> X = ut_mul_right(ut_mul_left(Lam, Rud), Lam);
        M2<R> Am = eye_minus(m.rd * X);
        M2<R> Bm = m.td * X;
        M2<R> Tun = inv(Am) * m.tu;
        Rud = m.ru + Bm * Tun;
        if (above) {
            if (jf == rl) {
                PC = Tun;
                pc0 = tu0n;
            } else if (jf > rl) {
                PC = ut_mul_right(PC, Lam) * Tun;
                pc0 = pc0 * ev * tu0n;
            }
        }
        U = D;
    }
    // U now holds the source layer
    const M2<R> RU = Rud;
    const C<R> RU0 = rud0;
    const SL<R> &S = U;
    const R zs = (R)A.zs, hs = (R)A.hs_layer;
    const Zd<R> Zs = zd<R>(A.zs), Zhs_s = zd<R>(A.hs_layer - A.zs), Zs_r = zd<R>(A.zs - A.zr),
                Zr_s = zd<R>(A.zr - A.zs), Zhs_r = zd<R>(A.hs_layer - A.zr);
    (void)hs;

    // ---------------- source terms (get_src_single / _tensor, green.cu:1271-1413)
    C<R> sexd1, sexu1;
    M2<R> Ldn = phase(S, Zhs_s, &sexd1), Lup = phase(S, Zs, &sexu1);
    M2<R> ED = ut_mul_right(ut_mul_left(Ldn, RD), Ldn);
    M2<R> EU = ut_mul_right(ut_mul_left(Lup, RU), Lup);
    const bool up = above || (same && A.zr <= A.zs);
    // the reverberation and source jump, on the side the receiver sees
    M2<R> ypsv = up ? inv(eye_minus(ED * EU)) : inv(eye_minus(EU * ED));
    C<R> y_sh = rcp(R(1) - sexd1 * RD0 * sexd1 * sexu1 * RU0 * sexu1);
    const R smu = S.mu;
    C<R> ssh = rcp(S.v * (R(2) * smu));
    C<R> fu = R(1) + sexd1 * RD0 * sexd1;       // 1 + e R^du e (SH)
    C<R> fd = sexu1 * RU0 * sexu1;              // e R^ud e (SH)
    // even / odd source vectors in this basis: f0 = 1/2 G^-1 e3, f1 = -1/2 H^-1 e2
    C<R> iG = rcp(S.detG), iH = rcp(S.detH);
    C<R> f1a = S.d1 * iH * R(0.5), f1b = -(S.r * iH * R(0.5));
    // W+ = I + E R E, W- = E R E - I (below) / I - E R E (above)
    M2<R> Wp = up ? eye_plus(ED) : eye_plus(EU);
    M2<R> Wm = up ? minus_eye(ED) : eye_minus(EU);

    // ---------------- receiver propagation (get_ypars_a_*)
    C<R> y0, y0t;
    M2<R> y1, y1t;
    if (same) {
        const SL<R> &Rv = S;
        if (A.zr <= A.zs) {
            C<R> e1v, e2v;
            M2<R> L1 = phase(Rv, Zr, &e1v), L2 = phase(Rv, Zs_r, &e2v);
            M2<R> L1t = dphase(Rv, Zr, R(-1), (const C<R> *)nullptr);
            M2<R> L2t = dphase(Rv, Zs_r, R(1), (const C<R> *)nullptr);
            M2<R> Ed = {{k, R(0)}, Rv.d0, Rv.p1, Rv.d1}, Eu = {{k, R(0)}, Rv.d0, -Rv.p1, -Rv.d1};
            M2<R> RL = ut_mul_right(RU, Lup);
            Urec = Ed * ut_mul_left(L1, RL) + Eu * L2;
            Utrec = Ed * ut_mul_left(L1t, RL) + Eu * L2t;
            u0 = e1v * RU0 * sexu1 + e2v;
            // green.cu:720 multiplies the up-going term by nu twice
            u0t = -(Rv.v * e1v * RU0 * sexu1) + ((A.fix & kFixDz) ? Rv.v * e2v : Rv.v * e2v * Rv.v);
        } else {
            C<R> e1v, e2v;
            M2<R> L1 = phase(Rv, Zr_s, &e1v), L2 = phase(Rv, Zhs_r, &e2v);
            M2<R> L1t = dphase(Rv, Zr_s, R(-1), (const C<R> *)nullptr);
            M2<R> L2t = dphase(Rv, Zhs_r, R(1), (const C<R> *)nullptr);
            M2<R> Ed = {{k, R(0)}, Rv.d0, Rv.p1, Rv.d1}, Eu = {{k, R(0)}, Rv.d0, -Rv.p1, -Rv.d1};
            M2<R> RL = ut_mul_right(RD, Ldn);
            Urec = Ed * L1 + Eu * ut_mul_left(L2, RL);
            Utrec = Ed * L1t + Eu * ut_mul_left(L2t, RL);
            u0 = e1v + e2v * RD0 * sexd1;
            u0t = -(Rv.v * e1v) + Rv.v * e2v * RD0 * sexd1;
        }
        y0 = u0 * y_sh;
        y0t = u0t * y_sh;
        y1 = Urec * ypsv;
        y1t = Utrec * ypsv;
    } else if (above) {
        C<R> yp0 = pc0 * sexu1 * y_sh;
        M2<R> yp1 = PC * ut_mul_left(Lup, ypsv);
        y0 = u0 * yp0;
        // green.cu:842 reuses the updated yu0
        y0t = (A.fix & kFixDz) ? u0t * yp0 : u0t * y0;
        y1 = Urec * yp1;
        y1t = Utrec * yp1;
    } else {
        C<R> yp0 = pd0 * sexd1 * y_sh;
        M2<R> yp1 = PD * ut_mul_left(Ldn, ypsv);
        y0 = u0 * yp0;
        y0t = u0t * yp0;
        y1 = Urec * yp1;
        y1t = Utrec * yp1;
    }

    const KOut out = make_kout(A, iw, j);
    if (single) {
        C<R> f0a = -(S.d0 * iG * R(0.5)), f0b = C<R>{k, R(0)} * iG * R(0.5);
        C<R> g0a, g0b, g1a, g1b;
        mv2(Wm, f0a, f0b, &g0a, &g0b);
        mv2(Wp, f1a, f1b, &g1a, &g1b);
        C<R> gsh = up ? fu * ssh : (fd + R(1)) * ssh;
        C<R> a00, a01, a10, a11;
        mv2(y1, g0a, g0b, &a00, &a01);
        mv2(y1, g1a, g1b, &a10, &a11);
        store_q<kSingle>(A, QS_B1, out, y0 * gsh);
        store_q<kSingle>(A, QS_A00, out, a00);
        store_q<kSingle>(A, QS_A01, out, a01);
        store_q<kSingle>(A, QS_A10, out, a10);
        store_q<kSingle>(A, QS_A11, out, a11);
        mv2(y1t, g0a, g0b, &a00, &a01);
        mv2(y1t, g1a, g1b, &a10, &a11);
        store_q<kSingle>(A, QS_B1T, out, y0t * gsh);
        store_q<kSingle>(A, QS_A0T0, out, a00);
        store_q<kSingle>(A, QS_A0T1, out, a01);
        store_q<kSingle>(A, QS_A1T0, out, a10);
        store_q<kSingle>(A, QS_A1T1, out, a11);
    } else {
        // s2 = k f1, s1 = -1/(2 mu) G^-1 e0, s0 = H^-1 (alpha', beta')
        C<R> s2a = f1a * k, s2b = f1b * k;
        C<R> s1a = -(S.d3 * iG * (R(0.5) / smu)), s1b = -(S.x * iG * R(0.5));
        C<R> sa = {T[s].a[0], T[s].a[1]}, sb = {T[s].b[0], T[s].b[1]};
        C<R> ba2 = (sb * sb) * rcp(sa * sa);
        C<R> al = ba2 * (R(-0.5) / smu);
        C<R> be = (ba2 * R(2) - R(1)) * (k * R(0.5));
        C<R> s0a = (S.d2 * al - S.d1 * be) * iH, s0b = (-(S.p2 * al) + S.p1 * be) * iH;
        C<R> q0a, q0b, q1a, q1b, q2a, q2b;
        mv2(Wp, s0a, s0b, &q0a, &q0b);
        mv2(Wm, s1a, s1b, &q1a, &q1b);
        mv2(Wp, s2a, s2b, &q2a, &q2b);
        // green.cu:1409-1412 give the m = 1 and m = 2 SH terms one factor;
        // GRT_FIX_SHSRC gives m = 1 a displacement jump's (1 - e R e up) and
        // m = 2 a traction jump's (e R e + 1 down), as the P-SV terms have
        C<R> shf = up ? fu : fd - R(1);
        C<R> shf1 = shf, shf2 = shf;
        if (A.fix & kFixShsrc) {
            if (up) shf1 = R(2) - fu;
            else shf2 = fd + R(1);
        }
        C<R> h1 = shf1 * S.v * ssh, h2 = shf2 * k * ssh;
        C<R> v0, v1;
        store_q<kTensor>(A, QT_B1, out, y0 * h1);
        store_q<kTensor>(A, QT_B2, out, y0 * h2);
        mv2(y1, q0a, q0b, &v0, &v1);
        store_q<kTensor>(A, QT_A00, out, v0);
        store_q<kTensor>(A, QT_A01, out, v1);
        mv2(y1, q1a, q1b, &v0, &v1);
        store_q<kTensor>(A, QT_A10, out, v0);
        store_q<kTensor>(A, QT_A11, out, v1);
        mv2(y1, q2a, q2b, &v0, &v1);
        store_q<kTensor>(A, QT_A20, out, v0);
        store_q<kTensor>(A, QT_A21, out, v1);
        if (fullq) {
            store_q<kTensor>(A, QT_N + QT_B1, out, y0t * h1);
            store_q<kTensor>(A, QT_N + QT_B2, out, y0t * h2);
            mv2(y1t, q0a, q0b, &v0, &v1);
            store_q<kTensor>(A, QT_N + QT_A00, out, v0);
            store_q<kTensor>(A, QT_N + QT_A01, out, v1);
            mv2(y1t, q1a, q1b, &v0, &v1);
            store_q<kTensor>(A, QT_N + QT_A10, out, v0);
            store_q<kTensor>(A, QT_N + QT_A11, out, v1);
            mv2(y1t, q2a, q2b, &v0, &v1);
            store_q<kTensor>(A, QT_N + QT_A20, out, v0);
            store_q<kTensor>(A, QT_N + QT_A21, out, v1);
        }
    }
    return PASS == 2 ? s : jlow + 2;
}

// add the layers the calling lanes evaluated to one of the kNlevSlots counters
__device__ __forceinline__ void count_levals(unsigned long long *c, int v)
{
    if (!c) return;
    const unsigned m = __activemask();
    const unsigned sum = __reduce_add_sync(m, (unsigned)v);
    if ((int)(threadIdx.x & 31) == __ffs(m) - 1) atomicAdd(c + (blockIdx.x % kNlevSlots), (unsigned long long)sum);
}

#ifndef GRT_POINT_MINB
#define GRT_POINT_MINB 1   // resident blocks per SM the register allocation must allow
#endif
// resident threads per SM the register allocation of the two passes must
// allow: pass 1 512 (128 registers, no spills), pass 2 GRT_PASS2_THREADS
// (512: 128 registers and 32 bytes of spills, 1-2 % faster than 384 with 167
// registers and none)
#ifndef GRT_PASS2_THREADS
#define GRT_PASS2_THREADS 512
#endif

// stage the layer table of (job, frequency) into shared memory with a TMA bulk
// copy issued by thread 0; every thread waits on the mbarrier phase
template <typename R>
__device__ __forceinline__ bool stage_table(const GrtArgs<R> &A, int iw, LayerW<R> *T, uint32_t sbar,
                                            uint32_t phase, bool wait)
{
    if (threadIdx.x == 0) {
        const unsigned bytes = (unsigned)(A.L * sizeof(LayerW<R>));
        const uint32_t sdst = (uint32_t)__cvta_generic_to_shared(T);
        const LayerW<R> *src = A.tab + (size_t)iw * A.L;
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(sbar), "r"(bytes) : "memory");
        asm volatile(
            "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(sdst),
            "l"(src), "r"(bytes), "r"(sbar)
            : "memory");
    }
    return wait ? mbar_wait(sbar, phase, A.err) : true;
}

// Tile lists written on the device (the host sends one offset per row):
// row r (a frequency of one job) has ceil(nk_r / nt) tiles from first[r] on.
// Plans: (frequency, first k); batches: (job, frequency, first k, 0).  One
// block per row.
static __global__ void plan_tiles_kernel(const int *nk, const long long *first, int nt, int2 *tiles)
{
    const int r = blockIdx.x;
    const int n = (nk[r] + nt - 1) / nt;
    int2 *out = tiles + first[r];
    for (int c = threadIdx.x; c < n; c += blockDim.x) out[c] = make_int2(r, c * nt);
}

static __global__ void batch_tiles_kernel(const int2 *row_id, const int *row_nk, const long long *first, int nt,
                                          int4 *tiles)
{
    const int r = blockIdx.x;
    const int2 id = row_id[r];
    const int n = (row_nk[r] + nt - 1) / nt;
    int4 *out = tiles + first[r];
    for (int c = threadIdx.x; c < n; c += blockDim.x) out[c] = make_int4(id.x, id.y, c * nt, 0);
}

// One job: one block per (frequency, block of kGrtThreads wavenumbers).
template <typename R, int SPEC = kSpecGeneric, int PASS = 0>
__global__ void __launch_bounds__(kGrtThreads, PASS == 1 ? 512 / kGrtThreads : PASS == 2 ? GRT_PASS2_THREADS / kGrtThreads : GRT_POINT_MINB) grt_point_kernel(GrtArgs<R> A)
{
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ __align__(8) unsigned long long bar;
    LayerW<R> *T = reinterpret_cast<LayerW<R> *>(smem_raw);
    const int2 tile = A.tiles[blockIdx.x];
    const int iw = tile.x;
    const int j = tile.y + threadIdx.x;
    const uint32_t sbar = (uint32_t)__cvta_generic_to_shared(&bar);
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(sbar) : "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    __syncthreads();
    stage_table(A, iw, T, sbar, 0, false);
    // lanes past the frequency's last wavenumber leave now (no block-wide
    // synchronisation follows; lane 0 of a tile is always valid and waits
    // for the table copy it issued): evaluating them would hold their warps
    if (j >= A.nk[iw]) return;
    if (!mbar_wait(sbar, 0, A.err)) return;
    count_levals(A.nlev, grt_point<R, SPEC, PASS>(A, T, iw, j));
}

// Many jobs in one launch.  tiles[t] = (job, frequency, first wavenumber
// index, 0), ordered job by job and frequency by frequency; NT threads per
// block evaluate NT consecutive wavenumbers of a tile.
//
// Persistent form (PERSIST, G blocks): the blocks take runs of kRun
// consecutive tiles round robin (block b: runs b, b + G, ...), so that the
// blocks in flight work on neighbouring frequencies and their writes of the
// coefficients stay within a few hundred MB, which the address translation
// covers; the job's arguments and layer table are restaged only when the
// (job, frequency) changes, behind a block barrier.  One-tile form: one
// block per tile, idle lanes leave at once, no barrier after the staging.
// The autotuner picks the form and shape on the batch.
constexpr int kRun = 4;
template <typename R, int NT, bool PERSIST, int SPEC = kSpecGeneric, int PASS = 0>
__global__ void __launch_bounds__(NT, PASS == 1 ? 512 / NT : PASS == 2 ? GRT_PASS2_THREADS / NT : 1) grt_batch_kernel(const GrtArgs<R> *__restrict__ jobs,
                                                           const int4 *__restrict__ tiles, int ntiles,
                                                           unsigned int *err)
{
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ __align__(8) unsigned long long bar;
    __shared__ GrtArgs<R> sA;                    // the current job's arguments (no aliasing with global stores)
    LayerW<R> *T = reinterpret_cast<LayerW<R> *>(smem_raw);
    const uint32_t sbar = (uint32_t)__cvta_generic_to_shared(&bar);
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(sbar) : "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    if constexpr (!PERSIST) {
        if (blockIdx.x >= ntiles) return;
        const int4 tl = tiles[blockIdx.x];
        if (threadIdx.x == 0) sA = jobs[tl.x];
        __syncthreads();
        stage_table(sA, tl.y, T, sbar, 0, false);
        const int j = tl.z + threadIdx.x;
        if (j >= sA.nk[tl.y]) return;              // lane 0 is valid: it waits for its copy
        if (!mbar_wait(sbar, 0, err)) return;
        count_levals(sA.nlev, grt_point<R, SPEC, PASS>(sA, T, tl.y, j));
        return;
    }
    __syncthreads();
    int cur_job = -1, cur_iw = -1;
    uint32_t phase = 0;
    for (long long c = blockIdx.x; c * kRun < ntiles; c += gridDim.x)
    for (int t = (int)(c * kRun); t < ntiles && t < (int)(c * kRun) + kRun; t++) {
        const int4 tl = tiles[t];
        if (tl.x != cur_job || tl.y != cur_iw) {
            __syncthreads();                       // every thread is done with the old table and arguments
            if (tl.x != cur_job && threadIdx.x == 0) sA = jobs[tl.x];
            const bool ok = stage_table(jobs[tl.x], tl.y, T, sbar, phase, true);
            if (__syncthreads_or(!ok)) {
                if (threadIdx.x == 0) atomicOr(err, 1u);
                return;
            }
            phase ^= 1u;
            cur_job = tl.x;
            cur_iw = tl.y;
        }
        const int j = tl.z + threadIdx.x;
        if (j < sA.nk[tl.y]) count_levals(sA.nlev, grt_point<R, SPEC, PASS>(sA, T, tl.y, j));
    }
}

}  // namespace grt
