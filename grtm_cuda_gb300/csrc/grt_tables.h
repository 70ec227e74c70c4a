// grt_tables.h -- host construction of the per-(frequency, layer) table the
// GRT kernel stages in shared memory.
#pragma once
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstring>
#include <functional>
#include <thread>
#include <vector>

#include "grt_job.h"
#include "grt_types.h"

namespace grt {

// Complex frequency w = 2 pi df f - i sigma of row iw (f = its frequency
// index); attenuated velocities by the reference's constant-Q dispersion
// (set_pars, green.cu:177-180); then (w/alpha)^2, (w/beta)^2, their difference
// and its inverse, rounded to R, with the double-float low words the FP32
// kernel needs.  tab: [nw][L].  Complex quotients by the textbook formula
// (these magnitudes are far from overflow), rows spread over host threads.
// w = 2 pi df f - i sigma and log(w / 2 pi) of frequency index f
struct RowFreq {
    double wr, wi, lwr, lwi;
};
inline RowFreq row_freq(const Job &J, int f)
{
    const double pi = 3.14159265358979323846;
    RowFreq w;
    w.wr = 2 * pi * J.df * f;
    w.wi = -J.sigma;
    w.lwr = std::log(std::hypot(w.wr, w.wi) / (2 * pi));
    w.lwi = std::atan2(w.wi, w.wr);
    return w;
}

template <typename R>
inline void layer_entry(const Job &J, const RowFreq &w, int i, LayerW<R> &t)
{
    const double pi = 3.14159265358979323846;
    auto lo = [](double x) { return (float)(x - (double)(float)x); };
    std::memset(&t, 0, sizeof t);
    // alpha = a0 (1 + lw / (pi qp) + i / (2 qp)), beta likewise with qs
    const double ar = J.a0[i] * (1.0 + w.lwr / (pi * J.qp[i]));
    const double ai = J.a0[i] * (w.lwi / (pi * J.qp[i]) + 0.5 / J.qp[i]);
    const double br = J.b0[i] * (1.0 + w.lwr / (pi * J.qs[i]));
    const double bi = J.b0[i] * (w.lwi / (pi * J.qs[i]) + 0.5 / J.qs[i]);
    // w / alpha, w / beta and their squares
    const double da = 1.0 / (ar * ar + ai * ai), db = 1.0 / (br * br + bi * bi);
    const double war = (w.wr * ar + w.wi * ai) * da, wai = (w.wi * ar - w.wr * ai) * da;
    const double wbr = (w.wr * br + w.wi * bi) * db, wbi = (w.wi * br - w.wr * bi) * db;
    const double a2r = war * war - wai * wai, a2i = 2 * war * wai;
    const double b2r = wbr * wbr - wbi * wbi, b2i = 2 * wbr * wbi;
    const double Wr = b2r - a2r, Wi = b2i - a2i, dW = 1.0 / (Wr * Wr + Wi * Wi);
    t.wa2x = a2r; t.wa2y = a2i; t.wb2x = b2r; t.wb2y = b2i;
    t.wa2[0] = (R)a2r; t.wa2[1] = (R)a2i;
    t.wb2[0] = (R)b2r; t.wb2[1] = (R)b2i;
    t.W[0] = (R)Wr; t.W[1] = (R)Wi;
    t.iW[0] = (R)(Wr * dW); t.iW[1] = (R)(-Wi * dW);
    t.a[0] = (R)ar; t.a[1] = (R)ai;
    t.b[0] = (R)br; t.b[1] = (R)bi;
    t.mu = (R)J.mu[i];
    t.h = (R)J.h[i];
    // low words: the FP64 kernel carries none
    if (sizeof(R) == 4) {
        t.wa2lo = lo(a2r);
        t.wb2lo = lo(b2r);
        t.wa2ylo = lo(a2i);
        t.wb2ylo = lo(b2i);
        t.hlo = lo(J.h[i]);
    }
}

template <typename R>
inline void fill_layer_rows(const Job &J, LayerW<R> *tab, int iw0, int iw1)
{
    for (int iw = iw0; iw < iw1; iw++) {
        const RowFreq w = row_freq(J, job_freq(J, iw));
        for (int i = 0; i < J.L; i++) layer_entry<R>(J, w, i, tab[(size_t)iw * J.L + i]);
    }
}

// Vertical wavenumbers nu_alpha, nu_beta (Re >= 0) of the receiver layer at
// w = -i sigma, k = 0 (frequency index 0, whatever rows a job keeps), as
// (re, im, re, im): the reference's slot-0 values its d/dz terms reuse.
inline void slot0_wavenumbers(const Job &J, double out[4])
{
    LayerW<double> t;
    layer_entry<double>(J, row_freq(J, 0), J.rl, t);
    std::complex<double> r0 = std::sqrt(std::complex<double>(-t.wa2x, -t.wa2y));
    std::complex<double> v0 = std::sqrt(std::complex<double>(-t.wb2x, -t.wb2y));
    if (r0.real() < 0) r0 = -r0;
    if (v0.real() < 0) v0 = -v0;
    out[0] = r0.real(); out[1] = r0.imag(); out[2] = v0.real(); out[3] = v0.imag();
}

template <typename R>
inline void fill_layer_table(const Job &J, LayerW<R> *tab)
{
    const long long work = (long long)J.nw * J.L;
    int nt = (int)std::min<long long>(16, std::max<long long>(1, work / 16384));
    nt = std::min(nt, (int)std::max(1u, std::thread::hardware_concurrency()));
    if (nt <= 1) {
        fill_layer_rows<R>(J, tab, 0, J.nw);
        return;
    }
    std::vector<std::thread> th;
    const int per = (J.nw + nt - 1) / nt;
    for (int t = 0; t < nt; t++) {
        const int a = t * per, b = std::min(J.nw, a + per);
        if (a < b) th.emplace_back(fill_layer_rows<R>, std::cref(J), tab, a, b);
    }
    for (auto &x : th) x.join();
}

}  // namespace grt
