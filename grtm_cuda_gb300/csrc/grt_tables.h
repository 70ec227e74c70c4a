// grt_tables.h -- host construction of the per-(frequency, layer) table the
// GRT kernel stages in shared memory.
#pragma once
#include <complex>
#include <cstring>

#include "grt_job.h"
#include "grt_types.h"

namespace grt {

// Complex frequency w = 2 pi df iw - i sigma; attenuated velocities by the
// reference's constant-Q dispersion (set_pars, green.cu:177-180); then
// (w/alpha)^2, (w/beta)^2, their difference and its inverse, rounded to R,
// with the double-float low words the FP32 kernel needs.  tab: [nw][L].
template <typename R>
inline void fill_layer_table(const Job &J, LayerW<R> *tab)
{
    using cd = std::complex<double>;
    const double pi = 3.14159265358979323846;
    const bool f32 = sizeof(R) == 4;
    auto lo = [](double x) { return (float)(x - (double)(float)x); };
    for (int iw = 0; iw < J.nw; iw++) {
        cd w(2 * pi * J.df * iw, -J.sigma);
        cd lw = std::log(w / (2 * pi));
        for (int i = 0; i < J.L; i++) {
            cd cs = 1.0 + lw / (pi * J.qs[i]) + cd(0, 1) / (2.0 * J.qs[i]);
            cd cp = 1.0 + lw / (pi * J.qp[i]) + cd(0, 1) / (2.0 * J.qp[i]);
            cd a = J.a0[i] * cp, b = J.b0[i] * cs;
            cd wa = w / a, wb = w / b;
            cd wa2 = wa * wa, wb2 = wb * wb, W = wb2 - wa2, iW = 1.0 / W;
            LayerW<R> &t = tab[(size_t)iw * J.L + i];
            std::memset(&t, 0, sizeof t);
            t.wa2x = wa2.real(); t.wa2y = wa2.imag(); t.wb2x = wb2.real(); t.wb2y = wb2.imag();
            t.wa2[0] = (R)wa2.real(); t.wa2[1] = (R)wa2.imag();
            t.wb2[0] = (R)wb2.real(); t.wb2[1] = (R)wb2.imag();
            t.W[0] = (R)W.real(); t.W[1] = (R)W.imag();
            t.iW[0] = (R)iW.real(); t.iW[1] = (R)iW.imag();
            t.a[0] = (R)a.real(); t.a[1] = (R)a.imag();
            t.b[0] = (R)b.real(); t.b[1] = (R)b.imag();
            t.mu = (R)J.mu[i];
            t.h = (R)J.h[i];
            // low words: the FP64 kernel carries none
            if (f32) {
                t.wa2lo = lo(wa2.real());
                t.wb2lo = lo(wb2.real());
                t.wa2ylo = lo(wa2.imag());
                t.wb2ylo = lo(wb2.imag());
                t.hlo = lo(J.h[i]);
            }
        }
    }
}

}  // namespace grt
