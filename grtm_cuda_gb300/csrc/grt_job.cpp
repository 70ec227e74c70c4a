// grt_job.cpp -- input parsing, source-interface insertion, grid and k grid.
// Rules follow the reference's host code in cusrc/popm/func/green.cu (cited
// per function) so that a reference input file gives the same layer table,
// the same (w,k) list and the same receiver/source placement.
#include "grt_job.h"

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdio>

namespace grt {

using cd = std::complex<double>;
static const double PI = 3.1415926535897932384626433;

// green.cu:2001-2049: a copy of the layer holding the source starts at hs when
// ztop[i-1] < hs < ztop[i]; then thicknesses and mu = b0^2 rho.  The
// reference always adds one layer, reading uninitialised memory when nothing
// was inserted; here the layer count is kept in that case.
static int finish(Job &J, int n, const double *zt, const double *vp, const double *vs, const double *rh,
                  const double *qp, const double *qs, std::string &err)
{
    if (n < 2) { err = "need at least one layer over a half-space"; return kErrModel; }
    for (int i = 1; i < n; i++)
        if (!(zt[i] > zt[i - 1])) { err = "layer tops must increase"; return kErrModel; }
    for (int i = 0; i < n; i++)
        if (!(vp[i] > 0 && vs[i] > 0 && rh[i] > 0 && qp[i] > 0 && qs[i] > 0 && vp[i] > vs[i])) {
            err = "layer " + std::to_string(i) + ": need vp > vs > 0, rho > 0, Q > 0";
            return kErrModel;
        }
    J.h.clear(); J.a0.clear(); J.b0.clear(); J.rho.clear(); J.qp.clear(); J.qs.clear();
    J.inserted = false;
    auto push = [&](double z, int i) {
        J.h.push_back(z); J.a0.push_back(vp[i]); J.b0.push_back(vs[i]);
        J.rho.push_back(rh[i]); J.qp.push_back(qp[i]); J.qs.push_back(qs[i]);
    };
    for (int i = 0; i < n; i++) {
        if (i > 0 && zt[i - 1] < J.hs && zt[i] > J.hs) { push(J.hs, i - 1); J.inserted = true; }
        push(zt[i], i);
    }
    if (!J.inserted && J.hs > zt[n - 1]) { err = "source in the half-space is not supported"; return kErrModel; }
    if (J.hs < 0 || J.hr < 0) { err = "depths must be >= 0"; return kErrModel; }
    J.L = (int)J.h.size();
    if (J.L > 256) { err = "too many layers (max 256 after insertion)"; return kErrModel; }
    J.vmax = 0; J.vmin = 100000;
    for (int i = 0; i < J.L; i++) {                      // green.cu:2034-2037
        J.vmax = std::max(J.vmax, J.a0[i]);
        J.vmin = std::min(J.vmin, J.b0[i]);
    }
    for (int i = 0; i < J.L - 1; i++) J.h[i] = J.h[i + 1] - J.h[i];
    J.mu.resize(J.L);
    for (int i = 0; i < J.L; i++) J.mu[i] = J.b0[i] * J.b0[i] * J.rho[i];
    return kOk;
}

int job_from_layers(int n, const double *ztop, const double *vp, const double *vs, const double *rho,
                    const double *qp, const double *qs, double hs, double hr, int src, Job &J,
                    std::string &err)
{
    if (!ztop || !vp || !vs || !rho || !qp || !qs) { err = "null layer array"; return kErrArg; }
    J = Job();
    J.hs = hs; J.hr = hr; J.src = src ? 1 : 0;
    return finish(J, n, ztop, vp, vs, rho, qp, qs, err);
}

int read_input(const char *path, RawInput &in, std::string &err)
{
    FILE *f = fopen(path, "r");
    if (!f) { err = std::string("cannot open ") + path; return kErrIo; }
    int n = 0;
    bool ok = fscanf(f, "%lf %lf %d", &in.hs, &in.hr, &n) == 3 && n >= 2 && n <= 255;
    if (ok) {
        in.zt.resize(n); in.vp.resize(n); in.vs.resize(n); in.rho.resize(n); in.qp.resize(n); in.qs.resize(n);
    }
    for (int i = 0; ok && i < n; i++)
        ok = fscanf(f, " %lf , %lf , %lf , %lf , %lf , %lf", &in.zt[i], &in.vp[i], &in.vs[i], &in.rho[i], &in.qp[i],
                    &in.qs[i]) == 6;
    ok = ok && fscanf(f, "%lf %lf %d %d %lf %d %lf %lf %d %d", &in.dt, &in.dist, &in.nf1, &in.nf2, &in.twin,
                      &in.log2n, &in.t0, &in.taper, &in.n_ptam, &in.src) == 10;
    fclose(f);
    if (!ok) { err = std::string("malformed input file ") + path; return kErrParse; }
    return kOk;
}

// cal_kmax, green.cu:108-162
static double cal_kmax(const Job &J, cd w, const std::vector<cd> &b, int nf)
{
    const int s = J.s, r = J.rl;
    double pmin = 0, dz = 0, kmax;
    auto sl = [&](int i) { return std::abs(w / b[i]); };
    if (r == s - 1) {
        pmin = std::max(sl(s), sl(s - 1));
        dz = std::min(J.zs, J.h[r] - J.zr);
    } else if (r < s - 1) {
        pmin = std::max(sl(s), sl(s - 1));
        dz = std::min(J.zs, J.hs - J.hr);
        for (int l = r; l <= s - 2; l++) {
            pmin = std::max(pmin, sl(l + 1));
            dz = std::min(dz, J.h[l]);
        }
    } else if (r == s) {
        pmin = sl(s);
        dz = std::fabs(J.hr - J.hs);
    } else if (r == s + 1) {
        pmin = std::max(sl(s), sl(s + 1));
        dz = std::min(J.h[s] - J.zs, J.zr);
    } else {
        pmin = std::max(sl(s), sl(s + 1));
        dz = std::min(J.h[s] - J.zs, std::fabs(J.hr - J.hs));
        for (int l = s + 1; l < r - 1; l++) {
            pmin = std::max(pmin, sl(l));
            dz = std::min(dz, J.h[l]);
        }
    }
    if (dz < 0.2) kmax = nf < 10 ? std::min(pmin + 2.0, 20. * pmin) : std::min(pmin + 2.0, 2.0 * pmin);
    else kmax = std::sqrt((3.0 / dz) * (3.0 / dz) + pmin * pmin);
    if (kmax - pmin < 0.5) kmax = pmin + 0.5;
    return kmax;
}

int job_setup(Job &J, double dt, int log2n, double t0, double taper, double sigma_factor, int k_mode,
              int nk_fixed, double dk_override, int fix, std::string &err, const int *nk_custom,
              const int *k_stride)
{
    if (k_stride && k_mode != 2) { err = "a k stride needs a custom grid (nk_custom)"; return kErrArg; }
    if (k_mode == 2 && !nk_custom) { err = "custom k grid needs nk_custom"; return kErrArg; }
    if (k_mode < 0 || k_mode > 2) { err = "unknown k grid mode"; return kErrArg; }
    if (!(dt > 0) || log2n < 2 || log2n > 15) { err = "need dt > 0 and 2 <= log2n <= 15"; return kErrArg; }
    if (!(taper >= 0 && taper <= 1)) { err = "taper must be in [0, 1]"; return kErrArg; }
    if (!(sigma_factor > 0)) { err = "sigma_factor must be > 0"; return kErrArg; }
    if (k_mode == 1 && nk_fixed < 2) { err = "fixed k grid needs nk >= 2"; return kErrArg; }
    J.dt = dt; J.log2n = log2n; J.t0 = t0; J.taper = taper; J.k_mode = k_mode; J.nk_fixed = nk_fixed;
    J.fix = fix;
    // green.cu:2065-2080
    J.nw = 1 << (log2n - 1);
    J.nwf = J.nw;
    J.fsel.clear();
    J.N = 2 * J.nw;
    const double T = J.N * dt;
    J.df = 1.0 / T;
    J.sigma = sigma_factor / T;
    const double vavg = 0.5 * (J.vmax + J.vmin);
    double Lw = 2.0 * (J.vmax * T + J.vmax / vavg * std::fabs(J.hs - J.hr) + 100.0);
    J.dk = dk_override > 0 ? dk_override : 2 * PI / Lw;
    // source layer, green.cu:2081-2090 (the source sits at the bottom of the
    // layer above an inserted interface)
    double hs = J.hs, hr = J.hr;
    J.s = -1;
    for (int i = 0; i < J.L; i++) {
        if (hs <= J.h[i]) { J.s = i; J.zs = hs; break; }
        hs -= J.h[i];
    }
    // receiver layer, green.cu:2092-2101: the reference tests the reduced
    // source depth; the corrected rule (fix bit 1) tests the receiver depth
    J.rl = -1;
    for (int i = 0; i < J.L; i++) {
        double probe = (fix & 1) ? hr : hs;
        if (probe <= J.h[i]) { J.rl = i; J.zr = hr; break; }
        hr -= J.h[i];
    }
    if (J.s < 0 || J.s > J.L - 2) { err = "source must lie above the half-space"; return kErrModel; }
    if (J.rl < 0) { err = "receiver layer not found"; return kErrModel; }
    // wavenumber grid: ragged per-frequency k_max (green.cu:2145-2194) or fixed
    J.nk.assign(J.nw, 0);
    J.koff.assign(J.nw, 0);
    J.ks.assign(J.nw, 1);
    J.nbrow = 0;
    long long tot = 0;
    J.nkmax = 0;
    std::vector<cd> b(J.L);
    for (int iw = 0; iw < J.nw; iw++) {
        int nk;
        if (k_mode == 2) {
            nk = nk_custom[iw];
            if (nk < 2 || nk > (1 << 24)) { err = "custom k grid: need 2 <= nk <= 2^24 at every frequency"; return kErrArg; }
        } else if (k_mode == 1) {
            nk = nk_fixed;
        } else {
            cd w(2 * PI * J.df * iw, -J.sigma);
            cd lw = std::log(w / (2 * PI));
            for (int i = 0; i < J.L; i++) b[i] = J.b0[i] * (1.0 + lw / (PI * J.qs[i]) + cd(0, 1) / (2.0 * J.qs[i]));
            double km = iw < 3 ? cal_kmax(J, cd(2 * PI * J.df * 3.0, -J.sigma), b, iw) : cal_kmax(J, w, b, iw);
            km *= 1.1;  // k_factor, green.cu:2063
            nk = (int)(km / J.dk) + 2;
        }
        if (k_stride) {
            if (k_stride[iw] < 1 || k_stride[iw] > 64) { err = "k stride must be in 1..64"; return kErrArg; }
            J.ks[iw] = k_stride[iw];
        }
        if ((long long)(nk - 1) * J.ks[iw] + 1 > (1 << 24)) { err = "k grid: (nk - 1) * stride + 1 beyond 2^24 wavenumbers"; return kErrArg; }
        J.nk[iw] = nk;
        J.koff[iw] = tot;
        tot += nk;
        J.nkmax = std::max(J.nkmax, nk);
        J.nbrow = std::max(J.nbrow, (nk - 1) * J.ks[iw] + 1);
    }
    J.nkw = tot;
    return kOk;
}

int job_select(Job &J, int n, const int *sel, std::string &err)
{
    if (n < 1 || !sel) { err = "empty frequency selection"; return kErrArg; }
    if (!J.fsel.empty() || J.nw != J.nwf) { err = "frequencies already selected"; return kErrArg; }
    std::vector<char> seen(J.nwf, 0);
    for (int i = 0; i < n; i++) {
        if (sel[i] < 0 || sel[i] >= J.nwf) { err = "selected frequency out of range (0..N/2-1)"; return kErrArg; }
        if (seen[sel[i]]) { err = "repeated selected frequency"; return kErrArg; }
        seen[sel[i]] = 1;
    }
    std::vector<int> nk(n), ks(n);
    std::vector<long long> koff(n);
    long long tot = 0;
    J.nkmax = 0;
    J.nbrow = 0;
    for (int i = 0; i < n; i++) {
        nk[i] = J.nk[sel[i]];
        ks[i] = J.ks[sel[i]];
        koff[i] = tot;
        tot += nk[i];
        J.nkmax = std::max(J.nkmax, nk[i]);
        J.nbrow = std::max(J.nbrow, (nk[i] - 1) * ks[i] + 1);
    }
    J.nk.swap(nk);
    J.ks.swap(ks);
    J.koff.swap(koff);
    J.nkw = tot;
    J.fsel.assign(sel, sel + n);
    J.nw = n;
    return kOk;
}

int flatten(int n, const double *ztop, const double *vp, const double *vs, double hs, double hr, double r_earth,
            double *ztop_f, double *vp_f, double *vs_f, double *hs_f, double *hr_f, std::string &err)
{
    if (n < 1 || !ztop || !vp || !vs || !ztop_f || !vp_f || !vs_f || !(r_earth > 0)) {
        err = "bad flattening arguments";
        return kErrArg;
    }
    // greent.py:13-47: a layer of thickness h whose bottom lies at radius r is
    // stretched by s = R / (r + h/2), and so are its velocities; the tops of the
    // flat model are the running sum of the stretched thicknesses; the half-space
    // takes the factor at its top
    double r = r_earth, top = 0.0;
    for (int i = 0; i < n; i++) {
        const double h = i + 1 < n ? ztop[i + 1] - ztop[i] : 0.0;
        if (!(h >= 0)) { err = "layer tops must increase"; return kErrModel; }
        r -= h;
        if (!(r > 0)) { err = "model deeper than the Earth radius"; return kErrModel; }
        const double sc = r_earth / (r + 0.5 * h);
        ztop_f[i] = top;
        vp_f[i] = vp[i] * sc;
        vs_f[i] = vs[i] * sc;
        top += h * sc;
    }
    // greent.py:65-67: depths by z_f = R ln(R / (R - z))
    auto fz = [&](double z) { return r_earth * std::log(r_earth / (r_earth - z)); };
    if (!(hs < r_earth) || !(hr < r_earth)) { err = "depth beyond the Earth radius"; return kErrModel; }
    if (hs_f) *hs_f = fz(hs);
    if (hr_f) *hr_f = fz(hr);
    return kOk;
}

}  // namespace grt
