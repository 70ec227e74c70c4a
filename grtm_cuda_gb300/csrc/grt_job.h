// grt_job.h -- host-side description of one GRT job: the layered model after
// source-interface insertion, the time/frequency grid and the wavenumber grid.
#pragma once
#include <string>
#include <vector>

namespace grt {

struct Job {
    // model (green.cu:1995-2049)
    int L = 0;                                   // layers after insertion
    std::vector<double> h, a0, b0, rho, qp, qs, mu;
    bool inserted = false;
    double hs = 0, hr = 0;                       // source / receiver depth as given
    int s = 0, rl = 0;                           // source / receiver layer
    double zs = 0, zr = 0;                       // depth below the layer top
    int src = 0;                                 // 0 single force, 1 moment tensor
    // fields of the input file that only the file writer uses
    double dist0 = 0, twin = 0;
    int nf1 = 0, nf2 = 0, n_ptam = 0;
    // time / frequency grid (green.cu:2051-2080)
    double dt = 0, t0 = 0, taper = 0;
    int log2n = 0, nw = 0, N = 0;                // nw: frequency rows evaluated
    int nwf = 0;                                 // positive frequencies of the grid (N/2)
    std::vector<int> fsel;                       // frequency of each row (empty: row = frequency)
    double df = 0, sigma = 0, dk = 0, vmax = 0, vmin = 0;
    // wavenumber grid
    int k_mode = 0, nk_fixed = 0, fix = 0;
    std::vector<int> nk;                         // per frequency
    std::vector<long long> koff;                 // prefix sums of nk
    long long nkw = 0;
    int nkmax = 0;
    std::vector<int> ks;                         // per frequency k stride m: k_j = j m dk
    int nbrow = 0;                               // Bessel-table rows: max (nk - 1) m + 1
};

// status codes (the public header repeats them)
enum { kOk = 0, kErrArg = 1, kErrIo = 2, kErrParse = 3, kErrModel = 4, kErrCuda = 5, kErrNoMem = 6,
       kErrTimeout = 7, kErrUnsupported = 8 };

// The reference's positional input file, as read (green.cu:1995-2060).
struct RawInput {
    double hs = 0, hr = 0;
    std::vector<double> zt, vp, vs, rho, qp, qs;   // layer tops and properties
    double dt = 0, dist = 0, twin = 0, t0 = 0, taper = 0;
    int nf1 = 0, nf2 = 0, log2n = 0, n_ptam = 0, src = 0;
};
int read_input(const char *path, RawInput &in, std::string &err);
// Layers given by depth-to-top (ztop[0] = 0; the last layer is the half-space).
int job_from_layers(int n, const double *ztop, const double *vp, const double *vs, const double *rho,
                    const double *qp, const double *qs, double hs, double hr, int src, Job &J,
                    std::string &err);
// Grid, layer location and k grid.  sigma = sigma_factor / T (reference: 2).
int job_setup(Job &J, double dt, int log2n, double t0, double taper, double sigma_factor, int k_mode,
              int nk_fixed, double dk_override, int fix, std::string &err, const int *nk_custom = nullptr,
              const int *k_stride = nullptr);

// Keep only the frequencies sel[0..n) (distinct, 0 <= sel[i] < N/2, any
// order) as the job's rows, with their wavenumber grids.
int job_select(Job &J, int n, const int *sel, std::string &err);
// frequency index of row iw
inline int job_freq(const Job &J, int iw) { return J.fsel.empty() ? iw : J.fsel[iw]; }

// Earth-flattening transform of a spherical layered model (the reference's
// caller-side step, greent.py:13-47 and 65-67); density and Q unchanged.
int flatten(int n, const double *ztop, const double *vp, const double *vs, double hs, double hr, double r_earth,
            double *ztop_f, double *vp_f, double *vs_f, double *hs_f, double *hr_f, std::string &err);

}  // namespace grt
