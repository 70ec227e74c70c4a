// grt_noalloc.cu -- Green's functions for callers that cannot allocate device
// memory.
//
// Some callers cannot call cudaMalloc: a host process whose GPU memory is
// reserved up front by another runtime (a framework's caching allocator, a
// service with a fixed device-memory budget), or code running where device
// allocation is not permitted.  grt_run_noalloc computes the same traces as
// grt_run for small jobs without allocating anything on the device: every
// intermediate buffer (per-frequency layer tables, the (w,k) coefficient
// columns, the Bessel table, the spectra and the traces before download)
// lives in one file-scope device array of kScratchBytes.  The host-side job
// tables are staged in a file-scope host array of kStageBytes.
//
// Set-up: every call makes its device current and looks up the array's device
// address there with cudaGetSymbolAddress (cheap, allocates nothing), so a
// context torn down and recreated by the caller (cudaDeviceReset) never leaves
// a stale address behind.  The call copies synchronously and waits for its
// kernels, so no part of it may be captured into a CUDA graph.  A device takes
// the array when the library's kernels are first loaded there (with CUDA's
// default lazy loading, at the first grt_run_noalloc call on that device;
// with CUDA_MODULE_LOADING=EAGER, when the context is created) and holds it
// until the process exits.  All calls share the array (and the host staging
// array): calls that overlap on the GPU, or run from several host threads at
// once, race.  The only scratch word that must start at zero (the device
// error flag) is cleared by every call; all other scratch is fully written
// before it is read.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstring>
#include <string>

#include "../../include/grtm_gb300.h"
#include "grt_fft.cuh"
#include "grt_launch.h"
#include "grt_integrate.cuh"
#include "grt_job.h"
#include "grt_kernel.cuh"
#include "grt_tables.h"

namespace {

constexpr size_t kScratchBytes = 32ull << 20;  // device scratch per GPU: 32 MiB
constexpr size_t kStageBytes = 4ull << 20;     // host staging of the job tables: 4 MiB
constexpr double PI = 3.1415926535897932384626433;

}  // namespace

static __device__ __align__(256) unsigned char g_grt_scratch[kScratchBytes];
alignas(256) static unsigned char g_grt_stage[kStageBytes];

static size_t up256(size_t n) { return (n + 255) & ~size_t(255); }

static int fail(int code, const std::string &msg)
{
    fprintf(stderr, "grt_run_noalloc: %s (%s)\n", grt_status_string(code), msg.c_str());
    return code;
}

#define CUN(call)                                                                        \
    do {                                                                                 \
        cudaError_t e_ = (call);                                                         \
        if (e_ != cudaSuccess) return fail(GRT_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

extern "C" GRT_API int grt_run_noalloc(int device, const grt_model *m, const grt_opts *o, int n_dist,
                                       const double *dist, double *traces)
{
    using grt::Job;
    using cd = std::complex<double>;
    if (!m || !o || !dist || !traces || n_dist < 1) return fail(GRT_ERR_ARG, "null argument or no receivers");
    if (device < 0) return fail(GRT_ERR_ARG, "device ordinal out of range");
    if (o->precision != GRT_FP32) return fail(GRT_ERR_ARG, "the allocation-free entry point runs in FP32 only");
    for (int i = 0; i < n_dist; i++)
        if (!(dist[i] > 0)) return fail(GRT_ERR_ARG, "distances must be > 0");

    // the scratch array's address on this device, looked up on every call with
    // the device current (host code must never pass g_grt_scratch itself: in
    // host code that name is a host-side stand-in, not a device address)
    CUN(cudaSetDevice(device));
    unsigned char *scratch = nullptr;
    {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_grt_scratch);
        if (e != cudaSuccess || !p)
            return fail(GRT_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
        scratch = (unsigned char *)p;
    }

    if (o->k_mode == GRT_K_CUSTOM || o->k_stride) return fail(GRT_ERR_UNSUPPORTED, "custom k grids need grt_run");
    if (o->fix & (GRT_FIX_COLS | GRT_FIX_COLS20)) return fail(GRT_ERR_UNSUPPORTED, "corrected column layouts need grt_run");
    if (o->n_freq_sel > 0 || o->freq_sel) return fail(GRT_ERR_UNSUPPORTED, "frequency selections need a plan");
    if (o->k_slice) return fail(GRT_ERR_UNSUPPORTED, "a fixed k_slice needs a plan");
    // the job on the host (same rules as grt_run)
    Job J;
    std::string err;
    int rc = grt::job_from_layers(m->n_layer, m->ztop, m->vp, m->vs, m->rho, m->qp, m->qs, m->hs, m->hr,
                                  m->src_type, J, err);
    if (!rc) rc = grt::job_setup(J, o->dt, o->log2n, o->t0, o->taper, o->sigma_factor, o->k_mode, o->nk_fixed,
                                 o->dk, o->fix, err);
    if (rc) return fail(rc, err);
    const int L = J.L, nw = J.nw, N = J.N, nd = n_dist;
    const int nc = J.src == 0 ? grt::kSingleNC : grt::kTensorNC;
    const int nq = J.src == 0 ? (int)grt::QS_N : (int)grt::QT_N;
    long long ntiles = 0;
    for (int iw = 0; iw < nw; iw++) ntiles += (J.nk[iw] + grt::kGrtThreads - 1) / grt::kGrtThreads;
    if ((size_t)N * sizeof(grt::C<float>) > 128 * 1024) return fail(GRT_ERR_UNSUPPORTED, "N above 16384");

    // layout: staged tables first (same offsets on host and device), then work buffers
    using LW = grt::LayerW<float>;
    size_t off = 0;
    const size_t o_tab = off; off = up256(off + (size_t)nw * L * sizeof(LW));
    const size_t o_tiles = off; off = up256(off + (size_t)ntiles * sizeof(int2));
    const size_t o_nk = off; off = up256(off + (size_t)nw * sizeof(int));
    const size_t o_koff = off; off = up256(off + (size_t)nw * sizeof(long long));
    const size_t o_dist = off; off = up256(off + (size_t)nd * sizeof(double));
    const size_t o_post = off; off = up256(off + (size_t)nw * 2 * sizeof(float));
    // twiddles: e^{2 pi i m/N} (N/2 complex), then the spectral kernel's pass table (< N/2)
    const size_t o_tw = off; off = up256(off + (size_t)2 * N * sizeof(float));
    const size_t o_damp = off; off = up256(off + (size_t)N * sizeof(float));
    const size_t staged = off;
    const size_t o_K = off; off = up256(off + (size_t)nq * J.nkw * 2 * sizeof(float));
    const size_t o_B = off; off = up256(off + (size_t)J.nkmax * grt::NBASIS * nd * sizeof(float));
    const size_t o_S = off; off = up256(off + (size_t)nd * nc * nw * 2 * sizeof(float));
    const size_t o_sig = off; off = up256(off + (size_t)nd * nc * N * sizeof(float));
    const size_t o_err = off; off = up256(off + sizeof(unsigned));
    if (off > kScratchBytes || staged > kStageBytes) {
        char msg[256];
        snprintf(msg, sizeof msg,
                 "job needs %.1f MiB of device scratch and %.1f MiB of host staging; this entry point holds "
                 "%zu MiB and %zu MiB (use grt_run for larger jobs)",
                 off / 1048576.0, staged / 1048576.0, kScratchBytes >> 20, kStageBytes >> 20);
        return fail(GRT_ERR_UNSUPPORTED, msg);
    }

    // per-frequency tables into the host staging array (attenuation green.cu:177-180,
    // phase/taper/scale 1905-1921, de-damping 2236-2237)
    unsigned char *h = g_grt_stage;
    LW *tab = (LW *)(h + o_tab);
    grt::fill_layer_table<float>(J, tab);
    int2 *tiles = (int2 *)(h + o_tiles);
    long long t = 0;
    for (int iw = 0; iw < nw; iw++)
        for (int j0 = 0; j0 < J.nk[iw]; j0 += grt::kGrtThreads) tiles[t++] = make_int2(iw, j0);
    memcpy(h + o_nk, J.nk.data(), (size_t)nw * sizeof(int));
    memcpy(h + o_koff, J.koff.data(), (size_t)nw * sizeof(long long));
    memcpy(h + o_dist, dist, (size_t)nd * sizeof(double));
    float *post = (float *)(h + o_post);
    const int wc = (int)((double)nw * (1 - J.taper));
    const double coef = J.df * nw / PI;
    for (int iw = 0; iw < nw; iw++) {
        double st0 = iw > wc ? 0.5 * (1. + std::cos((iw - wc + 1) * PI / (nw - wc + 1))) : 1.0;
        double phi = 2 * PI * J.df * iw * J.t0;
        post[2 * iw] = (float)(std::cos(phi) * st0 * coef);
        post[2 * iw + 1] = (float)(std::sin(phi) * st0 * coef);
    }
    float *tw = (float *)(h + o_tw);
    for (int k = 0; k < N / 2; k++) {
        tw[2 * k] = (float)std::cos(2 * PI * k / N);
        tw[2 * k + 1] = (float)std::sin(2 * PI * k / N);
    }
    grt::fft::pass_twiddles(J.log2n, tw + N);
    // the FP32 spectral stage takes the de-damping factors in FP32
    float *damp = (float *)(h + o_damp);
    for (int n = 0; n < N; n++) damp[n] = (float)(std::exp(n * J.dt * J.sigma) * std::exp(J.t0 * J.sigma) / (double)N);
    float slot0[4];
    {
        const LW &t0r = tab[J.rl];
        cd r0 = std::sqrt(cd(-t0r.wa2x, -t0r.wa2y)), v0 = std::sqrt(cd(-t0r.wb2x, -t0r.wb2y));
        if (r0.real() < 0) r0 = -r0;
        if (v0.real() < 0) v0 = -v0;
        slot0[0] = (float)r0.real(); slot0[1] = (float)r0.imag(); slot0[2] = (float)v0.real(); slot0[3] = (float)v0.imag();
    }

    // upload, clear the error word, run the four kernels on the default stream
    const cudaStream_t st = 0;
    CUN(cudaMemcpy(scratch, g_grt_stage, staged, cudaMemcpyHostToDevice));
    CUN(cudaMemsetAsync(scratch + o_err, 0, sizeof(unsigned), st));
    grt::GrtArgs<float> A{};
    A.tab = (const LW *)(scratch + o_tab);
    A.tiles = (const int2 *)(scratch + o_tiles);
    A.nk = (const int *)(scratch + o_nk);
    A.koff = (const long long *)(scratch + o_koff);
    A.K = (float *)(scratch + o_K);
    A.nkw = J.nkw;
    A.dk = J.dk;
    A.zs = J.zs;
    A.zr = J.zr;
    A.hs_layer = J.h[J.s];
    A.hr_layer = J.h[J.rl];
    A.L = L; A.s = J.s; A.rl = J.rl; A.src = J.src; A.fix = J.fix; A.nq = nq;
    for (int i = 0; i < 4; i++) A.slot0[i] = slot0[i];
    A.err = (unsigned *)(scratch + o_err);
    CUN(grt::grt_point_launch<float>(A, grt::kSpecGeneric, (unsigned)ntiles, (size_t)L * sizeof(LW), st, nullptr));
    {
        long long n = (long long)J.nkmax * nd;
        grt::bessel_table_kernel<float><<<(unsigned)((n + 255) / 256), 256, 0, st>>>(
            (float *)(scratch + o_B), J.nkmax, nd, J.dk, (const double *)(scratch + o_dist), 0, 0);
        CUN(cudaGetLastError());
    }
    {
        grt::KsumArgs<float> S{};
        S.K = (const float *)(scratch + o_K);
        S.B = (const float *)(scratch + o_B);
        S.nk = A.nk;
        S.koff = A.koff;
        S.dist = (const double *)(scratch + o_dist);
        S.S = (float *)(scratch + o_S);
        S.nkw = J.nkw; S.dk = J.dk; S.nw = nw; S.nr = nd;
        S.rt = 128;
        while (S.rt > 1 && S.rt / 2 >= nd) S.rt /= 2;
        S.jt = 128 / S.rt;
        unsigned grid = (unsigned)(nw * ((nd + S.rt - 1) / S.rt));
        if (J.src == 0) grt::ksum_kernel<float, grt::kSingle><<<grid, grt::kSumThreads, 0, st>>>(S);
        else grt::ksum_kernel<float, grt::kTensor><<<grid, grt::kSumThreads, 0, st>>>(S);
        CUN(cudaGetLastError());
    }
    {
        grt::fft::C2RArgs F{};
        F.S = (const float2 *)(scratch + o_S);
        F.post = (const float2 *)(scratch + o_post);
        F.tw = (const float2 *)(scratch + o_tw);
        F.twp = (const float2 *)(scratch + o_tw) + N / 2;
        F.damp = (const float *)(scratch + o_damp);
        F.out = (float *)(scratch + o_sig);
        CUN(grt::fft::launch_c2r(F, (long long)nd * nc, J.log2n, st));
    }
    CUN(cudaStreamSynchronize(st));
    unsigned herr = 0;
    CUN(cudaMemcpy(&herr, scratch + o_err, sizeof herr, cudaMemcpyDeviceToHost));
    if (herr) return fail(GRT_ERR_TIMEOUT, "a bounded device wait gave up (layer-table copy)");

    // download the FP32 traces into the front half of the caller's buffer and
    // widen them in place, from the end, to doubles
    const size_t nval = (size_t)nd * nc * N;
    CUN(cudaMemcpy(traces, scratch + o_sig, nval * sizeof(float), cudaMemcpyDeviceToHost));
    unsigned char *bytes = (unsigned char *)traces;
    for (size_t i = nval; i-- > 0;) {
        float v;
        memcpy(&v, bytes + i * sizeof(float), sizeof v);
        double d = v;
        memcpy(bytes + i * sizeof(double), &d, sizeof d);
    }
    return GRT_OK;
}
