// grt_api.cu -- C ABI: contexts, plans, kernel launches and the reference's
// file-to-file entry point green().
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <tuple>
#include <memory>
#include <string>
#include <type_traits>
#include <vector>

#include "../../include/grtm_gb300.h"
#include "grt_integrate.cuh"
#include "grt_job.h"
#include "grt_kernel.cuh"
#include "grt_tables.h"
#include "grt_ksum_tc.cuh"
#include "grt_fft.cuh"
#include "grt_launch.h"

using grt::Job;
using cd = std::complex<double>;
static const double PI = 3.1415926535897932384626433;

#include <cublas_v2.h>

#include "grt_ctx.h"

struct grt_plan {
    grt_ctx *ctx = nullptr;
    Job J;
    int prec = 0;
    int nd = 0, nc = 0, nq = 0, ntiles = 0;
    int rt = 128, jt = 1;
    int use_tc = 0, nsplit = 1, kslice = 0;   // tensor-core wavenumber sum and its split-K
    // plain FP32 sum as SGEMMs (unit k strides, outside batches): planar
    // coefficients [nq][2][nw][nkp], one Bessel operand [nkp][nd], pair products
    // [gslices][np][2][nw][nd]
    bool gemm_ok = false;
    float *Ag = nullptr, *Bg = nullptr, *Dg = nullptr;
    int nkp = 0, gslices = 1;
    int kslice_req = 0;                       // requested k per slice (0: chosen here)
    int tc_bf16 = 0;                          // tensor-core sum in the 3xBF16 form (else 3xTF32)
    int nsplit_default = 1;                   // the wave-filling split (before batch tuning)
    size_t P_bytes = 0;                       // capacity of the split-K partial sums
    int gspec = 0;                            // compiled form of the GRT evaluation (grt::GrtSpec)
    int bt_rows = 0;                          // > 0: Bessel table tiled by 32 receivers (unit strides)
    int cols = 0;                             // output column layout (grt::ColKind)
    void *P = nullptr;                        // split-K partial sums
    float *Kt = nullptr;                      // coefficients in GEMM operand layout
    long long *kt_base = nullptr;             // per frequency tile offset into Kt (floats)
    std::vector<double> dist;
    double slot0[4] = {0, 0, 0, 0};
    // device buffers
    void *tab = nullptr, *K = nullptr, *B = nullptr, *S = nullptr, *post = nullptr, *tw = nullptr;
    void *spec = nullptr, *sig = nullptr;
    int2 *tiles = nullptr;
    int *nk = nullptr, *ks = nullptr;
    long long *koff = nullptr, *tfirst = nullptr;
    double *ddist = nullptr, *damp = nullptr;
    float *dampf = nullptr;                   // FP32 plans: the de-damping factors in FP32 (c2r_kernel)
    float *twp = nullptr;                     // FP32 plans: the c2r_kernel's pass twiddles
    float *rdu = nullptr;                     // two-pass GRT evaluation: R^du at the source between the passes
    unsigned *derr = nullptr;
    bool own_derr = true;                     // false inside a batch (the batch's error word)
    bool ran = false;                         // executed at least once (traces on the device)
    bool spec_valid = false;                  // full plans: spec holds the last execute's spectra
    unsigned long long *nlev = nullptr;       // kNlevSlots counters of layers the GRT kernel evaluated
    bool own_nlev = true;                     // false inside a batch (the batch's counters)
    grt_report rep{};
};

static int set_err(grt_ctx *ctx, int code, const std::string &msg)
{
    if (ctx) ctx->err = msg;
    return code;
}

#define CU(call)                                                                                        \
    do {                                                                                                \
        cudaError_t e_ = (call);                                                                        \
        if (e_ != cudaSuccess)                                                                          \
            return set_err(ctx, e_ == cudaErrorMemoryAllocation ? GRT_ERR_NOMEM : GRT_ERR_CUDA,          \
                           std::string(#call) + ": " + cudaGetErrorString(e_));                        \
    } while (0)

// ------------------------------------------------------------------ device memory
// Plans and batches take their device memory from the context's cache:
// blocks a destroyed plan releases are kept (up to half the device memory)
// and handed to the next request of a similar size, so a plan or batch made
// per call pays neither cudaMalloc's page mapping nor cudaFree's device-wide
// synchronisation.  All work on a context's memory is ordered on its stream
// (batch graphs join their side streams back into it; the auxiliary stream's
// set-up and fetch work is queued after it by an event and synchronised by the
// host before the call returns), so a block is reused only by work queued
// after the work that last used it.
static size_t pool_round(size_t n)
{
    const size_t g = n < ((size_t)1 << 20) ? 256 : ((size_t)2 << 20);
    return (std::max<size_t>(n, 1) + g - 1) / g * g;
}

static void pool_trim(grt_ctx *ctx, size_t keep)
{
    while (ctx->pooled > keep && !ctx->pool.empty()) {
        auto it = std::prev(ctx->pool.end());   // largest first
        cudaFree(it->second);
        ctx->pooled -= it->first;
        ctx->pool.erase(it);
    }
}

template <typename T>
static cudaError_t dev_alloc(grt_ctx *ctx, T **out, size_t bytes)
{
    const size_t n = pool_round(bytes);
    void *p = nullptr;
    auto it = ctx->pool.lower_bound(n);
    if (it != ctx->pool.end() && it->first <= n + n / 8) {
        p = it->second;
        ctx->live[p] = it->first;
        ctx->pooled -= it->first;
        ctx->pool.erase(it);
        *out = (T *)p;
        return cudaSuccess;
    }
    cudaError_t e = cudaMalloc(&p, n);
    if (e == cudaErrorMemoryAllocation && ctx->pooled) {
        cudaGetLastError();
        pool_trim(ctx, 0);
        e = cudaMalloc(&p, n);
    }
    if (e != cudaSuccess) {
        *out = nullptr;
        return e;
    }
    ctx->live[p] = n;
    *out = (T *)p;
    return cudaSuccess;
}

static void dev_free(grt_ctx *ctx, void *p)
{
    if (!p) return;
    auto it = ctx->live.find(p);
    if (it == ctx->live.end()) {
        cudaFree(p);
        return;
    }
    ctx->pool.emplace(it->second, p);
    ctx->pooled += it->second;
    ctx->live.erase(it);
    if (ctx->pooled > ctx->pool_cap) pool_trim(ctx, ctx->pool_cap);
}

// set-up and fetch work runs on the context's auxiliary stream (grt_ctx.h)
static cudaError_t setup_stream(grt_ctx *ctx, cudaStream_t *st) { return grt_setup_stream(ctx, st); }

extern "C" void grt_trim(grt_ctx *ctx)
{
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    pool_trim(ctx, 0);
}

extern "C" const char *grt_status_string(int s)
{
    switch (s) {
    case GRT_OK: return "ok";
    case GRT_ERR_ARG: return "invalid argument";
    case GRT_ERR_IO: return "i/o error";
    case GRT_ERR_PARSE: return "malformed input file";
    case GRT_ERR_MODEL: return "unsupported layered model";
    case GRT_ERR_CUDA: return "CUDA error";
    case GRT_ERR_NOMEM: return "out of memory";
    case GRT_ERR_TIMEOUT: return "device wait timed out";
    case GRT_ERR_UNSUPPORTED: return "unsupported size";
    default: return "unknown status";
    }
}

extern "C" int grt_create(grt_ctx **out, int device)
{
    if (!out) return GRT_ERR_ARG;
    *out = nullptr;
    std::unique_ptr<grt_ctx> c(new grt_ctx);
    grt_ctx *ctx = c.get();
    c->device = device;
    CU(cudaSetDevice(device));
    CU(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
    int least = 0, greatest = 0;
    CU(cudaDeviceGetStreamPriorityRange(&least, &greatest));
    CU(cudaStreamCreateWithPriority(&c->aux, cudaStreamNonBlocking, greatest));
    CU(cudaEventCreateWithFlags(&c->aux_ev, cudaEventDisableTiming));
    for (auto &e : c->ev) CU(cudaEventCreate(&e));
    size_t free_b = 0, total_b = 0;
    CU(cudaMemGetInfo(&free_b, &total_b));
    c->pool_cap = total_b / 2;
    *out = c.release();
    return GRT_OK;
}

extern "C" void grt_destroy(grt_ctx *ctx)
{
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    for (auto &e : ctx->ev)
        if (e) cudaEventDestroy(e);
    if (ctx->stream) {
        cudaStreamSynchronize(ctx->stream);
        cudaStreamDestroy(ctx->stream);
    }
    if (ctx->aux) {
        cudaStreamSynchronize(ctx->aux);
        cudaStreamDestroy(ctx->aux);
    }
    if (ctx->aux_ev) cudaEventDestroy(ctx->aux_ev);
    if (ctx->blas) cublasDestroy((cublasHandle_t)ctx->blas);
    pool_trim(ctx, 0);
    delete ctx;
}

extern "C" int grt_device_synchronize(int device)
{
    cudaError_t e = cudaSetDevice(device);
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    return e == cudaSuccess ? GRT_OK : GRT_ERR_CUDA;
}

extern "C" int grt_set_priority(grt_ctx *ctx, int high)
{
    if (!ctx) return GRT_ERR_ARG;
    if (!ctx->live.empty()) return set_err(ctx, GRT_ERR_ARG, "grt_set_priority: the context holds plans or batches");
    CU(cudaSetDevice(ctx->device));
    int least = 0, greatest = 0;
    CU(cudaDeviceGetStreamPriorityRange(&least, &greatest));
    const int prio = high ? greatest : 0;
    if (prio == ctx->priority) return GRT_OK;
    cudaStream_t s = nullptr;
    CU(cudaStreamCreateWithPriority(&s, cudaStreamNonBlocking, prio));
    cudaStreamSynchronize(ctx->stream);
    cudaStreamDestroy(ctx->stream);
    ctx->stream = s;
    ctx->priority = prio;
    return GRT_OK;
}

extern "C" const char *grt_last_error(const grt_ctx *ctx) { return ctx ? ctx->err.c_str() : "no context"; }

extern "C" void grt_plan_destroy(grt_plan *p)
{
    if (!p) return;
    cudaSetDevice(p->ctx->device);
    cudaStreamSynchronize(p->ctx->aux);   // set-up left in flight by a failed creation
    void *bufs[] = {p->tab, p->K, p->B, p->S, p->post, p->tw, p->spec, p->sig, p->tiles, p->nk, p->koff, p->ddist,
                    p->damp, p->dampf, p->twp, p->rdu, p->own_derr ? p->derr : nullptr, p->P, p->Kt, p->kt_base, p->ks, p->tfirst,
                    p->Ag, p->Bg, p->Dg, p->own_nlev ? p->nlev : nullptr};
    for (void *b : bufs) dev_free(p->ctx, b);
    delete p;
}

// Raise a kernel's dynamic shared-memory limit (never lower it: a captured
// graph replays launches of several sizes).  One table for all contexts; a
// context itself is used from one host thread at a time.
template <typename F>
static cudaError_t raise_smem_limit(F *kernel, int bytes)
{
    static std::map<std::pair<int, const void *>, int> current;   // (device, kernel) -> limit set
    static std::mutex mu;   // contexts on other host threads share the table
    std::lock_guard<std::mutex> lock(mu);
    int dev = 0;
    cudaGetDevice(&dev);
    int &cur = current[{dev, (const void *)kernel}];
    if (bytes <= cur) return cudaSuccess;
    cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e == cudaSuccess) cur = bytes;
    return e;
}

// output column layout, count and coefficient columns of a job
static int col_kind(const Job &J)
{
    const bool fix = (J.fix & grt::kFixCols) != 0, fix20 = (J.fix & grt::kFixCols20) != 0;
    if (J.src == 0) return (fix || fix20) ? grt::kColSingleFix : grt::kColSingle;
    return fix ? grt::kColTensorFix : (fix20 ? grt::kColTensorFix20 : grt::kColTensor);
}
static int col_count(int kind)
{
    return kind == grt::kColTensorFix ? grt::kTensorFixNC
                                      : ((kind == grt::kColTensor || kind == grt::kColTensorFix20) ? grt::kTensorNC
                                                                                                : grt::kSingleNC);
}
// the tensor-core plan of a column layout (the 30-column layout has none: SIMT sums)
static grt::TcPlan tc_plan(int kind)
{
    static constexpr grt::TcPlan ts = grt::make_tcplan<grt::kColSingle>(), tt = grt::make_tcplan<grt::kColTensor>(),
                                 tsf = grt::make_tcplan<grt::kColSingleFix>(),
                                 tt20 = grt::make_tcplan<grt::kColTensorFix20>();
    switch (kind) {
    case grt::kColTensor: return tt;
    case grt::kColSingleFix: return tsf;
    case grt::kColTensorFix20: return tt20;
    case grt::kColTensorFix: {
        grt::TcPlan none{};
        for (int q = 0; q < 16; q++) none.qslot[q] = -1;
        return none;
    }
    default: return ts;
    }
}
// operand tiles per stage block of the tensor-core sum (coefficient columns it reads)
static int tc_tiles(int kind)
{
    return kind == grt::kColTensorFix ? 0 : tc_plan(kind).nqu;
}
static const grt::ColTerms kColTermsTab[5] = {grt::make_colterms<grt::kColSingle>(), grt::make_colterms<grt::kColTensor>(),
                                              grt::make_colterms<grt::kColSingleFix>(),
                                              grt::make_colterms<grt::kColTensorFix>(),
                                              grt::make_colterms<grt::kColTensorFix20>()};

static int coef_count(int kind)
{
    return kind == grt::kColTensorFix ? 2 * (int)grt::QT_N
                                      : ((kind == grt::kColTensor || kind == grt::kColTensorFix20) ? (int)grt::QT_N
                                                                                                : (int)grt::QS_N);
}

// ------------------------------------------------------------------ host tables
template <typename R>
static void build_tables(const Job &J, std::vector<grt::LayerW<R>> &tab, std::vector<R> &post, std::vector<R> &tw,
                         std::vector<double> &damp)
{
    const int L = J.L, nw = J.nw, nwf = J.nwf, N = J.N;
    tab.resize((size_t)nw * L);
    grt::fill_layer_table<R>(J, tab.data());
    // phase e^{i w_r t0}, cosine taper and scale df nw / pi (green.cu:1905-1921),
    // nw the grid's positive frequencies, at the frequency of each row
    post.resize(2 * (size_t)nw);
    const int wc = (int)((double)nwf * (1 - J.taper));
    const double coef = J.df * nwf / PI;
    for (int row = 0; row < nw; row++) {
        const int iw = grt::job_freq(J, row);
        double st0 = iw > wc ? 0.5 * (1. + std::cos((iw - wc + 1) * PI / (nwf - wc + 1))) : 1.0;
        double phi = 2 * PI * J.df * iw * J.t0;
        post[2 * row] = (R)(std::cos(phi) * st0 * coef);
        post[2 * row + 1] = (R)(std::sin(phi) * st0 * coef);
    }
    tw.resize(N);  // N/2 complex
    for (int m = 0; m < N / 2; m++) {
        tw[2 * m] = (R)std::cos(2 * PI * m / N);
        tw[2 * m + 1] = (R)std::sin(2 * PI * m / N);
    }
    // Re(x_n) / N e^{sigma n dt} e^{sigma t0} (green.cu:2236-2237)
    damp.resize(N);
    for (int n = 0; n < N; n++) damp[n] = std::exp(n * J.dt * J.sigma) * std::exp(J.t0 * J.sigma) / (double)N;
}

// the tensor-core sum's k split: at most 64 slices of at least 8 stages
static int tc_max_split(const grt_plan *p)
{
    const int KT = p->tc_bf16 ? grt::tc::TcPrec<grt::tc::kBF16>::KT : grt::tc::TcPrec<grt::tc::kTF32>::KT;
    return std::max(1, std::min(64, p->J.nkmax / (8 * KT)));
}
static void set_tc_split(grt_plan *p, int s)
{
    const int KT = p->tc_bf16 ? grt::tc::TcPrec<grt::tc::kBF16>::KT : grt::tc::TcPrec<grt::tc::kTF32>::KT;
    s = std::max(1, std::min(tc_max_split(p), s));
    p->kslice = ((p->J.nkmax + s - 1) / s + KT - 1) / KT * KT;
    p->nsplit = (p->J.nkmax + p->kslice - 1) / p->kslice;
    p->rep.k_slice = p->kslice;
}

template <typename R>
static int upload(grt_plan *p)
{
    grt_ctx *ctx = p->ctx;
    const Job &J = p->J;
    cudaStream_t st = nullptr;
    CU(setup_stream(ctx, &st));
    std::vector<grt::LayerW<R>> tab;
    std::vector<R> post, tw;
    std::vector<double> damp;
    build_tables<R>(J, tab, post, tw, damp);
    // slot-0 vertical wavenumbers (w = -i sigma, k = 0) of the receiver layer
    grt::slot0_wavenumbers(J, p->slot0);
    // tiles of kGrtThreads wavenumbers, listed on the device from one offset per frequency
    std::vector<long long> tfirst(J.nw);
    long long ntl = 0;
    for (int iw = 0; iw < J.nw; iw++) {
        tfirst[iw] = ntl;
        ntl += (J.nk[iw] + grt::kGrtThreads - 1) / grt::kGrtThreads;
    }
    if (ntl >= (1LL << 31)) return set_err(ctx, GRT_ERR_UNSUPPORTED, "too many (w,k) tiles for one launch");
    p->ntiles = (int)ntl;
    const size_t szK = (size_t)p->nq * J.nkw * 2 * sizeof(R);
    // the tensor-core sum reads the Bessel table in receiver tiles of 32 when
    // every frequency has a unit stride (a stage's rows are then contiguous)
    bool unit = true;
    for (int m : J.ks) unit = unit && m == 1;
    const int KT = p->tc_bf16 ? grt::tc::TcPrec<grt::tc::kBF16>::KT : grt::tc::TcPrec<grt::tc::kTF32>::KT;
    if (p->use_tc && unit) p->bt_rows = (J.nbrow + KT - 1) / KT * KT;
    const size_t szB = p->bt_rows ? (size_t)((p->nd + grt::kBesselTile - 1) / grt::kBesselTile) * grt::kBesselTile *
                                        p->bt_rows * grt::NBASIS * sizeof(R)
                                  : (size_t)J.nbrow * grt::NBASIS * p->nd * sizeof(R);
    const size_t ntr = (size_t)p->nd * p->nc;
    CU(dev_alloc(ctx, &p->tab, tab.size() * sizeof(tab[0])));
    CU(dev_alloc(ctx, &p->tiles, ntl * sizeof(int2)));
    CU(dev_alloc(ctx, &p->tfirst, J.nw * sizeof(long long)));
    CU(dev_alloc(ctx, &p->nk, J.nw * sizeof(int)));
    CU(dev_alloc(ctx, &p->koff, J.nw * sizeof(long long)));
    CU(dev_alloc(ctx, &p->ks, J.nw * sizeof(int)));
    CU(dev_alloc(ctx, &p->ddist, p->nd * sizeof(double)));
    if (!p->use_tc) CU(dev_alloc(ctx, &p->K, szK));
    CU(dev_alloc(ctx, &p->B, szB));
    if (p->bt_rows) CU(cudaMemsetAsync(p->B, 0, szB, st));   // padding rows and receivers stay zero
    CU(dev_alloc(ctx, &p->S, ntr * J.nw * 2 * sizeof(R)));
    CU(dev_alloc(ctx, &p->post, post.size() * sizeof(R)));
    CU(dev_alloc(ctx, &p->tw, tw.size() * sizeof(R)));
    CU(dev_alloc(ctx, &p->damp, damp.size() * sizeof(double)));
    std::vector<float> dampf, twp;
    if (std::is_same<R, float>::value) {
        dampf.assign(damp.begin(), damp.end());
        CU(dev_alloc(ctx, &p->dampf, dampf.size() * sizeof(float)));
        twp.resize(2 * (size_t)std::max(1, grt::fft::pass_twiddle_count(J.log2n - 1)), 0.f);
        grt::fft::pass_twiddles(J.log2n, twp.data());
        CU(dev_alloc(ctx, &p->twp, twp.size() * sizeof(float)));
    }
    // spectra-only plans (a frequency selection) keep [tr][row] spectra and no traces
    const bool sel = !J.fsel.empty();
    if (!sel) CU(dev_alloc(ctx, &p->sig, ntr * J.N * sizeof(R)));
    CU(dev_alloc(ctx, &p->spec, ntr * (sel ? J.nw : J.N) * 2 * sizeof(R)));
    CU(dev_alloc(ctx, &p->derr, sizeof(unsigned)));
    CU(dev_alloc(ctx, &p->nlev, grt::kNlevSlots * sizeof(unsigned long long)));
    if (p->use_tc) {
        // split the k range so that the CTA count (both column groups) fills whole
        // waves of the SMs (one CTA per SM)
        int nsm = 148;
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, ctx->device);
        const long long tiles =
            2LL * ((J.nw + grt::tc::kW - 1) / grt::tc::kW) * ((p->nd + grt::tc::kN - 1) / grt::tc::kN);
        int best = 1;
        double best_cost = 1e30;
        const int maxs = tc_max_split(p);
        for (int s = 1; s <= maxs; s++) {
            const long long n = tiles * s;
            const long long waves = (n + nsm - 1) / nsm;
            // time ~ waves x (k per CTA); small penalty per extra split for the reduction
            const double cost = (double)waves * ((double)J.nkmax / s + 64.0) + 2.0 * s;
            if (cost < best_cost) { best_cost = cost; best = s; }
        }
        p->nsplit_default = best;
        set_tc_split(p, best);
        if (p->kslice_req > 0) {
            p->kslice = p->kslice_req;
            p->nsplit = (J.nkmax + p->kslice - 1) / p->kslice;
        }
        p->rep.k_slice = p->kslice;
        // partial sums of every (k slice, column group)
        p->P_bytes = (size_t)p->nsplit * 2 * ntr * J.nw * 2 * sizeof(float);
        CU(dev_alloc(ctx, &p->P, p->P_bytes));
        // operand blocks of (frequency tile of 64, k stage of KT): nq x (hi, lo) x 4 KB each
        const int nwt = (J.nw + grt::tc::kW - 1) / grt::tc::kW;
        std::vector<long long> base(nwt);
        long long tot = 0;
        bool padded = (J.nw % grt::tc::kW) != 0;
        for (int t = 0; t < nwt; t++) {
            int mx = 0;
            for (int i = t * grt::tc::kW; i < std::min(J.nw, (t + 1) * grt::tc::kW); i++) mx = std::max(mx, J.nk[i]);
            const int ns = (mx + KT - 1) / KT;
            for (int i = t * grt::tc::kW; i < std::min(J.nw, (t + 1) * grt::tc::kW); i++)
                if (J.nk[i] != ns * KT) padded = true;
            base[t] = tot;
            tot += (long long)ns * tc_tiles(p->cols) * 2 * grt::tc::kM * grt::tc::kKT;
        }
        CU(dev_alloc(ctx, &p->Kt, (size_t)tot * sizeof(float)));
        CU(dev_alloc(ctx, &p->kt_base, nwt * sizeof(long long)));
        CU(cudaMemcpyAsync(p->kt_base, base.data(), nwt * sizeof(long long), cudaMemcpyHostToDevice, st));
        // slots beyond a frequency's k range stay zero: the GRT kernel only writes valid (w,k)
        if (padded) CU(cudaMemsetAsync(p->Kt, 0, (size_t)tot * sizeof(float), st));
        CU(cudaStreamSynchronize(st));
    }
    // the specialised FP32 evaluation runs as two passes (bottom-up, then the
    // rest): kRduPlanes floats per (w,k) between them
    if (p->gspec == grt::kSpecAboveTensor && std::is_same<R, float>::value)
        CU(dev_alloc(ctx, &p->rdu, (size_t)grt::kRduPlanes * J.nkw * sizeof(float)));
    CU(cudaMemcpyAsync(p->tab, tab.data(), tab.size() * sizeof(tab[0]), cudaMemcpyHostToDevice, st));
    CU(cudaMemcpyAsync(p->nk, J.nk.data(), J.nw * sizeof(int), cudaMemcpyHostToDevice, st));
    CU(cudaMemcpyAsync(p->tfirst, tfirst.data(), J.nw * sizeof(long long), cudaMemcpyHostToDevice, st));
    grt::plan_tiles_kernel<<<J.nw, 256, 0, st>>>(p->nk, p->tfirst, grt::kGrtThreads, p->tiles);
    CU(cudaGetLastError());
    CU(cudaMemcpyAsync(p->koff, J.koff.data(), J.nw * sizeof(long long), cudaMemcpyHostToDevice, st));
    CU(cudaMemcpyAsync(p->ks, J.ks.data(), J.nw * sizeof(int), cudaMemcpyHostToDevice, st));
    CU(cudaMemcpyAsync(p->ddist, p->dist.data(), p->nd * sizeof(double), cudaMemcpyHostToDevice, st));
    CU(cudaMemcpyAsync(p->post, post.data(), post.size() * sizeof(R), cudaMemcpyHostToDevice, st));
    CU(cudaMemcpyAsync(p->tw, tw.data(), tw.size() * sizeof(R), cudaMemcpyHostToDevice, st));
    CU(cudaMemcpyAsync(p->damp, damp.data(), damp.size() * sizeof(double), cudaMemcpyHostToDevice, st));
    if (p->dampf)
        CU(cudaMemcpyAsync(p->dampf, dampf.data(), dampf.size() * sizeof(float), cudaMemcpyHostToDevice, st));
    if (p->twp) CU(cudaMemcpyAsync(p->twp, twp.data(), twp.size() * sizeof(float), cudaMemcpyHostToDevice, st));
    CU(cudaMemsetAsync(p->derr, 0, sizeof(unsigned), st));
    p->rep.h2d_bytes = (long long)(tab.size() * sizeof(tab[0]) +
                                   J.nw * (2 * sizeof(int) + 2 * sizeof(long long)) + p->nd * sizeof(double) +
                                   (post.size() + tw.size()) * sizeof(R) + damp.size() * sizeof(double) +
                                   (dampf.size() + twp.size()) * sizeof(float));
    p->rep.d2h_bytes = (long long)(ntr * (sel ? 2 * J.nw : J.N) * sizeof(R));
    CU(cudaStreamSynchronize(st));
    return GRT_OK;
}

extern "C" int grt_plan_create(grt_ctx *ctx, const grt_model *m, const grt_opts *o, int n_dist, const double *dist,
                               grt_plan **out)
{
    if (!ctx || !m || !o || !out || n_dist < 1 || !dist) return set_err(ctx, GRT_ERR_ARG, "null argument or no receivers");
    *out = nullptr;
    for (int i = 0; i < n_dist; i++)
        if (!(dist[i] > 0)) return set_err(ctx, GRT_ERR_ARG, "distances must be > 0");
    if (o->precision != GRT_FP32 && o->precision != GRT_FP64) return set_err(ctx, GRT_ERR_ARG, "bad precision");
    std::unique_ptr<grt_plan> p(new grt_plan);
    p->ctx = ctx;
    std::string err;
    int rc = grt::job_from_layers(m->n_layer, m->ztop, m->vp, m->vs, m->rho, m->qp, m->qs, m->hs, m->hr, m->src_type,
                                  p->J, err);
    if (!rc)
        rc = grt::job_setup(p->J, o->dt, o->log2n, o->t0, o->taper, o->sigma_factor, o->k_mode, o->nk_fixed, o->dk,
                            o->fix, err, o->nk_custom, o->k_stride);
    if (!rc && (o->n_freq_sel > 0 || o->freq_sel)) rc = grt::job_select(p->J, o->n_freq_sel, o->freq_sel, err);
    if (rc) return set_err(ctx, rc, err);
    const Job &J = p->J;
    p->prec = o->precision;
    p->nd = n_dist;
    p->dist.assign(dist, dist + n_dist);
    p->cols = col_kind(J);
    p->nc = col_count(p->cols);
    p->nq = coef_count(p->cols);
    // FP32: the complex-to-real kernel takes every N the job accepts (up to 2^15);
    // FP64: the shared-memory FFT holds N complex doubles
    if (p->prec && (size_t)J.N * sizeof(grt::C<double>) > 128 * 1024)
        return set_err(ctx, GRT_ERR_UNSUPPORTED, "N too large for the shared-memory FFT at this precision");
    if (J.nkmax > (1 << 24)) return set_err(ctx, GRT_ERR_UNSUPPORTED, "too many wavenumbers");
    // receivers per block / k-lanes per receiver of the wavenumber sum
    p->rt = 128;
    while (p->rt > 1 && p->rt / 2 >= n_dist) p->rt /= 2;
    p->jt = 128 / p->rt;
    // FP32 plans sum over wavenumbers on the tensor cores unless GRT_KSUM=simt
    const char *ks = getenv("GRT_KSUM");
    // the corrected 30-column tensor layout needs 16 coefficient columns: beyond the
    // tensor-core sum's shared and tensor memory, it runs the SIMT sum
    p->use_tc = (p->prec == GRT_FP32) && !(ks && !strcmp(ks, "simt")) && p->cols != grt::kColTensorFix;
    if (o->tc_split != GRT_TC_3XTF32 && o->tc_split != GRT_TC_3XBF16) return set_err(ctx, GRT_ERR_ARG, "bad tc_split");
    p->tc_bf16 = o->tc_split == GRT_TC_3XBF16;
    const int kt_step = p->tc_bf16 ? 16 : 8;
    if (o->k_slice < 0 || o->k_slice % kt_step)
        return set_err(ctx, GRT_ERR_ARG, "k_slice must be a non-negative multiple of 8 (16 for the 3xBF16 sum)");
    if (o->k_slice > 0 && (J.nkmax + o->k_slice - 1) / o->k_slice > 4096)
        return set_err(ctx, GRT_ERR_ARG, "k_slice too small: more than 4096 slices");
    p->kslice_req = o->k_slice;
    // FP32 moment-tensor jobs with the receiver above the source's layer (and the
    // reference's 8 coefficient columns) run the GRT evaluation compiled for that case
    p->gspec = (p->prec == GRT_FP32 && J.src == 1 && J.rl < J.s && p->nq == grt::QT_N) ? grt::kSpecAboveTensor
                                                                                       : grt::kSpecGeneric;
    p->rep.ksum_impl = p->use_tc ? (p->tc_bf16 ? 3 : 1) : 0;
    // the plain FP32 sum runs as SGEMMs when every frequency has a unit k stride
    p->gemm_ok = p->prec == GRT_FP32 && !p->use_tc && p->cols != grt::kColTensorFix;
    for (int iw = 0; iw < J.nw; iw++) p->gemm_ok = p->gemm_ok && J.ks[iw] == 1;
    if (p->gemm_ok) p->rep.ksum_impl = 2;

    // the tensor-core sum multiplies a tile of 64 frequencies by one Bessel operand:
    // the frequencies of a tile share their k stride
    if (p->use_tc)
        for (int iw = 0; iw < J.nw; iw++)
            if (J.ks[iw] != J.ks[iw - iw % grt::tc::kW])
                return set_err(ctx, GRT_ERR_ARG, "k_stride must be constant on each aligned block of 64 frequencies");
    CU(cudaSetDevice(ctx->device));
    rc = p->prec ? upload<double>(p.get()) : upload<float>(p.get());
    if (rc) {
        grt_plan_destroy(p.release());
        return rc;
    }
    *out = p.release();
    return GRT_OK;
}


// tensor-core wavenumber sum (FP32 path): split-K partial sums, then TwoSum reduction
static int launch_ksum_tc(grt_plan *p, cudaStream_t st, int &launches)
{
    grt_ctx *ctx = p->ctx;
    const Job &J = p->J;
    grt::KsumTcArgs<float> T{};
    T.Kt = p->Kt;
    T.kt_base = p->kt_base;
    T.B = (const float *)p->B;
    T.bt_rows = p->bt_rows;
    T.nk = p->nk;
    T.ks = p->ks;
    T.koff = p->koff;
    T.dist = p->ddist;
    T.P = (float *)p->P;
    T.nkw = J.nkw;
    T.dk = J.dk;
    T.nw = J.nw;
    T.nr = p->nd;
    T.nkmax = J.nkmax;
    T.nsplit = p->nsplit;
    T.kslice = p->kslice;
    T.err = p->derr;
    const int nwt = (J.nw + grt::tc::kW - 1) / grt::tc::kW, nrt = (p->nd + grt::tc::kN - 1) / grt::tc::kN;
    const unsigned grid = (unsigned)(nwt * nrt * p->nsplit);
    // one launch for both column groups (grt_tc_tf32.cu, grt_tc_bf16.cu)
    CU(grt::ksum_tc_launch(p->cols == grt::kColTensorFix ? grt::kColTensor : p->cols, p->tc_bf16, T, grid, st));
    launches++;
    const long long n = (long long)p->nd * p->nc * J.nw * 2;
    grt::ksum_tc_reduce_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>((const float *)p->P, (float *)p->S, n,
                                                                             2 * p->nsplit);
    launches++;
    CU(cudaGetLastError());
    return GRT_OK;
}

// ------------------------------------------------------------------ stages
template <typename R>
static grt::GrtArgs<R> grt_args(const grt_plan *p)
{
    const Job &J = p->J;
    grt::GrtArgs<R> A{};
    A.tab = (const grt::LayerW<R> *)p->tab;
    A.tiles = p->tiles;
    A.nk = p->nk;
    A.ks = p->ks;
    A.koff = p->koff;
    A.K = (R *)p->K;
    A.nkw = J.nkw;
    A.dk = J.dk;
    A.zs = J.zs;
    A.zr = J.zr;
    A.hs_layer = J.h[J.s];
    A.hr_layer = J.h[J.rl];
    A.L = J.L; A.s = J.s; A.rl = J.rl; A.src = J.src; A.fix = J.fix; A.nq = p->nq;
    for (int i = 0; i < 4; i++) A.slot0[i] = (R)p->slot0[i];
    A.err = p->derr;
    A.nlev = p->nlev;
    A.Kt = p->use_tc ? p->Kt : nullptr;
    A.kt_base = p->kt_base;
    A.nqt = tc_tiles(p->cols);
    A.kt_bf16 = p->tc_bf16;
    {
        const grt::TcPlan tp = tc_plan(p->cols);
        for (int q = 0; q < 16; q++) A.qslot[q] = (signed char)tp.qslot[q];
    }
    A.rdu = (R *)p->rdu;
    return A;
}

template <typename R>
static int launch_bessel(grt_plan *p, cudaStream_t st, int &launches)
{
    grt_ctx *ctx = p->ctx;
    const Job &J = p->J;
    const long long n = (long long)J.nbrow * p->nd;
    const int blocks = (int)((n + 255) / 256);
    grt::bessel_table_kernel<R><<<blocks, 256, 0, st>>>((R *)p->B, J.nbrow, p->nd, J.dk, p->ddist, p->bt_rows,
                                                        (J.fix & (grt::kFixCols | grt::kFixCols20)) ? 1 : 0);
    launches++;
    CU(cudaGetLastError());
    return GRT_OK;
}

// plain FP32 sum as cuBLAS SGEMMs (see gemm_a_kernel): planar coefficient
// matrices, then per (power, Bessel function) class its operand and the
// products of every pair of the class, one per k slice, then the combination
template <int SRC>
static cudaError_t launch_gemm_combine(const grt_plan *p, cudaStream_t st)
{
    const long long n = (long long)p->J.nw * p->nd;
    grt::gemm_combine_kernel<SRC><<<(unsigned)((n + 255) / 256), 256, 0, st>>>(p->Dg, p->gslices, p->J.nw, p->nd,
                                                                              p->ddist, (float *)p->S);
    return cudaGetLastError();
}

static int launch_ksum_gemm(grt_plan *p, cudaStream_t st, int &launches)
{
    grt_ctx *ctx = p->ctx;
    const Job &J = p->J;
    if (!ctx->blas) {
        cublasHandle_t h = nullptr;
        if (cublasCreate(&h) != CUBLAS_STATUS_SUCCESS) return set_err(ctx, GRT_ERR_CUDA, "cublasCreate failed");
        cublasSetMathMode(h, CUBLAS_PEDANTIC_MATH);   // FP32 products and sums, no TF32
        ctx->blas = h;
    }
    cublasHandle_t h = (cublasHandle_t)ctx->blas;
    if (cublasSetStream(h, st) != CUBLAS_STATUS_SUCCESS) return set_err(ctx, GRT_ERR_CUDA, "cublasSetStream failed");
    const grt::ColTerms &CT = kColTermsTab[p->cols];
    if (!p->Ag) {
        // buffers on first use; k slices of at most 8192 wavenumbers
        p->nkp = (J.nkmax + 3) / 4 * 4;
        p->gslices = std::max(1, (p->nkp + 8191) / 8192);
        CU(dev_alloc(ctx, &p->Ag, (size_t)p->nq * 2 * J.nw * p->nkp * sizeof(float)));
        CU(dev_alloc(ctx, &p->Bg, (size_t)p->nkp * p->nd * sizeof(float)));
        CU(dev_alloc(ctx, &p->Dg, (size_t)p->gslices * CT.np * 2 * J.nw * p->nd * sizeof(float)));
    }
    const int nw = J.nw, nr = p->nd, nkp = p->nkp;
    {
        const long long n = (long long)p->nq * nw * nkp;
        grt::gemm_a_kernel<<<(unsigned)std::min<long long>((n + 255) / 256, 16384), 256, 0, st>>>(
            (const float *)p->K, p->nk, p->koff, J.nkw, nw, nkp, p->nq, p->Ag);
        CU(cudaGetLastError());
        launches++;
    }
    const int klen = (nkp + p->gslices - 1) / p->gslices;
    const float one = 1.f, zero = 0.f;
    bool done[48] = {};
    for (int p0 = 0; p0 < CT.np; p0++) {
        if (done[p0]) continue;
        const int kp = CT.pkp[p0], b = CT.pb[p0];
        const long long n = (long long)nkp * nr;
        grt::gemm_b_kernel<<<(unsigned)std::min<long long>((n + 255) / 256, 16384), 256, 0, st>>>(
            (const float *)p->B, J.nbrow, nr, nkp, J.dk, kp, b, p->Bg);
        CU(cudaGetLastError());
        launches++;
        for (int pp = p0; pp < CT.np; pp++) {
            if (done[pp] || CT.pkp[pp] != kp || CT.pb[pp] != b) continue;
            done[pp] = true;
            const float *Aq = p->Ag + (size_t)CT.pq[pp] * 2 * nw * nkp;
            for (int sl = 0; sl < p->gslices; sl++) {
                const int k0 = sl * klen, kl = std::min(klen, nkp - k0);
                float *Dp = p->Dg + ((size_t)sl * CT.np + pp) * 2 * nw * nr;
                if (kl <= 0) {
                    CU(cudaMemsetAsync(Dp, 0, (size_t)2 * nw * nr * sizeof(float), st));
                    continue;
                }
                // column-major: D^T [nr x 2nw] = Bc^T [nr x kl] * A^T [kl x 2nw]
                if (cublasSgemm(h, CUBLAS_OP_N, CUBLAS_OP_N, nr, 2 * nw, kl, &one, p->Bg + (size_t)k0 * nr, nr,
                                Aq + k0, nkp, &zero, Dp, nr) != CUBLAS_STATUS_SUCCESS)
                    return set_err(ctx, GRT_ERR_CUDA, "cublasSgemm failed");
                launches++;
            }
        }
    }
    switch (p->cols) {
    case grt::kColSingle: CU(launch_gemm_combine<grt::kColSingle>(p, st)); break;
    case grt::kColSingleFix: CU(launch_gemm_combine<grt::kColSingleFix>(p, st)); break;
    case grt::kColTensorFix: CU(launch_gemm_combine<grt::kColTensorFix>(p, st)); break;
    case grt::kColTensorFix20: CU(launch_gemm_combine<grt::kColTensorFix20>(p, st)); break;
    default: CU(launch_gemm_combine<grt::kColTensor>(p, st)); break;
    }
    launches++;
    return GRT_OK;
}

template <typename R>
static int launch_ksum(grt_plan *p, cudaStream_t st, int &launches)
{
    grt_ctx *ctx = p->ctx;
    const Job &J = p->J;
    if constexpr (std::is_same<R, float>::value) {
        if (p->use_tc) return launch_ksum_tc(p, st, launches);
    }
    grt::KsumArgs<R> S{};
    S.K = (const R *)p->K; S.B = (const R *)p->B; S.nk = p->nk; S.ks = p->ks; S.koff = p->koff; S.dist = p->ddist;
    S.S = (R *)p->S; S.nkw = J.nkw; S.dk = J.dk; S.nw = J.nw; S.nr = p->nd; S.rt = p->rt; S.jt = p->jt;
    if constexpr (std::is_same<R, float>::value) {
        // plans (not batch jobs, whose work is captured in a graph) on unit-stride grids
        if (p->gemm_ok && p->own_derr) return launch_ksum_gemm(p, st, launches);
    }
    const int grid = J.nw * ((p->nd + p->rt - 1) / p->rt);
    switch (p->cols) {
    case grt::kColSingle: grt::ksum_kernel<R, grt::kColSingle><<<grid, grt::kSumThreads, 0, st>>>(S); break;
    case grt::kColSingleFix: grt::ksum_kernel<R, grt::kColSingleFix><<<grid, grt::kSumThreads, 0, st>>>(S); break;
    case grt::kColTensorFix: grt::ksum_kernel<R, grt::kColTensorFix><<<grid, grt::kSumThreads, 0, st>>>(S); break;
    case grt::kColTensorFix20: grt::ksum_kernel<R, grt::kColTensorFix20><<<grid, grt::kSumThreads, 0, st>>>(S); break;
    default: grt::ksum_kernel<R, grt::kColTensor><<<grid, grt::kSumThreads, 0, st>>>(S); break;
    }
    launches++;
    CU(cudaGetLastError());
    return GRT_OK;
}

template <typename R>
static int launch_spectral(grt_plan *p, cudaStream_t st, int &launches)
{
    grt_ctx *ctx = p->ctx;
    const Job &J = p->J;
    grt::SpecArgs<R> S{};
    S.S = (const R *)p->S; S.post = (const R *)p->post; S.tw = (const R *)p->tw; S.damp = p->damp;
    // the full spectra are filled only when a caller fetches them (ensure_spec)
    S.spec_out = nullptr; S.sig_out = (R *)p->sig; S.nw = J.nw; S.logn = J.log2n;
    p->spec_valid = false;
    if (!J.fsel.empty()) {
        // spectra-only plan: phase, taper and scale of each selected frequency
        const long long n = (long long)p->nd * p->nc * J.nw;
        const unsigned blocks = (unsigned)std::min<long long>((n + 255) / 256, 65535);
        grt::select_kernel<R><<<blocks, 256, 0, st>>>((const R *)p->S, (const R *)p->post, (R *)p->spec, n, J.nw);
        launches++;
        CU(cudaGetLastError());
        return GRT_OK;
    }
    if constexpr (std::is_same<R, float>::value) {
        // FP32: the complex-to-real transform of half length, one CTA per trace
        grt::fft::C2RArgs F{};
        F.S = (const float2 *)p->S; F.post = (const float2 *)p->post; F.tw = (const float2 *)p->tw;
        F.twp = (const float2 *)p->twp; F.damp = p->dampf; F.out = (float *)p->sig;
        CU(grt::fft::launch_c2r(F, (long long)p->nd * p->nc, J.log2n, st));
        launches++;
        return GRT_OK;
    }
    const size_t smem2 = (size_t)J.N * sizeof(grt::C<R>);
    CU(raise_smem_limit(grt::spectral_kernel<R>, (int)smem2));
    const int threads = std::min(512, std::max(32, J.N / 2));
    grt::spectral_kernel<R><<<p->nd * p->nc, threads, smem2, st>>>(S);
    launches++;
    CU(cudaGetLastError());
    return GRT_OK;
}

// (the small reads below go through the auxiliary stream: a synchronous copy on
// the legacy stream waited behind other contexts' pending graph copies)
static int check_device_error(grt_ctx *ctx, const unsigned *derr)
{
    unsigned herr = 0;
    cudaStream_t st = nullptr;
    CU(setup_stream(ctx, &st));
    CU(cudaMemcpyAsync(&herr, derr, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
    CU(cudaStreamSynchronize(st));
    if (herr)
        return set_err(ctx, GRT_ERR_TIMEOUT,
                       std::string("a bounded device wait gave up: ") + ((herr & 1) ? "layer-table copy " : "") +
                           ((herr & 2) ? "tensor-core operand refill " : "") + ((herr & 4) ? "tensor-core issue " : "") +
                           ((herr & 8) ? "tensor-core drain" : ""));
    return GRT_OK;
}

// the layers the GRT kernel evaluated, summed over its counters
static cudaError_t read_nlev(grt_ctx *ctx, const unsigned long long *d, long long *out)
{
    unsigned long long h[grt::kNlevSlots];
    cudaStream_t st = nullptr;
    cudaError_t e = setup_stream(ctx, &st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(h, d, sizeof h, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return e;
    unsigned long long t = 0;
    for (unsigned long long v : h) t += v;
    *out = (long long)t;
    return cudaSuccess;
}

template <typename R>
static int execute(grt_plan *p)
{
    grt_ctx *ctx = p->ctx;
    const Job &J = p->J;
    cudaStream_t st = ctx->stream;
    int launches = 0, rc;
    // 1. per-(w,k) GRT kernel
    const grt::GrtArgs<R> A = grt_args<R>(p);
    const size_t smem = (size_t)J.L * sizeof(grt::LayerW<R>);
    CU(cudaMemsetAsync(p->nlev, 0, grt::kNlevSlots * sizeof(unsigned long long), st));
    CU(cudaEventRecord(ctx->ev[0], st));
    CU(grt::grt_point_launch<R>(A, p->gspec, (unsigned)p->ntiles, smem, st, &launches));
    CU(cudaEventRecord(ctx->ev[1], st));
    // 2. Bessel table, 3. wavenumber sum, 4. spectral stage + inverse DFT
    if ((rc = launch_bessel<R>(p, st, launches))) return rc;
    CU(cudaEventRecord(ctx->ev[2], st));
    if ((rc = launch_ksum<R>(p, st, launches))) return rc;
    CU(cudaEventRecord(ctx->ev[3], st));
    if ((rc = launch_spectral<R>(p, st, launches))) return rc;
    CU(cudaEventRecord(ctx->ev[4], st));
    CU(cudaEventSynchronize(ctx->ev[4]));
    if ((rc = check_device_error(ctx, p->derr))) return rc;
    float t[4];
    for (int i = 0; i < 4; i++) CU(cudaEventElapsedTime(&t[i], ctx->ev[i], ctx->ev[i + 1]));
    p->rep.ms_grt = t[0];
    p->rep.ms_bessel = t[1];
    p->rep.ms_ksum = t[2];
    p->rep.ms_spectral = t[3];
    p->rep.ms_total = t[0] + t[1] + t[2] + t[3];
    p->rep.kernel_launches = launches;
    CU(read_nlev(ctx, p->nlev, &p->rep.n_layer_evals));
    return GRT_OK;
}

extern "C" int grt_plan_info(const grt_plan *p, grt_report *r)
{
    if (!p || !r) return GRT_ERR_ARG;
    const Job &J = p->J;
    *r = p->rep;
    r->n_layer = J.L;
    r->s_layer = J.s;
    r->r_layer = J.rl;
    r->zs = J.zs;
    r->zr = J.zr;
    r->nw = J.nw;
    r->n_samples = J.N;
    r->n_cols = p->nc;
    r->n_wk = J.nkw;
    r->nk_max = J.nkmax;
    r->dk = J.dk;
    r->df = J.df;
    r->sigma = J.sigma;
    return GRT_OK;
}

extern "C" int grt_grid(const grt_model *m, const grt_opts *o, grt_report *r)
{
    if (!m || !o || !r) return GRT_ERR_ARG;
    Job J;
    std::string err;
    int rc = grt::job_from_layers(m->n_layer, m->ztop, m->vp, m->vs, m->rho, m->qp, m->qs, m->hs, m->hr, m->src_type,
                                  J, err);
    if (!rc)
        rc = grt::job_setup(J, o->dt, o->log2n, o->t0, o->taper, o->sigma_factor, o->k_mode, o->nk_fixed, o->dk,
                            o->fix, err, o->nk_custom, o->k_stride);
    if (!rc && (o->n_freq_sel > 0 || o->freq_sel)) rc = grt::job_select(J, o->n_freq_sel, o->freq_sel, err);
    if (rc) {
        fprintf(stderr, "grt_grid: %s\n", err.c_str());
        return rc;
    }
    *r = grt_report{};
    r->n_layer = J.L;
    r->s_layer = J.s;
    r->r_layer = J.rl;
    r->zs = J.zs;
    r->zr = J.zr;
    r->nw = J.nw;
    r->n_samples = J.N;
    r->n_cols = col_count(col_kind(J));
    r->n_wk = J.nkw;
    r->nk_max = J.nkmax;
    r->dk = J.dk;
    r->df = J.df;
    r->sigma = J.sigma;
    return GRT_OK;
}

extern "C" int grt_plan_execute(grt_plan *p, grt_report *r)
{
    if (!p) return GRT_ERR_ARG;
    grt_ctx *ctx = p->ctx;
    CU(cudaSetDevice(ctx->device));
    int rc = p->prec ? execute<double>(p) : execute<float>(p);
    if (rc) return rc;
    p->ran = true;
    if (r) grt_plan_info(p, r);
    return GRT_OK;
}

// full plans: fill the spectra of the last execute from its k-sums (taper,
// phase, scale and Hermitian fill), the first time a caller asks for them
template <typename R>
static int ensure_spec(grt_plan *p)
{
    grt_ctx *ctx = p->ctx;
    if (!p->J.fsel.empty() || p->spec_valid) return GRT_OK;
    const long long n = (long long)p->nd * p->nc * p->J.N;
    grt::spec_fill_kernel<R><<<(unsigned)std::min<long long>((n + 255) / 256, 65535), 256, 0, ctx->stream>>>(
        (const R *)p->S, (const R *)p->post, (R *)p->spec, (long long)p->nd * p->nc, p->J.nw);
    CU(cudaGetLastError());
    p->spec_valid = true;
    return GRT_OK;
}

template <typename R>
static int fetch(grt_plan *p, double *traces, double *spectra)
{
    grt_ctx *ctx = p->ctx;
    if (spectra) {
        int rc = ensure_spec<R>(p);
        if (rc) return rc;
    }
    const size_t n = (size_t)p->nd * p->nc * p->J.N;
    std::vector<R> h;
    if (traces) {
        h.resize(n);
        CU(cudaMemcpyAsync(h.data(), p->sig, n * sizeof(R), cudaMemcpyDeviceToHost, ctx->stream));
        CU(cudaStreamSynchronize(ctx->stream));
        for (size_t i = 0; i < n; i++) traces[i] = (double)h[i];
    }
    if (spectra) {
        h.resize(2 * n);
        CU(cudaMemcpyAsync(h.data(), p->spec, 2 * n * sizeof(R), cudaMemcpyDeviceToHost, ctx->stream));
        CU(cudaStreamSynchronize(ctx->stream));
        for (size_t i = 0; i < 2 * n; i++) spectra[i] = (double)h[i];
    }
    return GRT_OK;
}

template <typename R>
static int fetch_freqs(grt_plan *p, int n_freq, const int *freq_idx, double *spectra)
{
    grt_ctx *ctx = p->ctx;
    const size_t rows = (size_t)p->nd * p->nc;
    std::vector<grt::C<R>> h(rows * n_freq);
    // gathered on the device ([f][row]) and downloaded in one copy: full plans
    // from the k-sums and the phase/taper table (no full spectrum is filled),
    // spectra-only plans from their [row][selected frequency] spectra
    const Job &J = p->J;
    std::vector<int> idx(freq_idx, freq_idx + n_freq), sel;
    if (!J.fsel.empty())
        for (int f = 0; f < n_freq; f++)
            sel.push_back((int)(std::find(J.fsel.begin(), J.fsel.end(), freq_idx[f]) - J.fsel.begin()));
    int *d_idx = nullptr;
    R *d_out = nullptr;
    cudaError_t e = dev_alloc(ctx, &d_idx, 2 * (size_t)n_freq * sizeof(int));
    if (e == cudaSuccess) e = dev_alloc(ctx, &d_out, h.size() * 2 * sizeof(R));
    cudaStream_t st = nullptr;
    if (e == cudaSuccess) e = setup_stream(ctx, &st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_idx, idx.data(), n_freq * sizeof(int), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && !sel.empty())
        e = cudaMemcpyAsync(d_idx + n_freq, sel.data(), n_freq * sizeof(int), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) {
        const long long n = (long long)rows * n_freq;
        grt::gather_freqs_kernel<R><<<(unsigned)std::min<long long>((n + 255) / 256, 4096), 256, 0, st>>>(
            (const R *)p->S, (const R *)p->post, (const R *)p->spec, d_idx, sel.empty() ? nullptr : d_idx + n_freq,
            (long long)rows, J.nw, n_freq, d_out);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(h.data(), d_out, h.size() * sizeof(grt::C<R>), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    else if (st) cudaStreamSynchronize(st);   // nothing in flight when the blocks go back
    dev_free(ctx, d_idx);
    dev_free(ctx, d_out);
    CU(e);
    for (size_t r = 0; r < rows; r++)
        for (int f = 0; f < n_freq; f++) {
            spectra[2 * (r * n_freq + f)] = (double)h[f * rows + r].x;
            spectra[2 * (r * n_freq + f) + 1] = (double)h[f * rows + r].y;
        }
    return GRT_OK;
}

extern "C" int grt_plan_fetch_freqs(grt_plan *p, int n_freq, const int *freq_idx, double *spectra)
{
    if (!p || n_freq < 1 || !freq_idx || !spectra) return GRT_ERR_ARG;
    grt_ctx *ctx = p->ctx;
    for (int f = 0; f < n_freq; f++)
        if (freq_idx[f] < 0 || freq_idx[f] >= p->J.N ||
            (!p->J.fsel.empty() && std::find(p->J.fsel.begin(), p->J.fsel.end(), freq_idx[f]) == p->J.fsel.end()))
            return set_err(ctx, GRT_ERR_ARG, "frequency index out of range or not selected");
    CU(cudaSetDevice(ctx->device));
    return p->prec ? fetch_freqs<double>(p, n_freq, freq_idx, spectra) : fetch_freqs<float>(p, n_freq, freq_idx, spectra);
}

extern "C" int grt_plan_fetch(grt_plan *p, double *traces, double *spectra)
{
    if (!p) return GRT_ERR_ARG;
    grt_ctx *ctx = p->ctx;
    if (!p->J.fsel.empty()) return set_err(ctx, GRT_ERR_UNSUPPORTED, "a frequency-selection plan has spectra only");
    CU(cudaSetDevice(ctx->device));
    return p->prec ? fetch<double>(p, traces, spectra) : fetch<float>(p, traces, spectra);
}

// ------------------------------------------------------------------ error estimate
// Predicted relative L2 error of each receiver's traces against the FP64 path
// of the same method (the judge of the FP32 path; see noise_kernel).  The
// k-sum noise variance of every column, carried through the spectral stage
// (|post|^2, the Hermitian pair, the inverse DFT and the de-damping,
// E|dx|^2 = sum_n damp_n^2 * 2 sum_w |post_w|^2 v_w), over the trace's norm,
// times eps.  Receivers between two distance bands interpolate linearly.
// The coefficients' noise level eps(w, class, band) of an FP32 plan,
// measured: a spectra-only FP64 plan over kSpotFreqs spot frequencies (half
// spread geometrically over the lowest quarter of the band, where the far
// receivers' energy is, the rest evenly up to the last) evaluates the same
// (w, k) points; eps^2 = num / den of spot_noise_kernel per (spot, class,
// band), interpolated linearly in frequency between spots.
constexpr int kSpotFreqs = 16;

static int spot_noise(grt_plan *p, const grt::NoiseArgs<float> &A, std::vector<int> &rows, std::vector<double> &eps2,
                      const std::vector<int> &reps, std::vector<double> &s64)
// eps2: [spot][class][band]; s64: the k-sums of the receivers reps (indices
// into p->dist) at the spot rows in FP64, [rep][col][spot] complex
{
    grt_ctx *ctx = p->ctx;
    const Job &J = p->J;
    std::vector<int> sel;
    const int nlo = kSpotFreqs / 2;   // geometric over 1 .. nw/4 (the far receivers' band), the rest even above
    for (int i = 0; i < nlo; i++)
        sel.push_back((int)std::lround(std::exp(std::log(std::max(1, J.nw / 4)) * i / (nlo - 1.0))));
    for (int i = 1; i <= kSpotFreqs - nlo; i++)
        sel.push_back((int)std::lround(J.nw / 4.0 + (J.nw - 1 - J.nw / 4.0) * i / (kSpotFreqs - nlo)));
    for (int &v : sel) v = std::min(J.nw - 1, std::max(0, v));
    std::sort(sel.begin(), sel.end());
    sel.erase(std::unique(sel.begin(), sel.end()), sel.end());
    rows = sel;
    // the FP64 spot plan: this plan's job over the spot frequencies, one receiver
    std::unique_ptr<grt_plan> q(new grt_plan);
    q->ctx = ctx;
    q->J = J;
    std::string err;
    int rc = grt::job_select(q->J, (int)sel.size(), sel.data(), err);
    if (rc) return set_err(ctx, rc, err);
    q->prec = GRT_FP64;
    q->nd = (int)reps.size();
    q->dist.clear();
    for (int r : reps) q->dist.push_back(p->dist[r]);
    q->cols = p->cols;
    q->nc = p->nc;
    q->nq = p->nq;
    q->rt = 128;
    while (q->rt > 1 && q->rt / 2 >= q->nd) q->rt /= 2;
    q->jt = 128 / q->rt;
    if ((rc = upload<double>(q.get())) || (rc = execute<double>(q.get()))) {
        grt_plan_destroy(q.release());
        return rc;
    }
    const int ns = (int)sel.size();
    int *drows = nullptr;
    double *dout = nullptr;
    cudaError_t e = dev_alloc(ctx, &drows, ns * sizeof(int));
    constexpr int NB = grt::kNoiseBands;
    if (e == cudaSuccess) e = dev_alloc(ctx, &dout, (size_t)ns * A.ncls * 2 * NB * sizeof(double));
    cudaStream_t st = ctx->stream;
    std::vector<double> h((size_t)ns * A.ncls * 2 * NB);
    if (e == cudaSuccess) e = cudaMemcpyAsync(drows, sel.data(), ns * sizeof(int), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) {
        grt::spot_noise_kernel<float><<<(unsigned)(ns * A.ncls), grt::kNoiseThreads, 0, st>>>(
            A, (const double *)q->K, q->koff, q->J.nkw, drows, dout);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(h.data(), dout, h.size() * sizeof(double), cudaMemcpyDeviceToHost, st);
    s64.resize((size_t)q->nd * q->nc * ns * 2);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(s64.data(), q->S, s64.size() * sizeof(double), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    dev_free(ctx, drows);
    dev_free(ctx, dout);
    grt_plan_destroy(q.release());
    CU(e);
    eps2.assign((size_t)ns * A.ncls * NB, 0.0);
    for (int i = 0; i < ns; i++)
        for (int c = 0; c < A.ncls; c++)
            for (int b = 0; b < NB; b++) {
                const double *o = &h[((size_t)i * A.ncls + c) * 2 * NB];
                eps2[((size_t)i * A.ncls + c) * NB + b] = o[NB + b] > 0 ? o[b] / o[NB + b] : 0.0;
            }
    return GRT_OK;
}

template <typename R>
static int error_estimate(grt_plan *p, double eps, double *est)
{
    grt_ctx *ctx = p->ctx;
    const Job &J = p->J;
    const grt::ColTerms &CT = kColTermsTab[p->cols];
    constexpr int NB = grt::kNoiseBands;
    grt::NoiseArgs<R> A{};
    int tcls[48];
    A.ncls = 0;
    for (int t = 0; t < CT.nt; t++) {
        int c = 0;
        while (c < A.ncls && !(A.cls_q[c] == CT.q[t] && A.cls_p[c] == CT.kp[t])) c++;
        if (c == A.ncls) {
            A.cls_q[c] = CT.q[t];
            A.cls_p[c] = CT.kp[t];
            A.ncls++;
        }
        tcls[t] = c;
    }
    const double rmin = *std::min_element(p->dist.begin(), p->dist.end());
    const double rmax = *std::max_element(p->dist.begin(), p->dist.end());
    const double l0 = std::log(rmin), l1 = std::log(std::max(rmax, rmin * 1.0001));
    for (int b = 0; b < NB; b++) A.rb[b] = (float)std::exp(l0 + (l1 - l0) * b / (NB - 1));
    if (p->use_tc) {
        A.Kt = p->Kt;
        A.kt_base = p->kt_base;
        A.nqt = tc_tiles(p->cols);
        A.kt_bf16 = p->tc_bf16;
        const grt::TcPlan tp = tc_plan(p->cols);
        for (int q = 0; q < 16; q++) A.qslot[q] = tp.qslot[q];
    } else {
        A.K = (const R *)p->K;
    }
    A.nk = p->nk;
    A.ks = p->ks;
    A.koff = p->koff;
    A.nkw = J.nkw;
    A.dk = J.dk;
    A.nw = J.nw;
    // the coefficients' noise level: given, or measured against FP64 (FP32 plans)
    // eps^2 per (spot row, class, band)
    std::vector<int> srow;
    std::vector<double> seps2;
    const size_t per = (size_t)A.ncls * NB;
    // receivers checked directly at the spot frequencies: the one nearest (in
    // log distance) to each band distance
    std::vector<int> reps;
    std::vector<double> s64;
    bool measured = false;
    if (eps > 0 || !std::is_same<R, float>::value) {
        const double e0 = eps > 0 ? eps : GRT_EPS_FP64;
        srow.assign(1, 0);
        seps2.assign(per, e0 * e0);
    } else if constexpr (std::is_same<R, float>::value) {
        for (int b = 0; b < NB; b++) {
            int best = 0;
            for (int r = 1; r < p->nd; r++)
                if (std::fabs(std::log(p->dist[r] / A.rb[b])) < std::fabs(std::log(p->dist[best] / A.rb[b]))) best = r;
            if (std::find(reps.begin(), reps.end(), best) == reps.end()) reps.push_back(best);
        }
        int rc = spot_noise(p, A, srow, seps2, reps, s64);
        if (rc) return rc;
        measured = true;
    }
    // eps^2 at a row, interpolated between spot rows (constant beyond them)
    std::vector<double> e2row(per);
    auto eps2_at = [&](int row) {
        size_t i1 = std::upper_bound(srow.begin(), srow.end(), row) - srow.begin();
        if (i1 == 0 || i1 == srow.size()) {
            const size_t i = i1 == 0 ? 0 : srow.size() - 1;
            for (size_t x = 0; x < per; x++) e2row[x] = seps2[i * per + x];
        } else {
            const double f = (double)(row - srow[i1 - 1]) / (srow[i1] - srow[i1 - 1]);
            for (size_t x = 0; x < per; x++) e2row[x] = (1 - f) * seps2[(i1 - 1) * per + x] + f * seps2[i1 * per + x];
        }
    };
    float *H = nullptr;
    double *nrm = nullptr;
    CU(dev_alloc(ctx, &H, (size_t)J.nw * A.ncls * NB * sizeof(float)));
    A.H = H;
    cudaError_t e = dev_alloc(ctx, &nrm, (size_t)p->nd * sizeof(double));
    if (e != cudaSuccess) {
        dev_free(ctx, H);
        CU(e);
    }
    cudaStream_t st = ctx->stream;
    grt::noise_kernel<R><<<(unsigned)(J.nw * A.ncls), grt::kNoiseThreads, 0, st>>>(A);
    grt::trace_norm_kernel<R><<<(unsigned)p->nd, 256, 0, st>>>((const R *)p->sig, (long long)p->nc * J.N, nrm);
    std::vector<float> h((size_t)J.nw * A.ncls * NB);
    std::vector<double> n2(p->nd);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(h.data(), H, h.size() * sizeof(float), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(n2.data(), nrm, n2.size() * sizeof(double), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    dev_free(ctx, H);
    dev_free(ctx, nrm);
    CU(e);
    // G[c][b] = sum_w eps^2(w) 2 |post_w|^2 H[w][c][b]
    const int wc = (int)((double)J.nwf * (1 - J.taper));
    const double coef = J.df * J.nwf / PI;
    std::vector<double> G((size_t)A.ncls * NB, 0.0);
    for (int row = 0; row < J.nw; row++) {
        const int iw = grt::job_freq(J, row);
        const double st0 = iw > wc ? 0.5 * (1. + std::cos((iw - wc + 1) * PI / (J.nwf - wc + 1))) : 1.0;
        const double wgt = 2.0 * (st0 * coef) * (st0 * coef);
        eps2_at(row);
        for (size_t i = 0; i < G.size(); i++) G[i] += wgt * e2row[i] * h[(size_t)row * A.ncls * NB + i];
    }
    double damp2 = 0.0;
    for (int n = 0; n < J.N; n++) {
        const double d = std::exp(J.sigma * (n * J.dt + J.t0)) / J.N;
        damp2 += d * d;
    }
    // the wavenumber sum's own rounding (FP32: 3xTF32 products and TMEM chains, or
    // compensated SIMT / SGEMM slices), a floor under the coefficients' noise
    const double floor = p->prec ? 0.0 : (p->use_tc ? 3e-5 : 3e-6);
    // band position of a distance and the modelled variance of receiver r,
    // summed over frequencies with weights gsum (G) or at one row
    auto band_at = [&](double d, int &b0, double &f) {
        const double x = l1 > l0 ? (std::log(d) - l0) / (l1 - l0) * (NB - 1) : 0.0;
        b0 = std::min(NB - 2, std::max(0, (int)x));
        f = std::min(1.0, std::max(0.0, x - b0));
    };
    auto model_var = [&](double d, const double *g_cls_band) {
        int b0;
        double f;
        band_at(d, b0, f);
        double var = 0.0;
        for (int t = 0; t < CT.nt; t++) {
            const double g = (1 - f) * g_cls_band[(size_t)tcls[t] * NB + b0] + f * g_cls_band[(size_t)tcls[t] * NB + b0 + 1];
            var += CT.coef[t] * CT.coef[t] * std::pow(d, -2.0 * CT.rpow[t]) * g;
        }
        return var;
    };
    // The noise model assumes errors independent from one wavenumber to the
    // next; where they are not, the actual error of a sum differs from the
    // model by a factor that depends on the distance.  Measured: the FP32
    // k-sums of the representative receivers at the spot rows against the FP64
    // spot plan's, over the model's prediction at the same rows (both weighted
    // as the trace weighs the rows); the factor of a receiver is interpolated
    // in log distance between the representatives (ends held), kept within
    // [0.5, 64].
    std::vector<double> cfac(reps.size(), 1.0);
    if (measured && !reps.empty()) {
        const int ns = (int)srow.size(), nc = p->nc;
        std::vector<float> s32((size_t)nc * J.nw * 2);
        std::vector<double> gs(per);
        for (size_t i = 0; i < reps.size(); i++) {
            CU(cudaMemcpy(s32.data(), (const float *)p->S + (size_t)reps[i] * nc * J.nw * 2, s32.size() * sizeof(float),
                          cudaMemcpyDeviceToHost));
            double act = 0.0, mod = 0.0;
            for (int si = 0; si < ns; si++) {
                const int row = srow[si];
                const int iw = grt::job_freq(J, row);
                const double st0 = iw > wc ? 0.5 * (1. + std::cos((iw - wc + 1) * PI / (J.nwf - wc + 1))) : 1.0;
                const double wgt = 2.0 * (st0 * coef) * (st0 * coef);
                double a = 0.0;
                for (int c = 0; c < nc; c++) {
                    const double *z = &s64[(((size_t)i * nc + c) * ns + si) * 2];
                    const double dr = s32[((size_t)c * J.nw + row) * 2] - z[0];
                    const double di = s32[((size_t)c * J.nw + row) * 2 + 1] - z[1];
                    a += dr * dr + di * di;
                }
                for (size_t x = 0; x < per; x++) gs[x] = seps2[(size_t)si * per + x] * h[(size_t)row * per + x];
                act += wgt * a;
                mod += wgt * model_var(p->dist[reps[i]], gs.data());
            }
            if (mod > 0 && act > 0) cfac[i] = std::min(64.0, std::max(0.5, act / mod));
        }
    }
    std::vector<int> order(reps.size());
    for (size_t i = 0; i < order.size(); i++) order[i] = (int)i;
    std::sort(order.begin(), order.end(), [&](int a, int b) { return p->dist[reps[a]] < p->dist[reps[b]]; });
    auto cfac_at = [&](double d) {
        if (order.empty()) return 1.0;
        if (d <= p->dist[reps[order.front()]]) return cfac[order.front()];
        if (d >= p->dist[reps[order.back()]]) return cfac[order.back()];
        for (size_t i = 1; i < order.size(); i++) {
            const double d0 = p->dist[reps[order[i - 1]]], d1 = p->dist[reps[order[i]]];
            if (d <= d1) {
                const double f = d1 > d0 ? std::log(d / d0) / std::log(d1 / d0) : 1.0;
                return (1 - f) * cfac[order[i - 1]] + f * cfac[order[i]];
            }
        }
        return cfac[order.back()];
    };
    for (int r = 0; r < p->nd; r++) {
        const double var = model_var(p->dist[r], G.data()) * cfac_at(p->dist[r]);
        est[r] = n2[r] > 0 ? std::sqrt(var * damp2 / n2[r] + floor * floor) : HUGE_VAL;
    }
    return GRT_OK;
}

static int plan_error_estimate(grt_plan *p, double eps, double *est)
{
    grt_ctx *ctx = p->ctx;
    if (!p->J.fsel.empty()) return set_err(ctx, GRT_ERR_UNSUPPORTED, "a frequency-selection plan has no traces");
    if (!p->ran) return set_err(ctx, GRT_ERR_ARG, "execute the plan first");
    if (!(eps >= 0)) return set_err(ctx, GRT_ERR_ARG, "eps must be >= 0");
    CU(cudaSetDevice(ctx->device));
    return p->prec ? error_estimate<double>(p, eps, est) : error_estimate<float>(p, eps, est);
}

extern "C" int grt_plan_error_estimate(grt_plan *p, double eps, double *est)
{
    if (!p || !est) return GRT_ERR_ARG;
    return plan_error_estimate(p, eps, est);
}

// ------------------------------------------------------------------ convergence sweep
// One block per (selected frequency, distance band): envelope of the weighted
// integrand g(k) = max_q |K_q(w,k)| (1+k)^2 min(1, (k r)^-1/2) and its total;
// the smallest k_c whose tail sum_{k >= k_c} g stays within a threshold (tol
// times the total, or an absolute threshold per pair); the tail fraction at
// a given wavenumber (a prediction to judge); and, if asked, the aliasing of
// coarser steps: with S_q^(s) = s dk sum_{j = 0 mod s, j < k_c/dk} K_q(j dk)
// J0(j dk r), alias[0] = max_q |S_q^(1)| and alias[s] = max_q |S_q^(2^s) -
// S_q^(1)| for s = 1..5 (the step's spatial aliasing at distance r).
constexpr int kStrides = 6;
constexpr int kSweepThreads = 128;

__device__ double block_sum(double v, double *red)
{
    red[threadIdx.x] = v;
    __syncthreads();
    for (int h = blockDim.x / 2; h > 0; h >>= 1) {
        if ((int)threadIdx.x < h) red[threadIdx.x] += red[threadIdx.x + h];
        __syncthreads();
    }
    const double r = red[0];
    __syncthreads();
    return r;
}

struct SweepOut {
    const double *tol_abs, *kjudge;
    double *kmax, *tail, *env, *alias;
};

__global__ void __launch_bounds__(kSweepThreads) sweep_kmax_kernel(
    const float *K, long long nkw, int nq, const int *nk, const long long *koff, const int *fidx, int nf,
    const double *band_r, int nb, double dk, double tol, SweepOut O)
{
    __shared__ double red[kSweepThreads];
    __shared__ double chunk[kSweepThreads + 1];   // suffix sums of the threads' chunks
    __shared__ int jc_s;
    __shared__ double tail_at_s;
    const int t = blockIdx.x;
    if (t >= nf * nb) return;
    const int f = t / nb, b = t % nb, iw = fidx[f];
    const int n = nk[iw];
    const long long off = koff[iw];
    const double r = band_r[b];
    const grt::C<float> *Kc = reinterpret_cast<const grt::C<float> *>(K);
    auto g = [&](int j) {
        float m = 0.f;
        for (int q = 0; q < nq; q++) {
            const grt::C<float> v = Kc[(long long)q * nkw + off + j];
            m = fmaxf(m, sqrtf(v.x * v.x + v.y * v.y));
        }
        const double k = dk * j, kr = k * r;
        return (double)m * (1.0 + k) * (1.0 + k) * (kr > 1.0 ? 1.0 / sqrt(kr) : 1.0);
    };
    // thread c owns the contiguous chunk [c n / T, (c + 1) n / T)
    const int T = blockDim.x, c = threadIdx.x;
    const int j0 = (int)((long long)c * n / T), j1 = (int)((long long)(c + 1) * n / T);
    double s = 0.0;
    for (int j = j0; j < j1; j++) s += g(j);
    chunk[c] = s;
    __syncthreads();
    if (c == 0) {
        chunk[T] = 0.0;
        for (int i = T - 1; i >= 0; i--) chunk[i] += chunk[i + 1];   // chunk[i] = sum over chunks >= i
        jc_s = 0;
        tail_at_s = 0.0;
    }
    __syncthreads();
    const double tot = chunk[0];
    const double thr = O.tol_abs ? O.tol_abs[t] : tol * tot;
    // the crossing tail(j) > thr lies in the last chunk whose suffix exceeds it
    if (chunk[c] > thr && !(chunk[c + 1] > thr)) {
        double tail = chunk[c + 1];
        int jc = j0;
        for (int j = j1 - 1; j >= j0; j--) {
            tail += g(j);
            if (tail > thr) { jc = j + 1; break; }
        }
        jc_s = jc;
    }
    const int jj = O.kjudge ? (int)ceil(O.kjudge[t] / dk) : n;
    if (jj < n && jj >= j0 && jj < j1) {
        double tail = chunk[c + 1];
        for (int j = j1 - 1; j >= jj; j--) tail += g(j);
        tail_at_s = tail;
    }
    __syncthreads();
    const int jc = jc_s;
    if (c == 0) {
        O.kmax[t] = dk * jc;
        if (O.tail) O.tail[t] = (tot > 0 && jj < n) ? tail_at_s / tot : 0.0;
        if (O.env) O.env[t] = tot;
    }
    if (!O.alias) return;
    // stride sums over the grid up to k_c (the part a sampler keeps)
    const int ne = jc > 0 ? jc : n;
    double emax[kStrides] = {}, ref = 0.0;
    for (int q = 0; q < nq; q++) {
        double sx[kStrides] = {}, sy[kStrides] = {};
        for (int j = c; j < ne; j += T) {
            const grt::C<float> v = Kc[(long long)q * nkw + off + j];
            const double w = (j == 0 ? 0.5 : 1.0) * dk * grt::bj0_ref(dk * j * r);
            const double x = w * v.x, y = w * v.y;
#pragma unroll
            for (int st = 0; st < kStrides; st++)
                if ((j & ((1 << st) - 1)) == 0) {
                    sx[st] += x * (1 << st);
                    sy[st] += y * (1 << st);
                }
        }
#pragma unroll
        for (int st = 0; st < kStrides; st++) {
            sx[st] = block_sum(sx[st], red);
            sy[st] = block_sum(sy[st], red);
        }
        ref = fmax(ref, hypot(sx[0], sy[0]));
        for (int st = 1; st < kStrides; st++) emax[st] = fmax(emax[st], hypot(sx[st] - sx[0], sy[st] - sy[0]));
    }
    if (c == 0) {
        O.alias[(long long)t * kStrides] = ref;
        for (int st = 1; st < kStrides; st++) O.alias[(long long)t * kStrides + st] = emax[st];
    }
}

extern "C" int grt_sweep_kmax(grt_ctx *ctx, const grt_model *m, const grt_opts *o, int n_freq, const int *freq_idx,
                              int n_band, const double *band_r, double tol, const double *tol_abs,
                              const double *k_judge, double *kmax_out, double *tail_out, double *env_out,
                              double *alias_out)
{
    if (!ctx || !m || !o || !freq_idx || !band_r || !kmax_out || n_freq < 1 || n_band < 1 || !(tol > 0))
        return set_err(ctx, GRT_ERR_ARG, "bad sweep arguments");
    if (o->k_stride) return set_err(ctx, GRT_ERR_ARG, "sweeps run on a unit-stride grid (k_stride must be NULL)");
    Job J;
    std::string err;
    int rc = grt::job_from_layers(m->n_layer, m->ztop, m->vp, m->vs, m->rho, m->qp, m->qs, m->hs, m->hr, m->src_type,
                                  J, err);
    if (!rc)
        rc = grt::job_setup(J, o->dt, o->log2n, o->t0, o->taper, o->sigma_factor, o->k_mode, o->nk_fixed, o->dk,
                            o->fix, err, o->nk_custom, o->k_stride);
    if (rc) return set_err(ctx, rc, err);
    // keep only the selected frequencies as rows: tables, offsets and tiles for them alone
    if (o->n_freq_sel > 0 || o->freq_sel) return set_err(ctx, GRT_ERR_ARG, "sweeps take their frequencies from freq_idx");
    rc = grt::job_select(J, n_freq, freq_idx, err);
    if (rc) return set_err(ctx, rc, err);
    std::vector<int> rows(n_freq);
    std::vector<int2> tiles;
    for (int f = 0; f < n_freq; f++) {
        rows[f] = f;
        for (int j0 = 0; j0 < J.nk[f]; j0 += grt::kGrtThreads) tiles.push_back(make_int2(f, j0));
    }
    const long long tot = J.nkw;
    const int nq = J.src == 0 ? (int)grt::QS_N : (int)grt::QT_N;
    std::vector<grt::LayerW<float>> tab;
    std::vector<float> post, tw;
    std::vector<double> damp;
    build_tables<float>(J, tab, post, tw, damp);
    struct Bufs {
        grt_ctx *c;
        std::vector<void *> v;
        ~Bufs() { for (void *p : v) dev_free(c, p); }
    } bufs{ctx, {}};
    auto dalloc = [&](size_t n) -> void * {
        void *p = nullptr;
        if (dev_alloc(ctx, &p, n) != cudaSuccess) return nullptr;
        bufs.v.push_back(p);
        return p;
    };
    CU(cudaSetDevice(ctx->device));
    void *d_tab = dalloc(tab.size() * sizeof(tab[0])), *d_tiles = dalloc(tiles.size() * sizeof(int2));
    void *d_nk = dalloc(J.nw * sizeof(int)), *d_koff = dalloc(J.nw * sizeof(long long));
    void *d_K = dalloc((size_t)nq * tot * 2 * sizeof(float)), *d_err = dalloc(sizeof(unsigned));
    void *d_f = dalloc(n_freq * sizeof(int)), *d_r = dalloc(n_band * sizeof(double));
    const size_t nt_ = (size_t)n_freq * n_band;
    void *d_out = dalloc(nt_ * (3 + kStrides) * sizeof(double));
    void *d_judge = k_judge ? dalloc(nt_ * sizeof(double)) : nullptr;
    void *d_tabs = tol_abs ? dalloc(nt_ * sizeof(double)) : nullptr;
    if (!d_tab || !d_tiles || !d_nk || !d_koff || !d_K || !d_err || !d_f || !d_r || !d_out || (k_judge && !d_judge) ||
        (tol_abs && !d_tabs))
        return set_err(ctx, GRT_ERR_NOMEM, "sweep buffers");
    cudaStream_t st = ctx->stream;
    CU(cudaMemcpyAsync(d_tab, tab.data(), tab.size() * sizeof(tab[0]), cudaMemcpyHostToDevice, st));
    CU(cudaMemcpyAsync(d_tiles, tiles.data(), tiles.size() * sizeof(int2), cudaMemcpyHostToDevice, st));
    CU(cudaMemcpyAsync(d_nk, J.nk.data(), J.nw * sizeof(int), cudaMemcpyHostToDevice, st));
    CU(cudaMemcpyAsync(d_koff, J.koff.data(), J.nw * sizeof(long long), cudaMemcpyHostToDevice, st));
    CU(cudaMemcpyAsync(d_f, rows.data(), n_freq * sizeof(int), cudaMemcpyHostToDevice, st));
    CU(cudaMemcpyAsync(d_r, band_r, n_band * sizeof(double), cudaMemcpyHostToDevice, st));
    if (k_judge) CU(cudaMemcpyAsync(d_judge, k_judge, nt_ * sizeof(double), cudaMemcpyHostToDevice, st));
    if (tol_abs) CU(cudaMemcpyAsync(d_tabs, tol_abs, nt_ * sizeof(double), cudaMemcpyHostToDevice, st));
    CU(cudaMemsetAsync(d_err, 0, sizeof(unsigned), st));
    grt::GrtArgs<float> A{};
    A.tab = (const grt::LayerW<float> *)d_tab;
    A.tiles = (const int2 *)d_tiles;
    A.nk = (const int *)d_nk;
    A.koff = (const long long *)d_koff;
    A.K = (float *)d_K;
    A.nkw = tot;
    A.dk = J.dk;
    A.zs = J.zs;
    A.zr = J.zr;
    A.hs_layer = J.h[J.s];
    A.hr_layer = J.h[J.rl];
    A.L = J.L; A.s = J.s; A.rl = J.rl; A.src = J.src; A.fix = J.fix; A.nq = nq;
    {
        double s0[4];
        grt::slot0_wavenumbers(J, s0);
        for (int i = 0; i < 4; i++) A.slot0[i] = (float)s0[i];
    }
    A.err = (unsigned *)d_err;
    CU(grt::grt_point_launch<float>(A, grt::kSpecGeneric, (unsigned)tiles.size(), (size_t)J.L * sizeof(grt::LayerW<float>),
                                    st, nullptr));
    const int nt = n_freq * n_band;
    SweepOut O{};
    O.tol_abs = (const double *)d_tabs;
    O.kjudge = (const double *)d_judge;
    O.kmax = (double *)d_out;
    O.tail = tail_out ? (double *)d_out + nt : nullptr;
    O.env = env_out ? (double *)d_out + 2 * nt : nullptr;
    O.alias = alias_out ? (double *)d_out + 3 * nt : nullptr;
    sweep_kmax_kernel<<<nt, kSweepThreads, 0, st>>>((const float *)d_K, tot, nq, (const int *)d_nk,
                                                    (const long long *)d_koff, (const int *)d_f, n_freq,
                                                    (const double *)d_r, n_band, J.dk, tol, O);
    CU(cudaGetLastError());
    CU(cudaMemcpyAsync(kmax_out, O.kmax, nt * sizeof(double), cudaMemcpyDeviceToHost, st));
    if (tail_out) CU(cudaMemcpyAsync(tail_out, O.tail, nt * sizeof(double), cudaMemcpyDeviceToHost, st));
    if (env_out) CU(cudaMemcpyAsync(env_out, O.env, nt * sizeof(double), cudaMemcpyDeviceToHost, st));
    if (alias_out) CU(cudaMemcpyAsync(alias_out, O.alias, (size_t)nt * kStrides * sizeof(double), cudaMemcpyDeviceToHost, st));
    unsigned herr = 0;
    CU(cudaMemcpyAsync(&herr, d_err, sizeof herr, cudaMemcpyDeviceToHost, st));
    CU(cudaStreamSynchronize(st));
    if (herr) return set_err(ctx, GRT_ERR_TIMEOUT, "a bounded device wait gave up (layer-table copy)");
    return GRT_OK;
}

extern "C" int grt_run(grt_ctx *ctx, const grt_model *m, const grt_opts *o, int n_dist, const double *dist,
                       double *traces, double *spectra, grt_report *r)
{
    grt_plan *p = nullptr;
    int rc = grt_plan_create(ctx, m, o, n_dist, dist, &p);
    if (rc) return rc;
    rc = grt_plan_execute(p, r);
    if (!rc) rc = grt_plan_fetch(p, traces, spectra);
    grt_plan_destroy(p);
    return rc;
}

// ------------------------------------------------------------------ green()
static int green_impl(const char *iname, const char *oname_w, const char *oname_t, std::string &msg)
{
    if (!iname || !oname_w || !oname_t) { msg = "null file name"; return GRT_ERR_ARG; }
    grt::RawInput in;
    int rc = grt::read_input(iname, in, msg);
    if (rc) return rc;
    const char *pe = getenv("GRT_PRECISION");
    grt_opts o{};
    o.dt = in.dt; o.log2n = in.log2n; o.t0 = in.t0; o.taper = in.taper; o.sigma_factor = 2.0;
    o.k_mode = GRT_K_REFERENCE; o.precision = (pe && !strcmp(pe, "fp64")) ? GRT_FP64 : GRT_FP32; o.fix = 0;
    grt_model m{(int)in.zt.size(), in.zt.data(), in.vp.data(), in.vs.data(), in.rho.data(), in.qp.data(), in.qs.data(),
                in.hs, in.hr, in.src};
    grt_ctx *ctx = nullptr;
    rc = grt_create(&ctx, 0);
    if (rc) { msg = "cannot create a CUDA context"; return rc; }
    grt_plan *p = nullptr;
    rc = grt_plan_create(ctx, &m, &o, 1, &in.dist, &p);
    std::vector<double> sig, spec;
    int N = 0, nc = 0;
    if (!rc) {
        N = p->J.N;
        nc = p->nc;
        sig.resize((size_t)nc * N);
        spec.resize((size_t)nc * N * 2);
        rc = grt_plan_execute(p, nullptr);
        if (!rc) rc = grt_plan_fetch(p, sig.data(), spec.data());
        grt_plan_destroy(p);
    }
    if (rc) msg = grt_last_error(ctx);
    grt_destroy(ctx);
    if (rc) return rc;
    // writers, green.cu:2242-2258: 30 columns, undefined ones as zero
    FILE *f = fopen(oname_t, "w");
    if (!f) { msg = std::string("cannot write ") + oname_t; return GRT_ERR_IO; }
    for (int n = 0; n < N; n++) {
        for (int c = 0; c < 30; c++) fprintf(f, "%.18e,", c < nc ? sig[(size_t)c * N + n] : 0.0);
        fprintf(f, "\n");
    }
    fclose(f);
    f = fopen(oname_w, "w");
    if (!f) { msg = std::string("cannot write ") + oname_w; return GRT_ERR_IO; }
    for (int n = 0; n < N; n++) {
        for (int c = 0; c < 30; c++) {
            double re = c < nc ? spec[((size_t)c * N + n) * 2] : 0.0, im = c < nc ? spec[((size_t)c * N + n) * 2 + 1] : 0.0;
            fprintf(f, "%.18e,%.18e,", re, im);
        }
        fprintf(f, "\n");
    }
    fclose(f);
    return GRT_OK;
}

extern "C" int grt_green(const char *iname, const char *oname_w, const char *oname_t)
{
    std::string msg;
    int rc = green_impl(iname, oname_w, oname_t, msg);
    if (rc) fprintf(stderr, "grt_green: %s (%s)\n", grt_status_string(rc), msg.c_str());
    return rc;
}

extern "C" void green(char *iname, char *oname_w, char *oname_t) { (void)grt_green(iname, oname_w, oname_t); }

// ------------------------------------------------------------------ batches
// Many jobs (models of any layer count, receiver sets, grids and lengths)
// executed together: one persistent launch of the batched GRT kernel over the
// tiles of every job, then each job's Bessel table, wavenumber sum and
// spectral stage on one of four side streams (the Bessel tables overlap the
// GRT launch).  The whole execution is captured once into a CUDA graph and
// replayed.  The GRT launch shape (threads per block = wavenumbers per tile,
// persistent grid size) is chosen by timing the candidates on the batch.
namespace {
constexpr int kSide = 4;
constexpr int kNtOpts[3] = {64, 128, 256};
}

struct grt_batch {
    grt_ctx *ctx = nullptr;
    std::vector<grt_plan *> jobs;
    int prec = 0, maxL = 0, nsm = 0;
    int nspec[3] = {};               // leading tiles (per block width) of jobs that allow the specialised
                                     // two-pass GRT form (their rows come first in the tile lists)
    void *d_args = nullptr;          // GrtArgs<R>[n_jobs]
    void *d_rows = nullptr;          // per (job, frequency) row: id, nk, first tile of each width
    int4 *d_tiles[3] = {};           // tile lists for 64 / 128 / 256 threads per block
    int ntiles[3] = {};
    long long points = 0;
    unsigned *derr = nullptr;
    unsigned long long *nlev = nullptr;  // counters of layers the GRT launch evaluated
    cudaStream_t side[kSide] = {};
    cudaStream_t copy = nullptr;     // trace downloads started by grt_batch_fetch_f32_async
    std::vector<float *> outs;       // per job: page-locked destination the graph downloads into (or null)
    std::vector<cudaEvent_t> done;   // per job: its stages finished (orders the in-graph download)
    bool has_out = false;
    cudaEvent_t ev_start = nullptr, ev_grt = nullptr, ev_end = nullptr;    // timing (graph event-record nodes)
    cudaEvent_t fork0 = nullptr, fork1 = nullptr, join[kSide] = {};         // dependencies between streams
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    bool launched = false, staged = false;   // grt_batch_launch / grt_batch_wait_stages done
    grt_tune tune{};
    grt_report rep{};
};

extern "C" void grt_batch_destroy(grt_batch *b)
{
    if (!b) return;
    cudaSetDevice(b->ctx->device);
    cudaStreamSynchronize(b->ctx->aux);   // set-up left in flight by a failed creation
    if (b->launched) cudaStreamSynchronize(b->ctx->stream);   // a launch never waited for
    if (b->copy) {
        cudaStreamSynchronize(b->copy);
        cudaStreamDestroy(b->copy);
    }
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    for (grt_plan *p : b->jobs) grt_plan_destroy(p);
    dev_free(b->ctx, b->d_args);
    dev_free(b->ctx, b->d_rows);
    for (auto *t : b->d_tiles) dev_free(b->ctx, t);
    dev_free(b->ctx, b->derr);
    dev_free(b->ctx, b->nlev);
    for (auto &s : b->side)
        if (s) cudaStreamDestroy(s);
    cudaEvent_t evs[] = {b->ev_start, b->ev_grt, b->ev_end, b->fork0, b->fork1};
    for (auto e : evs)
        if (e) cudaEventDestroy(e);
    for (auto e : b->join)
        if (e) cudaEventDestroy(e);
    for (auto e : b->done)
        if (e) cudaEventDestroy(e);
    delete b;
}

// GRT launch shapes the autotuner chooses from: (threads per block, persistent)
namespace {
struct Shape { int nt; bool persist; };
constexpr Shape kShapes[5] = {{64, false}, {128, false}, {256, false}, {128, true}, {256, true}};
int nt_index(int nt) { return nt == 64 ? 0 : nt == 128 ? 1 : 2; }
}

// the GRT launch of a batch in shape `shape` (grt_launch.h; the kernels live
// in grt_grt_f32.cu / grt_grt_f64.cu); *launches counts the kernels
template <typename R>
static int batch_launch_grt(grt_batch *b, int shape, int grid, int ntiles, cudaStream_t st, int *launches = nullptr)
{
    grt_ctx *ctx = b->ctx;
    const size_t smem = (size_t)b->maxL * sizeof(grt::LayerW<R>);
    const Shape sh = kShapes[shape < 0 || shape > 4 ? 4 : shape];
    CU(grt::grt_batch_launch<R>((const grt::GrtArgs<R> *)b->d_args, std::min(ntiles, b->nspec[nt_index(sh.nt)]),
                                sh.nt, sh.persist, b->d_tiles[nt_index(sh.nt)], ntiles, grid, smem, b->derr, st,
                                launches));
    return GRT_OK;
}

template <typename R>
static int batch_occupancy(int shape, size_t smem, int *blocks)
{
    *blocks = 1;
    if (shape != 3 && shape != 4) return GRT_OK;
    return grt::grt_batch_occupancy<R>(kShapes[shape].nt, smem, blocks) == cudaSuccess ? GRT_OK : GRT_ERR_CUDA;
}

template <typename R>
static cudaError_t raise_batch_limits(int smem)
{
    return grt::grt_batch_limits<R>(smem);
}

// Time the candidate shapes on a prefix of the tiles (up to 3e8 points: the
// coefficient writes of a smaller sample would fit the address translation
// better than the full batch does and favour the wrong shape).  The choice is
// remembered for batches of the same precision and depth on the device.
// Autotuner choices are kept per device for the process, not per context: they
// depend on the kernels and the GPU.  A second context (one that builds its
// batches beside another context's running graph, say) reuses a choice
// instead of timing candidates while the GPU is shared.
static std::mutex g_tune_mu;
static std::map<std::tuple<int, int, int>, std::pair<int, int>> g_tuned;   // (device, sizeof R, deepest) -> shape, blocks
static std::map<std::pair<int, int>, double> g_tuned_tc;                    // (device, deepest) -> k split ratio

extern "C" void grt_tune_clear(void)
{
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tuned.clear();
    g_tuned_tc.clear();
}

template <typename R>
static int batch_autotune(grt_batch *b, bool run)
{
    grt_ctx *ctx = b->ctx;
    cudaStream_t st = ctx->stream;
    const size_t smem = (size_t)b->maxL * sizeof(grt::LayerW<R>);
    const auto key = std::make_tuple(ctx->device, (int)sizeof(R), b->maxL);
    if (run) {
        std::pair<int, int> hit{-1, 0};
        {
            std::lock_guard<std::mutex> lk(g_tune_mu);
            auto it = g_tuned.find(key);
            if (it != g_tuned.end()) hit = it->second;
        }
        if (hit.first >= 0) {   // batches of this kind were tuned on this device
            b->tune.grt_shape = hit.first;
            b->tune.grt_blocks = hit.second;
            b->tune.grt_threads = kShapes[b->tune.grt_shape].nt;
            b->tune.tuned = 2;
            b->tune.n_cand = 0;
            return GRT_OK;
        }
    }
    const double frac = std::min(1.0, 3.0e8 / (double)std::max(1LL, b->points));
    int n = 0;
    float best = 1e30f;
    for (int sh = 0; sh < 5; sh++) {
        int occ = 1;
        if (batch_occupancy<R>(sh, smem, &occ)) return set_err(ctx, GRT_ERR_CUDA, "occupancy query failed");
        const int nt_all = b->ntiles[nt_index(kShapes[sh].nt)];
        for (int m = 1; m <= (kShapes[sh].persist ? 2 : 1); m++) {
            const int nt = std::max(1, (int)(nt_all * frac));
            const int grid = kShapes[sh].persist ? b->nsm * occ * m : nt_all;
            float ms = 0.f;
            if (run) {
                if (n == 0) {   // warm-up of the first shape
                    int rc = batch_launch_grt<R>(b, sh, grid, nt, st);
                    if (rc) return rc;
                }
                CU(cudaEventRecord(ctx->ev[0], st));
                int rc = batch_launch_grt<R>(b, sh, grid, nt, st);
                if (rc) return rc;
                CU(cudaEventRecord(ctx->ev[1], st));
                CU(cudaEventSynchronize(ctx->ev[1]));
                CU(cudaEventElapsedTime(&ms, ctx->ev[0], ctx->ev[1]));
            }
            if (n < GRT_TUNE_MAX) {
                b->tune.cand_threads[n] = kShapes[sh].nt;
                b->tune.cand_blocks[n] = kShapes[sh].persist ? grid : 0;
                b->tune.cand_ms[n] = ms;
            }
            n++;
            const bool pick = run ? ms < best : sh == 1;
            if (pick) {
                best = ms;
                b->tune.grt_shape = sh;
                b->tune.grt_threads = kShapes[sh].nt;
                b->tune.grt_blocks = kShapes[sh].persist ? grid : 0;
            }
        }
    }
    b->tune.n_cand = std::min(n, GRT_TUNE_MAX);
    b->tune.tuned = run;
    b->tune.sample_fraction = run ? frac : 0.0;
    if (run) {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        g_tuned[key] = std::make_pair(b->tune.grt_shape, b->tune.grt_blocks);
    }
    return check_device_error(ctx, b->derr);
}

// FP32 batches: the tensor-core sums' k split, timed.  Candidates around the
// wave-filling default of the largest job (in (w,k) points x receivers); the
// best one's ratio to the default is applied to every job that did not fix its
// k_slice, and it is remembered per device and deepest model.
static int tc_ensure_P(grt_plan *p)
{
    grt_ctx *ctx = p->ctx;
    const size_t need = (size_t)p->nsplit * 2 * p->nd * p->nc * p->J.nw * 2 * sizeof(float);
    if (need <= p->P_bytes) return GRT_OK;
    dev_free(ctx, p->P);
    p->P = nullptr;
    CU(dev_alloc(ctx, &p->P, need));
    p->P_bytes = need;
    return GRT_OK;
}

static int tc_autotune(grt_batch *b, bool run)
{
    grt_ctx *ctx = b->ctx;
    cudaStream_t st = ctx->stream;
    grt_plan *big = nullptr;
    for (grt_plan *p : b->jobs)
        if (p->use_tc && !p->kslice_req &&
            (!big || (double)p->J.nkw * p->nd > (double)big->J.nkw * big->nd))
            big = p;
    b->tune.tc_tuned = 0;
    b->tune.tc_n_cand = 0;
    if (!big) return GRT_OK;
    double ratio = 1.0, hit = 0.0;
    if (run) {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        auto it = g_tuned_tc.find(std::make_pair(ctx->device, b->maxL));
        if (it != g_tuned_tc.end()) hit = it->second;
    }
    if (hit > 0.0) {
        ratio = hit;
        b->tune.tc_tuned = 2;
    } else if (run) {
        const int s0 = big->nsplit_default;
        const int cand[4] = {s0, std::max(1, s0 / 2), std::max(1, (3 * s0 + 2) / 4), s0 * 2};
        float best = 1e30f;
        int sbest = s0;
        std::vector<int> seen;
        for (int c : cand) {
            set_tc_split(big, c);
            if (std::find(seen.begin(), seen.end(), big->nsplit) != seen.end()) continue;
            seen.push_back(big->nsplit);
            int rc = tc_ensure_P(big), launches = 0;
            if (!rc) rc = launch_ksum_tc(big, st, launches);                 // warm-up
            if (rc) return rc;
            CU(cudaEventRecord(ctx->ev[0], st));
            if ((rc = launch_ksum_tc(big, st, launches))) return rc;
            CU(cudaEventRecord(ctx->ev[1], st));
            CU(cudaEventSynchronize(ctx->ev[1]));
            float ms = 0.f;
            CU(cudaEventElapsedTime(&ms, ctx->ev[0], ctx->ev[1]));
            const int i = b->tune.tc_n_cand++;
            b->tune.tc_cand_split[i] = big->nsplit;
            b->tune.tc_cand_ms[i] = ms;
            if (ms < best) {
                best = ms;
                sbest = c;
            }
        }
        ratio = (double)sbest / s0;
        {
            std::lock_guard<std::mutex> lk(g_tune_mu);
            g_tuned_tc[std::make_pair(ctx->device, b->maxL)] = ratio;
        }
        b->tune.tc_tuned = 1;
    }
    for (grt_plan *p : b->jobs)
        if (p->use_tc && !p->kslice_req) {
            set_tc_split(p, (int)std::lround(p->nsplit_default * ratio));
            int rc = tc_ensure_P(p);
            if (rc) return rc;
        }
    b->tune.tc_nsplit = big->nsplit;
    return check_device_error(ctx, b->derr);
}

// a timing event: inside a stream capture it must become a graph node (external)
static cudaError_t record_timing(cudaEvent_t ev, cudaStream_t st)
{
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    cudaError_t e = cudaStreamIsCapturing(st, &cs);
    if (e != cudaSuccess) return e;
    return cs == cudaStreamCaptureStatusActive ? cudaEventRecordWithFlags(ev, st, cudaEventRecordExternal)
                                               : cudaEventRecord(ev, st);
}

template <typename R>
static int batch_record(grt_batch *b, cudaStream_t st)
{
    grt_ctx *ctx = b->ctx;
    int launches = 0, rc;
    const int sh = b->tune.grt_shape;
    // timing events are recorded as graph nodes (external), the fork/join
    // events only order the streams
    CU(cudaMemsetAsync(b->nlev, 0, grt::kNlevSlots * sizeof(unsigned long long), st));
    CU(record_timing(b->ev_start, st));
    CU(cudaEventRecord(b->fork0, st));
    for (int s = 0; s < kSide; s++) CU(cudaStreamWaitEvent(b->side[s], b->fork0, 0));
    // Bessel tables depend on the receivers only: they run beside the GRT launch
    for (size_t j = 0; j < b->jobs.size(); j++)
        if ((rc = launch_bessel<R>(b->jobs[j], b->side[j % kSide], launches))) return rc;
    if ((rc = batch_launch_grt<R>(b, sh, b->tune.grt_blocks, b->ntiles[nt_index(kShapes[sh].nt)], st, &launches)))
        return rc;
    CU(record_timing(b->ev_grt, st));
    CU(cudaEventRecord(b->fork1, st));
    for (int s = 0; s < kSide; s++) CU(cudaStreamWaitEvent(b->side[s], b->fork1, 0));
    if (b->has_out) {
        // with download destinations the jobs' sums run one after another on
        // side stream 0 (after every Bessel table), and each job's download,
        // on another side stream, overlaps the next jobs' work
        for (int s = 1; s < kSide; s++) {
            CU(cudaEventRecord(b->join[s], b->side[s]));
            CU(cudaStreamWaitEvent(b->side[0], b->join[s], 0));
        }
        for (size_t j = 0; j < b->jobs.size(); j++) {
            grt_plan *p = b->jobs[j];
            if ((rc = launch_ksum<R>(p, b->side[0], launches))) return rc;
            if ((rc = launch_spectral<R>(p, b->side[0], launches))) return rc;
            // the last job's download follows the graph (grt_batch_wait_stages):
            // a caller may start its next work while it drains
            if (b->outs[j] && j + 1 < b->jobs.size()) {
                cudaStream_t cs = b->side[1 + j % (kSide - 1)];
                CU(cudaEventRecord(b->done[j], b->side[0]));
                CU(cudaStreamWaitEvent(cs, b->done[j], 0));
                CU(cudaMemcpyAsync(b->outs[j], p->sig, (size_t)p->nd * p->nc * p->J.N * sizeof(R),
                                   cudaMemcpyDeviceToHost, cs));
            }
        }
        // the device time ends with the last job's stages; the graph with the downloads
        CU(cudaEventRecord(b->join[0], b->side[0]));
        CU(cudaStreamWaitEvent(st, b->join[0], 0));
        CU(record_timing(b->ev_end, st));
        for (int s = 1; s < kSide; s++) {
            CU(cudaEventRecord(b->join[s], b->side[s]));
            CU(cudaStreamWaitEvent(st, b->join[s], 0));
        }
    } else {
        for (size_t j = 0; j < b->jobs.size(); j++) {
            cudaStream_t ss = b->side[j % kSide];
            if ((rc = launch_ksum<R>(b->jobs[j], ss, launches))) return rc;
            if ((rc = launch_spectral<R>(b->jobs[j], ss, launches))) return rc;
        }
        for (int s = 0; s < kSide; s++) {
            CU(cudaEventRecord(b->join[s], b->side[s]));
            CU(cudaStreamWaitEvent(st, b->join[s], 0));
        }
        CU(record_timing(b->ev_end, st));
    }
    b->rep.kernel_launches = launches;
    return GRT_OK;
}

template <typename R>
static int batch_build(grt_batch *b, int autotune)
{
    grt_ctx *ctx = b->ctx;
    cudaStream_t st = nullptr;   // the set-up; the graph is captured on the main stream
    CU(setup_stream(ctx, &st));
    // per-job arguments in device memory; every job reports waits to the batch's error word
    std::vector<grt::GrtArgs<R>> args;
    for (grt_plan *p : b->jobs) {
        // all of the job's kernels report bounded-wait failures to the batch's word
        if (p->own_derr) dev_free(ctx, p->derr);
        p->derr = b->derr;
        p->own_derr = false;
        if (p->own_nlev) dev_free(ctx, p->nlev);
        p->nlev = b->nlev;
        p->own_nlev = false;
        args.push_back(grt_args<R>(p));
    }
    CU(dev_alloc(ctx, &b->d_args, args.size() * sizeof(args[0])));
    CU(cudaMemcpyAsync(b->d_args, args.data(), args.size() * sizeof(args[0]), cudaMemcpyHostToDevice, st));
    // tile lists for each block width, written on the device from one offset per
    // (job, frequency): the rows of jobs that allow the specialised two-pass
    // GRT form first (a prefix the one-tile forms launch as such), then the others
    std::vector<int2> row_id;
    std::vector<int> row_nk;
    size_t nrow_spec = 0;
    for (int cls = 0; cls < 2; cls++)
        for (size_t j = 0; j < b->jobs.size(); j++) {
            const grt_plan *p = b->jobs[j];
            if ((p->gspec == grt::kSpecAboveTensor && std::is_same<R, float>::value) != (cls == 0)) continue;
            const Job &J = p->J;
            for (int iw = 0; iw < J.nw; iw++) {
                row_id.push_back(make_int2((int)j, iw));
                row_nk.push_back(J.nk[iw]);
            }
            if (cls == 0) nrow_spec = row_id.size();
        }
    const size_t nrow = row_id.size();
    CU(dev_alloc(ctx, &b->d_rows, nrow * (sizeof(int2) + sizeof(int) + 3 * sizeof(long long)) + 8));
    int2 *d_id = (int2 *)b->d_rows;
    int *d_nk = (int *)(d_id + nrow);
    long long *d_first = (long long *)(((uintptr_t)(d_nk + nrow) + 7) & ~(uintptr_t)7);
    CU(cudaMemcpyAsync(d_id, row_id.data(), nrow * sizeof(int2), cudaMemcpyHostToDevice, st));
    CU(cudaMemcpyAsync(d_nk, row_nk.data(), nrow * sizeof(int), cudaMemcpyHostToDevice, st));
    std::vector<long long> first(3 * nrow);
    for (int w = 0; w < 3; w++) {
        long long n = 0;
        for (size_t r = 0; r < nrow; r++) {
            if (r == nrow_spec) b->nspec[w] = (int)n;
            first[w * nrow + r] = n;
            n += (row_nk[r] + kNtOpts[w] - 1) / kNtOpts[w];
        }
        if (nrow_spec == nrow) b->nspec[w] = (int)n;
        if (n >= (1LL << 31)) return set_err(ctx, GRT_ERR_UNSUPPORTED, "too many (w,k) tiles for one launch");
        b->ntiles[w] = (int)n;
        CU(dev_alloc(ctx, &b->d_tiles[w], n * sizeof(int4)));
    }
    CU(cudaMemcpyAsync(d_first, first.data(), 3 * nrow * sizeof(long long), cudaMemcpyHostToDevice, st));
    for (int w = 0; w < 3; w++) {
        grt::batch_tiles_kernel<<<(unsigned)nrow, 256, 0, st>>>(d_id, d_nk, d_first + w * nrow, kNtOpts[w],
                                                                b->d_tiles[w]);
        CU(cudaGetLastError());
    }
    CU(raise_batch_limits<R>((int)((size_t)b->maxL * sizeof(grt::LayerW<R>))));
    CU(cudaStreamSynchronize(st));
    int rc = batch_autotune<R>(b, autotune != 0);
    if (rc) return rc;
    if (std::is_same<R, float>::value && (rc = tc_autotune(b, autotune != 0))) return rc;
    // kernel attributes are set before the capture (a captured graph replays
    // every job's launch sizes)
    for (grt_plan *p : b->jobs) {
        if (std::is_same<R, float>::value) CU(grt::fft::c2r_prepare(p->J.log2n));
        else CU(raise_smem_limit(grt::spectral_kernel<R>, (int)((size_t)p->J.N * sizeof(grt::C<R>))));
        if (p->use_tc) {
            CU(grt::ksum_tc_limits(grt::kColSingle, p->tc_bf16));
            CU(grt::ksum_tc_limits(grt::kColSingleFix, p->tc_bf16));
            CU(grt::ksum_tc_limits(grt::kColTensorFix20, p->tc_bf16));
            CU(grt::ksum_tc_limits(grt::kColTensor, p->tc_bf16));
        }
    }
    CU(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    rc = batch_record<R>(b, ctx->stream);
    cudaGraph_t g = nullptr;
    cudaError_t ce = cudaStreamEndCapture(ctx->stream, &g);
    if (rc) {
        if (g) cudaGraphDestroy(g);
        return rc;
    }
    CU(ce);
    b->graph = g;
    CU(cudaGraphInstantiate(&b->exec, g, 0));
    return GRT_OK;
}

extern "C" int grt_batch_create(grt_ctx *ctx, int n_jobs, const grt_job *jobs, int autotune, grt_batch **out)
{
    if (!ctx || !jobs || !out || n_jobs < 1) return set_err(ctx, GRT_ERR_ARG, "bad batch arguments");
    *out = nullptr;
    std::unique_ptr<grt_batch, void (*)(grt_batch *)> b(new grt_batch, grt_batch_destroy);
    b->ctx = ctx;
    CU(cudaSetDevice(ctx->device));
    for (int j = 0; j < n_jobs; j++) {
        if (!jobs[j].model || !jobs[j].opts) return set_err(ctx, GRT_ERR_ARG, "batch job without model or options");
        if (j > 0 && jobs[j].opts->precision != jobs[0].opts->precision)
            return set_err(ctx, GRT_ERR_ARG, "all jobs of a batch share one precision");
        grt_plan *p = nullptr;
        int rc = grt_plan_create(ctx, jobs[j].model, jobs[j].opts, jobs[j].n_dist, jobs[j].dist, &p);
        if (rc) return set_err(ctx, rc, "job " + std::to_string(j) + ": " + ctx->err);
        b->jobs.push_back(p);
        b->outs.push_back(jobs[j].out_f32);
        if (jobs[j].out_f32) {
            if (p->prec != GRT_FP32) return set_err(ctx, GRT_ERR_ARG, "out_f32 needs an FP32 batch");
            if (!p->J.fsel.empty()) return set_err(ctx, GRT_ERR_ARG, "a frequency-selection job has no traces");
            b->has_out = true;
        }
        b->maxL = std::max(b->maxL, p->J.L);
        b->points += p->J.nkw;
    }
    b->prec = jobs[0].opts->precision;

    CU(cudaDeviceGetAttribute(&b->nsm, cudaDevAttrMultiProcessorCount, ctx->device));
    CU(dev_alloc(ctx, &b->derr, sizeof(unsigned)));
    cudaStream_t su = nullptr;
    CU(setup_stream(ctx, &su));
    CU(cudaMemsetAsync(b->derr, 0, sizeof(unsigned), su));
    CU(cudaStreamSynchronize(su));
    CU(dev_alloc(ctx, &b->nlev, grt::kNlevSlots * sizeof(unsigned long long)));
    for (auto &s : b->side) CU(cudaStreamCreateWithPriority(&s, cudaStreamNonBlocking, ctx->priority));
    CU(cudaStreamCreateWithPriority(&b->copy, cudaStreamNonBlocking, ctx->priority));
    b->done.assign(b->jobs.size(), nullptr);
    for (auto &e : b->done) CU(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    CU(cudaEventCreate(&b->ev_start));
    CU(cudaEventCreate(&b->ev_grt));
    CU(cudaEventCreate(&b->ev_end));
    CU(cudaEventCreateWithFlags(&b->fork0, cudaEventDisableTiming));
    CU(cudaEventCreateWithFlags(&b->fork1, cudaEventDisableTiming));
    for (auto &e : b->join) CU(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    int rc = b->prec ? batch_build<double>(b.get(), autotune) : batch_build<float>(b.get(), autotune);
    if (rc) return rc;
    *out = b.release();
    return GRT_OK;
}

extern "C" int grt_batch_launch(grt_batch *b)
{
    if (!b) return GRT_ERR_ARG;
    grt_ctx *ctx = b->ctx;
    CU(cudaSetDevice(ctx->device));
    if (b->launched) CU(cudaStreamSynchronize(ctx->stream));   // an execution left unfinished
    b->launched = b->staged = false;
    CU(cudaStreamSynchronize(b->copy));     // downloads of the previous results are done
    CU(cudaGraphLaunch(b->exec, ctx->stream));
    b->launched = true;
    return GRT_OK;
}

extern "C" int grt_batch_wait_stages(grt_batch *b)
{
    if (!b) return GRT_ERR_ARG;
    grt_ctx *ctx = b->ctx;
    if (!b->launched) return set_err(ctx, GRT_ERR_ARG, "grt_batch_wait_stages: no launch pending");
    CU(cudaSetDevice(ctx->device));
    CU(cudaStreamSynchronize(ctx->stream));  // the graph, its in-graph downloads included
    b->launched = false;
    const size_t last = b->jobs.size() - 1;
    if (b->outs[last]) {
        const grt_plan *p = b->jobs[last];
        CU(cudaMemcpyAsync(b->outs[last], p->sig, (size_t)p->nd * p->nc * p->J.N * sizeof(float),
                           cudaMemcpyDeviceToHost, b->copy));
    }
    b->staged = true;
    return GRT_OK;
}

extern "C" int grt_batch_finish(grt_batch *b, grt_report *r)
{
    if (!b) return GRT_ERR_ARG;
    grt_ctx *ctx = b->ctx;
    if (!b->staged) return set_err(ctx, GRT_ERR_ARG, "grt_batch_finish: grt_batch_wait_stages has not returned");
    CU(cudaSetDevice(ctx->device));
    CU(cudaStreamSynchronize(b->copy));      // the last job's download
    b->staged = false;
    int rc = check_device_error(ctx, b->derr);
    if (rc) return rc;
    float t_grt = 0.f, t_all = 0.f;
    CU(cudaEventElapsedTime(&t_grt, b->ev_start, b->ev_grt));
    CU(cudaEventElapsedTime(&t_all, b->ev_start, b->ev_end));
    b->rep.ms_grt = t_grt;
    b->rep.ms_total = t_all;
    CU(read_nlev(ctx, b->nlev, &b->rep.n_layer_evals));
    b->rep.ms_bessel = b->rep.ms_ksum = b->rep.ms_spectral = 0.f;
    long long nwk = 0, h2d = 0, d2h = 0;
    int ncol = 0;
    for (grt_plan *p : b->jobs) {
        nwk += p->J.nkw;
        h2d += p->rep.h2d_bytes;
        d2h += p->rep.d2h_bytes;
        ncol = std::max(ncol, p->nc);
        p->ran = true;
        p->spec_valid = false;
    }
    b->rep.n_wk = nwk;
    b->rep.h2d_bytes = h2d;
    b->rep.d2h_bytes = d2h;
    b->rep.n_cols = ncol;
    b->rep.ksum_impl = b->jobs[0]->use_tc;
    if (r) *r = b->rep;
    return GRT_OK;
}

extern "C" int grt_batch_execute(grt_batch *b, grt_report *r)
{
    int rc = grt_batch_launch(b);
    if (!rc) rc = grt_batch_wait_stages(b);
    if (!rc) rc = grt_batch_finish(b, r);
    return rc;
}

extern "C" int grt_batch_fetch(grt_batch *b, int job, double *traces, double *spectra)
{
    if (!b || job < 0 || job >= (int)b->jobs.size()) return GRT_ERR_ARG;
    return grt_plan_fetch(b->jobs[job], traces, spectra);
}

extern "C" int grt_batch_fetch_freqs(grt_batch *b, int job, int n_freq, const int *freq_idx, double *spectra)
{
    if (!b || job < 0 || job >= (int)b->jobs.size()) return GRT_ERR_ARG;
    return grt_plan_fetch_freqs(b->jobs[job], n_freq, freq_idx, spectra);
}

extern "C" int grt_batch_error_estimate(grt_batch *b, int job, double eps, double *est)
{
    if (!b || job < 0 || job >= (int)b->jobs.size() || !est) return GRT_ERR_ARG;
    return plan_error_estimate(b->jobs[job], eps, est);
}

extern "C" int grt_batch_info(const grt_batch *b, int job, grt_report *r, grt_tune *t)
{
    if (!b || job < -1 || job >= (int)b->jobs.size()) return GRT_ERR_ARG;
    if (r) {
        if (job < 0) *r = b->rep;
        else grt_plan_info(b->jobs[job], r);
    }
    if (t) *t = b->tune;
    return GRT_OK;
}

// ------------------------------------------------------------------ seismograms
// Moment tensor of a double couple (Aki & Richards, Box 4.4; x north, y east,
// z down): strike, dip, rake in degrees, scalar moment m0.
extern "C" void grt_dc_moment(double strike, double dip, double rake, double m0, double *m)
{
    if (!m) return;
    const double d2r = PI / 180.0;
    const double f = strike * d2r, d = dip * d2r, l = rake * d2r;
    const double sd = std::sin(d), cd = std::cos(d), s2d = std::sin(2 * d), c2d = std::cos(2 * d);
    const double sl = std::sin(l), cl = std::cos(l), sf = std::sin(f), cf = std::cos(f);
    const double s2f = std::sin(2 * f), c2f = std::cos(2 * f);
    m[0] = -m0 * (sd * cl * s2f + s2d * sl * sf * sf);          // Mxx
    m[1] = m0 * (sd * cl * s2f - s2d * sl * cf * cf);           // Myy
    m[2] = m0 * s2d * sl;                                       // Mzz
    m[3] = m0 * (sd * cl * c2f + 0.5 * s2d * sl * s2f);         // Mxy
    m[4] = -m0 * (cd * cl * cf + c2d * sl * sf);                // Mxz
    m[5] = -m0 * (cd * cl * sf - c2d * sl * cf);                // Myz
}

// weights of the displacement columns (0-9) of the moment-tensor output for
// component Z (up), R (away from the source), T (clockwise) at azimuth phi (the
// receiver's azimuth from the source, degrees clockwise from north).  The
// horizontal-isotropic term (columns 2, 9) and the m = 1 terms (1, 5, 7) take a
// minus sign: the m = 0 and m = 2 parts of the horizontal moments share the
// coefficients a2, u_z = a2z k (h J0 - c2 J2), and the m = 1 columns carry the
// opposite orientation; with these signs every family equals the displacement
// that reciprocity with the single-force solution gives.
static void mt_weights(const double *m, double phi_deg, double w[3][grt::kTensorFixNC])
{
    for (int i = 0; i < 3; i++)
        for (int c = 0; c < grt::kTensorFixNC; c++) w[i][c] = 0.0;
    const double ph = phi_deg * PI / 180.0;
    const double w2c = 0.5 * (m[0] - m[1]), w2s = m[3], w1c = -m[4], w1s = -m[5], w0 = m[2],
                 w0h = -0.5 * (m[0] + m[1]);
    const double c2 = w2c * std::cos(2 * ph) + w2s * std::sin(2 * ph), s2 = -w2c * std::sin(2 * ph) + w2s * std::cos(2 * ph);
    const double c1 = w1c * std::cos(ph) + w1s * std::sin(ph), s1 = -w1c * std::sin(ph) + w1s * std::cos(ph);
    // Z: m = 2, 1, 0 families and the horizontal-isotropic part of the m = 2 family
    w[0][6] = c2; w[0][7] = c1; w[0][8] = w0; w[0][9] = w0h;
    // R
    w[1][0] = c2; w[1][1] = c1; w[1][3] = w0; w[1][2] = w0h;
    // T
    w[2][4] = s2; w[2][5] = s1;
}

// weights [3 (Z up, R away, T clockwise)][15] of the single-force displacement
// columns (0: R and 2: T and 3: Z of a horizontal force, 1: R and 4: Z of a
// vertical one) for force f = (Fx, Fy, Fz; x north, y east, z down) at the
// receiver's azimuth from the source; the same orientation as mt_weights,
// checked against the reciprocal displacement
extern "C" void grt_sf_weights(const double *f, double azimuth, double *w)
{
    if (!f || !w) return;
    for (int i = 0; i < 3 * grt::kSingleNC; i++) w[i] = 0.0;
    const double ph = azimuth * PI / 180.0;
    const double fr = f[0] * std::cos(ph) + f[1] * std::sin(ph), ft = -f[0] * std::sin(ph) + f[1] * std::cos(ph);
    w[0 * grt::kSingleNC + 3] = fr; w[0 * grt::kSingleNC + 4] = f[2];
    w[1 * grt::kSingleNC + 0] = fr; w[1 * grt::kSingleNC + 1] = f[2];
    w[2 * grt::kSingleNC + 2] = ft;
}

extern "C" void grt_mt_weights(const double *m, double azimuth, double *w)
{
    if (!m || !w) return;
    double t[3][grt::kTensorFixNC];
    mt_weights(m, azimuth, t);
    for (int i = 0; i < 3; i++)
        for (int c = 0; c < grt::kTensorFixNC; c++) w[i * grt::kTensorFixNC + c] = t[i][c];
}

template <typename R>
static int synth(grt_plan *p, const grt_source *src, const double *azimuth, double *seis)
{
    grt_ctx *ctx = p->ctx;
    const Job &J = p->J;
    const int nd = p->nd, nc = p->nc, N = J.N, nw = J.nw;
    std::vector<R> W((size_t)nd * 3 * nc, R(0));
    for (int r = 0; r < nd; r++) {
        if (J.src == 0) {
            // single force: the weights of its displacement columns (15)
            double w[3 * grt::kSingleNC];
            grt_sf_weights(src->f, azimuth[r], w);
            for (int i = 0; i < 3; i++)
                for (int c = 0; c < nc && c < grt::kSingleNC; c++)
                    W[((size_t)r * 3 + i) * nc + c] = (R)w[i * grt::kSingleNC + c];
            continue;
        }
        double w[3][grt::kTensorFixNC];
        mt_weights(src->m, azimuth[r], w);
        for (int i = 0; i < 3; i++)
            for (int c = 0; c < nc; c++) W[((size_t)r * 3 + i) * nc + c] = (R)w[i][c];
    }
    // source-time spectrum at the complex frequency: dt sum_n s_n e^{-sigma n dt} e^{-i w n dt}
    std::vector<R> stf;
    if (src->n_stf > 0) {
        stf.resize(2 * (size_t)nw);
        for (int k = 0; k < nw; k++) {
            cd acc(0, 0);
            const double wk = 2 * PI * J.df * k;
            for (int n = 0; n < src->n_stf; n++) {
                const double t = n * J.dt;
                acc += src->stf[n] * std::exp(-J.sigma * t) * std::exp(cd(0, -wk * t));
            }
            acc *= J.dt;
            stf[2 * k] = (R)acc.real();
            stf[2 * k + 1] = (R)acc.imag();
        }
    }
    struct Bufs {
        grt_ctx *c;
        std::vector<void *> v;
        ~Bufs() { for (void *q : v) dev_free(c, q); }
    } bufs{ctx, {}};
    void *dW = nullptr, *dS = nullptr, *dO = nullptr;
    CU(dev_alloc(ctx, &dW, W.size() * sizeof(R))); bufs.v.push_back(dW);
    if (!stf.empty()) { CU(dev_alloc(ctx, &dS, stf.size() * sizeof(R))); bufs.v.push_back(dS); }
    const size_t nout = (size_t)nd * 3 * N;
    CU(dev_alloc(ctx, &dO, nout * sizeof(R))); bufs.v.push_back(dO);
    cudaStream_t st = ctx->stream;
    CU(cudaMemcpyAsync(dW, W.data(), W.size() * sizeof(R), cudaMemcpyHostToDevice, st));
    if (dS) CU(cudaMemcpyAsync(dS, stf.data(), stf.size() * sizeof(R), cudaMemcpyHostToDevice, st));
    grt::SynthArgs<R> A{};
    A.S = (const R *)p->S; A.W = (const R *)dW; A.stf = (const R *)dS; A.post = (const R *)p->post;
    A.tw = (const R *)p->tw; A.damp = p->damp; A.out = (R *)dO;
    A.nw = nw; A.logn = J.log2n; A.nc = nc; A.nout = 3;
    const size_t smem = (size_t)N * sizeof(grt::C<R>);
    CU(raise_smem_limit(grt::synth_kernel<R>, (int)smem));
    const int threads = std::min(512, std::max(32, N / 2));
    grt::synth_kernel<R><<<nd * 3, threads, smem, st>>>(A);
    CU(cudaGetLastError());
    std::vector<R> h(nout);
    CU(cudaMemcpyAsync(h.data(), dO, nout * sizeof(R), cudaMemcpyDeviceToHost, st));
    CU(cudaStreamSynchronize(st));
    for (size_t i = 0; i < nout; i++) seis[i] = (double)h[i];
    return GRT_OK;
}

extern "C" int grt_plan_synth(grt_plan *p, const grt_source *src, const double *azimuth, double *seis)
{
    if (!p || !src || !azimuth || !seis) return GRT_ERR_ARG;
    grt_ctx *ctx = p->ctx;
    if (!p->J.fsel.empty()) return set_err(ctx, GRT_ERR_UNSUPPORTED, "a frequency-selection plan has spectra only");
    if (src->n_stf < 0 || (src->n_stf > 0 && !src->stf) || src->n_stf > p->J.N)
        return set_err(ctx, GRT_ERR_ARG, "source-time function: 0 <= n_stf <= N samples");
    // the seismogram kernel holds one trace's N complex values in shared memory
    if ((size_t)p->J.N * (p->prec ? sizeof(grt::C<double>) : sizeof(grt::C<float>)) > 128 * 1024)
        return set_err(ctx, GRT_ERR_UNSUPPORTED, "seismograms: N too large for the shared-memory FFT");
    CU(cudaSetDevice(ctx->device));
    return p->prec ? synth<double>(p, src, azimuth, seis) : synth<float>(p, src, azimuth, seis);
}

extern "C" int grt_batch_synth(grt_batch *b, int job, const grt_source *src, const double *azimuth, double *seis)
{
    if (!b || job < 0 || job >= (int)b->jobs.size()) return GRT_ERR_ARG;
    return grt_plan_synth(b->jobs[job], src, azimuth, seis);
}

extern "C" int grt_flatten(int n_layer, const double *ztop, const double *vp, const double *vs, double hs, double hr,
                           double r_earth, double *ztop_f, double *vp_f, double *vs_f, double *hs_f, double *hr_f)
{
    std::string err;
    const int rc = grt::flatten(n_layer, ztop, vp, vs, hs, hr, r_earth, ztop_f, vp_f, vs_f, hs_f, hr_f, err);
    if (rc) fprintf(stderr, "grt_flatten: %s\n", err.c_str());
    return rc;
}

// ------------------------------------------------------------------ binary output
// "GRTMBIN1", int32 version (1), n_dist, n_cols, N, float64 dt, t0, sigma,
// float64 dist[n_dist], then the traces as float32 [n_dist][n_cols][N]
// (little-endian, as the host writes them).  FP64 plans store their traces
// rounded to float32.
extern "C" int grt_plan_write(grt_plan *p, const char *path)
{
    if (!p || !path) return GRT_ERR_ARG;
    grt_ctx *ctx = p->ctx;
    const Job &J = p->J;
    if (!J.fsel.empty()) return set_err(ctx, GRT_ERR_UNSUPPORTED, "a frequency-selection plan has spectra only");
    const size_t n = (size_t)p->nd * p->nc * J.N;
    std::vector<float> tr(n);
    CU(cudaSetDevice(ctx->device));
    if (p->prec) {
        std::vector<double> h(n);
        CU(cudaMemcpy(h.data(), p->sig, n * sizeof(double), cudaMemcpyDeviceToHost));
        for (size_t i = 0; i < n; i++) tr[i] = (float)h[i];
    } else {
        CU(cudaMemcpy(tr.data(), p->sig, n * sizeof(float), cudaMemcpyDeviceToHost));
    }
    FILE *f = fopen(path, "wb");
    if (!f) return set_err(ctx, GRT_ERR_IO, std::string("cannot write ") + path);
    const int32_t hdr[4] = {1, p->nd, p->nc, J.N};
    const double par[3] = {J.dt, J.t0, J.sigma};
    bool ok = fwrite("GRTMBIN1", 1, 8, f) == 8 && fwrite(hdr, sizeof hdr, 1, f) == 1 && fwrite(par, sizeof par, 1, f) == 1 &&
              fwrite(p->dist.data(), sizeof(double), p->nd, f) == (size_t)p->nd &&
              fwrite(tr.data(), sizeof(float), n, f) == n;
    ok = (fclose(f) == 0) && ok;
    return ok ? GRT_OK : set_err(ctx, GRT_ERR_IO, std::string("short write to ") + path);
}

// traces as float32 (the working precision of FP32 plans: no widening on the host)
extern "C" int grt_plan_fetch_f32(grt_plan *p, float *traces)
{
    if (!p || !traces) return GRT_ERR_ARG;
    grt_ctx *ctx = p->ctx;
    if (!p->J.fsel.empty()) return set_err(ctx, GRT_ERR_UNSUPPORTED, "a frequency-selection plan has spectra only");
    const size_t n = (size_t)p->nd * p->nc * p->J.N;
    CU(cudaSetDevice(ctx->device));
    if (p->prec) {
        std::vector<double> h(n);
        CU(cudaMemcpy(h.data(), p->sig, n * sizeof(double), cudaMemcpyDeviceToHost));
        for (size_t i = 0; i < n; i++) traces[i] = (float)h[i];
        return GRT_OK;
    }
    CU(cudaMemcpyAsync(traces, p->sig, n * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
    CU(cudaStreamSynchronize(ctx->stream));
    return GRT_OK;
}

extern "C" int grt_host_alloc(size_t bytes, void **ptr)
{
    if (!ptr || bytes == 0) return GRT_ERR_ARG;
    *ptr = nullptr;
    const cudaError_t e = cudaHostAlloc(ptr, bytes, cudaHostAllocPortable);
    if (e != cudaSuccess) {
        *ptr = nullptr;
        return e == cudaErrorMemoryAllocation ? GRT_ERR_NOMEM : GRT_ERR_CUDA;
    }
    return GRT_OK;
}

extern "C" void grt_host_free(void *ptr)
{
    if (ptr) cudaFreeHost(ptr);
}

extern "C" int grt_batch_fetch_f32_async(grt_batch *b, int job, float *traces)
{
    if (!b || job < 0 || job >= (int)b->jobs.size() || !traces) return GRT_ERR_ARG;
    grt_plan *p = b->jobs[job];
    grt_ctx *ctx = b->ctx;
    if (p->prec != GRT_FP32) return set_err(ctx, GRT_ERR_UNSUPPORTED, "asynchronous fetches are for FP32 batches");
    if (!p->J.fsel.empty()) return set_err(ctx, GRT_ERR_UNSUPPORTED, "a frequency-selection plan has spectra only");
    CU(cudaSetDevice(ctx->device));
    // grt_batch_execute returned after the graph finished: the traces are final
    const size_t n = (size_t)p->nd * p->nc * p->J.N;
    CU(cudaMemcpyAsync(traces, p->sig, n * sizeof(float), cudaMemcpyDeviceToHost, b->copy));
    return GRT_OK;
}

extern "C" int grt_batch_wait(grt_batch *b)
{
    if (!b) return GRT_ERR_ARG;
    grt_ctx *ctx = b->ctx;
    CU(cudaSetDevice(ctx->device));
    CU(cudaStreamSynchronize(b->copy));
    return GRT_OK;
}

extern "C" int grt_batch_fetch_f32(grt_batch *b, int job, float *traces)
{
    if (!b || job < 0 || job >= (int)b->jobs.size()) return GRT_ERR_ARG;
    return grt_plan_fetch_f32(b->jobs[job], traces);
}
