// grt_mlp.cu -- the learned wavenumber sampler's network: a small MLP
// (n_in -> 64 -> 64 -> 64 -> n_out, SiLU hidden activations, linear output)
// with hand-written FP32 CUDA kernels for inference, backpropagation and Adam.
//
// Parameter vector layout: W1[64][n_in], b1[64], W2[64][64], b2[64],
// W3[64][64], b3[64], W4[n_out][64], b4[n_out].  Loss: mean squared error
// over samples and outputs.  Forward and delta kernels run one thread per
// sample with the weights in shared memory; the gradient kernel runs one
// thread per parameter.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <string>
#include <utility>
#include <vector>

#include "../../include/grtm_gb300.h"
#include "grt_ctx.h"

namespace {

constexpr int H = 64;
constexpr int kMaxIn = 32, kMaxOut = 4;
constexpr int kThreads = 64;

struct Layout {
    int ni, no;
    int w1, b1, w2, b2, w3, b3, w4, b4, n;
    __host__ __device__ Layout(int ni_, int no_) : ni(ni_), no(no_)
    {
        w1 = 0; b1 = w1 + H * ni; w2 = b1 + H; b2 = w2 + H * H; w3 = b2 + H; b3 = w3 + H * H;
        w4 = b3 + H; b4 = w4 + no * H; n = b4 + no;
    }
};

__device__ __forceinline__ float sig(float z) { return 1.f / (1.f + __expf(-z)); }

// z = W h + b over 64 outputs; in/out in registers
template <int NIN>
__device__ __forceinline__ void dense(const float *W, const float *b, const float *in, float *z)
{
#pragma unroll 4
    for (int o = 0; o < H; o++) {
        float s = b[o];
#pragma unroll
        for (int i = 0; i < NIN; i++) s = fmaf(W[o * NIN + i], in[i], s);
        z[o] = s;
    }
}

// forward for samples idx[i] (or i), saving pre-activations z1..z3 and the output
__global__ void __launch_bounds__(kThreads) mlp_forward(const float *P, int ni, int no, int n, const float *X,
                                                       const int *idx, float *Y, float *act)
{
    extern __shared__ float sp[];
    const Layout Lo(ni, no);
    for (int i = threadIdx.x; i < Lo.n; i += blockDim.x) sp[i] = P[i];
    __syncthreads();
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const int row = idx ? idx[s] : s;
    float x[kMaxIn], h[H], z[H];
    for (int i = 0; i < kMaxIn; i++) x[i] = i < ni ? X[(long long)row * ni + i] : 0.f;
    // layer 1 (n_in inputs, generic loop)
    for (int o = 0; o < H; o++) {
        float acc = sp[Lo.b1 + o];
        for (int i = 0; i < ni; i++) acc = fmaf(sp[Lo.w1 + o * ni + i], x[i], acc);
        z[o] = acc;
    }
    float *a = act ? act + (long long)s * 3 * H : nullptr;
#pragma unroll
    for (int o = 0; o < H; o++) {
        if (a) a[o] = z[o];
        h[o] = z[o] * sig(z[o]);
    }
    dense<H>(sp + Lo.w2, sp + Lo.b2, h, z);
#pragma unroll
    for (int o = 0; o < H; o++) {
        if (a) a[H + o] = z[o];
        h[o] = z[o] * sig(z[o]);
    }
    dense<H>(sp + Lo.w3, sp + Lo.b3, h, z);
#pragma unroll
    for (int o = 0; o < H; o++) {
        if (a) a[2 * H + o] = z[o];
        h[o] = z[o] * sig(z[o]);
    }
    for (int o = 0; o < no; o++) {
        float acc = sp[Lo.b4 + o];
#pragma unroll
        for (int i = 0; i < H; i++) acc = fmaf(sp[Lo.w4 + o * H + i], h[i], acc);
        Y[(long long)s * no + o] = acc;
    }
}

// backward, per sample: output error, loss share and the deltas of all
// four layers, D[s] = (d1[64], d2[64], d3[64], d4[n_out])
constexpr int kDS = 3 * H + kMaxOut;

__device__ __forceinline__ float dsilu(float z)
{
    const float g = sig(z);
    return g * (1.f + z * (1.f - g));
}

__global__ void __launch_bounds__(kThreads) mlp_delta(const float *P, int ni, int no, int n, float scale,
                                                     const float *T, const int *idx, const float *Y,
                                                     const float *act, float *D, float *lsum)
{
    extern __shared__ float sp[];
    const Layout Lo(ni, no);
    for (int i = threadIdx.x; i < Lo.n; i += blockDim.x) sp[i] = P[i];
    __syncthreads();
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const int row = idx ? idx[s] : s;
    const float *a = act + (long long)s * 3 * H;
    float *dd = D + (long long)s * kDS;
    float d4[kMaxOut], l = 0.f;
    for (int o = 0; o < kMaxOut; o++) {
        float e = 0.f;
        if (o < no) e = Y[(long long)s * no + o] - T[(long long)row * no + o];
        l += e * e;
        d4[o] = 2.f * e * scale;
        if (o < no) dd[3 * H + o] = d4[o];
    }
    lsum[s] = l * scale;
    float cur[H], nxt[H];
#pragma unroll 4
    for (int i = 0; i < H; i++) {
        float acc = 0.f;
        for (int o = 0; o < no; o++) acc = fmaf(sp[Lo.w4 + o * H + i], d4[o], acc);
        cur[i] = acc * dsilu(a[2 * H + i]);
        dd[2 * H + i] = cur[i];
    }
#pragma unroll 4
    for (int i = 0; i < H; i++) {
        float acc = 0.f;
#pragma unroll
        for (int o = 0; o < H; o++) acc = fmaf(sp[Lo.w3 + o * H + i], cur[o], acc);
        nxt[i] = acc * dsilu(a[H + i]);
        dd[H + i] = nxt[i];
    }
#pragma unroll 4
    for (int i = 0; i < H; i++) {
        float acc = 0.f;
#pragma unroll
        for (int o = 0; o < H; o++) acc = fmaf(sp[Lo.w2 + o * H + i], nxt[o], acc);
        dd[i] = acc * dsilu(a[i]);
    }
}

// gradient, one thread per parameter: the batch sum of delta x layer input
// (deterministic, no atomics); thread Lo.n sums the loss
__global__ void mlp_grad(int ni, int no, int n, const float *X, const int *idx, const float *act,
                         const float *D, const float *lsum, float *G, float *loss)
{
    const Layout Lo(ni, no);
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p > Lo.n) return;
    if (p == Lo.n) {
        float t = 0.f;
        for (int s = 0; s < n; s++) t += lsum[s];
        *loss = t;
        return;
    }
    int layer, o, i = -1;   // i < 0: bias
    if (p < Lo.b1) { layer = 1; o = p / ni; i = p % ni; }
    else if (p < Lo.w2) { layer = 1; o = p - Lo.b1; }
    else if (p < Lo.b2) { layer = 2; o = (p - Lo.w2) / H; i = (p - Lo.w2) % H; }
    else if (p < Lo.w3) { layer = 2; o = p - Lo.b2; }
    else if (p < Lo.b3) { layer = 3; o = (p - Lo.w3) / H; i = (p - Lo.w3) % H; }
    else if (p < Lo.w4) { layer = 3; o = p - Lo.b3; }
    else if (p < Lo.b4) { layer = 4; o = (p - Lo.w4) / H; i = (p - Lo.w4) % H; }
    else { layer = 4; o = p - Lo.b4; }
    const int doff = (layer - 1) * H + o;
    float g = 0.f;
    for (int s = 0; s < n; s++) {
        float in = 1.f;
        if (i >= 0) {
            if (layer == 1) {
                in = X[(long long)(idx ? idx[s] : s) * ni + i];
            } else {
                const float z = act[(long long)s * 3 * H + (layer - 2) * H + i];
                in = z * sig(z);
            }
        }
        g = fmaf(D[(long long)s * kDS + doff], in, g);
    }
    G[p] = g;
}

__global__ void adam_step(float *P, const float *G, float *M, float *V, int n, float lr, float b1, float b2, float eps,
                          float c1, float c2)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float g = G[i];
    const float m = b1 * M[i] + (1.f - b1) * g, v = b2 * V[i] + (1.f - b2) * g * g;
    M[i] = m;
    V[i] = v;
    P[i] -= lr * (m / c1) / (sqrtf(v / c2) + eps);
}

}  // namespace

struct grt_mlp {
    grt_ctx *ctx = nullptr;
    int device = 0;
    Layout lo{1, 1};
    float *P = nullptr, *G = nullptr, *M = nullptr, *V = nullptr, *loss = nullptr;
    // the forward pass's inputs and outputs, kept between calls (grown when a
    // call needs more): a cudaFree per call would wait for the whole device
    float *fx = nullptr, *fy = nullptr;
    size_t fx_n = 0, fy_n = 0;
    long long step = 0;
    grt_mlp(int ni, int no) : lo(ni, no) {}
};

static int mfail(grt_ctx *ctx, int code, const std::string &m)
{
    if (ctx) ctx->err = m;
    return code;
}
#define CUM(call)                                                                                     \
    do {                                                                                              \
        cudaError_t e_ = (call);                                                                      \
        if (e_ != cudaSuccess) return mfail(ctx, GRT_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

// device buffers freed when the helper leaves scope
struct DevBufs {
    std::vector<void *> v;
    void *get(size_t n)
    {
        void *p = nullptr;
        if (cudaMalloc(&p, n ? n : 4) != cudaSuccess) return nullptr;
        v.push_back(p);
        return p;
    }
    ~DevBufs()
    {
        for (void *p : v) cudaFree(p);
    }
};

extern "C" int grt_mlp_create(grt_ctx *ctx, int n_in, int n_out, unsigned long long seed, grt_mlp **out)
{
    if (!ctx || !out || n_in < 1 || n_in > kMaxIn || n_out < 1 || n_out > kMaxOut)
        return mfail(ctx, GRT_ERR_ARG, "mlp: 1 <= n_in <= 32, 1 <= n_out <= 4");
    std::unique_ptr<grt_mlp> m(new grt_mlp(n_in, n_out));
    m->ctx = ctx;
    m->device = ctx->device;
    const int n = m->lo.n;
    CUM(cudaSetDevice(ctx->device));
    CUM(cudaMalloc(&m->P, n * sizeof(float)));
    CUM(cudaMalloc(&m->G, n * sizeof(float)));
    CUM(cudaMalloc(&m->M, n * sizeof(float)));
    CUM(cudaMalloc(&m->V, n * sizeof(float)));
    CUM(cudaMalloc(&m->loss, sizeof(float)));
    // uniform(-a, a) weights with a = sqrt(3 / fan_in), zero biases (splitmix64 stream)
    std::vector<float> h(n, 0.f);
    unsigned long long st = seed ? seed : 0x9E3779B97F4A7C15ull;
    auto uni = [&]() {
        st += 0x9E3779B97F4A7C15ull;
        unsigned long long z = st;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        return (double)(z >> 11) / 9007199254740992.0;
    };
    auto fill = [&](int off, int count, int fan) {
        const double a = std::sqrt(3.0 / fan);
        for (int i = 0; i < count; i++) h[off + i] = (float)((2 * uni() - 1) * a);
    };
    const Layout &L = m->lo;
    fill(L.w1, H * n_in, n_in);
    fill(L.w2, H * H, H);
    fill(L.w3, H * H, H);
    fill(L.w4, n_out * H, H);
    CUM(cudaMemcpy(m->P, h.data(), n * sizeof(float), cudaMemcpyHostToDevice));
    CUM(cudaMemset(m->M, 0, n * sizeof(float)));
    CUM(cudaMemset(m->V, 0, n * sizeof(float)));
    *out = m.release();
    return GRT_OK;
}

extern "C" void grt_mlp_destroy(grt_mlp *m)
{
    if (!m) return;
    cudaSetDevice(m->device);
    cudaFree(m->P); cudaFree(m->G); cudaFree(m->M); cudaFree(m->V); cudaFree(m->loss);
    cudaFree(m->fx); cudaFree(m->fy);
    delete m;
}

extern "C" int grt_mlp_n_params(const grt_mlp *m) { return m ? m->lo.n : 0; }

extern "C" int grt_mlp_get_params(grt_mlp *m, float *host)
{
    if (!m || !host) return GRT_ERR_ARG;
    grt_ctx *ctx = m->ctx;
    CUM(cudaMemcpy(host, m->P, m->lo.n * sizeof(float), cudaMemcpyDeviceToHost));
    return GRT_OK;
}

extern "C" int grt_mlp_set_params(grt_mlp *m, const float *host)
{
    if (!m || !host) return GRT_ERR_ARG;
    grt_ctx *ctx = m->ctx;
    CUM(cudaMemcpy(m->P, host, m->lo.n * sizeof(float), cudaMemcpyHostToDevice));
    CUM(cudaMemset(m->M, 0, m->lo.n * sizeof(float)));
    CUM(cudaMemset(m->V, 0, m->lo.n * sizeof(float)));
    m->step = 0;
    return GRT_OK;
}

static size_t fwd_smem(const Layout &L) { return (size_t)L.n * sizeof(float); }
// per-sample work floats of a backward pass: pre-activations, deltas, loss share
static size_t work_floats(int n) { return (size_t)n * (3 * H + kDS + 1); }

// forward (and, with dT, backward into m->G / m->loss) over n samples;
// work: work_floats(n) floats (only for the backward)
static int launch_fb(grt_mlp *m, int n, const float *dX, const float *dT, const int *didx, float *dY, float *work,
                     cudaStream_t st)
{
    grt_ctx *ctx = m->ctx;
    const Layout &L = m->lo;
    const unsigned grid = (unsigned)((n + kThreads - 1) / kThreads);
    float *act = dT ? work : nullptr, *D = work + (size_t)n * 3 * H, *ls = D + (size_t)n * kDS;
    CUM(cudaFuncSetAttribute(mlp_forward, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)fwd_smem(L)));
    mlp_forward<<<grid, kThreads, fwd_smem(L), st>>>(m->P, L.ni, L.no, n, dX, didx, dY, act);
    CUM(cudaGetLastError());
    if (dT) {
        CUM(cudaFuncSetAttribute(mlp_delta, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)fwd_smem(L)));
        mlp_delta<<<grid, kThreads, fwd_smem(L), st>>>(m->P, L.ni, L.no, n, 1.f / ((float)n * L.no), dT,
                                                                 didx, dY, act, D, ls);
        CUM(cudaGetLastError());
        mlp_grad<<<(L.n + 1 + 127) / 128, 128, 0, st>>>(L.ni, L.no, n, dX, didx, act, D, ls, m->G, m->loss);
        CUM(cudaGetLastError());
    }
    return GRT_OK;
}

extern "C" int grt_mlp_forward(grt_mlp *m, int n, const float *x, float *y)
{
    if (!m || !x || !y || n < 1) return GRT_ERR_ARG;
    grt_ctx *ctx = m->ctx;
    CUM(cudaSetDevice(m->device));
    cudaStream_t st = nullptr;
    CUM(grt_setup_stream(ctx, &st));
    const size_t nx = (size_t)n * m->lo.ni, ny = (size_t)n * m->lo.no;
    if (nx > m->fx_n || ny > m->fy_n) {
        CUM(cudaStreamSynchronize(st));
        const size_t gx = std::max(nx, 2 * m->fx_n), gy = std::max(ny, 2 * m->fy_n);
        cudaFree(m->fx);
        cudaFree(m->fy);
        m->fx = m->fy = nullptr;
        m->fx_n = m->fy_n = 0;
        if (cudaMalloc(&m->fx, gx * sizeof(float)) != cudaSuccess || cudaMalloc(&m->fy, gy * sizeof(float)) != cudaSuccess) {
            cudaGetLastError();
            return mfail(ctx, GRT_ERR_NOMEM, "mlp forward buffers");
        }
        m->fx_n = gx;
        m->fy_n = gy;
    }
    CUM(cudaMemcpyAsync(m->fx, x, nx * sizeof(float), cudaMemcpyHostToDevice, st));
    int rc = launch_fb(m, n, m->fx, nullptr, nullptr, m->fy, nullptr, st);
    if (rc) {
        cudaStreamSynchronize(st);
        return rc;
    }
    CUM(cudaMemcpyAsync(y, m->fy, ny * sizeof(float), cudaMemcpyDeviceToHost, st));
    CUM(cudaStreamSynchronize(st));
    return GRT_OK;
}

extern "C" int grt_mlp_loss_grad(grt_mlp *m, int n, const float *x, const float *t, float *loss, float *grad)
{
    if (!m || !x || !t || n < 1) return GRT_ERR_ARG;
    grt_ctx *ctx = m->ctx;
    const Layout &L = m->lo;
    DevBufs b;
    float *dX = (float *)b.get((size_t)n * L.ni * sizeof(float)), *dT = (float *)b.get((size_t)n * L.no * sizeof(float));
    float *dY = (float *)b.get((size_t)n * L.no * sizeof(float)), *dA = (float *)b.get(work_floats(n) * sizeof(float));
    if (!dX || !dT || !dY || !dA) return mfail(ctx, GRT_ERR_NOMEM, "mlp gradient buffers");
    CUM(cudaMemcpyAsync(dX, x, (size_t)n * L.ni * sizeof(float), cudaMemcpyHostToDevice, ctx->stream));
    CUM(cudaMemcpyAsync(dT, t, (size_t)n * L.no * sizeof(float), cudaMemcpyHostToDevice, ctx->stream));
    int rc = launch_fb(m, n, dX, dT, nullptr, dY, dA, ctx->stream);
    if (rc) return rc;
    if (loss) CUM(cudaMemcpyAsync(loss, m->loss, sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
    if (grad) CUM(cudaMemcpyAsync(grad, m->G, L.n * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
    CUM(cudaStreamSynchronize(ctx->stream));
    return GRT_OK;
}

extern "C" int grt_mlp_train(grt_mlp *m, int n, const float *x, const float *t, int epochs, int batch, float lr,
                             unsigned long long seed, float *loss_out)
{
    if (!m || !x || !t || n < 1 || epochs < 1 || batch < 1) return GRT_ERR_ARG;
    grt_ctx *ctx = m->ctx;
    const Layout &L = m->lo;
    batch = std::min(batch, n);
    DevBufs b;
    float *dX = (float *)b.get((size_t)n * L.ni * sizeof(float)), *dT = (float *)b.get((size_t)n * L.no * sizeof(float));
    float *dY = (float *)b.get((size_t)batch * L.no * sizeof(float)), *dA = (float *)b.get(work_floats(batch) * sizeof(float));
    int *dI = (int *)b.get((size_t)n * sizeof(int));
    if (!dX || !dT || !dY || !dA || !dI) return mfail(ctx, GRT_ERR_NOMEM, "mlp training buffers");
    CUM(cudaMemcpyAsync(dX, x, (size_t)n * L.ni * sizeof(float), cudaMemcpyHostToDevice, ctx->stream));
    CUM(cudaMemcpyAsync(dT, t, (size_t)n * L.no * sizeof(float), cudaMemcpyHostToDevice, ctx->stream));
    std::vector<int> perm(n);
    for (int i = 0; i < n; i++) perm[i] = i;
    unsigned long long st = seed ? seed : 1;
    float last = 0.f;
    for (int ep = 0; ep < epochs; ep++) {
        for (int i = n - 1; i > 0; i--) {   // Fisher-Yates with an xorshift stream
            st ^= st << 13; st ^= st >> 7; st ^= st << 17;
            const int j = (int)(st % (unsigned long long)(i + 1));
            std::swap(perm[i], perm[j]);
        }
        CUM(cudaMemcpyAsync(dI, perm.data(), (size_t)n * sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
        CUM(cudaStreamSynchronize(ctx->stream));
        for (int s0 = 0; s0 + batch <= n; s0 += batch) {
            int rc = launch_fb(m, batch, dX, dT, dI + s0, dY, dA, ctx->stream);
            if (rc) return rc;
            m->step++;
            const float b1 = 0.9f, b2 = 0.999f;
            const float c1 = 1.f - std::pow(b1, (float)m->step), c2 = 1.f - std::pow(b2, (float)m->step);
            adam_step<<<(L.n + 255) / 256, 256, 0, ctx->stream>>>(m->P, m->G, m->M, m->V, L.n, lr, b1, b2, 1e-8f, c1, c2);
            CUM(cudaGetLastError());
        }
        CUM(cudaMemcpyAsync(&last, m->loss, sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
    }
    CUM(cudaStreamSynchronize(ctx->stream));
    if (loss_out) *loss_out = last;
    return GRT_OK;
}
