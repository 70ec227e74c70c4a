// grt_ctx.h -- the context object behind grt_ctx* (shared by the library's
// translation units).
#pragma once
#include <cuda_runtime.h>

#include <map>
#include <string>

struct grt_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    int priority = 0;   // CUDA stream priority of the context's streams (0: the default)
    // set-up and fetch work (uploads, tile lists, spectra gathers): a stream of
    // the device's greatest priority, ordered after the main stream by aux_ev
    cudaStream_t aux = nullptr;
    cudaEvent_t aux_ev = nullptr;
    cudaEvent_t ev[6] = {};
    std::string err;
    // device blocks released by plans and batches, kept for reuse (by size),
    // and the blocks handed out from this cache
    std::multimap<size_t, void *> pool;
    std::map<void *, size_t> live;
    size_t pooled = 0, pool_cap = 0;
    // cuBLAS handle of the plain FP32 wavenumber sum (created on first use)
    void *blas = nullptr;
};

// The context's auxiliary stream, ordered after all work queued so far on its
// main stream: set-up work (uploads, tile lists), spectra gathers and the
// sampler network's forward pass.  At the greatest priority their small
// kernels are scheduled ahead of another context's pending blocks instead of
// after each of its long kernels.  Callers synchronise it before they return.
inline cudaError_t grt_setup_stream(grt_ctx *ctx, cudaStream_t *st)
{
    cudaError_t e = cudaEventRecord(ctx->aux_ev, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(ctx->aux, ctx->aux_ev, 0);
    *st = ctx->aux;
    return e;
}
