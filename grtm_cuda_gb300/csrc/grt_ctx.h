// grt_ctx.h -- the context object behind grt_ctx* (shared by the library's
// translation units).
#pragma once
#include <cuda_runtime.h>

#include <map>
#include <string>

struct grt_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev[6] = {};
    std::string err;
    // batch launch shapes picked by the autotuner, by (precision, deepest model)
    std::map<std::pair<int, int>, std::pair<int, int>> tuned;
    // tensor-core k split picked for batches, as a ratio to the wave-filling default, by deepest model
    std::map<int, double> tuned_tc;
    // device blocks released by plans and batches, kept for reuse (by size),
    // and the blocks handed out from this cache
    std::multimap<size_t, void *> pool;
    std::map<void *, size_t> live;
    size_t pooled = 0, pool_cap = 0;
    // cuBLAS handle of the plain FP32 wavenumber sum (created on first use)
    void *blas = nullptr;
};
