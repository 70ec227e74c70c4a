// grt_tc_impl.cuh -- launchers of the tensor-core wavenumber sum for one
// split form, included by its translation unit (grt_tc_tf32.cu, grt_tc_bf16.cu).
#pragma once
#include <map>
#include <mutex>
#include <utility>

#include "grt_ksum_tc.cuh"
#include "grt_launch.h"

namespace grt {
namespace tc_detail {

// raise a kernel's dynamic shared-memory limit, never lowering it (a captured
// graph replays launches of several sizes); one table for all contexts
template <typename F>
cudaError_t raise_smem(F *kernel, int bytes)
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

template <int SRC, int PREC>
cudaError_t form_launch(const KsumTcArgs<float> &T, unsigned grid, cudaStream_t st)
{
    cudaError_t e = raise_smem(ksum_tc_kernel<SRC, PREC>, tc::smem_bytes<SRC, PREC>());
    if (e != cudaSuccess) return e;
    ksum_tc_kernel<SRC, PREC><<<2 * grid, tc::kThreads, tc::smem_bytes<SRC, PREC>(), st>>>(T);
    return cudaGetLastError();
}

}  // namespace tc_detail

template <int PREC>
cudaError_t ksum_tc_launch_form(int cols, const KsumTcArgs<float> &T, unsigned grid, cudaStream_t st)
{
    using tc_detail::form_launch;
    switch (cols) {
    case kColSingle: return form_launch<kColSingle, PREC>(T, grid, st);
    case kColSingleFix: return form_launch<kColSingleFix, PREC>(T, grid, st);
    case kColTensorFix20: return form_launch<kColTensorFix20, PREC>(T, grid, st);
    case kColTensor: return form_launch<kColTensor, PREC>(T, grid, st);
    default: return cudaErrorInvalidValue;
    }
}

template <int PREC>
cudaError_t ksum_tc_limits_form(int cols)
{
    using tc_detail::raise_smem;
    switch (cols) {
    case kColSingle: return raise_smem(ksum_tc_kernel<kColSingle, PREC>, tc::smem_bytes<kColSingle, PREC>());
    case kColSingleFix: return raise_smem(ksum_tc_kernel<kColSingleFix, PREC>, tc::smem_bytes<kColSingleFix, PREC>());
    case kColTensorFix20:
        return raise_smem(ksum_tc_kernel<kColTensorFix20, PREC>, tc::smem_bytes<kColTensorFix20, PREC>());
    case kColTensor: return raise_smem(ksum_tc_kernel<kColTensor, PREC>, tc::smem_bytes<kColTensor, PREC>());
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace grt
