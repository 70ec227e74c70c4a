// grt_grt_impl.cuh -- definitions of the GRT launchers (grt_launch.h),
// included by the per-precision translation units.
#pragma once
#include <map>
#include <mutex>
#include <type_traits>
#include <utility>

#include "grt_kernel.cuh"
#include "grt_launch.h"

namespace grt {
namespace launch_detail {

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

template <typename R, int NT, bool P>
void batch(const GrtArgs<R> *jobs, int nspec, const int4 *tiles, int ntiles, int grid, size_t smem, unsigned *err,
           cudaStream_t st, int *launches)
{
    // one-tile forms: the leading tiles of jobs that allow the specialised
    // evaluation in two passes (bottom-up, then the rest; GrtArgs::rdu
    // between), the remaining tiles in the generic one
    if constexpr (!P && std::is_same<R, float>::value) {
        if (nspec > 0) {
            grt_batch_kernel<R, NT, P, kSpecAboveTensor, 1><<<nspec, NT, smem, st>>>(jobs, tiles, nspec, err);
            grt_batch_kernel<R, NT, P, kSpecAboveTensor, 2><<<nspec, NT, smem, st>>>(jobs, tiles, nspec, err);
            if (launches) *launches += 2;
        }
        if (ntiles > nspec) {
            grt_batch_kernel<R, NT, P><<<ntiles - nspec, NT, smem, st>>>(jobs, tiles + nspec, ntiles - nspec, err);
            if (launches) *launches += 1;
        }
        return;
    }
    grt_batch_kernel<R, NT, P><<<grid, NT, smem, st>>>(jobs, tiles, ntiles, err);
    if (launches) *launches += 1;
}

}  // namespace launch_detail

template <typename R>
cudaError_t grt_point_launch(const GrtArgs<R> &A, int spec, unsigned nblocks, size_t smem, cudaStream_t st,
                             int *launches)
{
    if constexpr (std::is_same<R, float>::value) {
        if (spec == kSpecAboveTensor) {
            grt_point_kernel<R, kSpecAboveTensor, 1><<<nblocks, kGrtThreads, smem, st>>>(A);
            grt_point_kernel<R, kSpecAboveTensor, 2><<<nblocks, kGrtThreads, smem, st>>>(A);
            if (launches) *launches += 2;
            return cudaGetLastError();
        }
    }
    grt_point_kernel<R><<<nblocks, kGrtThreads, smem, st>>>(A);
    if (launches) *launches += 1;
    return cudaGetLastError();
}

template <typename R>
cudaError_t grt_batch_launch(const GrtArgs<R> *jobs, int nspec, int nt, bool persist, const int4 *tiles, int ntiles,
                             int grid, size_t smem, unsigned *err, cudaStream_t st, int *launches)
{
    using namespace launch_detail;
    if (ntiles <= 0) return cudaSuccess;
    nspec = nspec < 0 ? 0 : nspec > ntiles ? ntiles : nspec;
    if (!persist) {
        if (nt == 64) batch<R, 64, false>(jobs, nspec, tiles, ntiles, ntiles, smem, err, st, launches);
        else if (nt == 128) batch<R, 128, false>(jobs, nspec, tiles, ntiles, ntiles, smem, err, st, launches);
        else batch<R, 256, false>(jobs, nspec, tiles, ntiles, ntiles, smem, err, st, launches);
    } else {
        if (nt == 128) batch<R, 128, true>(jobs, nspec, tiles, ntiles, grid, smem, err, st, launches);
        else batch<R, 256, true>(jobs, nspec, tiles, ntiles, grid, smem, err, st, launches);
    }
    return cudaGetLastError();
}

template <typename R>
cudaError_t grt_batch_occupancy(int nt, size_t smem, int *blocks)
{
    *blocks = 1;
    cudaError_t e = nt == 128 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, grt_batch_kernel<R, 128, true>,
                                                                             128, smem)
                              : cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, grt_batch_kernel<R, 256, true>,
                                                                             256, smem);
    if (*blocks < 1) *blocks = 1;
    return e;
}

template <typename R>
cudaError_t grt_batch_limits(int smem)
{
    using launch_detail::raise_smem;
    cudaError_t e;
    if ((e = raise_smem(grt_batch_kernel<R, 64, false>, smem)) != cudaSuccess) return e;
    if ((e = raise_smem(grt_batch_kernel<R, 128, false>, smem)) != cudaSuccess) return e;
    if ((e = raise_smem(grt_batch_kernel<R, 256, false>, smem)) != cudaSuccess) return e;
    if ((e = raise_smem(grt_batch_kernel<R, 128, true>, smem)) != cudaSuccess) return e;
    if constexpr (std::is_same<R, float>::value) {
        if ((e = raise_smem(grt_batch_kernel<R, 64, false, kSpecAboveTensor, 1>, smem)) != cudaSuccess) return e;
        if ((e = raise_smem(grt_batch_kernel<R, 128, false, kSpecAboveTensor, 1>, smem)) != cudaSuccess) return e;
        if ((e = raise_smem(grt_batch_kernel<R, 256, false, kSpecAboveTensor, 1>, smem)) != cudaSuccess) return e;
        if ((e = raise_smem(grt_batch_kernel<R, 64, false, kSpecAboveTensor, 2>, smem)) != cudaSuccess) return e;
        if ((e = raise_smem(grt_batch_kernel<R, 128, false, kSpecAboveTensor, 2>, smem)) != cudaSuccess) return e;
        if ((e = raise_smem(grt_batch_kernel<R, 256, false, kSpecAboveTensor, 2>, smem)) != cudaSuccess) return e;
    }
    return raise_smem(grt_batch_kernel<R, 256, true>, smem);
}

}  // namespace grt
