// grt_launch.h -- host launchers of the GRT kernels (grt_kernel.cuh).
//
// The kernels are instantiated in their own translation units, one per
// precision (grt_grt_f32.cu, grt_grt_f64.cu), which the build compiles in
// parallel with the rest of the library; callers see only these functions.
#pragma once
#include <cuda_runtime.h>

#include "grt_types.h"

namespace grt {

// One job: nblocks tiles of kGrtThreads wavenumbers; spec kSpecAboveTensor
// (FP32) runs the two-pass form (A.rdu set).  *launches counts the kernels.
template <typename R>
cudaError_t grt_point_launch(const GrtArgs<R> &A, int spec, unsigned nblocks, size_t smem, cudaStream_t st,
                             int *launches);

// Many jobs: nt threads per block (64, 128, 256), one block per tile
// (grid = ntiles) or persistent (grid blocks).  The first nspec tiles belong to
// FP32 jobs that allow the specialised form: the one-tile forms run them in
// two passes and the rest in one; the persistent forms run every tile in one.
template <typename R>
cudaError_t grt_batch_launch(const GrtArgs<R> *jobs, int nspec, int nt, bool persist, const int4 *tiles, int ntiles,
                             int grid, size_t smem, unsigned *err, cudaStream_t st, int *launches);

// resident blocks per SM of a persistent batch form
template <typename R>
cudaError_t grt_batch_occupancy(int nt, size_t smem, int *blocks);

// raise the dynamic shared-memory limit of every batch form to smem bytes
// (never lowered; before a stream capture)
template <typename R>
cudaError_t grt_batch_limits(int smem);

extern template cudaError_t grt_point_launch<float>(const GrtArgs<float> &, int, unsigned, size_t, cudaStream_t, int *);
extern template cudaError_t grt_point_launch<double>(const GrtArgs<double> &, int, unsigned, size_t, cudaStream_t,
                                                     int *);
extern template cudaError_t grt_batch_launch<float>(const GrtArgs<float> *, int, int, bool, const int4 *, int, int,
                                                    size_t, unsigned *, cudaStream_t, int *);
extern template cudaError_t grt_batch_launch<double>(const GrtArgs<double> *, int, int, bool, const int4 *, int, int,
                                                     size_t, unsigned *, cudaStream_t, int *);
extern template cudaError_t grt_batch_occupancy<float>(int, size_t, int *);
extern template cudaError_t grt_batch_occupancy<double>(int, size_t, int *);
extern template cudaError_t grt_batch_limits<float>(int);
extern template cudaError_t grt_batch_limits<double>(int);

}  // namespace grt

namespace grt {

template <typename R> struct KsumTcArgs;

// The tensor-core wavenumber sum (grt_ksum_tc.cuh), instantiated in
// grt_tc_tf32.cu and grt_tc_bf16.cu: one launch for both column groups
// (2 CTAs per frequency tile, receiver tile and k slice; grid counts the
// triples) of column layout cols (ColKind) in the 3xTF32 (bf16 = 0) or 3xBF16
// form.
cudaError_t ksum_tc_launch(int cols, int bf16, const KsumTcArgs<float> &T, unsigned grid, cudaStream_t st);
// raise the shared-memory limit of that form (before a stream capture)
cudaError_t ksum_tc_limits(int cols, int bf16);
// the same for one form (PREC: tc::kTF32 or tc::kBF16)
template <int PREC>
cudaError_t ksum_tc_launch_form(int cols, const KsumTcArgs<float> &T, unsigned grid, cudaStream_t st);
template <int PREC>
cudaError_t ksum_tc_limits_form(int cols);

}  // namespace grt
