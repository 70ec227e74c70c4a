// grt_tc_tf32.cu -- the 3xTF32 tensor-core wavenumber sums and the
// dispatch of both split forms (grt_launch.h).
#include "grt_tc_impl.cuh"

namespace grt {

template cudaError_t ksum_tc_launch_form<tc::kTF32>(int, const KsumTcArgs<float> &, unsigned, cudaStream_t);
template cudaError_t ksum_tc_limits_form<tc::kTF32>(int);
// the 3xBF16 form is compiled in grt_tc_bf16.cu
extern template cudaError_t ksum_tc_launch_form<tc::kBF16>(int, const KsumTcArgs<float> &, unsigned, cudaStream_t);
extern template cudaError_t ksum_tc_limits_form<tc::kBF16>(int);

cudaError_t ksum_tc_launch(int cols, int bf16, const KsumTcArgs<float> &T, unsigned grid, cudaStream_t st)
{
    return bf16 ? ksum_tc_launch_form<tc::kBF16>(cols, T, grid, st) : ksum_tc_launch_form<tc::kTF32>(cols, T, grid, st);
}

cudaError_t ksum_tc_limits(int cols, int bf16)
{
    return bf16 ? ksum_tc_limits_form<tc::kBF16>(cols) : ksum_tc_limits_form<tc::kTF32>(cols);
}

}  // namespace grt
