// grt_tc_bf16.cu -- the 3xBF16 tensor-core wavenumber sums (grt_launch.h).
#include "grt_tc_impl.cuh"

namespace grt {
template cudaError_t ksum_tc_launch_form<tc::kBF16>(int, const KsumTcArgs<float> &, unsigned, cudaStream_t);
template cudaError_t ksum_tc_limits_form<tc::kBF16>(int);
}  // namespace grt
