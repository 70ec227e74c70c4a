// grt_grt_f32.cu -- the FP32 GRT kernels and their launchers (grt_launch.h).
#include "grt_grt_impl.cuh"

namespace grt {
template cudaError_t grt_point_launch<float>(const GrtArgs<float> &, int, unsigned, size_t, cudaStream_t, int *);
template cudaError_t grt_batch_launch<float>(const GrtArgs<float> *, int, int, bool, const int4 *, int, int, size_t,
                                             unsigned *, cudaStream_t, int *);
template cudaError_t grt_batch_occupancy<float>(int, size_t, int *);
template cudaError_t grt_batch_limits<float>(int);
}  // namespace grt
