// grt_grt_f64.cu -- the FP64 GRT kernels and their launchers (grt_launch.h).
#include "grt_grt_impl.cuh"

namespace grt {
template cudaError_t grt_point_launch<double>(const GrtArgs<double> &, int, unsigned, size_t, cudaStream_t, int *);
template cudaError_t grt_batch_launch<double>(const GrtArgs<double> *, int, int, bool, const int4 *, int, int, size_t,
                                              unsigned *, cudaStream_t, int *);
template cudaError_t grt_batch_occupancy<double>(int, size_t, int *);
template cudaError_t grt_batch_limits<double>(int);
}  // namespace grt
