// FP32 instantiation of the step kernels (built with --fmad=false like FP64), plus the
// double <-> float conversions used when FP32 contexts exchange Arr3d (double) arrays.
#include "ark_kernels.cuh"

namespace ark {
template struct Launch<float>;
template void convert_from_double<float>(float *, const double *, int64_t, double, cudaStream_t);
template void convert_to_double<float>(double *, const float *, int64_t, double, cudaStream_t);
template void face_density_to_double<float>(double *, const float *, int64_t, double, double, cudaStream_t);
} // namespace ark
