// FP32 instantiation of the step kernels (FMA contraction allowed), plus the
// double <-> float conversions used when FP32 contexts exchange Arr3d (double) arrays.
#include "ark_kernels.cuh"

namespace ark {
template struct Launch<float>;
template void convert_from_double<float>(float *, const double *, int64_t, cudaStream_t);
template void convert_to_double<float>(double *, const float *, int64_t, cudaStream_t);
} // namespace ark
