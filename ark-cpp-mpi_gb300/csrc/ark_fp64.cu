// FP64 instantiation of the step kernels.  Built with --fmad=false: no a*b+c is fused, so
// every operation rounds as the reference's does when built with -ffp-contract=off.
#include "ark_kernels.cuh"

namespace ark {
template struct Launch<double>;
} // namespace ark
