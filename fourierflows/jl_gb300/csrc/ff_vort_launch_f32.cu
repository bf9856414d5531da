// Fused vorticity kernels instantiated for FP32: passes A and B.
#include "ff_vort_launch_impl.cuh"

namespace ff {
FF_INSTANTIATE_VORT_LAUNCH_AB(float)
}  // namespace ff
