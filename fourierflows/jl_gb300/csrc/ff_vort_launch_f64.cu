// Fused vorticity kernels instantiated for FP64.
#include "ff_vort_launch_impl.cuh"

namespace ff {
FF_INSTANTIATE_VORT_LAUNCH(double)
}  // namespace ff
