// Fused vorticity kernels instantiated for FP64: pass C with the epilogues of
// the RK4 substeps and the LSRK54 stage.
#define FF_C_FAMILY_ETD 0
#define FF_C_FAMILY_RK 1
#include "ff_vort_launch_impl.cuh"

namespace ff {
FF_INSTANTIATE_VORT_LAUNCH_C(double, rk_f64)
}  // namespace ff
