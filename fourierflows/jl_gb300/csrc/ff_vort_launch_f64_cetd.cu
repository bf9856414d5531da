// Fused vorticity kernels instantiated for FP64: pass C with the epilogues of
// the bare calcN! and the ETDRK4 substeps.
#define FF_C_FAMILY_ETD 1
#define FF_C_FAMILY_RK 0
#include "ff_vort_launch_impl.cuh"

namespace ff {
FF_INSTANTIATE_VORT_LAUNCH_C(double, etd_f64)
}  // namespace ff
