// Launch helpers of the fused vorticity passes.  The kernels are instantiated per
// precision in ff_vort_launch_f32.cu / ff_vort_launch_f64.cu (compiled in parallel);
// the host logic in ff_vorticity.cu only sees these declarations.
#pragma once

#include <cuda_runtime.h>

namespace ff {

struct PassLaunch {
  int grid, threads;
  size_t smem;
  int tile;   // generic path: tile width / rows per CTA
  bool reg;   // register-resident power-of-two kernels
  bool fuse = false;  // pass C, register path: also the next substep's pass A
  bool split = false; // pass C, register path, not fused: kept tiles split by field
};

struct EpiArgs {  // precision-independent copy of EpiScalars
  double c, b, dt;
  int first, use_filter;
};

template <typename T>
int vort_launch_a(const PassLaunch& L, const void* probs, const void* work, int nwork, const void* inputs,
                  cudaStream_t s);
template <typename T>
int vort_launch_b(const PassLaunch& L, const void* probs, const void* work, int nwork, cudaStream_t s);
// epi: one of the Epilogue values of ff_vorticity.cuh (0..4: bare calcN! and ETDRK4,
// 5..9: RK4 and LSRK54); each family is instantiated in its own translation unit
int vort_launch_c_etd_f32(const PassLaunch&, int, const void*, const void*, int, const EpiArgs&, cudaStream_t);
int vort_launch_c_rk_f32(const PassLaunch&, int, const void*, const void*, int, const EpiArgs&, cudaStream_t);
int vort_launch_c_etd_f64(const PassLaunch&, int, const void*, const void*, int, const EpiArgs&, cudaStream_t);
int vort_launch_c_rk_f64(const PassLaunch&, int, const void*, const void*, int, const EpiArgs&, cudaStream_t);
const void* vort_kernel_c_etd_f32(bool reg, int epi, bool fuse, bool split);
const void* vort_kernel_c_rk_f32(bool reg, int epi, bool fuse, bool split);
const void* vort_kernel_c_etd_f64(bool reg, int epi, bool fuse, bool split);
const void* vort_kernel_c_rk_f64(bool reg, int epi, bool fuse, bool split);

template <typename T>
inline int vort_launch_c(const PassLaunch& L, int epi, const void* probs, const void* work, int nwork,
                         const EpiArgs& S, cudaStream_t s) {
  const bool etd = epi <= 4;
  if (sizeof(T) == 8)
    return etd ? vort_launch_c_etd_f64(L, epi, probs, work, nwork, S, s)
               : vort_launch_c_rk_f64(L, epi, probs, work, nwork, S, s);
  return etd ? vort_launch_c_etd_f32(L, epi, probs, work, nwork, S, s)
             : vort_launch_c_rk_f32(L, epi, probs, work, nwork, S, s);
}

// kernel entry points (for occupancy queries and shared-memory limits)
template <typename T> const void* vort_kernel_a(bool reg);
template <typename T> const void* vort_kernel_b(bool reg);
template <typename T> inline const void* vort_kernel_c(bool reg, int epi, bool fuse = false, bool split = false) {
  const bool etd = epi <= 4;
  if (sizeof(T) == 8)
    return etd ? vort_kernel_c_etd_f64(reg, epi, fuse, split) : vort_kernel_c_rk_f64(reg, epi, fuse, split);
  return etd ? vort_kernel_c_etd_f32(reg, epi, fuse, split) : vort_kernel_c_rk_f32(reg, epi, fuse, split);
}

constexpr int kNumEpilogues = 10;

}  // namespace ff
