// Definitions of the launch helpers declared in ff_vort_launch.cuh, instantiated for one
// precision by ff_vort_launch_f32.cu / ff_vort_launch_f64.cu.
#pragma once

#include "ff_vort_launch.cuh"
#include "ff_vorticity.cuh"

namespace ff {

template <typename T> static EpiScalars<T> to_scalars(const EpiArgs& a) {
  EpiScalars<T> S;
  S.c = (T)a.c;
  S.b = (T)a.b;
  S.dt = (T)a.dt;
  S.first = a.first;
  S.use_filter = a.use_filter;
  return S;
}

template <typename T>
int vort_launch_a(const PassLaunch& L, const void* probs, const void* work, int nwork, const void* inputs,
                  cudaStream_t s) {
  const auto* P = (const VortProb<T>*)probs;
  if (L.reg)
    k_vort_a_r<T><<<L.grid, L.threads, L.smem, s>>>(P, (const WorkItem*)work, nwork, (const cx<T>* const*)inputs);
  else
    k_vort_a<T><<<L.grid, L.threads, L.smem, s>>>(P, (const WorkItem*)work, nwork, L.tile,
                                                  (const cx<T>* const*)inputs);
  FF_LAUNCHED("k_vort_a");
  return FF_OK;
}

template <typename T>
int vort_launch_b(const PassLaunch& L, const void* probs, const void* work, int nwork, cudaStream_t s) {
  const auto* P = (const VortProb<T>*)probs;
  if (L.reg) k_vort_b_r<T><<<L.grid, L.threads, L.smem, s>>>(P, (const WorkItem*)work, nwork);
  else k_vort_b<T><<<L.grid, L.threads, L.smem, s>>>(P, (const WorkItem*)work, nwork, L.tile);
  FF_LAUNCHED("k_vort_b");
  return FF_OK;
}

template <typename T, int EPI>
static void launch_c_epi(const PassLaunch& L, const VortProb<T>* P, const WorkItem* work, int nwork,
                         const EpiScalars<T>& S, cudaStream_t s) {
  if (L.reg) {
    if constexpr (EPI != EPI_N && EPI != EPI_ETD4 && EPI != EPI_RK4) {
      if (L.fuse) {
        k_vort_c_r<T, EPI, true><<<L.grid, L.threads, L.smem, s>>>(P, work, nwork, S);
        return;
      }
    }
    if constexpr (!FuseA<T>::value) {  // the split form exists where pass C runs unfused
      if (L.split) {
        k_vort_c_rs<T, EPI><<<L.grid, L.threads, L.smem, s>>>(P, work, nwork, S);
        return;
      }
    }
    k_vort_c_r<T, EPI, false><<<L.grid, L.threads, L.smem, s>>>(P, work, nwork, S);
  } else {
    k_vort_c<T, EPI><<<L.grid, L.threads, L.smem, s>>>(P, work, nwork, L.tile, S);
  }
}

#if FF_C_FAMILY_ETD || FF_C_FAMILY_RK
// pass C launchers of one family of epilogues (compiled in their own translation units):
// ETD = the bare calcN! and the ETDRK4 substeps, RK = the RK4 substeps and the LSRK54 stage
template <typename T>
int vort_launch_c_family(const PassLaunch& L, int epi, const void* probs, const void* work, int nwork,
                         const EpiArgs& a, cudaStream_t s) {
  const auto* P = (const VortProb<T>*)probs;
  const auto* w = (const WorkItem*)work;
  const EpiScalars<T> S = to_scalars<T>(a);
  switch (epi) {
#define FF_EPI_CASE(E) \
  case E: launch_c_epi<T, E>(L, P, w, nwork, S, s); break;
#if FF_C_FAMILY_ETD
    FF_EPI_CASE(EPI_N) FF_EPI_CASE(EPI_ETD1) FF_EPI_CASE(EPI_ETD2) FF_EPI_CASE(EPI_ETD3) FF_EPI_CASE(EPI_ETD4)
#endif
#if FF_C_FAMILY_RK
    FF_EPI_CASE(EPI_RK1) FF_EPI_CASE(EPI_RK2) FF_EPI_CASE(EPI_RK3) FF_EPI_CASE(EPI_RK4) FF_EPI_CASE(EPI_LS)
#endif
#undef FF_EPI_CASE
    default: set_error("vort_launch_c: epilogue %d is not in this family", epi); return FF_ERR_ARG;
  }
  FF_LAUNCHED("k_vort_c");
  return FF_OK;
}

template <typename T, int EPI> static const void* fuse_ptr(bool fuse, bool split) {
  if constexpr (EPI != EPI_N && EPI != EPI_ETD4 && EPI != EPI_RK4) {
    if (fuse) return (const void*)k_vort_c_r<T, EPI, true>;
  }
  if constexpr (!FuseA<T>::value) {
    if (split) return (const void*)k_vort_c_rs<T, EPI>;
  }
  return (const void*)k_vort_c_r<T, EPI, false>;
}

template <typename T> const void* vort_kernel_c_family(bool reg, int epi, bool fuse, bool split) {
  switch (epi) {
#define FF_EPI_PTR(E) \
  case E: return !reg ? (const void*)k_vort_c<T, E> : fuse_ptr<T, E>(fuse, split);
#if FF_C_FAMILY_ETD
    FF_EPI_PTR(EPI_N) FF_EPI_PTR(EPI_ETD1) FF_EPI_PTR(EPI_ETD2) FF_EPI_PTR(EPI_ETD3) FF_EPI_PTR(EPI_ETD4)
#endif
#if FF_C_FAMILY_RK
    FF_EPI_PTR(EPI_RK1) FF_EPI_PTR(EPI_RK2) FF_EPI_PTR(EPI_RK3) FF_EPI_PTR(EPI_RK4) FF_EPI_PTR(EPI_LS)
#endif
#undef FF_EPI_PTR
    default: return nullptr;
  }
}

#endif

template <typename T> const void* vort_kernel_a(bool reg) {
  return reg ? (const void*)k_vort_a_r<T> : (const void*)k_vort_a<T>;
}
template <typename T> const void* vort_kernel_b(bool reg) {
  return reg ? (const void*)k_vort_b_r<T> : (const void*)k_vort_b<T>;
}

// passes A and B, and pass C, in separate translation units (they compile in parallel)
#define FF_INSTANTIATE_VORT_LAUNCH_AB(T)                                                                         \
  template int vort_launch_a<T>(const PassLaunch&, const void*, const void*, int, const void*, cudaStream_t);    \
  template int vort_launch_b<T>(const PassLaunch&, const void*, const void*, int, cudaStream_t);                 \
  template const void* vort_kernel_a<T>(bool);                                                                   \
  template const void* vort_kernel_b<T>(bool);
#define FF_INSTANTIATE_VORT_LAUNCH_C(T, NAME)                                                                    \
  int vort_launch_c_##NAME(const PassLaunch& L, int epi, const void* probs, const void* work, int nwork,          \
                           const EpiArgs& a, cudaStream_t s) {                                                   \
    return vort_launch_c_family<T>(L, epi, probs, work, nwork, a, s);                                            \
  }                                                                                                              \
  const void* vort_kernel_c_##NAME(bool reg, int epi, bool fuse, bool split) {                                  \
    return vort_kernel_c_family<T>(reg, epi, fuse, split);                                                       \
  }

}  // namespace ff
