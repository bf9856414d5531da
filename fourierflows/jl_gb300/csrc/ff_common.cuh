// Shared definitions for libfourierflows_gb300: complex helpers, status codes and the
// per-thread last-error buffer behind ff_last_error().
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

#include "../../../include/fourierflows_gb300.h"

namespace ff {

// ---------------------------------------------------------------------------------------
// complex numbers as interleaved (re, im) pairs: float2 / double2
// ---------------------------------------------------------------------------------------
template <typename T> struct V2;
template <> struct V2<float> { using type = float2; };
template <> struct V2<double> { using type = double2; };
template <typename T> using cx = typename V2<T>::type;

template <typename T> __host__ __device__ __forceinline__ cx<T> mk(T a, T b) {
  cx<T> r;
  r.x = a;
  r.y = b;
  return r;
}

// Overloads for both storage types so that argument deduction works at call sites.
#define FF_CX_OPS(C, R)                                                                     \
  __device__ __forceinline__ C add(C a, C b) { C r; r.x = a.x + b.x; r.y = a.y + b.y; return r; } \
  __device__ __forceinline__ C sub(C a, C b) { C r; r.x = a.x - b.x; r.y = a.y - b.y; return r; } \
  __device__ __forceinline__ C cmul(C a, C b) {                                              \
    C r;                                                                                     \
    r.x = fma(a.x, b.x, -a.y * b.y);                                                         \
    r.y = fma(a.x, b.y, a.y * b.x);                                                          \
    return r;                                                                                \
  }                                                                                          \
  /* a * conj(b) */                                                                          \
  __device__ __forceinline__ C cmulc(C a, C b) {                                             \
    C r;                                                                                     \
    r.x = fma(a.x, b.x, a.y * b.y);                                                          \
    r.y = fma(a.y, b.x, -a.x * b.y);                                                         \
    return r;                                                                                \
  }                                                                                          \
  __device__ __forceinline__ C conj(C a) { C r; r.x = a.x; r.y = -a.y; return r; }           \
  __device__ __forceinline__ C scl(C a, R s) { C r; r.x = a.x * s; r.y = a.y * s; return r; } \
  /* multiply by +i and by -i */                                                             \
  __device__ __forceinline__ C mul_i(C a) { C r; r.x = -a.y; r.y = a.x; return r; }          \
  __device__ __forceinline__ C mul_mi(C a) { C r; r.x = a.y; r.y = -a.x; return r; }

FF_CX_OPS(float2, float)
FF_CX_OPS(double2, double)
#undef FF_CX_OPS

template <typename T> __device__ __forceinline__ cx<T> czero() { return mk<T>(T(0), T(0)); }

// ---------------------------------------------------------------------------------------
// L2 prefetch hints (no register result, no completion to wait for)
// ---------------------------------------------------------------------------------------
__device__ __forceinline__ void prefetch_l2(const void* p) { asm volatile("prefetch.global.L2 [%0];" ::"l"(p)); }

// every 128-byte line of a contiguous span, spread over the threads of the CTA
template <typename E> __device__ __forceinline__ void prefetch_lines(const E* p, int n, int lane, int lanes) {
  const uintptr_t a = reinterpret_cast<uintptr_t>(p) & ~uintptr_t(127);
  const uintptr_t e = reinterpret_cast<uintptr_t>(p + n);
  for (uintptr_t x = a + (uintptr_t)lane * 128; x < e; x += (uintptr_t)lanes * 128)
    prefetch_l2(reinterpret_cast<const void*>(x));
}

// ---------------------------------------------------------------------------------------
// errors
// ---------------------------------------------------------------------------------------
void set_error(const char* fmt, ...);
int cuda_status(cudaError_t e, const char* what);

#define FF_CHECK_ARG(cond, ...)     \
  do {                              \
    if (!(cond)) {                  \
      ::ff::set_error(__VA_ARGS__); \
      return FF_ERR_ARG;            \
    }                               \
  } while (0)

#define FF_CUDA(call)                                             \
  do {                                                            \
    cudaError_t e__ = (call);                                     \
    if (e__ != cudaSuccess) return ::ff::cuda_status(e__, #call); \
  } while (0)

#define FF_LAUNCHED(what)                                        \
  do {                                                           \
    cudaError_t e__ = cudaGetLastError();                        \
    if (e__ != cudaSuccess) return ::ff::cuda_status(e__, what); \
  } while (0)

inline int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }

// grid size for flat elementwise kernels: a multiple of the SM count, capped by the work
int elementwise_grid(int64_t n, int threads);
int sm_count();

}  // namespace ff
