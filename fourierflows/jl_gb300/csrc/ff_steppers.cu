// Elementwise kernels of the generic time-stepping path: each reference broadcast group
// of a substep (src/timesteppers.jl) becomes one pass over HBM, plus dealias!, the
// spectral helpers of the Diffusion module and the Parseval reductions.
//
// Arithmetic follows the reference broadcasts' evaluation order so that FP64 results
// agree with the CPU restatement to rounding.
#include <mutex>
#include <vector>

#include "ff_common.cuh"

namespace ff {

// per-mode coefficient (see ff_coef); the kind is uniform across the launch
template <typename T> struct Coef {
  const void* p;
  int kind;
  T re, im;
  __device__ __forceinline__ cx<T> mul(cx<T> v, int64_t i) const {
    switch (kind) {
      case FF_COEF_REAL: return scl(v, static_cast<const T*>(p)[i]);
      case FF_COEF_COMPLEX: return cmul(static_cast<const cx<T>*>(p)[i], v);
      case FF_COEF_SCALAR: return im == T(0) ? scl(v, re) : cmul(mk<T>(re, im), v);
      default: return czero<T>();
    }
  }
};

template <typename T> static Coef<T> coef(const ff_coef& c) {
  Coef<T> r;
  r.p = c.ptr;
  r.kind = c.kind;
  r.re = (T)c.re;
  r.im = (T)c.im;
  return r;
}

static int check_coef(const ff_coef& c, const char* what) {
  FF_CHECK_ARG(c.kind >= FF_COEF_NONE && c.kind <= FF_COEF_SCALAR, "%s: bad coefficient kind %d", what, c.kind);
  FF_CHECK_ARG(!(c.kind == FF_COEF_REAL || c.kind == FF_COEF_COMPLEX) || c.ptr != nullptr,
               "%s: coefficient array is null", what);
  return FF_OK;
}

#define GRID_STRIDE(i, n) for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < (n); i += (int64_t)gridDim.x * blockDim.x)

template <typename T>
__global__ void k_euler(int64_t n, cx<T>* sol, const cx<T>* __restrict__ N, Coef<T> L, T dt, const T* filter) {
  GRID_STRIDE(i, n) {
    const cx<T> s = sol[i];
    cx<T> v;
    if (filter) v = scl(add(s, scl(add(N[i], L.mul(s, i)), dt)), filter[i]);
    else v = add(s, scl(add(L.mul(s, i), N[i]), dt));
    sol[i] = v;
  }
}

template <typename T>
__global__ void k_rk4_substep(int64_t n, cx<T>* RHS, Coef<T> L, const cx<T>* x, const cx<T>* sol, cx<T>* newsol,
                              T c) {
  GRID_STRIDE(i, n) {
    const cx<T> r = add(RHS[i], L.mul(x[i], i));
    RHS[i] = r;
    if (newsol) newsol[i] = add(sol[i], scl(r, c));
  }
}

template <typename T>
__global__ void k_rk4_update(int64_t n, cx<T>* sol, cx<T>* RHS4, Coef<T> L, const cx<T>* x, const cx<T>* R1,
                             const cx<T>* R2, const cx<T>* R3, T c6, const T* filter) {
  GRID_STRIDE(i, n) {
    const cx<T> r4 = add(RHS4[i], L.mul(x[i], i));
    RHS4[i] = r4;
    const cx<T> acc = add(add(add(R1[i], scl(R2[i], T(2))), scl(R3[i], T(2))), r4);
    cx<T> v = add(sol[i], scl(acc, c6));
    if (filter) v = scl(v, filter[i]);
    sol[i] = v;
  }
}

template <typename T>
__global__ void k_lsrk54(int64_t n, cx<T>* sol, cx<T>* RHS, cx<T>* S2, Coef<T> L, T A, T B, T dt, int first,
                         const T* filter) {
  GRID_STRIDE(i, n) {
    const cx<T> s = sol[i];
    const cx<T> r = add(RHS[i], L.mul(s, i));
    RHS[i] = r;
    const cx<T> q = first ? scl(r, dt) : add(scl(S2[i], A), scl(r, dt));
    S2[i] = q;
    cx<T> v = add(s, scl(q, B));
    if (filter) v = scl(v, filter[i]);
    sol[i] = v;
  }
}

template <typename T>
__global__ void k_etd12(int64_t n, cx<T>* out, Coef<T> eh, const cx<T>* sol, Coef<T> z, const cx<T>* N) {
  GRID_STRIDE(i, n) out[i] = add(eh.mul(sol[i], i), z.mul(N[i], i));
}

template <typename T>
__global__ void k_etd3(int64_t n, cx<T>* out, Coef<T> eh, const cx<T>* sol1, Coef<T> z, const cx<T>* N1,
                       const cx<T>* N3) {
  GRID_STRIDE(i, n) out[i] = add(eh.mul(sol1[i], i), z.mul(sub(scl(N3[i], T(2)), N1[i]), i));
}

template <typename T>
__global__ void k_etd_update(int64_t n, cx<T>* sol, Coef<T> eL, Coef<T> a, Coef<T> b, Coef<T> g,
                             const cx<T>* N1, const cx<T>* N2, const cx<T>* N3, const cx<T>* N4, const T* filter) {
  GRID_STRIDE(i, n) {
    // expL sol + alpha N1 + (2 beta)(N2 + N3) + Gamma N4
    cx<T> v = add(eL.mul(sol[i], i), a.mul(N1[i], i));
    v = add(v, scl(b.mul(add(N2[i], N3[i]), i), T(2)));
    v = add(v, g.mul(N4[i], i));
    if (filter) v = scl(v, filter[i]);
    sol[i] = v;
  }
}

template <typename T>
__global__ void k_ab3(int64_t n, cx<T>* sol, cx<T>* RHS, cx<T>* Rm1, cx<T>* Rm2, Coef<T> L, T dt, int euler,
                      T h1, T h2, T h3, const T* filter) {
  GRID_STRIDE(i, n) {
    const cx<T> s = sol[i];
    const cx<T> r = add(RHS[i], L.mul(s, i));
    RHS[i] = r;
    const cx<T> m1 = Rm1[i];
    cx<T> v;
    if (euler) v = add(s, scl(r, dt));
    else v = add(s, scl(add(sub(scl(r, h1), scl(m1, h2)), scl(Rm2[i], h3)), dt));
    if (filter) v = scl(v, filter[i]);
    sol[i] = v;
    Rm2[i] = m1;
    Rm1[i] = r;
  }
}

template <typename T> __global__ void k_filter(int64_t n, cx<T>* sol, const T* __restrict__ f) {
  GRID_STRIDE(i, n) sol[i] = scl(sol[i], f[i]);
}

// ---- whole steps of a linear equation (N = 0): one pass for nsteps steps -----------------
// The Diffusion module's constant-kappa calcN! sets N = 0 (src/diffusion.jl:129-133).  An
// ETDRK4 step then reduces exactly to sol = [filter] exp(L dt) sol: every term in N1..N4
// of ETDRK4update! adds an exact zero (src/timesteppers.jl:501-504,552).  An RK4 step is
// its four linear stages, computed in registers in the order the generic kernels take them
// (k_rk4_substep three times, then k_rk4_update), so both give the generic path's bits.
template <typename T>
__global__ void k_linear_etd(int64_t n, cx<T>* sol, Coef<T> eL, const T* __restrict__ filter, int nsteps) {
  GRID_STRIDE(i, n) {
    cx<T> v = sol[i];
    for (int k = 0; k < nsteps; ++k) {
      v = eL.mul(v, i);
      if (filter) v = scl(v, filter[i]);
    }
    sol[i] = v;
  }
}

// FP32 state with a real exp(L dt): two modes per thread per iteration (16-byte state and
// 8-byte coefficient loads), four iterations in flight per thread
__global__ void k_linear_etd_f32x2(int64_t npairs, float4* sol, const float2* __restrict__ eL,
                                   const float2* __restrict__ filter, int nsteps) {
  constexpr int U = 4;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i0 = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i0 < npairs; i0 += U * stride) {
    float4 v[U];
    float2 e[U], f[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int64_t i = i0 + u * stride;
      if (i < npairs) {
        v[u] = sol[i];
        e[u] = eL[i];
        f[u] = filter ? filter[i] : make_float2(1.f, 1.f);
      }
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int64_t i = i0 + u * stride;
      if (i < npairs) {
        float4 x = v[u];
        for (int k = 0; k < nsteps; ++k) {
          x.x *= e[u].x;
          x.y *= e[u].x;
          x.z *= e[u].y;
          x.w *= e[u].y;
          if (filter) {
            x.x *= f[u].x;
            x.y *= f[u].x;
            x.z *= f[u].y;
            x.w *= f[u].y;
          }
        }
        sol[i] = x;
      }
    }
  }
}

__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }

// L x rounded on its own, as the generic kernels' RHS = N + L x with N = 0 rounds it: a
// bare product must not be contracted into the add that consumes it
template <typename T> __device__ __forceinline__ cx<T> lin(const Coef<T>& L, cx<T> v, int64_t i) {
  if (L.kind == FF_COEF_REAL) {
    const T c = static_cast<const T*>(L.p)[i];
    return mk<T>(mul_rn(v.x, c), mul_rn(v.y, c));
  }
  if (L.kind == FF_COEF_SCALAR && L.im == T(0)) return mk<T>(mul_rn(v.x, L.re), mul_rn(v.y, L.re));
  return L.mul(v, i);
}

template <typename T>
__global__ void k_linear_rk4(int64_t n, cx<T>* sol, Coef<T> L, T half, T dt, T c6, const T* __restrict__ filter,
                             int nsteps) {
  GRID_STRIDE(i, n) {
    cx<T> s = sol[i];
    for (int k = 0; k < nsteps; ++k) {
      const cx<T> r1 = lin(L, s, i);
      cx<T> x = add(s, scl(r1, half));
      const cx<T> r2 = lin(L, x, i);
      x = add(s, scl(r2, half));
      const cx<T> r3 = lin(L, x, i);
      x = add(s, scl(r3, dt));
      const cx<T> r4 = lin(L, x, i);
      const cx<T> acc = add(add(add(r1, scl(r2, T(2))), scl(r3, T(2))), r4);
      s = add(s, scl(acc, c6));
      if (filter) s = scl(s, filter[i]);
    }
    sol[i] = s;
  }
}

template <typename T>
__global__ void k_dealias(cx<T>* fh, int64_t d0, int64_t d1, int64_t d2, int64_t total, int64_t lo0, int64_t hi0,
                          int64_t lo1, int64_t hi1, int64_t lo2, int64_t hi2) {
  GRID_STRIDE(i, total) {
    const int64_t i0 = i % d0;
    const int64_t r = i / d0;
    const int64_t i1 = r % d1;
    const int64_t i2 = (r / d1) % d2;
    if ((i0 >= lo0 && i0 < hi0) || (i1 >= lo1 && i1 < hi1) || (i2 >= lo2 && i2 < hi2)) fh[i] = czero<T>();
  }
}

template <typename T>
__global__ void k_mul_ik(int64_t n0, int64_t total, cx<T>* out, const cx<T>* in, const T* __restrict__ k) {
  GRID_STRIDE(i, total) out[i] = mul_i(scl(in[i], k[i % n0]));
}

// ---- ETDRK4 coefficients by the Kassam-Trefethen contour means, in FP64 ------------------
// For each mode, z_j = dt L + r exp(2 pi i (j + 1/2) / M), j < M, and
//   zeta  = dt mean((e^{z/2} - 1) / z)
//   alpha = dt mean((-4 - z + e^z (4 - 3z + z^2)) / z^3)
//   beta  = dt mean(( 2 + z + e^z (-2 + z)) / z^3)
//   Gamma = dt mean((-4 - 3z - z^2 + e^z (4 - z)) / z^3)
// (the reference's getetdcoeffs, src/timesteppers.jl:689-718; real parts for real L).
struct Circle {
  double2 c[64];
  int m;
};

__device__ __forceinline__ double2 cexp64(double2 z) {
  double s, c;
  sincos(z.y, &s, &c);
  const double e = exp(z.x);
  return make_double2(e * c, e * s);
}

__device__ __forceinline__ double2 cdiv64(double2 a, double2 b) {
  const double d = b.x * b.x + b.y * b.y;
  return make_double2((a.x * b.x + a.y * b.y) / d, (a.y * b.x - a.x * b.y) / d);
}

template <typename T>
__global__ void k_etd_coefs(int64_t n, const T* __restrict__ L, T dt, Circle circ, T* zeta, T* alpha, T* beta,
                            T* gamma) {
  GRID_STRIDE(i, n) {
    const double dtl = (double)(T)(dt * L[i]);  // dt L in L's precision, then FP64
    double2 sz = make_double2(0, 0), sa = sz, sb = sz, sg = sz;
    for (int j = 0; j < circ.m; ++j) {
      const double2 z = make_double2(dtl + circ.c[j].x, circ.c[j].y);
      const double2 ez = cexp64(z);
      const double2 eh = cexp64(make_double2(0.5 * z.x, 0.5 * z.y));
      const double2 z2 = cmul(z, z);
      const double2 z3 = cmul(z2, z);
      sz = add(sz, cdiv64(make_double2(eh.x - 1.0, eh.y), z));
      // -4 - z + e^z (4 - 3z + z^2)
      const double2 pa = add(make_double2(-4.0 - z.x, -z.y), cmul(ez, make_double2(4.0 - 3.0 * z.x + z2.x,
                                                                                   -3.0 * z.y + z2.y)));
      // 2 + z + e^z (-2 + z)
      const double2 pb = add(make_double2(2.0 + z.x, z.y), cmul(ez, make_double2(-2.0 + z.x, z.y)));
      // -4 - 3z - z^2 + e^z (4 - z)
      const double2 pg = add(make_double2(-4.0 - 3.0 * z.x - z2.x, -3.0 * z.y - z2.y),
                             cmul(ez, make_double2(4.0 - z.x, -z.y)));
      sa = add(sa, cdiv64(pa, z3));
      sb = add(sb, cdiv64(pb, z3));
      sg = add(sg, cdiv64(pg, z3));
    }
    const double f = (double)dt / circ.m;
    zeta[i] = (T)(f * sz.x);
    alpha[i] = (T)(f * sa.x);
    beta[i] = (T)(f * sb.x);
    gamma[i] = (T)(f * sg.x);
  }
}

// u_hat = i l zeta_hat / K^2, v_hat = -i kr zeta_hat / K^2 (psi_hat = -zeta_hat / K^2)
template <typename T>
__global__ void k_velocities(int64_t nkr, int64_t n, const cx<T>* __restrict__ zh, const T* __restrict__ kr,
                             const T* __restrict__ l, const T* __restrict__ invK, cx<T>* uh, cx<T>* vh) {
  GRID_STRIDE(i, n) {
    const cx<T> z = zh[i];
    const int64_t c = i % nkr, j = i / nkr;
    uh[i] = mul_i(scl(z, l[j] * invK[i]));
    vh[i] = mul_mi(scl(z, kr[c] * invK[i]));
  }
}

template <typename T> __global__ void k_real_mul(int64_t n, int64_t na, T* x, const T* __restrict__ a) {
  GRID_STRIDE(i, n) x[i] *= a[i % na];
}

// ---- deterministic two-pass reduction ---------------------------------------------------
// pass 1: each CTA writes one FP64 partial; pass 2: one CTA sums the partials in order.
#define FF_RED_THREADS 256
#define FF_RED_MAXBLOCKS 1024

__device__ __forceinline__ double block_sum(double v) {
  __shared__ double sh[FF_RED_THREADS / 32];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) sh[w] = v;
  __syncthreads();
  v = 0.0;
  if (w == 0) {
    v = l < (int)(blockDim.x >> 5) ? sh[l] : 0.0;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  }
  return v;
}

// mode 0: |u|^2 [* wt]; mode 1: Re u.  rfft_form weights rows 1..n0-2 by 2.
// On GB300 FP64 runs at 2 instructions per SM per cycle, so with FP64 data this reduction
// is bound by the FP64 pipe before HBM: each mode costs two FMAs into one of two
// accumulators (rows counted once, rows counted twice; the factor 2 is applied once at the
// end), one more with a weight.  The row index i0 = i mod n0 advances by S mod n0 (S = the
// grid's thread count) instead of a 64-bit division per mode.
template <typename T>
__device__ __forceinline__ void parseval_add(const cx<T>* __restrict__ uh, const T* __restrict__ wt, int64_t i,
                                             bool twice, int mode, double& a1, double& a2) {
  const cx<T> u = uh[i];
  const double x = (double)u.x, y = (double)u.y;
  double& a = twice ? a2 : a1;
  if (mode != 0) a += x;
  else if (wt) a = fma(fma(x, x, y * y), (double)wt[i], a);
  else a = fma(y, y, fma(x, x, a));
}

template <typename T>
__global__ void k_parseval_partial(const cx<T>* __restrict__ uh, int64_t n0, int64_t total, int rfft_form, int mode,
                                   const T* __restrict__ wt, double* partial) {
  const int64_t S = (int64_t)gridDim.x * blockDim.x, s0 = S % n0;
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  int64_t i0 = i % n0;
  double a1 = 0.0, a2 = 0.0;
  for (; i < total; i += S) {
    parseval_add(uh, wt, i, rfft_form && i0 > 0 && i0 < n0 - 1, mode, a1, a2);
    i0 += s0;
    if (i0 >= n0) i0 -= n0;
  }
  const double acc = block_sum(a1 + 2.0 * a2);
  if (threadIdx.x == 0) partial[blockIdx.x] = acc;
}

__global__ void k_sum_partials(const double* __restrict__ partial, int n, double norm, double* out) {
  double acc = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) acc += partial[i];
  acc = block_sum(acc);
  if (threadIdx.x == 0) *out = acc * norm;
}

// per-device reduction scratch, allocated on first use and kept until exit
static double* reduction_scratch() {
  static std::mutex mu;
  static std::vector<double*> bufs;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return nullptr;
  std::lock_guard<std::mutex> lk(mu);
  if ((int)bufs.size() <= dev) bufs.resize(dev + 1, nullptr);
  if (!bufs[dev]) {
    void* p = nullptr;
    if (cudaMalloc(&p, (FF_RED_MAXBLOCKS + 8) * sizeof(double)) != cudaSuccess) return nullptr;
    bufs[dev] = (double*)p;
  }
  return bufs[dev];
}

template <typename T>
static int parseval(const void* uh, int64_t n0, int64_t nrest, int rfft_form, int mode, double norm, double* out,
                    cudaStream_t s, const void* wt = nullptr, double* dev_out = nullptr) {
  const int64_t total = n0 * nrest;
  double* scratch = reduction_scratch();
  if (!scratch) {
    set_error("parsevalsum: reduction scratch allocation failed");
    return FF_ERR_ALLOC;
  }
  int blocks = elementwise_grid(total, FF_RED_THREADS);
  if (blocks > FF_RED_MAXBLOCKS) blocks = FF_RED_MAXBLOCKS;
  k_parseval_partial<T><<<blocks, FF_RED_THREADS, 0, s>>>((const cx<T>*)uh, n0, total, rfft_form, mode,
                                                           (const T*)wt, scratch);
  FF_LAUNCHED("k_parseval_partial");
  double* res = dev_out ? dev_out : scratch + FF_RED_MAXBLOCKS;
  k_sum_partials<<<1, FF_RED_THREADS, 0, s>>>(scratch, blocks, norm, res);
  FF_LAUNCHED("k_sum_partials");
  if (dev_out) return FF_OK;
  FF_CUDA(cudaMemcpyAsync(out, res, sizeof(double), cudaMemcpyDeviceToHost, s));
  FF_CUDA(cudaStreamSynchronize(s));
  return FF_OK;
}

}  // namespace ff

using namespace ff;

#define FF_PREC_DISPATCH(prec, CALL_F64, CALL_F32)                      \
  do {                                                                  \
    FF_CHECK_ARG((prec) == FF_F64 || (prec) == FF_F32, "bad precision %d", (prec)); \
    if ((prec) == FF_F64) { CALL_F64; } else { CALL_F32; }              \
  } while (0)

#define LAUNCH1D(kernel, n, ...)                                            \
  do {                                                                      \
    if ((n) <= 0) return FF_OK;                                             \
    kernel<<<elementwise_grid((n), 256), 256, 0, (cudaStream_t)stream>>>(__VA_ARGS__); \
    FF_LAUNCHED(#kernel);                                                   \
  } while (0)

extern "C" {

int ff_euler_update(int prec, int64_t n, void* sol, const void* N, ff_coef L, double dt, const void* filter,
                    void* stream) {
  FF_CHECK_ARG(sol && N, "ff_euler_update: null array");
  if (int st = check_coef(L, "ff_euler_update")) return st;
  FF_PREC_DISPATCH(prec,
      LAUNCH1D(k_euler<double>, n, n, (double2*)sol, (const double2*)N, coef<double>(L), dt, (const double*)filter),
      LAUNCH1D(k_euler<float>, n, n, (float2*)sol, (const float2*)N, coef<float>(L), (float)dt, (const float*)filter));
  return FF_OK;
}

int ff_rk4_substep(int prec, int64_t n, void* RHS, ff_coef L, const void* x, const void* sol, void* newsol, double c,
                   void* stream) {
  FF_CHECK_ARG(RHS && x && (!newsol || sol), "ff_rk4_substep: null array");
  if (int st = check_coef(L, "ff_rk4_substep")) return st;
  FF_PREC_DISPATCH(prec,
      LAUNCH1D(k_rk4_substep<double>, n, n, (double2*)RHS, coef<double>(L), (const double2*)x, (const double2*)sol,
               (double2*)newsol, c),
      LAUNCH1D(k_rk4_substep<float>, n, n, (float2*)RHS, coef<float>(L), (const float2*)x, (const float2*)sol,
               (float2*)newsol, (float)c));
  return FF_OK;
}

int ff_rk4_update(int prec, int64_t n, void* sol, void* RHS4, ff_coef L, const void* x, const void* RHS1,
                  const void* RHS2, const void* RHS3, double c6, const void* filter, void* stream) {
  FF_CHECK_ARG(sol && RHS4 && x && RHS1 && RHS2 && RHS3, "ff_rk4_update: null array");
  if (int st = check_coef(L, "ff_rk4_update")) return st;
  FF_PREC_DISPATCH(prec,
      LAUNCH1D(k_rk4_update<double>, n, n, (double2*)sol, (double2*)RHS4, coef<double>(L), (const double2*)x,
               (const double2*)RHS1, (const double2*)RHS2, (const double2*)RHS3, c6, (const double*)filter),
      LAUNCH1D(k_rk4_update<float>, n, n, (float2*)sol, (float2*)RHS4, coef<float>(L), (const float2*)x,
               (const float2*)RHS1, (const float2*)RHS2, (const float2*)RHS3, (float)c6, (const float*)filter));
  return FF_OK;
}

int ff_lsrk54_stage(int prec, int64_t n, void* sol, void* RHS, void* S2, ff_coef L, double A, double B, double dt,
                    int first, const void* filter, void* stream) {
  FF_CHECK_ARG(sol && RHS && S2, "ff_lsrk54_stage: null array");
  if (int st = check_coef(L, "ff_lsrk54_stage")) return st;
  FF_PREC_DISPATCH(prec,
      LAUNCH1D(k_lsrk54<double>, n, n, (double2*)sol, (double2*)RHS, (double2*)S2, coef<double>(L), A, B, dt, first,
               (const double*)filter),
      LAUNCH1D(k_lsrk54<float>, n, n, (float2*)sol, (float2*)RHS, (float2*)S2, coef<float>(L), (float)A, (float)B,
               (float)dt, first, (const float*)filter));
  return FF_OK;
}

int ff_etdrk4_substep12(int prec, int64_t n, void* out, ff_coef e_half, const void* sol, ff_coef zeta,
                        const void* N, void* stream) {
  FF_CHECK_ARG(out && sol && N, "ff_etdrk4_substep12: null array");
  if (int st = check_coef(e_half, "ff_etdrk4_substep12")) return st;
  if (int st = check_coef(zeta, "ff_etdrk4_substep12")) return st;
  FF_PREC_DISPATCH(prec,
      LAUNCH1D(k_etd12<double>, n, n, (double2*)out, coef<double>(e_half), (const double2*)sol, coef<double>(zeta),
               (const double2*)N),
      LAUNCH1D(k_etd12<float>, n, n, (float2*)out, coef<float>(e_half), (const float2*)sol, coef<float>(zeta),
               (const float2*)N));
  return FF_OK;
}

int ff_etdrk4_substep3(int prec, int64_t n, void* out, ff_coef e_half, const void* sol1, ff_coef zeta,
                       const void* N1, const void* N3, void* stream) {
  FF_CHECK_ARG(out && sol1 && N1 && N3, "ff_etdrk4_substep3: null array");
  if (int st = check_coef(e_half, "ff_etdrk4_substep3")) return st;
  if (int st = check_coef(zeta, "ff_etdrk4_substep3")) return st;
  FF_PREC_DISPATCH(prec,
      LAUNCH1D(k_etd3<double>, n, n, (double2*)out, coef<double>(e_half), (const double2*)sol1, coef<double>(zeta),
               (const double2*)N1, (const double2*)N3),
      LAUNCH1D(k_etd3<float>, n, n, (float2*)out, coef<float>(e_half), (const float2*)sol1, coef<float>(zeta),
               (const float2*)N1, (const float2*)N3));
  return FF_OK;
}

int ff_etdrk4_update(int prec, int64_t n, void* sol, ff_coef expL, ff_coef alpha, ff_coef beta, ff_coef Gamma,
                     const void* N1, const void* N2, const void* N3, const void* N4, const void* filter,
                     void* stream) {
  FF_CHECK_ARG(sol && N1 && N2 && N3 && N4, "ff_etdrk4_update: null array");
  for (const ff_coef* c : {&expL, &alpha, &beta, &Gamma})
    if (int st = check_coef(*c, "ff_etdrk4_update")) return st;
  FF_PREC_DISPATCH(prec,
      LAUNCH1D(k_etd_update<double>, n, n, (double2*)sol, coef<double>(expL), coef<double>(alpha), coef<double>(beta),
               coef<double>(Gamma), (const double2*)N1, (const double2*)N2, (const double2*)N3, (const double2*)N4,
               (const double*)filter),
      LAUNCH1D(k_etd_update<float>, n, n, (float2*)sol, coef<float>(expL), coef<float>(alpha), coef<float>(beta),
               coef<float>(Gamma), (const float2*)N1, (const float2*)N2, (const float2*)N3, (const float2*)N4,
               (const float*)filter));
  return FF_OK;
}

int ff_ab3_update(int prec, int64_t n, void* sol, void* RHS, void* RHSm1, void* RHSm2, ff_coef L, double dt,
                  int euler, const void* filter, void* stream) {
  FF_CHECK_ARG(sol && RHS && RHSm1 && RHSm2, "ff_ab3_update: null array");
  if (int st = check_coef(L, "ff_ab3_update")) return st;
  const double h1 = 23.0 / 12.0, h2 = 16.0 / 12.0, h3 = 5.0 / 12.0;
  FF_PREC_DISPATCH(prec,
      LAUNCH1D(k_ab3<double>, n, n, (double2*)sol, (double2*)RHS, (double2*)RHSm1, (double2*)RHSm2, coef<double>(L), dt,
               euler, h1, h2, h3, (const double*)filter),
      LAUNCH1D(k_ab3<float>, n, n, (float2*)sol, (float2*)RHS, (float2*)RHSm1, (float2*)RHSm2, coef<float>(L),
               (float)dt, euler, (float)h1, (float)h2, (float)h3, (const float*)filter));
  return FF_OK;
}

int ff_linear_step(int prec, int stepper, int64_t n, void* sol, ff_coef c, double dt, const void* filter,
                   int64_t nsteps, void* stream) {
  FF_CHECK_ARG(sol, "ff_linear_step: null state");
  FF_CHECK_ARG(stepper == FF_STEP_ETDRK4 || stepper == FF_STEP_RK4, "ff_linear_step: ETDRK4 or RK4 only (got %d)",
               stepper);
  FF_CHECK_ARG(nsteps >= 0 && nsteps <= (1 << 20), "ff_linear_step: nsteps out of range");
  FF_CHECK_ARG(c.kind != FF_COEF_NONE, "ff_linear_step: missing coefficient");
  if (int st = check_coef(c, "ff_linear_step")) return st;
  if (n <= 0 || nsteps == 0) return FF_OK;
  auto s = (cudaStream_t)stream;
  const int ns = (int)nsteps;
  if (stepper == FF_STEP_ETDRK4) {
    const bool vec = prec == FF_F32 && c.kind == FF_COEF_REAL && ((uintptr_t)sol % 16) == 0 &&
                     ((uintptr_t)c.ptr % 8) == 0 && ((uintptr_t)filter % 8) == 0;
    if (vec) {
      const int64_t np = n / 2;
      if (np > 0) {
        k_linear_etd_f32x2<<<elementwise_grid(np, 256), 256, 0, s>>>(np, (float4*)sol, (const float2*)c.ptr,
                                                                       (const float2*)filter, ns);
        FF_LAUNCHED("k_linear_etd_f32x2");
      }
      if (n % 2) {  // the last mode of an odd count
        ff_coef t = c;
        t.ptr = (const float*)c.ptr + (n - 1);
        k_linear_etd<float><<<1, 32, 0, s>>>(1, (float2*)sol + (n - 1), coef<float>(t),
                                             filter ? (const float*)filter + (n - 1) : nullptr, ns);
        FF_LAUNCHED("k_linear_etd");
      }
      return FF_OK;
    }
    FF_PREC_DISPATCH(prec,
        LAUNCH1D(k_linear_etd<double>, n, n, (double2*)sol, coef<double>(c), (const double*)filter, ns),
        LAUNCH1D(k_linear_etd<float>, n, n, (float2*)sol, coef<float>(c), (const float*)filter, ns));
    return FF_OK;
  }
  // RK4: the stage constants rounded to the state precision as the generic path's are
  FF_PREC_DISPATCH(prec,
      LAUNCH1D(k_linear_rk4<double>, n, n, (double2*)sol, coef<double>(c), dt / 2.0, dt, dt / 6.0,
               (const double*)filter, ns),
      LAUNCH1D(k_linear_rk4<float>, n, n, (float2*)sol, coef<float>(c), (float)dt / 2.0f, (float)dt,
               (float)dt / 6.0f, (const float*)filter, ns));
  return FF_OK;
}

int ff_filter_mul(int prec, int64_t n, void* sol, const void* filter, void* stream) {
  FF_CHECK_ARG(sol && filter, "ff_filter_mul: null array");
  FF_PREC_DISPATCH(prec, LAUNCH1D(k_filter<double>, n, n, (double2*)sol, (const double*)filter),
                   LAUNCH1D(k_filter<float>, n, n, (float2*)sol, (const float*)filter));
  return FF_OK;
}

int ff_dealias(int prec, void* fh, const int64_t dims[4], const int64_t lo[3], const int64_t hi[3], void* stream) {
  FF_CHECK_ARG(fh && dims && lo && hi, "ff_dealias: null argument");
  for (int d = 0; d < 4; ++d) FF_CHECK_ARG(dims[d] >= 1, "ff_dealias: dims[%d] must be >= 1", d);
  const int64_t total = dims[0] * dims[1] * dims[2] * dims[3];
  FF_PREC_DISPATCH(prec,
      LAUNCH1D(k_dealias<double>, total, (double2*)fh, dims[0], dims[1], dims[2], total, lo[0], hi[0], lo[1], hi[1],
               lo[2], hi[2]),
      LAUNCH1D(k_dealias<float>, total, (float2*)fh, dims[0], dims[1], dims[2], total, lo[0], hi[0], lo[1], hi[1],
               lo[2], hi[2]));
  return FF_OK;
}

int ff_mul_ik(int prec, int64_t n0, int64_t nrest, void* out, const void* in, const void* k, void* stream) {
  FF_CHECK_ARG(out && in && k && n0 >= 1 && nrest >= 1, "ff_mul_ik: bad argument");
  const int64_t total = n0 * nrest;
  FF_PREC_DISPATCH(prec, LAUNCH1D(k_mul_ik<double>, total, n0, total, (double2*)out, (const double2*)in, (const double*)k),
                   LAUNCH1D(k_mul_ik<float>, total, n0, total, (float2*)out, (const float2*)in, (const float*)k));
  return FF_OK;
}

int ff_real_mul(int prec, int64_t n, int64_t na, void* x, const void* a, void* stream) {
  FF_CHECK_ARG(x && a && na >= 1 && n % na == 0, "ff_real_mul: bad argument");
  FF_PREC_DISPATCH(prec, LAUNCH1D(k_real_mul<double>, n, n, na, (double*)x, (const double*)a),
                   LAUNCH1D(k_real_mul<float>, n, n, na, (float*)x, (const float*)a));
  return FF_OK;
}

int ff_parsevalsum2(int prec, const void* uh, int64_t n0, int64_t nrest, int rfft_form, double norm, double* out,
                    void* stream) {
  FF_CHECK_ARG(uh && out && n0 >= 1 && nrest >= 1, "ff_parsevalsum2: bad argument");
  FF_PREC_DISPATCH(prec, return parseval<double>(uh, n0, nrest, rfft_form, 0, norm, out, (cudaStream_t)stream),
                   return parseval<float>(uh, n0, nrest, rfft_form, 0, norm, out, (cudaStream_t)stream));
  return FF_OK;
}

int ff_parsevalsum2_weighted(int prec, const void* uh, const void* wt, int64_t n0, int64_t nrest, int rfft_form,
                             double norm, double* out, double* dev_out, void* stream) {
  FF_CHECK_ARG(uh && (out || dev_out) && n0 >= 1 && nrest >= 1, "ff_parsevalsum2_weighted: bad argument");
  FF_PREC_DISPATCH(prec,
      return parseval<double>(uh, n0, nrest, rfft_form, 0, norm, out, (cudaStream_t)stream, wt, dev_out),
      return parseval<float>(uh, n0, nrest, rfft_form, 0, norm, out, (cudaStream_t)stream, wt, dev_out));
  return FF_OK;
}

int ff_etdrk4_coefficients(int prec, int64_t n, const void* L, double dt, int ncirc, double rcirc, void* zeta,
                           void* alpha, void* beta, void* gamma, void* stream) {
  FF_CHECK_ARG(L && zeta && alpha && beta && gamma && n >= 1, "ff_etdrk4_coefficients: bad argument");
  FF_CHECK_ARG(ncirc >= 1 && ncirc <= 64, "ff_etdrk4_coefficients: ncirc must be in 1..64");
  Circle circ;
  circ.m = ncirc;
  const long double pi = 3.141592653589793238462643383279502884L;
  for (int j = 0; j < ncirc; ++j) {
    const long double a = 2.0L * pi * ((long double)j + 0.5L) / (long double)ncirc;
    circ.c[j] = make_double2((double)(rcirc * cosl(a)), (double)(rcirc * sinl(a)));
  }
  FF_PREC_DISPATCH(prec,
      LAUNCH1D(k_etd_coefs<double>, n, n, (const double*)L, dt, circ, (double*)zeta, (double*)alpha, (double*)beta,
               (double*)gamma),
      LAUNCH1D(k_etd_coefs<float>, n, n, (const float*)L, (float)dt, circ, (float*)zeta, (float*)alpha, (float*)beta,
               (float*)gamma));
  return FF_OK;
}

int ff_vort_velocities(int prec, int64_t nkr, int64_t ny, const void* zh, const void* kr, const void* l,
                       const void* invK, void* uh, void* vh, void* stream) {
  FF_CHECK_ARG(zh && kr && l && invK && uh && vh && nkr >= 1 && ny >= 1, "ff_vort_velocities: bad argument");
  const int64_t n = nkr * ny;
  FF_PREC_DISPATCH(prec,
      LAUNCH1D(k_velocities<double>, n, nkr, n, (const double2*)zh, (const double*)kr, (const double*)l,
               (const double*)invK, (double2*)uh, (double2*)vh),
      LAUNCH1D(k_velocities<float>, n, nkr, n, (const float2*)zh, (const float*)kr, (const float*)l,
               (const float*)invK, (float2*)uh, (float2*)vh));
  return FF_OK;
}

int ff_parsevalsum(int prec, const void* uh, int64_t n0, int64_t nrest, int rfft_form, double norm, double* out,
                   void* stream) {
  FF_CHECK_ARG(uh && out && n0 >= 1 && nrest >= 1, "ff_parsevalsum: bad argument");
  FF_PREC_DISPATCH(prec, return parseval<double>(uh, n0, nrest, rfft_form, 1, norm, out, (cudaStream_t)stream),
                   return parseval<float>(uh, n0, nrest, rfft_form, 1, norm, out, (cudaStream_t)stream));
  return FF_OK;
}

}  // extern "C"
