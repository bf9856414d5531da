// radialspectrum (src/utils.jl:239-283): a 2D spectrum bilinearly interpolated onto a
// polar (rho, theta) grid and integrated over theta, as one binned reduction.
//
// One CTA per radius rho_i (i >= 1): its threads walk the theta samples, interpolate
// the spectrum at (rho cos theta, rho sin theta) straight from the unshifted array (the
// fftshift is index arithmetic), and reduce in FP64.  The reference interpolates with
// Interpolations.jl's scaled linear B-spline on the shifted wavenumber ranges; inside the
// range that is bilinear interpolation between the four neighbouring grid values.
#include <math.h>

#include <algorithm>

#include "ff_common.cuh"

namespace {

using namespace ff;

template <typename E> struct Acc;  // an element read as FP64 (re, im)
template <> struct Acc<float> {
  static __device__ double2 get(const float* p, int64_t e) { return make_double2(p[e], 0.0); }
};
template <> struct Acc<double> {
  static __device__ double2 get(const double* p, int64_t e) { return make_double2(p[e], 0.0); }
};
template <> struct Acc<float2> {
  static __device__ double2 get(const float2* p, int64_t e) { return make_double2(p[e].x, p[e].y); }
};
template <> struct Acc<double2> {
  static __device__ double2 get(const double2* p, int64_t e) { return make_double2(p[e].x, p[e].y); }
};

template <typename E> __device__ void put(E* out, int64_t i, double2 v);
template <> __device__ void put<float>(float* out, int64_t i, double2 v) { out[i] = (float)v.x; }
template <> __device__ void put<double>(double* out, int64_t i, double2 v) { out[i] = v.x; }
template <> __device__ void put<float2>(float2* out, int64_t i, double2 v) { out[i] = make_float2((float)v.x, (float)v.y); }
template <> __device__ void put<double2>(double2* out, int64_t i, double2 v) { out[i] = v; }

struct Polar {
  int64_t n0, n1;      // array sizes (nkr or nk, nl)
  int rfft;            // 1: conjugate-symmetric form (no shift along dimension 0)
  double k0, dk, l0, dl;  // first wavenumber and spacing of the shifted ranges
  int64_t nrho, ntheta;
  double rhomax, theta0, dtheta, fac;
};

// lower grid index (0-based, clamped to [0, n-2]) and weight of coordinate x
__device__ __forceinline__ void lin_index(double x, double x0, double dx, int64_t n, int64_t& i, double& w) {
  const double u = (x - x0) / dx;
  double fi = floor(u);
  fi = fmin(fmax(fi, 0.0), (double)(n - 2));
  i = (int64_t)fi;
  w = u - fi;
}

// shifted index -> storage index: fftshift(x)[s] = x[(s - n/2) mod n]
__device__ __forceinline__ int64_t unshift(int64_t s, int64_t n) { return (s - n / 2 + n) % n; }

template <typename E>
__global__ void __launch_bounds__(256) k_radialspectrum(const E* __restrict__ fh, Polar P, E* __restrict__ out) {
  __shared__ double2 red[256 / 32];
  for (int64_t ir = 1 + blockIdx.x; ir < P.nrho; ir += gridDim.x) {
    const double rho = (double)ir * P.rhomax / (double)(P.nrho - 1);
    double2 acc = make_double2(0.0, 0.0);
    for (int64_t it = threadIdx.x; it < P.ntheta; it += blockDim.x) {
      const double th = P.theta0 + (double)it * P.dtheta;
      int64_t i, j;
      double wi, wj;
      lin_index(rho * cos(th), P.k0, P.dk, P.n0, i, wi);
      lin_index(rho * sin(th), P.l0, P.dl, P.n1, j, wj);
      const int64_t i0 = P.rfft ? i : unshift(i, P.n0), i1 = P.rfft ? i + 1 : unshift(i + 1, P.n0);
      const int64_t j0 = unshift(j, P.n1), j1 = unshift(j + 1, P.n1);
      const double2 a = Acc<E>::get(fh, i0 + j0 * P.n0), b = Acc<E>::get(fh, i1 + j0 * P.n0);
      const double2 c = Acc<E>::get(fh, i0 + j1 * P.n0), d = Acc<E>::get(fh, i1 + j1 * P.n0);
      const double w00 = (1 - wi) * (1 - wj), w10 = wi * (1 - wj), w01 = (1 - wi) * wj, w11 = wi * wj;
      acc.x += w00 * a.x + w10 * b.x + w01 * c.x + w11 * d.x;
      acc.y += w00 * a.y + w10 * b.y + w01 * c.y + w11 * d.y;
    }
    for (int o = 16; o > 0; o >>= 1) {
      acc.x += __shfl_down_sync(0xffffffffu, acc.x, o);
      acc.y += __shfl_down_sync(0xffffffffu, acc.y, o);
    }
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
      double2 s = make_double2(0.0, 0.0);
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
        s.x += red[w].x;
        s.y += red[w].y;
      }
      const double f = P.fac * rho * P.dtheta;
      put<E>(out, ir, make_double2(f * s.x, f * s.y));
    }
    __syncthreads();
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) put<E>(out, 0, Acc<E>::get(fh, 0));
}

template <typename E> int launch(const void* fh, const Polar& P, void* out, cudaStream_t s) {
  const int grid = (int)std::min<int64_t>(P.nrho - 1 > 0 ? P.nrho - 1 : 1, 8 * (int64_t)sm_count());
  k_radialspectrum<E><<<grid, 256, 0, s>>>((const E*)fh, P, (E*)out);
  FF_LAUNCHED("k_radialspectrum");
  return FF_OK;
}

}  // namespace

extern "C" int ff_radialspectrum(int prec, int is_complex, const void* fh, int64_t n0, int64_t nk, int64_t nl,
                                 double Lx, double Ly, int64_t nrho, int64_t ntheta, void* out, void* stream) {
  FF_CHECK_ARG(prec == FF_F64 || prec == FF_F32, "ff_radialspectrum: bad precision %d", prec);
  FF_CHECK_ARG(fh && out, "ff_radialspectrum: null pointer");
  FF_CHECK_ARG(nk >= 4 && nl >= 4 && nk % 2 == 0 && nl % 2 == 0, "ff_radialspectrum: grid %lld x %lld",
               (long long)nk, (long long)nl);
  FF_CHECK_ARG(n0 == nk / 2 + 1 || n0 == nk, "ff_radialspectrum: first dimension %lld is neither nkr nor nk",
               (long long)n0);
  FF_CHECK_ARG(nrho >= 2 && ntheta >= 2, "ff_radialspectrum: need at least 2 radii and 2 angles");
  Polar P;
  P.n0 = n0;
  P.n1 = nl;
  P.rfft = n0 == nk / 2 + 1;
  const double pi = 3.14159265358979323846;
  P.dk = 2 * pi / Lx;
  P.dl = 2 * pi / Ly;
  P.k0 = P.rfft ? 0.0 : -(double)(nk / 2) * P.dk;
  P.l0 = -(double)(nl / 2) * P.dl;
  P.nrho = nrho;
  P.ntheta = ntheta;
  P.rhomax = std::min((double)(nk / 2 - 1) * P.dk, (double)(nl / 2 - 1) * P.dl);
  P.theta0 = P.rfft ? -pi / 2 : 0.0;
  P.dtheta = (P.rfft ? pi : 2 * pi) / (double)(ntheta - 1);
  P.fac = P.rfft ? 2.0 : 1.0;
  auto s = (cudaStream_t)stream;
  if (prec == FF_F64) return is_complex ? launch<double2>(fh, P, out, s) : launch<double>(fh, P, out, s);
  return is_complex ? launch<float2>(fh, P, out, s) : launch<float>(fh, P, out, s);
}
