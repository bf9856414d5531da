// A stand-in for FourierFlows.jl's own GPU path (CUDA.jl broadcasts + CUFFT plans), used
// only as a comparator arm of bench.py: the 2D vorticity ETDRK4 step in FP64, unfused,
// one kernel per Julia broadcast and one cuFFT call per transform, launched from the host
// one after another on one stream, as CUDA.jl enqueues them.
//
// Reference op sequence restated here (paths relative to the FourierFlows.jl tree):
//   ETDRK4 substeps and update   src/timesteppers.jl:501-547 (one broadcast each)
//   rfft plan: plan_rfft on a CuArray -> a cuFFT D2Z plan; ldiv! with it -> the C2R
//     (Z2D) plan followed by the 1/(nx ny) scaling of AbstractFFTs' ScaledPlan
//                                 src/domains.jl:5,208
//   dealias!: two broadcasts, fh[kralias, :] = 0 and fh[:, lalias] = 0
//                                 src/domains.jl:457-458
//   calcN! of the vorticity term on the Jacobian convention of jacobianh
//     (src/utils.jl:190-205): zh = dealias(sol); uh = i l zh / K^2; vh = -i kr zh / K^2;
//     u, v, zeta = irfft(...); u zeta, v zeta; N = -(i kr rfft(u zeta) + i l rfft(v zeta));
//     dealias!(N)  -- the same function the library's fused path and the oracle compute.
//
// cuFFT's C2R overwrites its input; every C2R input here is a temporary that is not read
// again, so no protective copy is made (CUDA.jl may copy there: this stand-in is, if
// anything, faster than the path it stands for).
#include <cuda_runtime.h>
#include <cufft.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

namespace {

thread_local char g_err[512] = "";

int fail(const char* what, int code) {
  snprintf(g_err, sizeof(g_err), "%s (code %d)", what, code);
  return code == 0 ? -1 : code;
}

#define U_CUDA(x)                                                    \
  do {                                                               \
    cudaError_t e__ = (x);                                           \
    if (e__ != cudaSuccess) return fail(#x, (int)e__);               \
  } while (0)
#define U_FFT(x)                                                     \
  do {                                                               \
    cufftResult r__ = (x);                                           \
    if (r__ != CUFFT_SUCCESS) return fail(#x, 1000 + (int)r__);      \
  } while (0)

constexpr int kThreads = 256;

int blocks(int64_t n) { return (int)((n + kThreads - 1) / kThreads); }

// ---- one kernel per broadcast --------------------------------------------------------
__global__ void k_copy(double2* __restrict__ y, const double2* __restrict__ x, int64_t n) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) y[i] = x[i];
}

// fh[kralias, :] = 0: rows [k0, nkr) of every column (kr fastest)
__global__ void k_zero_kr(double2* __restrict__ f, int nkr, int ny, int k0) {
  const int w = nkr - k0;
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < (int64_t)w * ny) {
    const int64_t j = i / w, k = k0 + i % w;
    f[k + j * nkr] = make_double2(0.0, 0.0);
  }
}

// fh[:, lalias] = 0: columns [la, lb)
__global__ void k_zero_l(double2* __restrict__ f, int nkr, int la, int lb) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < (int64_t)nkr * (lb - la)) f[(int64_t)la * nkr + i] = make_double2(0.0, 0.0);
}

// uh = i l invKrsq zh   (u = -d psi / dy, psi_hat = -zh invKrsq)
__global__ void k_uh(double2* __restrict__ uh, const double2* __restrict__ zh, const double* __restrict__ l,
                     const double* __restrict__ invK, int nkr, int64_t n) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) {
    const double s = l[i / nkr] * invK[i];
    const double2 z = zh[i];
    uh[i] = make_double2(-s * z.y, s * z.x);
  }
}

// vh = -i kr invKrsq zh   (v = d psi / dx)
__global__ void k_vh(double2* __restrict__ vh, const double2* __restrict__ zh, const double* __restrict__ kr,
                     const double* __restrict__ invK, int nkr, int64_t n) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) {
    const double s = kr[i % nkr] * invK[i];
    const double2 z = zh[i];
    vh[i] = make_double2(s * z.y, -s * z.x);
  }
}

// rmul!(y, 1 / (nx ny)) of the scaled inverse plan
__global__ void k_scale(double* __restrict__ y, double s, int64_t n) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) y[i] *= s;
}

// a .*= b (physical)
__global__ void k_mul(double* __restrict__ a, const double* __restrict__ b, int64_t n) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) a[i] *= b[i];
}

// N = -i kr uzh - i l vzh
__global__ void k_flux(double2* __restrict__ N, const double2* __restrict__ a, const double2* __restrict__ b,
                       const double* __restrict__ kr, const double* __restrict__ l, int nkr, int64_t n) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) {
    const double k = kr[i % nkr], m = l[i / nkr];
    const double2 x = a[i], y = b[i];
    // -i k x - i m y = (k x.y + m y.y, -(k x.x + m y.x))
    N[i] = make_double2(k * x.y + m * y.y, -(k * x.x + m * y.x));
  }
}

// sol1 = exp(L dt / 2) sol + zeta N   (ETDRK4substep12!)
__global__ void k_substep12(double2* __restrict__ s1, const double* __restrict__ eh, const double2* __restrict__ s,
                            const double* __restrict__ zc, const double2* __restrict__ N, int64_t n) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) {
    const double a = eh[i], b = zc[i];
    const double2 x = s[i], y = N[i];
    s1[i] = make_double2(a * x.x + b * y.x, a * x.y + b * y.y);
  }
}

// sol2 = exp(L dt / 2) sol1 + zeta (2 N3 - N1)   (ETDRK4substep3!)
__global__ void k_substep3(double2* __restrict__ s2, const double* __restrict__ eh, const double2* __restrict__ s1,
                           const double* __restrict__ zc, const double2* __restrict__ N1,
                           const double2* __restrict__ N3, int64_t n) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) {
    const double a = eh[i], b = zc[i];
    const double2 x = s1[i], p = N1[i], q = N3[i];
    const double2 d = make_double2(2.0 * q.x - p.x, 2.0 * q.y - p.y);
    s2[i] = make_double2(a * x.x + b * d.x, a * x.y + b * d.y);
  }
}

// sol = exp(L dt) sol + alpha N1 + 2 beta (N2 + N3) + Gamma N4   (ETDRK4update!)
__global__ void k_update(double2* __restrict__ s, const double* __restrict__ eL, const double* __restrict__ al,
                         const double* __restrict__ be, const double* __restrict__ ga, const double2* __restrict__ N1,
                         const double2* __restrict__ N2, const double2* __restrict__ N3,
                         const double2* __restrict__ N4, int64_t n) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) {
    const double e = eL[i], a = al[i], b2 = 2.0 * be[i], g = ga[i];
    const double2 x = s[i], p = N1[i], q = N2[i], r = N3[i], t = N4[i];
    double re = e * x.x + a * p.x;
    double im = e * x.y + a * p.y;
    re = re + b2 * (q.x + r.x);
    im = im + b2 * (q.y + r.y);
    s[i] = make_double2(re + g * t.x, im + g * t.y);
  }
}

}  // namespace

struct ffu {
  int nx = 0, ny = 0, nkr = 0, k0 = 0, la = 0, lb = 0;
  int64_t nc = 0, nr = 0;
  const double *kr = nullptr, *l = nullptr, *invK = nullptr;
  const double *eL = nullptr, *eh = nullptr, *zc = nullptr, *al = nullptr, *be = nullptr, *ga = nullptr;
  double2 *s1 = nullptr, *s2 = nullptr, *N[4] = {nullptr, nullptr, nullptr, nullptr};
  double2 *zh = nullptr, *uh = nullptr, *vh = nullptr;
  double *u = nullptr, *v = nullptr, *z = nullptr;
  cufftHandle fwd = 0, inv = 0;
  bool have_fwd = false, have_inv = false;
  int launches = 0;  // kernels + cuFFT executions enqueued by the last ffu_step
};

namespace {

void destroy(ffu* h) {
  if (!h) return;
  if (h->have_fwd) cufftDestroy(h->fwd);
  if (h->have_inv) cufftDestroy(h->inv);
  void* bufs[] = {h->s1, h->s2, h->N[0], h->N[1], h->N[2], h->N[3], h->zh, h->uh, h->vh, h->u, h->v, h->z};
  for (void* p : bufs)
    if (p) cudaFree(p);
  delete h;
}

int dealias(ffu* h, double2* f, cudaStream_t s) {
  if (h->k0 < h->nkr) {
    k_zero_kr<<<blocks((int64_t)(h->nkr - h->k0) * h->ny), kThreads, 0, s>>>(f, h->nkr, h->ny, h->k0);
    ++h->launches;
  }
  if (h->lb > h->la) {
    k_zero_l<<<blocks((int64_t)h->nkr * (h->lb - h->la)), kThreads, 0, s>>>(f, h->nkr, h->la, h->lb);
    ++h->launches;
  }
  U_CUDA(cudaGetLastError());
  return 0;
}

int irfft(ffu* h, double2* in, double* out, cudaStream_t s) {
  U_FFT(cufftExecZ2D(h->inv, (cufftDoubleComplex*)in, out));
  k_scale<<<blocks(h->nr), kThreads, 0, s>>>(out, 1.0 / ((double)h->nx * h->ny), h->nr);
  h->launches += 2;
  U_CUDA(cudaGetLastError());
  return 0;
}

int calcN(ffu* h, double2* N, const double2* sol, cudaStream_t s) {
  const int64_t n = h->nc;
  k_copy<<<blocks(n), kThreads, 0, s>>>(h->zh, sol, n);
  ++h->launches;
  if (int st = dealias(h, h->zh, s)) return st;
  k_uh<<<blocks(n), kThreads, 0, s>>>(h->uh, h->zh, h->l, h->invK, h->nkr, n);
  k_vh<<<blocks(n), kThreads, 0, s>>>(h->vh, h->zh, h->kr, h->invK, h->nkr, n);
  h->launches += 2;
  if (int st = irfft(h, h->uh, h->u, s)) return st;
  if (int st = irfft(h, h->vh, h->v, s)) return st;
  if (int st = irfft(h, h->zh, h->z, s)) return st;
  k_mul<<<blocks(h->nr), kThreads, 0, s>>>(h->u, h->z, h->nr);
  k_mul<<<blocks(h->nr), kThreads, 0, s>>>(h->v, h->z, h->nr);
  h->launches += 2;
  U_FFT(cufftExecD2Z(h->fwd, h->u, (cufftDoubleComplex*)h->uh));
  U_FFT(cufftExecD2Z(h->fwd, h->v, (cufftDoubleComplex*)h->vh));
  h->launches += 2;
  k_flux<<<blocks(n), kThreads, 0, s>>>(N, h->uh, h->vh, h->kr, h->l, h->nkr, n);
  ++h->launches;
  U_CUDA(cudaGetLastError());
  return dealias(h, N, s);
}

}  // namespace

extern "C" {

const char* ffu_last_error(void) { return g_err; }

// nx, ny: grid; kr (nkr), l (ny), invKrsq (nkr*ny): device FP64 wavenumber arrays;
// k0: first aliased kr row (nkr if none), [la, lb): aliased l columns (la == lb if none);
// coef[6] = exp(L dt), exp(L dt / 2), zeta, alpha, beta, Gamma: device FP64 (nkr*ny).
// The arrays stay owned by the caller and must outlive the handle.
int ffu_create(int64_t nx, int64_t ny, const double* kr, const double* l, const double* invKrsq, int64_t k0,
               int64_t la, int64_t lb, const double* const coef[6], ffu** out) {
  if (!out || !kr || !l || !invKrsq || !coef) return fail("ffu_create: null argument", -1);
  if (nx < 2 || ny < 2 || nx % 2 || ny % 2) return fail("ffu_create: nx, ny must be even", -1);
  for (int i = 0; i < 6; ++i)
    if (!coef[i]) return fail("ffu_create: null coefficient array", -1);
  *out = nullptr;
  ffu* h = new ffu();
  h->nx = (int)nx;
  h->ny = (int)ny;
  h->nkr = (int)(nx / 2 + 1);
  h->k0 = (int)k0;
  h->la = (int)la;
  h->lb = (int)lb;
  h->nc = (int64_t)h->nkr * ny;
  h->nr = nx * ny;
  h->kr = kr;
  h->l = l;
  h->invK = invKrsq;
  h->eL = coef[0];
  h->eh = coef[1];
  h->zc = coef[2];
  h->al = coef[3];
  h->be = coef[4];
  h->ga = coef[5];
  const size_t cb = sizeof(double2) * h->nc, rb = sizeof(double) * h->nr;
  double2** cbufs[] = {&h->s1, &h->s2, &h->N[0], &h->N[1], &h->N[2], &h->N[3], &h->zh, &h->uh, &h->vh};
  double** rbufs[] = {&h->u, &h->v, &h->z};
  int st = 0;
  for (double2** p : cbufs)
    if (!st && cudaMalloc((void**)p, cb) != cudaSuccess) st = fail("ffu_create: cudaMalloc", -2);
  for (double** p : rbufs)
    if (!st && cudaMalloc((void**)p, rb) != cudaSuccess) st = fail("ffu_create: cudaMalloc", -2);
  // column-major (nkr, ny) with kr fastest is row-major [ny][nkr]: a 2D plan of (ny, nx)
  if (!st && cufftPlan2d(&h->fwd, (int)ny, (int)nx, CUFFT_D2Z) != CUFFT_SUCCESS) st = fail("cufftPlan2d D2Z", -3);
  else if (!st) h->have_fwd = true;
  if (!st && cufftPlan2d(&h->inv, (int)ny, (int)nx, CUFFT_Z2D) != CUFFT_SUCCESS) st = fail("cufftPlan2d Z2D", -3);
  else if (!st) h->have_inv = true;
  if (st) {
    destroy(h);
    return st;
  }
  *out = h;
  return 0;
}

int ffu_destroy(ffu* h) {
  destroy(h);
  return 0;
}

// nsteps ETDRK4 steps of the state `sol` (device, (nkr, ny) complex FP64) on `stream`
int ffu_step(ffu* h, void* sol_, int64_t nsteps, void* stream) {
  if (!h || !sol_) return fail("ffu_step: null argument", -1);
  auto s = (cudaStream_t)stream;
  U_FFT(cufftSetStream(h->fwd, s));
  U_FFT(cufftSetStream(h->inv, s));
  auto* sol = (double2*)sol_;
  const int64_t n = h->nc;
  for (int64_t k = 0; k < nsteps; ++k) {
    h->launches = 0;
    if (int st = calcN(h, h->N[0], sol, s)) return st;
    k_substep12<<<blocks(n), kThreads, 0, s>>>(h->s1, h->eh, sol, h->zc, h->N[0], n);
    if (int st = calcN(h, h->N[1], h->s1, s)) return st;
    k_substep12<<<blocks(n), kThreads, 0, s>>>(h->s2, h->eh, sol, h->zc, h->N[1], n);
    if (int st = calcN(h, h->N[2], h->s2, s)) return st;
    k_substep3<<<blocks(n), kThreads, 0, s>>>(h->s2, h->eh, h->s1, h->zc, h->N[0], h->N[2], n);
    if (int st = calcN(h, h->N[3], h->s2, s)) return st;
    k_update<<<blocks(n), kThreads, 0, s>>>(sol, h->eL, h->al, h->be, h->ga, h->N[0], h->N[1], h->N[2], h->N[3], n);
    h->launches += 4;
    U_CUDA(cudaGetLastError());
  }
  return 0;
}

// kernels and cuFFT executions one step enqueues
int ffu_launches_per_step(const ffu* h) { return h ? h->launches : -1; }

}  // extern "C"
