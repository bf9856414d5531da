// Discrete adjoint of the 2D vorticity nonlinear term, and the FP64 reduction of the
// viscosity gradient of an ETDRK4 step.
//
// The state is the stored half spectrum s (nkr x ny complex) read as a real vector of its
// real and imaginary parts, <a, b> = sum Re(conj(a) b).  The forward term is
//     N(s) = P (Dx F(u z) + Dy F(v z)),  z = irfft(P s), u = irfft(Au P s), v = irfft(Av P s)
// with the 2/3 mask P, Dx = -i kr, Dy = -i l, Au = i l/K^2, Av = -i kr/K^2, F = rfft.
// With the normalised irfft, F^T(g) = nx ny irfft(g / w) and irfft^T(y) = w F(y) / (nx ny),
// where w = 1 on the kr = 0 and kr = nx/2 columns and 2 elsewhere (the half-spectrum
// weights of parsevalsum2).  Hence the transpose of the linearisation at s applied to lam:
//     gx = irfft(i kr P lam / w),  gy = irfft(i l P lam / w)
//     J^T lam = P [ w ( -i l/K^2 F(z gx) + i kr/K^2 F(z gy) + F(u gx + v gy) ) ]
// computed as one prep kernel, a batched inverse transform of 5 fields, one product
// kernel, a batched forward transform of 3 fields and one combine kernel.
#include <mutex>
#include <vector>

#include "ff_common.cuh"

namespace ff {

#define GRID_STRIDE_ADJ(i, n) \
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < (n); i += (int64_t)gridDim.x * blockDim.x)

struct AdjGrid {
  int64_t nkr, ny, nkd, la, lb;
};

__device__ __forceinline__ bool kept(const AdjGrid& g, int64_t c, int64_t j) {
  return c < g.nkd && (j < g.la || j >= g.lb);
}

__device__ __forceinline__ double half_weight(const AdjGrid& g, int64_t c) {
  return (c == 0 || c == g.nkr - 1) ? 1.0 : 2.0;
}

// X5 = [Au P s, Av P s, P s, i kr P lam / w, i l P lam / w]
template <typename T>
__global__ void k_adj_prep(AdjGrid g, const cx<T>* __restrict__ s, const cx<T>* __restrict__ lam,
                           const T* __restrict__ kr, const T* __restrict__ l, const T* __restrict__ invK,
                           cx<T>* __restrict__ X5) {
  const int64_t n = g.nkr * g.ny;
  GRID_STRIDE_ADJ(e, n) {
    const int64_t c = e % g.nkr, j = e / g.nkr;
    cx<T> z = czero<T>(), m = czero<T>();
    if (kept(g, c, j)) {
      z = s[e];
      m = lam[e];
    }
    const T ik = invK[e];
    const T rw = (T)(1.0 / half_weight(g, c));
    X5[e] = mul_i(scl(z, l[j] * ik));
    X5[n + e] = mul_mi(scl(z, kr[c] * ik));
    X5[2 * n + e] = z;
    X5[3 * n + e] = mul_i(scl(m, kr[c] * rw));
    X5[4 * n + e] = mul_i(scl(m, l[j] * rw));
  }
}

// physical: [u, v, z, gx, gy] -> [z gx, z gy, u gx + v gy] (first three slots, in place)
template <typename T> __global__ void k_adj_prod(int64_t np, T* Y) {
  GRID_STRIDE_ADJ(i, np) {
    const T u = Y[i], v = Y[np + i], z = Y[2 * np + i], gx = Y[3 * np + i], gy = Y[4 * np + i];
    Y[i] = z * gx;
    Y[np + i] = z * gy;
    Y[2 * np + i] = u * gx + v * gy;
  }
}

// out = P [ w ( -i l/K^2 X0 + i kr/K^2 X1 + X2 ) ]
template <typename T>
__global__ void k_adj_combine(AdjGrid g, const cx<T>* __restrict__ X3, const T* __restrict__ kr,
                              const T* __restrict__ l, const T* __restrict__ invK, cx<T>* __restrict__ out) {
  const int64_t n = g.nkr * g.ny;
  GRID_STRIDE_ADJ(e, n) {
    const int64_t c = e % g.nkr, j = e / g.nkr;
    cx<T> r = czero<T>();
    if (kept(g, c, j)) {
      const T ik = invK[e];
      r = add(add(mul_mi(scl(X3[e], l[j] * ik)), mul_i(scl(X3[n + e], kr[c] * ik))), X3[2 * n + e]);
      r = scl(r, (T)half_weight(g, c));
    }
    out[e] = r;
  }
}

// viscosity-gradient terms of one adjoint ETDRK4 step (see ff_vort_adj_nu_terms)
template <typename T> struct NuArgs {
  const cx<T>* lam;  // adjoint of the new state
  const cx<T>* la;   // adjoint of sol1 (a)
  const cx<T>* lb;   // adjoint of the first sol2 (b)
  const cx<T>* lc;   // adjoint of the second sol2 (c)
  const cx<T>* s;
  const cx<T>* a;
  const cx<T>* n1;
  const cx<T>* n2;
  const cx<T>* n3;
  const cx<T>* n4;
  const T* dE;   // d expLdt / d nu
  const T* dE2;  // d exp_half_Ldt / d nu
  const T* dZ;   // d zeta / d nu
  const T* dA;   // d alpha / d nu
  const T* dB;   // d beta / d nu
  const T* dG;   // d Gamma / d nu
};

// Re(conj(a) b) in FP64
__device__ __forceinline__ double redot(float2 a, float2 b) {
  return (double)a.x * (double)b.x + (double)a.y * (double)b.y;
}
__device__ __forceinline__ double redot(double2 a, double2 b) { return a.x * b.x + a.y * b.y; }

#define FF_ADJ_THREADS 256
#define FF_ADJ_MAXBLOCKS 1024

__device__ __forceinline__ double adj_block_sum(double v) {
  __shared__ double sh[FF_ADJ_THREADS / 32];
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

template <typename T> __global__ void k_adj_nu_partial(int64_t n, NuArgs<T> A, double* partial) {
  double acc = 0.0;
  GRID_STRIDE_ADJ(e, n) {
    const double dE = A.dE[e], dE2 = A.dE2[e], dZ = A.dZ[e], dA = A.dA[e], dB = A.dB[e], dG = A.dG[e];
    const cx<T> s = A.s[e], n1 = A.n1[e], n2 = A.n2[e], n3 = A.n3[e];
    // s' = E s + alpha N1 + 2 beta (N2 + N3) + Gamma N4
    acc += redot(A.lam[e], s) * dE + redot(A.lam[e], n1) * dA + 2.0 * dB * (redot(A.lam[e], n2) + redot(A.lam[e], n3)) +
           redot(A.lam[e], A.n4[e]) * dG;
    // c = E2 a + Z (2 N3 - N1)
    acc += redot(A.lc[e], A.a[e]) * dE2 + dZ * (2.0 * redot(A.lc[e], n3) - redot(A.lc[e], n1));
    // b = E2 s + Z N2,  a = E2 s + Z N1
    acc += redot(A.lb[e], s) * dE2 + redot(A.lb[e], n2) * dZ;
    acc += redot(A.la[e], s) * dE2 + redot(A.la[e], n1) * dZ;
  }
  acc = adj_block_sum(acc);
  if (threadIdx.x == 0) partial[blockIdx.x] = acc;
}

__global__ void k_adj_accumulate(const double* __restrict__ partial, int n, double scale, double* acc_out) {
  double acc = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) acc += partial[i];
  acc = adj_block_sum(acc);
  if (threadIdx.x == 0) *acc_out += acc * scale;
}

}  // namespace ff

struct ff_vadj {
  int prec = FF_F64, dev = 0;
  ff::AdjGrid g{};
  int64_t nx = 0;
  const void* kr = nullptr;
  const void* l = nullptr;
  const void* invK = nullptr;
  ff_plan* inv5 = nullptr;  // irfft of 5 stacked fields
  ff_plan* fwd3 = nullptr;  // rfft of 3 stacked fields
  void* X5 = nullptr;
  void* Y5 = nullptr;
  void* X3 = nullptr;
  double* partial = nullptr;
};

static void vadj_free(ff_vadj* h) {
  if (!h) return;
  if (h->inv5) ff_plan_destroy(h->inv5);
  if (h->fwd3) ff_plan_destroy(h->fwd3);
  for (void* p : {h->X5, h->Y5, h->X3, (void*)h->partial})
    if (p) cudaFree(p);
  delete h;
}

template <typename T> static int vadj_apply_t(ff_vadj* h, const void* s, const void* lam, void* out, cudaStream_t st) {
  using namespace ff;
  const int64_t n = h->g.nkr * h->g.ny, np = h->nx * h->g.ny;
  const int th = 256;
  k_adj_prep<T><<<elementwise_grid(n, th), th, 0, st>>>(h->g, (const cx<T>*)s, (const cx<T>*)lam, (const T*)h->kr,
                                                        (const T*)h->l, (const T*)h->invK, (cx<T>*)h->X5);
  FF_LAUNCHED("k_adj_prep");
  if (int e = ff_irfft(h->inv5, h->X5, h->Y5, st)) return e;
  k_adj_prod<T><<<elementwise_grid(np, th), th, 0, st>>>(np, (T*)h->Y5);
  FF_LAUNCHED("k_adj_prod");
  if (int e = ff_rfft(h->fwd3, h->Y5, h->X3, st)) return e;
  k_adj_combine<T><<<elementwise_grid(n, th), th, 0, st>>>(h->g, (const cx<T>*)h->X3, (const T*)h->kr,
                                                           (const T*)h->l, (const T*)h->invK, (cx<T>*)out);
  FF_LAUNCHED("k_adj_combine");
  return FF_OK;
}

template <typename T>
static int vadj_nu_t(ff_vadj* h, const ff_adj_nu* a, double scale, double* acc, cudaStream_t st) {
  using namespace ff;
  NuArgs<T> A;
  A.lam = (const cx<T>*)a->lam;
  A.la = (const cx<T>*)a->lam_a;
  A.lb = (const cx<T>*)a->lam_b;
  A.lc = (const cx<T>*)a->lam_c;
  A.s = (const cx<T>*)a->s;
  A.a = (const cx<T>*)a->a;
  A.n1 = (const cx<T>*)a->n1;
  A.n2 = (const cx<T>*)a->n2;
  A.n3 = (const cx<T>*)a->n3;
  A.n4 = (const cx<T>*)a->n4;
  A.dE = (const T*)a->dE;
  A.dE2 = (const T*)a->dE2;
  A.dZ = (const T*)a->dZ;
  A.dA = (const T*)a->dA;
  A.dB = (const T*)a->dB;
  A.dG = (const T*)a->dG;
  const int64_t n = h->g.nkr * h->g.ny;
  int blocks = elementwise_grid(n, FF_ADJ_THREADS);
  if (blocks > FF_ADJ_MAXBLOCKS) blocks = FF_ADJ_MAXBLOCKS;
  k_adj_nu_partial<T><<<blocks, FF_ADJ_THREADS, 0, st>>>(n, A, h->partial);
  FF_LAUNCHED("k_adj_nu_partial");
  k_adj_accumulate<<<1, FF_ADJ_THREADS, 0, st>>>(h->partial, blocks, scale, acc);
  FF_LAUNCHED("k_adj_accumulate");
  return FF_OK;
}

extern "C" {

int ff_vadj_create(int prec, int64_t nx, int64_t ny, int64_t nkd, int64_t la, int64_t lb, const void* kr,
                   const void* l, const void* invKrsq, ff_vadj** out) {
  FF_CHECK_ARG(out, "ff_vadj_create: null output");
  *out = nullptr;
  FF_CHECK_ARG(prec == FF_F64 || prec == FF_F32, "ff_vadj_create: bad precision %d", prec);
  FF_CHECK_ARG(nx >= 2 && ny >= 2 && nx % 2 == 0, "ff_vadj_create: bad grid %lld x %lld", (long long)nx,
               (long long)ny);
  FF_CHECK_ARG(nkd >= 1 && nkd <= nx / 2 + 1 && la >= 0 && la <= lb && lb <= ny, "ff_vadj_create: bad alias ranges");
  FF_CHECK_ARG(kr && l && invKrsq, "ff_vadj_create: null wavenumber array");
  ff_vadj* h = new ff_vadj();
  h->prec = prec;
  h->nx = nx;
  h->g = ff::AdjGrid{nx / 2 + 1, ny, nkd, la, lb};
  h->kr = kr;
  h->l = l;
  h->invK = invKrsq;
  cudaGetDevice(&h->dev);
  const int64_t dims[3] = {nx, ny, 1};
  int st = ff_plan_create(2, dims, prec, 5, &h->inv5);
  if (!st) st = ff_plan_create(2, dims, prec, 3, &h->fwd3);
  const size_t es = prec == FF_F64 ? 16 : 8;
  const size_t nc = (size_t)h->g.nkr * ny, np = (size_t)nx * ny;
  cudaError_t e = cudaSuccess;
  if (!st) e = cudaMalloc(&h->X5, 5 * nc * es);
  if (!st && e == cudaSuccess) e = cudaMalloc(&h->Y5, 5 * np * es / 2);
  if (!st && e == cudaSuccess) e = cudaMalloc(&h->X3, 3 * nc * es);
  if (!st && e == cudaSuccess) e = cudaMalloc(&h->partial, FF_ADJ_MAXBLOCKS * sizeof(double));
  if (!st && e != cudaSuccess) st = ff::cuda_status(e, "ff_vadj_create: workspace");
  if (st) {
    vadj_free(h);
    return st;
  }
  *out = h;
  return FF_OK;
}

int ff_vadj_destroy(ff_vadj* h) {
  vadj_free(h);
  return FF_OK;
}

int ff_vadj_apply(ff_vadj* h, const void* s, const void* lam, void* out, void* stream) {
  FF_CHECK_ARG(h && s && lam && out, "ff_vadj_apply: null argument");
  auto st = (cudaStream_t)stream;
  return h->prec == FF_F64 ? vadj_apply_t<double>(h, s, lam, out, st) : vadj_apply_t<float>(h, s, lam, out, st);
}

int ff_vort_adj_nu_terms(ff_vadj* h, const ff_adj_nu* args, double scale, double* dev_acc, void* stream) {
  FF_CHECK_ARG(h && args && dev_acc, "ff_vort_adj_nu_terms: null argument");
  const void* ptrs[] = {args->lam, args->lam_a, args->lam_b, args->lam_c, args->s, args->a, args->n1, args->n2,
                        args->n3, args->n4, args->dE, args->dE2, args->dZ, args->dA, args->dB, args->dG};
  for (const void* p : ptrs) FF_CHECK_ARG(p, "ff_vort_adj_nu_terms: null array");
  auto st = (cudaStream_t)stream;
  return h->prec == FF_F64 ? vadj_nu_t<double>(h, args, scale, dev_acc, st) : vadj_nu_t<float>(h, args, scale, dev_acc, st);
}

}  // extern "C"
