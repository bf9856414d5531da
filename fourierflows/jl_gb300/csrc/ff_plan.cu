// Generic FFT plans behind ff_rfft / ff_irfft / ff_fft / ff_ifft.
//
// A d-dimensional transform is a sequence of line passes, x first (the reference's
// rfft/irfft order): a contiguous "row" pass over dimension 0 and one strided "column"
// pass per further dimension.  Each pass reads its input once from HBM and writes its
// output once; the transform itself runs in shared memory (ff_fft.cuh).
//
//   rfft  : rows R2C (in -> out), cols y (out, in place), cols z (out, in place)
//   irfft : cols z (in -> work), cols y (work, in place), rows C2R (work -> out, scaled)
//           -- the input is never written (FFTW's c2r may destroy it; callers in the
//              reference guard with deepcopy, src/diffusion.jl:154-155)
//   fft   : rows C2C (in -> out), cols y, cols z (in place)
//   ifft  : the same with the inverse direction, the last pass scaled by 1/N.
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <mutex>
#include <set>
#include <utility>

#include "ff_plan.cuh"

namespace ff {

// ---------------------------------------------------------------------------------------
// host-side set-up
// ---------------------------------------------------------------------------------------
bool factorize(int n, LinePlan& P) {
  P.n = n;
  P.nst = 0;
  int m = n;
  while (m % 8 == 0 && m > 1) { P.radix[P.nst++] = 8; m /= 8; }
  while (m % 4 == 0) { P.radix[P.nst++] = 4; m /= 4; }
  while (m % 2 == 0) { P.radix[P.nst++] = 2; m /= 2; }
  for (int p = 3; m > 1; p += 2) {
    while (m % p == 0) {
      if (p > FF_MAX_GENERIC_RADIX || P.nst >= FF_MAX_STAGES) return false;
      P.radix[P.nst++] = p;
      m /= p;
    }
  }
  return true;
}

static const long double kPiL = 3.141592653589793238462643383279502884L;

// exp(-2 pi i e / n) with the quarter turns exact
static void twiddle(long double e, long double n, double& re, double& im) {
  long double a = -2.0L * kPiL * e / n;
  re = (double)cosl(a);
  im = (double)sinl(a);
  long double q = 4.0L * e / n;
  if (q == 0.0L) { re = 1.0; im = 0.0; }
  else if (q == 1.0L) { re = 0.0; im = -1.0; }
  else if (q == 2.0L) { re = -1.0; im = 0.0; }
  else if (q == 3.0L) { re = 0.0; im = 1.0; }
}

void host_twiddles(int n, std::vector<double>& t) {
  t.resize(2 * (size_t)n);
  for (int e = 0; e < n; ++e) twiddle(e, n, t[2 * e], t[2 * e + 1]);
  // For the register-resident FFT of a power-of-two length 16..4096, the twiddles of each
  // radix-8 stage of span NS > 1 follow, stage by stage and r-major: entry
  // n + (NS - R0) + (r - 1) NS + k = W_n^(k r n / (8 NS)), r = 1..7, k < NS, where R0 is the
  // first stage's radix (the spans are R0, 8 R0, ..., n/8; see ff_regfft.cuh).  A warp's
  // threads then read consecutive entries of one stage and r.
  if (n >= 16 && n <= 4096 && (n & (n - 1)) == 0) {
    int L = 0;
    while ((1 << L) < n) ++L;
    const int R0 = (L % 3) ? (1 << (L % 3)) : 8;
    for (int NS = R0; NS * 8 <= n; NS *= 8) {
      const int tws = n / (NS * 8);
      for (int r = 1; r < 8; ++r)
        for (int k = 0; k < NS; ++k) {
          double re, im;
          twiddle((long double)k * r * tws, n, re, im);
          t.push_back(re);
          t.push_back(im);
        }
    }
  }
}

void host_real_twiddles(int N, std::vector<double>& t) {
  const int h = N / 2;
  t.resize(2 * (size_t)(h + 1));
  for (int k = 0; k <= h; ++k) twiddle(k, N, t[2 * k], t[2 * k + 1]);
}

int upload_table(const std::vector<double>& t, int prec, void** dev) {
  const size_t count = t.size() / 2;
  *dev = nullptr;
  if (count == 0) return FF_OK;
  if (prec == FF_F64) {
    FF_CUDA(cudaMalloc(dev, count * sizeof(double2)));
    FF_CUDA(cudaMemcpy(*dev, t.data(), count * sizeof(double2), cudaMemcpyHostToDevice));
  } else {
    std::vector<float> f(t.size());
    for (size_t i = 0; i < t.size(); ++i) f[i] = (float)t[i];
    FF_CUDA(cudaMalloc(dev, count * sizeof(float2)));
    FF_CUDA(cudaMemcpy(*dev, f.data(), count * sizeof(float2), cudaMemcpyHostToDevice));
  }
  return FF_OK;
}

int ensure_smem(const void* func, size_t bytes) {
  if (bytes <= 32 * 1024) return FF_OK;  // inside the default 48 KB with any static use here
  FF_CHECK_ARG(bytes <= 227 * 1024, "shared memory request of %zu bytes exceeds 227 KB", bytes);
  static std::mutex mu;
  static std::set<std::pair<const void*, int>> done;
  int dev = 0;
  FF_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(mu);
  auto key = std::make_pair(func, dev);
  if (done.count(key)) return FF_OK;
  // both limits, the default 48 KB and the opt-in 227 KB, cover static and dynamic
  // shared memory together
  cudaFuncAttributes fa;
  FF_CUDA(cudaFuncGetAttributes(&fa, func));
  if (bytes + fa.sharedSizeBytes <= 48 * 1024) return FF_OK;
  const size_t cap = 227 * 1024 - fa.sharedSizeBytes;
  FF_CHECK_ARG(bytes <= cap, "shared memory request of %zu bytes exceeds the kernel's %zu", bytes, cap);
  FF_CUDA(cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)cap));
  done.insert(key);
  return FF_OK;
}

static int round_threads(int64_t t) {
  int64_t r = ((t + 31) / 32) * 32;
  if (r < 64) r = 64;
  if (r > 512) r = 512;
  return (int)r;
}

ColGeom col_geom(int n, int prec, int tl_hint) {
  const size_t elem = prec == FF_F64 ? 16 : 8;
  ColGeom g;
  g.tl = tl_hint > 0 ? tl_hint : (prec == FF_F64 ? 2 : 4);
  while (g.tl > 1 && 2 * (size_t)g.tl * n * elem > 160 * 1024) g.tl /= 2;
  g.nth = round_threads((int64_t)g.tl * n / 8);
  g.smem = 2 * (size_t)g.tl * n * elem;
  return g;
}

RowGeom row_geom(int h, int prec) {
  const int elem = prec == FF_F64 ? 16 : 8;
  RowGeom g;
  int hh = h > 0 ? h : 1;
  g.tlr = 512 / hh;
  if (g.tlr < 1) g.tlr = 1;
  if (g.tlr > 32) g.tlr = 32;
  while (g.tlr > 1 && 2 * (size_t)g.tlr * rows_stride(hh, elem) * elem > 160 * 1024) g.tlr /= 2;
  g.nth = round_threads((int64_t)g.tlr * hh / 8);
  g.smem = 2 * (size_t)g.tlr * rows_stride(hh, elem) * elem;
  return g;
}

// ---------------------------------------------------------------------------------------
// kernels
// ---------------------------------------------------------------------------------------
// R2C along contiguous rows of nx reals -> nx/2+1 complex
template <typename T>
__global__ void k_r2c_rows(const T* __restrict__ in, cx<T>* __restrict__ out, int64_t nrows, int nx, LinePlan P,
                           const cx<T>* __restrict__ tw, const cx<T>* __restrict__ rtw, int tlr) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int h = nx / 2, nkr = h + 1;
  const AddrRows ad{rows_stride(h, sizeof(cx<T>)), rows_pad_shift(sizeof(cx<T>))};
  cx<T>* A = reinterpret_cast<cx<T>*>(smem_raw);
  cx<T>* B = A + tlr * ad.stride;
  const int64_t row0 = (int64_t)blockIdx.x * tlr;
  for (int idx = threadIdx.x; idx < tlr * h; idx += blockDim.x) {
    const int ln = idx / h, m = idx - ln * h;
    const int64_t row = row0 + ln;
    cx<T> v = czero<T>();
    if (row < nrows) v = reinterpret_cast<const cx<T>*>(in + row * nx)[m];
    A[ad(ln, m)] = v;
  }
  __syncthreads();
  const cx<T>* Z = fft_lines<T, -1>(A, B, tw, P, tlr, ad);
  const int half = h / 2 + 1;
  for (int idx = threadIdx.x; idx < tlr * half; idx += blockDim.x) {
    const int ln = idx / half, k = idx - ln * half;
    const int64_t row = row0 + ln;
    if (row >= nrows) continue;
    cx<T>* o = out + row * nkr;
    if (k == 0) {
      const cx<T> z = Z[ad(ln, 0)];
      o[0] = mk<T>(z.x + z.y, T(0));
      o[h] = mk<T>(z.x - z.y, T(0));
    } else {
      cx<T> xk, xhk;
      r2c_pair<T>(Z[ad(ln, k)], Z[ad(ln, h - k)], __ldg(&rtw[k]), xk, xhk);
      o[k] = xk;
      if (h - k != k) o[h - k] = xhk;
    }
  }
}

// C2R along rows: nx/2+1 complex -> nx reals, scaled
template <typename T>
__global__ void k_c2r_rows(const cx<T>* __restrict__ in, T* __restrict__ out, int64_t nrows, int nx, LinePlan P,
                           const cx<T>* __restrict__ tw, const cx<T>* __restrict__ rtw, int tlr, T scale) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int h = nx / 2, nkr = h + 1;
  const AddrRows ad{rows_stride(h, sizeof(cx<T>)), rows_pad_shift(sizeof(cx<T>))};
  cx<T>* A = reinterpret_cast<cx<T>*>(smem_raw);
  cx<T>* B = A + tlr * ad.stride;
  const int64_t row0 = (int64_t)blockIdx.x * tlr;
  for (int idx = threadIdx.x; idx < tlr * h; idx += blockDim.x) {
    const int ln = idx / h, k = idx - ln * h;
    const int64_t row = row0 + ln;
    cx<T> v = czero<T>();
    if (row < nrows) {
      const cx<T>* r = in + row * nkr;
      v = c2r_pre<T>(r[k], r[h - k], __ldg(&rtw[k]), k);
    }
    A[ad(ln, k)] = v;
  }
  __syncthreads();
  const cx<T>* Z = fft_lines<T, 1>(A, B, tw, P, tlr, ad);
  for (int idx = threadIdx.x; idx < tlr * h; idx += blockDim.x) {
    const int ln = idx / h, m = idx - ln * h;
    const int64_t row = row0 + ln;
    if (row >= nrows) continue;
    const cx<T> z = Z[ad(ln, m)];
    reinterpret_cast<cx<T>*>(out + row * nx)[m] = mk<T>(z.x * scale, z.y * scale);
  }
}

// C2C along contiguous rows (in may alias out)
template <typename T, int DIR>
__global__ void k_c2c_rows(const cx<T>* in, cx<T>* out, int64_t nrows, int n, LinePlan P,
                           const cx<T>* __restrict__ tw, int tlr, T scale) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const AddrRows ad{rows_stride(n, sizeof(cx<T>)), rows_pad_shift(sizeof(cx<T>))};
  cx<T>* A = reinterpret_cast<cx<T>*>(smem_raw);
  cx<T>* B = A + tlr * ad.stride;
  const int64_t row0 = (int64_t)blockIdx.x * tlr;
  for (int idx = threadIdx.x; idx < tlr * n; idx += blockDim.x) {
    const int ln = idx / n, m = idx - ln * n;
    const int64_t row = row0 + ln;
    A[ad(ln, m)] = row < nrows ? in[row * n + m] : czero<T>();
  }
  __syncthreads();
  const cx<T>* Z = fft_lines<T, DIR>(A, B, tw, P, tlr, ad);
  for (int idx = threadIdx.x; idx < tlr * n; idx += blockDim.x) {
    const int ln = idx / n, m = idx - ln * n;
    const int64_t row = row0 + ln;
    if (row < nrows) out[row * n + m] = scl(Z[ad(ln, m)], scale);
  }
}

// C2C along a strided axis: tiles of tl adjacent columns (in may alias out)
template <typename T, int DIR>
__global__ void k_cols(const cx<T>* in, cx<T>* out, int64_t ncols, int n, int64_t stride, int64_t nouter,
                       int64_t outer_stride, LinePlan P, const cx<T>* __restrict__ tw, int tl, T scale) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const AddrTile ad{tl};
  cx<T>* A = reinterpret_cast<cx<T>*>(smem_raw);
  cx<T>* B = A + tl * n;
  const int64_t c0 = (int64_t)blockIdx.x * tl;
  for (int64_t o = blockIdx.y; o < nouter; o += gridDim.y) {
    const int64_t base = o * outer_stride;
    for (int idx = threadIdx.x; idx < tl * n; idx += blockDim.x) {
      const int ln = idx % tl, j = idx / tl;
      const int64_t c = c0 + ln;
      A[ad(ln, j)] = c < ncols ? in[base + c + j * stride] : czero<T>();
    }
    __syncthreads();
    const cx<T>* Z = fft_lines<T, DIR>(A, B, tw, P, tl, ad);
    for (int idx = threadIdx.x; idx < tl * n; idx += blockDim.x) {
      const int ln = idx % tl, j = idx / tl;
      const int64_t c = c0 + ln;
      if (c < ncols) out[base + c + j * stride] = scl(Z[ad(ln, j)], scale);
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------------------
template <typename T> static int prec_of() { return sizeof(T) == 8 ? FF_F64 : FF_F32; }

bool plan_generic_forced() {
  const char* e = getenv("FF_PLAN_GENERIC");
  return e && e[0] == '1';
}

template <typename T>
int launch_r2c_rows(const T* in, cx<T>* out, int64_t nrows, int nx, const LinePlan& P, const cx<T>* tw,
                    const cx<T>* rtw, cudaStream_t s) {
  if (nrows <= 0) return FF_OK;
  // FP64 real rows are FP64-pipe bound on either path and measured faster on the shared-
  // memory kernels (4096^2: 671 us against 737 us); FP32 rows take the register path
  if (sizeof(T) == 4 && reg_rows_ok(nx / 2) && !plan_generic_forced())
    return launch_r2c_rows_reg<T>(in, out, nrows, nx, tw, rtw, s);
  const RowGeom g = row_geom(nx / 2, prec_of<T>());
  int st = ensure_smem((const void*)k_r2c_rows<T>, g.smem);
  if (st) return st;
  k_r2c_rows<T><<<(unsigned)ceil_div(nrows, g.tlr), g.nth, g.smem, s>>>(in, out, nrows, nx, P, tw, rtw, g.tlr);
  FF_LAUNCHED("k_r2c_rows");
  return FF_OK;
}

template <typename T>
int launch_c2r_rows(const cx<T>* in, T* out, int64_t nrows, int nx, const LinePlan& P, const cx<T>* tw,
                    const cx<T>* rtw, T scale, cudaStream_t s) {
  if (nrows <= 0) return FF_OK;
  if (sizeof(T) == 4 && reg_rows_ok(nx / 2) && !plan_generic_forced())
    return launch_c2r_rows_reg<T>(in, out, nrows, nx, tw, rtw, scale, s);
  const RowGeom g = row_geom(nx / 2, prec_of<T>());
  int st = ensure_smem((const void*)k_c2r_rows<T>, g.smem);
  if (st) return st;
  k_c2r_rows<T><<<(unsigned)ceil_div(nrows, g.tlr), g.nth, g.smem, s>>>(in, out, nrows, nx, P, tw, rtw, g.tlr,
                                                                         scale);
  FF_LAUNCHED("k_c2r_rows");
  return FF_OK;
}

template <typename T, int DIR>
int launch_c2c_rows(const cx<T>* in, cx<T>* out, int64_t nrows, int n, const LinePlan& P, const cx<T>* tw,
                    T scale, cudaStream_t s) {
  if (nrows <= 0) return FF_OK;
  if (reg_line_ok(n) && !plan_generic_forced()) return launch_c2c_rows_reg<T, DIR>(in, out, nrows, n, tw, scale, s);
  const RowGeom g = row_geom(n, prec_of<T>());
  // row_geom sizes for a line of length n here (not n/2)
  int st = ensure_smem((const void*)k_c2c_rows<T, DIR>, g.smem);
  if (st) return st;
  k_c2c_rows<T, DIR><<<(unsigned)ceil_div(nrows, g.tlr), g.nth, g.smem, s>>>(in, out, nrows, n, P, tw, g.tlr,
                                                                              scale);
  FF_LAUNCHED("k_c2c_rows");
  return FF_OK;
}

template <typename T, int DIR>
int launch_cols(const cx<T>* in, cx<T>* out, int64_t ncols, int n, int64_t stride, int64_t nouter,
                int64_t outer_stride, const LinePlan& P, const cx<T>* tw, T scale, cudaStream_t s) {
  if (ncols <= 0 || nouter <= 0) return FF_OK;
  if (reg_line_ok(n) && !plan_generic_forced())
    return launch_cols_reg<T, DIR>(in, out, ncols, n, stride, nouter, outer_stride, tw, scale, s);
  const ColGeom g = col_geom(n, prec_of<T>());
  int st = ensure_smem((const void*)k_cols<T, DIR>, g.smem);
  if (st) return st;
  dim3 grid((unsigned)ceil_div(ncols, g.tl), (unsigned)(nouter < 65535 ? nouter : 65535));
  k_cols<T, DIR><<<grid, g.nth, g.smem, s>>>(in, out, ncols, n, stride, nouter, outer_stride, P, tw, g.tl, scale);
  FF_LAUNCHED("k_cols");
  return FF_OK;
}

template int launch_r2c_rows<float>(const float*, float2*, int64_t, int, const LinePlan&, const float2*,
                                    const float2*, cudaStream_t);
template int launch_r2c_rows<double>(const double*, double2*, int64_t, int, const LinePlan&, const double2*,
                                     const double2*, cudaStream_t);
template int launch_c2r_rows<float>(const float2*, float*, int64_t, int, const LinePlan&, const float2*,
                                    const float2*, float, cudaStream_t);
template int launch_c2r_rows<double>(const double2*, double*, int64_t, int, const LinePlan&, const double2*,
                                     const double2*, double, cudaStream_t);
template int launch_cols<float, -1>(const float2*, float2*, int64_t, int, int64_t, int64_t, int64_t,
                                    const LinePlan&, const float2*, float, cudaStream_t);
template int launch_cols<float, 1>(const float2*, float2*, int64_t, int, int64_t, int64_t, int64_t,
                                   const LinePlan&, const float2*, float, cudaStream_t);
template int launch_cols<double, -1>(const double2*, double2*, int64_t, int, int64_t, int64_t, int64_t,
                                     const LinePlan&, const double2*, double, cudaStream_t);
template int launch_cols<double, 1>(const double2*, double2*, int64_t, int, int64_t, int64_t, int64_t,
                                    const LinePlan&, const double2*, double, cudaStream_t);

}  // namespace ff

// =========================================================================================
// ff_plan
// =========================================================================================
struct ff_plan {
  int ndim = 0, prec = FF_F64, real = 1, device = 0;
  int64_t n[3] = {1, 1, 1};
  int64_t batch = 1;
  ff::LinePlan lp[3];
  void* tw[3] = {nullptr, nullptr, nullptr};
  void* rtw = nullptr;
  void* work = nullptr;
};

static int plan_free(ff_plan* p) {
  if (!p) return FF_OK;
  for (int d = 0; d < 3; ++d)
    if (p->tw[d]) cudaFree(p->tw[d]);
  if (p->rtw) cudaFree(p->rtw);
  if (p->work) cudaFree(p->work);
  delete p;
  return FF_OK;
}

static int plan_create(int real, int ndim, const int64_t* n, int prec, int64_t batch, ff_plan** out) {
  FF_CHECK_ARG(out != nullptr, "ff_plan_create: null output pointer");
  *out = nullptr;
  FF_CHECK_ARG(ndim >= 1 && ndim <= 3, "ff_plan_create: ndim must be 1, 2 or 3 (got %d)", ndim);
  FF_CHECK_ARG(prec == FF_F64 || prec == FF_F32, "ff_plan_create: prec must be FF_F64 or FF_F32");
  FF_CHECK_ARG(batch >= 1, "ff_plan_create: batch must be >= 1");
  const int64_t maxn = prec == FF_F64 ? 4096 : 8192;
  for (int d = 0; d < ndim; ++d) {
    FF_CHECK_ARG(n[d] >= 1, "ff_plan_create: n[%d] = %lld must be positive", d, (long long)n[d]);
    const int64_t lim = (real && d == 0) ? 2 * maxn : maxn;
    if (n[d] > lim) {
      ff::set_error("ff_plan_create: n[%d] = %lld exceeds the single-pass limit %lld", d, (long long)n[d],
                    (long long)lim);
      return FF_ERR_UNSUPPORTED;
    }
  }
  if (real) FF_CHECK_ARG(n[0] % 2 == 0, "ff_plan_create: n[0] = %lld must be even", (long long)n[0]);
  ff_plan* p = new ff_plan();
  p->ndim = ndim;
  p->prec = prec;
  p->real = real;
  p->batch = batch;
  for (int d = 0; d < ndim; ++d) p->n[d] = n[d];
  cudaGetDevice(&p->device);
  int st = FF_OK;
  for (int d = 0; d < ndim && st == FF_OK; ++d) {
    const int len = (int)((real && d == 0) ? n[0] / 2 : n[d]);
    if (!ff::factorize(len, p->lp[d])) {
      ff::set_error("ff_plan_create: n[%d] = %lld has a prime factor above %d", d, (long long)n[d],
                    FF_MAX_GENERIC_RADIX);
      st = FF_ERR_UNSUPPORTED;
      break;
    }
    std::vector<double> t;
    ff::host_twiddles(len, t);
    st = ff::upload_table(t, prec, &p->tw[d]);
  }
  if (st == FF_OK && real) {
    std::vector<double> t;
    ff::host_real_twiddles((int)n[0], t);
    st = ff::upload_table(t, prec, &p->rtw);
  }
  if (st == FF_OK && real && ndim > 1) {
    const size_t elem = prec == FF_F64 ? 16 : 8;
    size_t count = (size_t)(n[0] / 2 + 1) * batch;
    for (int d = 1; d < ndim; ++d) count *= (size_t)n[d];
    cudaError_t e = cudaMalloc(&p->work, count * elem);
    if (e != cudaSuccess) st = ff::cuda_status(e, "ff_plan_create: workspace");
  }
  if (st != FF_OK) {
    plan_free(p);
    return st;
  }
  *out = p;
  return FF_OK;
}

template <typename T> using cxT = ff::cx<T>;

static int check_ptr(const void* p, size_t align, const char* what) {
  FF_CHECK_ARG(p != nullptr, "%s: null pointer", what);
  FF_CHECK_ARG(((uintptr_t)p % align) == 0, "%s: pointer %p is not %zu-byte aligned", what, p, align);
  return FF_OK;
}

template <typename T>
static int exec_rfft(const ff_plan* p, const T* in, cxT<T>* out, cudaStream_t s) {
  const int64_t nx = p->n[0], ny = p->n[1], nz = p->n[2], nkr = nx / 2 + 1, B = p->batch;
  const auto* tw0 = (const cxT<T>*)p->tw[0];
  int st = ff::launch_r2c_rows<T>(in, out, ny * nz * B, (int)nx, p->lp[0], tw0, (const cxT<T>*)p->rtw, s);
  if (st || p->ndim == 1) return st;
  st = ff::launch_cols<T, -1>(out, out, nkr, (int)ny, nkr, nz * B, nkr * ny, p->lp[1], (const cxT<T>*)p->tw[1],
                              T(1), s);
  if (st || p->ndim == 2) return st;
  return ff::launch_cols<T, -1>(out, out, nkr * ny, (int)nz, nkr * ny, B, nkr * ny * nz, p->lp[2],
                                (const cxT<T>*)p->tw[2], T(1), s);
}

template <typename T>
static int exec_irfft(const ff_plan* p, const cxT<T>* in, T* out, cudaStream_t s) {
  const int64_t nx = p->n[0], ny = p->n[1], nz = p->n[2], nkr = nx / 2 + 1, B = p->batch;
  const T scale = (T)(1.0 / ((double)nx * (double)ny * (double)nz));
  const cxT<T>* src = in;
  auto* work = (cxT<T>*)p->work;
  int st = FF_OK;
  if (p->ndim == 3) {
    st = ff::launch_cols<T, 1>(src, work, nkr * ny, (int)nz, nkr * ny, B, nkr * ny * nz, p->lp[2],
                               (const cxT<T>*)p->tw[2], T(1), s);
    if (st) return st;
    src = work;
  }
  if (p->ndim >= 2) {
    st = ff::launch_cols<T, 1>(src, work, nkr, (int)ny, nkr, nz * B, nkr * ny, p->lp[1], (const cxT<T>*)p->tw[1],
                               T(1), s);
    if (st) return st;
    src = work;
  }
  return ff::launch_c2r_rows<T>(src, out, ny * nz * B, (int)nx, p->lp[0], (const cxT<T>*)p->tw[0],
                                (const cxT<T>*)p->rtw, scale, s);
}

template <typename T, int DIR>
static int exec_fft(const ff_plan* p, const cxT<T>* in, cxT<T>* out, cudaStream_t s) {
  const int64_t nx = p->n[0], ny = p->n[1], nz = p->n[2], B = p->batch;
  const T one = T(1);
  const T scale = DIR > 0 ? (T)(1.0 / ((double)nx * (double)ny * (double)nz)) : one;
  int st = ff::launch_c2c_rows<T, DIR>(in, out, ny * nz * B, (int)nx, p->lp[0], (const cxT<T>*)p->tw[0],
                                       p->ndim == 1 ? scale : one, s);
  if (st || p->ndim == 1) return st;
  st = ff::launch_cols<T, DIR>(out, out, nx, (int)ny, nx, nz * B, nx * ny, p->lp[1], (const cxT<T>*)p->tw[1],
                               p->ndim == 2 ? scale : one, s);
  if (st || p->ndim == 2) return st;
  return ff::launch_cols<T, DIR>(out, out, nx * ny, (int)nz, nx * ny, B, nx * ny * nz, p->lp[2],
                                 (const cxT<T>*)p->tw[2], scale, s);
}

static int check_plan(const ff_plan* p, int real, const char* what) {
  FF_CHECK_ARG(p != nullptr, "%s: null plan", what);
  FF_CHECK_ARG(p->real == real, "%s: plan kind mismatch (real plan %d)", what, p->real);
  int dev = 0;
  FF_CUDA(cudaGetDevice(&dev));
  FF_CHECK_ARG(dev == p->device, "%s: plan was created on device %d, current device is %d", what, p->device,
               dev);
  return FF_OK;
}

extern "C" {

int ff_plan_create(int ndim, const int64_t n[3], int prec, int64_t batch, ff_plan** plan) {
  return plan_create(1, ndim, n, prec, batch, plan);
}

int ff_cplan_create(int ndim, const int64_t n[3], int prec, int64_t batch, ff_plan** plan) {
  return plan_create(0, ndim, n, prec, batch, plan);
}

int ff_plan_destroy(ff_plan* plan) { return plan_free(plan); }

int ff_rfft(const ff_plan* p, const void* in, void* out, void* stream) {
  int st = check_plan(p, 1, "ff_rfft");
  if (st) return st;
  const size_t es = p->prec == FF_F64 ? 8 : 4;
  if ((st = check_ptr(in, 2 * es, "ff_rfft input")) || (st = check_ptr(out, 2 * es, "ff_rfft output"))) return st;
  FF_CHECK_ARG(in != out, "ff_rfft: in-place real transforms are not supported");
  auto s = (cudaStream_t)stream;
  return p->prec == FF_F64 ? exec_rfft<double>(p, (const double*)in, (double2*)out, s)
                           : exec_rfft<float>(p, (const float*)in, (float2*)out, s);
}

int ff_irfft(const ff_plan* p, const void* in, void* out, void* stream) {
  int st = check_plan(p, 1, "ff_irfft");
  if (st) return st;
  const size_t es = p->prec == FF_F64 ? 8 : 4;
  if ((st = check_ptr(in, 2 * es, "ff_irfft input")) || (st = check_ptr(out, 2 * es, "ff_irfft output")))
    return st;
  FF_CHECK_ARG(in != out, "ff_irfft: in-place real transforms are not supported");
  auto s = (cudaStream_t)stream;
  return p->prec == FF_F64 ? exec_irfft<double>(p, (const double2*)in, (double*)out, s)
                           : exec_irfft<float>(p, (const float2*)in, (float*)out, s);
}

int ff_fft(const ff_plan* p, const void* in, void* out, void* stream) {
  int st = check_plan(p, 0, "ff_fft");
  if (st) return st;
  const size_t es = p->prec == FF_F64 ? 8 : 4;
  if ((st = check_ptr(in, 2 * es, "ff_fft input")) || (st = check_ptr(out, 2 * es, "ff_fft output"))) return st;
  auto s = (cudaStream_t)stream;
  return p->prec == FF_F64 ? exec_fft<double, -1>(p, (const double2*)in, (double2*)out, s)
                           : exec_fft<float, -1>(p, (const float2*)in, (float2*)out, s);
}

int ff_ifft(const ff_plan* p, const void* in, void* out, void* stream) {
  int st = check_plan(p, 0, "ff_ifft");
  if (st) return st;
  const size_t es = p->prec == FF_F64 ? 8 : 4;
  if ((st = check_ptr(in, 2 * es, "ff_ifft input")) || (st = check_ptr(out, 2 * es, "ff_ifft output"))) return st;
  auto s = (cudaStream_t)stream;
  return p->prec == FF_F64 ? exec_fft<double, 1>(p, (const double2*)in, (double2*)out, s)
                           : exec_fft<float, 1>(p, (const float2*)in, (float2*)out, s);
}

}  // extern "C"
