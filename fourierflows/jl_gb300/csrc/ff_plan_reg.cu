// Register-resident kernels of the rfft / fft plans for power-of-two line lengths: the
// transforms behind mul! / ldiv! with a grid's rfftplan or fftplan (src/domains.jl:2-5).
//
// Each thread holds eight elements of one line (regfft, ff_regfft.cuh): a CTA of nt
// threads transforms nt * 8 / N lines of length N.  Elements go straight from HBM to
// registers and back; shared memory carries only the exchanges between radix stages (and,
// for the real forward transform, the one that pairs Z[k] with Z[h - k] for the unpack).
// The shared-memory Stockham kernels of ff_plan.cu keep the other lengths.
#include "ff_plan.cuh"
#include "ff_regfft.cuh"

namespace ff {

namespace {

constexpr int kRegThreads = 256;  // threads per CTA of the row kernels, unless one line needs more
constexpr int kMaxThreads = 512;  // one line of 4096 complex values

template <typename T> constexpr int row_shift() { return sizeof(T) == 8 ? 3 : 4; }

// R2C of rows of nx = 2H reals: the half-length complex FFT of z[m] = x[2m] + i x[2m+1],
// then X[k] = E + W O from Z[k] and Z[H - k] (r2c_pair), X[0] and X[H] from Z[0]
template <typename T, int H>
__device__ __forceinline__ void r2c_row(const T* __restrict__ in, cx<T>* __restrict__ out, int64_t nrows,
                                        const cx<T>* __restrict__ tw, const cx<T>* __restrict__ rtw, cx<T>* smem) {
  constexpr int PP = H / 8, SH = row_shift<T>(), STRIDE = H + (H >> SH) + 1;
  const int rows = blockDim.x / PP, ln = threadIdx.x / PP, t = threadIdx.x & (PP - 1);
  const int64_t row = (int64_t)blockIdx.x * rows + ln;
  const bool live = row < nrows;
  const cx<T>* src = reinterpret_cast<const cx<T>*>(in + (live ? row : 0) * (2 * (int64_t)H));
  cx<T> v[1][8];
#pragma unroll
  for (int q = 0; q < 8; ++q) v[0][q] = live ? src[t + q * PP] : czero<T>();
  cx<T>* const buf[1] = {smem};
  const XRow xr{ln * STRIDE, SH};
  regfft<T, 1, H, -1>(v, t, tw, buf, xr);
#pragma unroll
  for (int q = 0; q < 8; ++q) smem[xr(t + q * PP)] = v[0][q];
  __syncthreads();
  if (live) {
    cx<T>* o = out + row * (int64_t)(H + 1);
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const int k = t + q * PP;
      if (k == 0) {
        const cx<T> z = v[0][0];
        o[0] = mk<T>(z.x + z.y, T(0));
        o[H] = mk<T>(z.x - z.y, T(0));
      } else {
        cx<T> xk, xhk;
        r2c_pair<T>(v[0][q], smem[xr(H - k)], __ldg(&rtw[k]), xk, xhk);
        o[k] = xk;
      }
    }
  }
}

// C2R of rows of H + 1 complex values -> 2H reals, times scale
template <typename T, int H>
__device__ __forceinline__ void c2r_row(const cx<T>* __restrict__ in, T* __restrict__ out, int64_t nrows,
                                        const cx<T>* __restrict__ tw, const cx<T>* __restrict__ rtw, T scale,
                                        cx<T>* smem) {
  constexpr int PP = H / 8, SH = row_shift<T>(), STRIDE = H + (H >> SH) + 1;
  const int rows = blockDim.x / PP, ln = threadIdx.x / PP, t = threadIdx.x & (PP - 1);
  const int64_t row = (int64_t)blockIdx.x * rows + ln;
  const bool live = row < nrows;
  const cx<T>* r = in + (live ? row : 0) * (int64_t)(H + 1);
  const XRow xr{ln * STRIDE, SH};
  // packing by pairs: k = t + q PP (q < 4) gives Z[k] = A + i P and Z[H-k] = conj(A) + i conj(P)
  // from A = X[k] + conj X[H-k] and P = (X[k] - conj X[H-k]) conj(W^k); the partner value
  // reaches its owner through shared memory, Z[0] and the self-paired Z[H/2] directly
  cx<T> v[1][8];
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int k = t + q * PP;
    cx<T> zk = czero<T>(), zh = czero<T>();
    if (live) {
      if (k == 0) {
        zk = c2r_pre<T>(r[0], r[H], __ldg(&rtw[0]), 0);
      } else {
        const cx<T> b = conj(r[H - k]);
        const cx<T> xk = r[k];
        const cx<T> a = add(xk, b);
        const cx<T> pp = cmulc(sub(xk, b), __ldg(&rtw[k]));
        zk = add(a, mul_i(pp));
        zh = mk<T>(a.x + pp.y, pp.x - a.y);
      }
    }
    v[0][q] = zk;
    if (k != 0) smem[xr(H - k)] = zh;
  }
  if (t == 0) smem[xr(H / 2)] = live ? c2r_pre<T>(r[H / 2], r[H / 2], __ldg(&rtw[H / 2]), H / 2) : czero<T>();
  __syncthreads();
#pragma unroll
  for (int q = 4; q < 8; ++q) v[0][q] = smem[xr(t + q * PP)];
  __syncthreads();
  cx<T>* const buf[1] = {smem};
  regfft<T, 1, H, 1>(v, t, tw, buf, xr);
  if (live) {
    cx<T>* o = reinterpret_cast<cx<T>*>(out + row * (2 * (int64_t)H));
#pragma unroll
    for (int q = 0; q < 8; ++q) o[t + q * PP] = scl(v[0][q], scale);
  }
}

// C2C of contiguous rows of N complex values (in may alias out: every element is read
// into registers before the first exchange and written after the last)
template <typename T, int N, int DIR>
__device__ __forceinline__ void c2c_row(const cx<T>* in, cx<T>* out, int64_t nrows, const cx<T>* __restrict__ tw,
                                        T scale, cx<T>* smem) {
  constexpr int PP = N / 8, SH = row_shift<T>(), STRIDE = N + (N >> SH) + 1;
  const int rows = blockDim.x / PP, ln = threadIdx.x / PP, t = threadIdx.x & (PP - 1);
  const int64_t row = (int64_t)blockIdx.x * rows + ln;
  const bool live = row < nrows;
  const cx<T>* src = in + (live ? row : 0) * (int64_t)N;
  cx<T> v[1][8];
#pragma unroll
  for (int q = 0; q < 8; ++q) v[0][q] = live ? src[t + q * PP] : czero<T>();
  cx<T>* const buf[1] = {smem};
  regfft<T, 1, N, DIR>(v, t, tw, buf, XRow{ln * STRIDE, SH});
  if (live) {
    cx<T>* o = out + row * (int64_t)N;
#pragma unroll
    for (int q = 0; q < 8; ++q) o[t + q * PP] = scl(v[0][q], scale);
  }
}

// C2C along a strided axis: a tile of tl adjacent columns, thread (t, ln) holding rows
// t + q N/8 of column c0 + ln (a warp's loads touch tl adjacent columns of 32/tl rows)
template <typename T, int N, int DIR>
__device__ __forceinline__ void col_tile(const cx<T>* in, cx<T>* out, int64_t ncols, int64_t stride, int64_t base,
                                         const cx<T>* __restrict__ tw, T scale, cx<T>* smem) {
  constexpr int PP = N / 8;
  const int tl = blockDim.x / PP, ln = threadIdx.x & (tl - 1), t = threadIdx.x / tl;
  const int64_t c = (int64_t)blockIdx.x * tl + ln;
  const bool live = c < ncols;
  cx<T> v[1][8];
#pragma unroll
  for (int q = 0; q < 8; ++q) v[0][q] = live ? in[base + c + (int64_t)(t + q * PP) * stride] : czero<T>();
  cx<T>* const buf[1] = {smem};
  regfft<T, 1, N, DIR>(v, t, tw, buf, XCol{tl, ln});
  if (live) {
#pragma unroll
    for (int q = 0; q < 8; ++q) out[base + c + (int64_t)(t + q * PP) * stride] = scl(v[0][q], scale);
  }
}

#define FF_PLAN_ROW_CASES(X) X(16) X(32) X(64) X(128) X(256) X(512) X(1024) X(2048)
#define FF_PLAN_LINE_CASES(X) X(16) X(32) X(64) X(128) X(256) X(512) X(1024) X(2048) X(4096)

template <typename T>
__global__ void __launch_bounds__(kMaxThreads) k_r2c_rows_r(const T* __restrict__ in, cx<T>* __restrict__ out,
                                                           int64_t nrows, int h, const cx<T>* __restrict__ tw,
                                                           const cx<T>* __restrict__ rtw) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cx<T>* smem = reinterpret_cast<cx<T>*>(smem_raw);
  switch (h) {
#define FF_CASE(H) \
  case H: r2c_row<T, H>(in, out, nrows, tw, rtw, smem); break;
    FF_PLAN_ROW_CASES(FF_CASE)
#undef FF_CASE
    default: break;
  }
}

template <typename T>
__global__ void __launch_bounds__(kMaxThreads) k_c2r_rows_r(const cx<T>* __restrict__ in, T* __restrict__ out,
                                                           int64_t nrows, int h, const cx<T>* __restrict__ tw,
                                                           const cx<T>* __restrict__ rtw, T scale) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cx<T>* smem = reinterpret_cast<cx<T>*>(smem_raw);
  switch (h) {
#define FF_CASE(H) \
  case H: c2r_row<T, H>(in, out, nrows, tw, rtw, scale, smem); break;
    FF_PLAN_ROW_CASES(FF_CASE)
#undef FF_CASE
    default: break;
  }
}

template <typename T, int DIR>
__global__ void __launch_bounds__(kMaxThreads) k_c2c_rows_r(const cx<T>* in, cx<T>* out, int64_t nrows, int n,
                                                           const cx<T>* __restrict__ tw, T scale) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cx<T>* smem = reinterpret_cast<cx<T>*>(smem_raw);
  switch (n) {
#define FF_CASE(N) \
  case N: c2c_row<T, N, DIR>(in, out, nrows, tw, scale, smem); break;
    FF_PLAN_LINE_CASES(FF_CASE)
#undef FF_CASE
    default: break;
  }
}

template <typename T, int DIR>
__global__ void __launch_bounds__(kMaxThreads) k_cols_r(const cx<T>* in, cx<T>* out, int64_t ncols, int n, int64_t stride,
                                               int64_t nouter, int64_t outer_stride, const cx<T>* __restrict__ tw,
                                               T scale) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cx<T>* smem = reinterpret_cast<cx<T>*>(smem_raw);
  for (int64_t o = blockIdx.y; o < nouter; o += gridDim.y) {
    switch (n) {
#define FF_CASE(N) \
  case N: col_tile<T, N, DIR>(in, out, ncols, stride, o * outer_stride, tw, scale, smem); break;
      FF_PLAN_LINE_CASES(FF_CASE)
#undef FF_CASE
      default: break;
    }
    __syncthreads();
  }
}

// threads for lines of length n: one line needs n/8; several short lines share a CTA
int line_threads(int n, int cap) {
  int t = n / 8;
  while (t * 2 <= cap) t *= 2;
  return t;
}

}  // namespace

bool reg_rows_ok(int h) { return regfft_ok(h) && h <= 2048; }
bool reg_line_ok(int n) { return regfft_ok(n); }

template <typename T>
int launch_r2c_rows_reg(const T* in, cx<T>* out, int64_t nrows, int nx, const cx<T>* tw, const cx<T>* rtw,
                        cudaStream_t s) {
  const int h = nx / 2, nt = line_threads(h, kRegThreads), rows = nt * 8 / h;
  const size_t smem = (size_t)rows * (h + (h >> row_shift<T>()) + 1) * sizeof(cx<T>);
  if (int st = ensure_smem((const void*)k_r2c_rows_r<T>, smem)) return st;
  k_r2c_rows_r<T><<<(unsigned)ceil_div(nrows, rows), nt, smem, s>>>(in, out, nrows, h, tw, rtw);
  FF_LAUNCHED("k_r2c_rows_r");
  return FF_OK;
}

template <typename T>
int launch_c2r_rows_reg(const cx<T>* in, T* out, int64_t nrows, int nx, const cx<T>* tw, const cx<T>* rtw, T scale,
                        cudaStream_t s) {
  const int h = nx / 2, nt = line_threads(h, kRegThreads), rows = nt * 8 / h;
  const size_t smem = (size_t)rows * (h + (h >> row_shift<T>()) + 1) * sizeof(cx<T>);
  if (int st = ensure_smem((const void*)k_c2r_rows_r<T>, smem)) return st;
  k_c2r_rows_r<T><<<(unsigned)ceil_div(nrows, rows), nt, smem, s>>>(in, out, nrows, h, tw, rtw, scale);
  FF_LAUNCHED("k_c2r_rows_r");
  return FF_OK;
}

template <typename T, int DIR>
int launch_c2c_rows_reg(const cx<T>* in, cx<T>* out, int64_t nrows, int n, const cx<T>* tw, T scale,
                        cudaStream_t s) {
  const int nt = line_threads(n, kRegThreads), rows = nt * 8 / n;
  const size_t smem = (size_t)rows * (n + (n >> row_shift<T>()) + 1) * sizeof(cx<T>);
  if (int st = ensure_smem((const void*)k_c2c_rows_r<T, DIR>, smem)) return st;
  k_c2c_rows_r<T, DIR><<<(unsigned)ceil_div(nrows, rows), nt, smem, s>>>(in, out, nrows, n, tw, scale);
  FF_LAUNCHED("k_c2c_rows_r");
  return FF_OK;
}

template <typename T, int DIR>
int launch_cols_reg(const cx<T>* in, cx<T>* out, int64_t ncols, int n, int64_t stride, int64_t nouter,
                    int64_t outer_stride, const cx<T>* tw, T scale, cudaStream_t s) {
  // tiles of tl adjacent columns (32-byte row segments: 2 FP64 or 4 FP32 columns), more for
  // short columns so that a CTA has at least 64 threads, fewer where a CTA would pass 512
  const int pp = n / 8;
  int tl = sizeof(T) == 8 ? 2 : 4;
  while (tl * pp < 64) tl *= 2;
  while (tl > 1 && tl * pp > kMaxThreads) tl /= 2;
  const int nt = tl * pp;
  const size_t smem = (size_t)(n + n / 8) * tl * sizeof(cx<T>);
  if (int st = ensure_smem((const void*)k_cols_r<T, DIR>, smem)) return st;
  dim3 grid((unsigned)ceil_div(ncols, tl), (unsigned)(nouter < 65535 ? nouter : 65535));
  k_cols_r<T, DIR><<<grid, nt, smem, s>>>(in, out, ncols, n, stride, nouter, outer_stride, tw, scale);
  FF_LAUNCHED("k_cols_r");
  return FF_OK;
}

#define FF_INST(T)                                                                                            \
  template int launch_r2c_rows_reg<T>(const T*, cx<T>*, int64_t, int, const cx<T>*, const cx<T>*, cudaStream_t); \
  template int launch_c2r_rows_reg<T>(const cx<T>*, T*, int64_t, int, const cx<T>*, const cx<T>*, T,             \
                                      cudaStream_t);                                                           \
  template int launch_c2c_rows_reg<T, -1>(const cx<T>*, cx<T>*, int64_t, int, const cx<T>*, T, cudaStream_t);    \
  template int launch_c2c_rows_reg<T, 1>(const cx<T>*, cx<T>*, int64_t, int, const cx<T>*, T, cudaStream_t);     \
  template int launch_cols_reg<T, -1>(const cx<T>*, cx<T>*, int64_t, int, int64_t, int64_t, int64_t,           \
                                      const cx<T>*, T, cudaStream_t);                                          \
  template int launch_cols_reg<T, 1>(const cx<T>*, cx<T>*, int64_t, int, int64_t, int64_t, int64_t, const cx<T>*, \
                                     T, cudaStream_t);
FF_INST(float)
FF_INST(double)
#undef FF_INST

}  // namespace ff
