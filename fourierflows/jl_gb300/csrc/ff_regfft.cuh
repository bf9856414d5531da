// Register-resident Stockham FFT for power-of-two line lengths N (16 .. 4096).
//
// A line of length N is held by P = N/8 threads; thread t owns x[t + q P], q = 0..7, in
// registers.  Stages run small radix first (2 or 4 when log2 N is not a multiple of 3),
// then radix 8.  In the Stockham order, butterfly j of a radix-R stage reads positions
// j + r N/R; with j = t + m P (m < 8/R) those are exactly thread t's slots m + r (8/R), so
// every butterfly of every stage is computed from the owning thread's own registers.
// Between stages the outputs are scattered to shared memory at their Stockham positions
//     (j - k) R + k + r Ns,   k = j mod Ns
// and gathered back in the t + q P pattern: one exchange (two barriers) per stage except
// the last.  The last stage is radix 8 with Ns = P, whose outputs t + r P are thread t's
// own slots, so a transform ends with the result in natural order in registers.
//
// F independent lines per thread (fields) share each exchange's barriers.  All index
// arithmetic is compile-time shifts and masks.  Twiddles come from the per-length table
// W_N^e of the host (ff_plan.cu).
#pragma once

#include "ff_fft.cuh"

namespace ff {

__host__ __device__ constexpr int ilog2c(int n) { return n <= 1 ? 0 : 1 + ilog2c(n / 2); }

__host__ __device__ constexpr bool regfft_ok(int n) { return n >= 16 && n <= 4096 && (n & (n - 1)) == 0; }

// shared-memory slot of position p of a line: columns interleave tl lines (line fastest),
// rows keep lines contiguous; one pad slot every 8 (columns) or 2^sh (rows) positions
struct XCol {
  int tl, ln;
  __device__ __forceinline__ int operator()(int p) const { return (p + (p >> 3)) * tl + ln; }
};
struct XRow {
  int base, sh;
  __device__ __forceinline__ int operator()(int p) const { return base + p + (p >> sh); }
};

// twiddles W_N^(k r N/(8 NS)), r = 1..7, of a radix-8 stage of span NS > 1 (k = t mod NS):
// the only stages with twiddles, since a smaller radix only ever opens a transform.  The
// table holds W_N^e for e < N and then these stage by stage, r-major (host_twiddles):
// entry N + (NS - R0) + (r - 1) NS + k, R0 the first stage's radix, so consecutive threads
// read consecutive entries.
template <typename T, int N, int NS>
__device__ __forceinline__ void stage_twiddles(int t, const cx<T>* __restrict__ tw, cx<T> (&w)[8]) {
  constexpr int L = ilog2c(N);
  constexpr int R0 = (L % 3) != 0 ? (1 << (L % 3)) : 8;
  const int k = t & (NS - 1);
  const cx<T>* stage = tw + N + (NS - R0);
#pragma unroll
  for (int r = 1; r < 8; ++r) w[r] = __ldg(&stage[(r - 1) * NS + k]);
}

// one stage of span NS with its twiddles w already in registers; the next stage's
// twiddles are loaded before the exchange so that their latency hides behind it
template <typename T, int F, int N, int DIR, int NS, class X>
__device__ __forceinline__ void regfft_from(cx<T> (&v)[F][8], int t, const cx<T>* __restrict__ tw,
                                            cx<T>* const* buf, X x, const cx<T> (&w)[8]) {
  constexpr int L = ilog2c(N);
  constexpr int R = (NS == 1 && (L % 3) != 0) ? (1 << (L % 3)) : 8;
  constexpr int M = 8 / R;
  constexpr int P = N / 8;
#pragma unroll
  for (int m = 0; m < M; ++m) {
#pragma unroll
    for (int f = 0; f < F; ++f) {
      cx<T> u[R];
#pragma unroll
      for (int r = 0; r < R; ++r) u[r] = v[f][m + r * M];
      if constexpr (NS > 1 && R == 8 && FF_TWIDDLE_FMA && sizeof(T) == 8) {
        Dft8Tw<T, DIR>::run(u, w);  // FP64: the twiddles inside the first butterfly layer
      } else {
        if (NS > 1) {
#pragma unroll
          for (int r = 1; r < R; ++r) u[r] = DIR < 0 ? cmul(u[r], w[r]) : cmulc(u[r], w[r]);
        }
        Dft<T, R, DIR>::run(u);
      }
#pragma unroll
      for (int r = 0; r < R; ++r) v[f][m + r * M] = u[r];
    }
  }
  if constexpr (NS * R < N) {
    cx<T> wn[8];
    stage_twiddles<T, N, NS * R>(t, tw, wn);
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const int m = q % M, r = q / M;
      const int j = t + m * P;
      const int k = j & (NS - 1);
      const int pos = (j - k) * R + k + r * NS;
#pragma unroll
      for (int f = 0; f < F; ++f) buf[f][x(pos)] = v[f][q];
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < 8; ++q)
#pragma unroll
      for (int f = 0; f < F; ++f) v[f][q] = buf[f][x(t + q * P)];
    __syncthreads();
    regfft_from<T, F, N, DIR, NS * R, X>(v, t, tw, buf, x, wn);
  }
}

// v[f][q] = x_f[t + q N/8] in; X_f[t + q N/8] out (DIR -1: forward, +1: unnormalised inverse)
template <typename T, int F, int N, int DIR, class X>
__device__ __forceinline__ void regfft(cx<T> (&v)[F][8], int t, const cx<T>* __restrict__ tw, cx<T>* const* buf,
                                       X x) {
  const cx<T> none[8] = {};
  regfft_from<T, F, N, DIR, 1, X>(v, t, tw, buf, x, none);
}

}  // namespace ff
