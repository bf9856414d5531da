// Line-FFT engine: mixed-radix Stockham transforms of several lines held in shared memory.
//
// A "line" is one 1D complex transform of length n.  A CTA loads a tile of lines into a
// shared-memory buffer, runs every radix stage of the plan with all of its threads
// (ping-pong between two buffers, one barrier per stage) and stores the tile back.  The
// kernels that call this engine decide how a tile is gathered from HBM and how it is
// scattered, which is where the physics of the fused passes is folded in.
//
// Stage s with radix R and span Ns (product of the earlier radices) maps butterfly j of
// a line (j in [0, n/R)) to
//     inputs   src[j + r*n/R],                   r = 0..R-1
//     twiddle  W_n^{k r n/(Ns R)},  k = j mod Ns
//     outputs  dst[(j - k) R + k + r Ns]
// which is the self-sorting (Stockham) decimation-in-time order: the result comes out
// in natural order without a bit-reversal pass.
//
// Twiddles are read from a per-length table tw[e] = exp(-2 pi i e / n) built on the host
// in extended precision; the inverse direction conjugates them.  No transcendental
// function is evaluated on the device.
#pragma once

#include "ff_common.cuh"

namespace ff {

#define FF_MAX_STAGES 24
#define FF_MAX_GENERIC_RADIX 31

struct LinePlan {
  int n;                       // complex length of a line
  int nst;                     // number of stages
  int radix[FF_MAX_STAGES];    // radix of each stage, in execution order
};

// butterfly constants (exact decimal expansions rounded by the compiler)
#define FF_SQRT1_2 0.707106781186547524400844362105
#define FF_SQRT3_2 0.866025403784438646763723170753
#define FF_C5_1 0.309016994374947424102293417183
#define FF_C5_2 (-0.809016994374947424102293417183)
#define FF_S5_1 0.951056516295153572116439333379
#define FF_S5_2 0.587785252292473129168705954639

// multiply by -i for the forward transform (DIR = -1), by +i for the inverse (DIR = +1)
template <int DIR, typename C> __device__ __forceinline__ C rot(C a) { return DIR < 0 ? mul_mi(a) : mul_i(a); }

// ---------------------------------------------------------------------------------------
// small DFTs on registers, v[q] <- sum_r v[r] exp(DIR 2 pi i r q / R)
// ---------------------------------------------------------------------------------------
template <typename T, int R, int DIR> struct Dft;

template <typename T, int DIR> struct Dft<T, 2, DIR> {
  static __device__ __forceinline__ void run(cx<T>* v) {
    cx<T> a = v[0], b = v[1];
    v[0] = add(a, b);
    v[1] = sub(a, b);
  }
};

template <typename T, int DIR> struct Dft<T, 4, DIR> {
  static __device__ __forceinline__ void run(cx<T>* v) {
    cx<T> s02 = add(v[0], v[2]), d02 = sub(v[0], v[2]);
    cx<T> s13 = add(v[1], v[3]), d13 = rot<DIR>(sub(v[1], v[3]));
    v[0] = add(s02, s13);
    v[2] = sub(s02, s13);
    v[1] = add(d02, d13);
    v[3] = sub(d02, d13);
  }
};

// FP64 twiddled radix-8 stages fold their twiddle products into the butterfly's first
// layer (Dft8Tw), and pass B's packing and unpacking fold theirs into FMA chains; 0
// restores product-then-add everywhere
#ifndef FF_TWIDDLE_FMA
#define FF_TWIDDLE_FMA 1
#endif

// the radix-8 butterfly after its first layer: a[r] = v[r] + v[r+4], b[r] = v[r] - v[r+4]
template <typename T, int DIR> __device__ __forceinline__ void dft8_rest(cx<T> (&a)[4], cx<T> (&b)[4], cx<T>* v);

template <typename T, int DIR> struct Dft<T, 8, DIR> {
  static __device__ __forceinline__ void run(cx<T>* v) {
    cx<T> a[4], b[4];
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      a[r] = add(v[r], v[r + 4]);
      b[r] = sub(v[r], v[r + 4]);
    }
    dft8_rest<T, DIR>(a, b, v);
  }
};

// a + u w (DIR < 0) or a + u conj(w) (DIR > 0) as two FMA chains (four FMAs where a product
// and an add take six operations)
template <int DIR, typename C> __device__ __forceinline__ C fma_tw(C a, C u, C w) {
  C r;
  if (DIR < 0) {
    r.x = fma(u.x, w.x, fma(-u.y, w.y, a.x));
    r.y = fma(u.x, w.y, fma(u.y, w.x, a.y));
  } else {
    r.x = fma(u.x, w.x, fma(u.y, w.y, a.x));
    r.y = fma(u.y, w.x, fma(-u.x, w.y, a.y));
  }
  return r;
}
// 2 t - s (one FMA per part; 2 t is exact)
template <typename C> __device__ __forceinline__ C twice_minus(C t, C s) {
  C r;
  r.x = fma(decltype(t.x)(2), t.x, -s.x);
  r.y = fma(decltype(t.y)(2), t.y, -s.y);
  return r;
}

// Radix-8 butterfly of a twiddled stage, the twiddles w[1..7] applied inside its first
// layer: with t_r = u_r w_r (t_0 = u_0), a[r] = t_r + u_{r+4} w_{r+4} by FMA chains and
// b[r] = 2 t_r - a[r], 36 instead of 44 FP64 operations for the twiddles and that layer.
// Used for FP64, whose kernels are bound by the FP64 pipe; the rounding differs from
// twiddle-then-butterfly within the FFT's usual error.
template <typename T, int DIR> struct Dft8Tw {
  static __device__ __forceinline__ void run(cx<T>* v, const cx<T>* w) {
    cx<T> a[4], b[4];
    a[0] = fma_tw<DIR>(v[0], v[4], w[4]);
    b[0] = twice_minus(v[0], a[0]);
#pragma unroll
    for (int r = 1; r < 4; ++r) {
      const cx<T> t = DIR < 0 ? cmul(v[r], w[r]) : cmulc(v[r], w[r]);
      a[r] = fma_tw<DIR>(t, v[r + 4], w[r + 4]);
      b[r] = twice_minus(t, a[r]);
    }
    dft8_rest<T, DIR>(a, b, v);
  }
};

template <typename T, int DIR> __device__ __forceinline__ void dft8_rest(cx<T> (&a)[4], cx<T> (&b)[4], cx<T>* v) {
  const T h = T(FF_SQRT1_2);
  Dft<T, 4, DIR>::run(a);
  if constexpr (sizeof(T) == 8 && FF_TWIDDLE_FMA) {
    // FP64: b[1] W8 = h r1 and b[3] W8^3 = h r3 with r1, r3 the unscaled rotations; the
    // factor h then enters the radix-4 butterfly's output FMAs (20 instead of 24 operations)
    const cx<T> r1 = DIR < 0 ? mk<T>(b[1].x + b[1].y, b[1].y - b[1].x) : mk<T>(b[1].x - b[1].y, b[1].y + b[1].x);
    const cx<T> r3 = DIR < 0 ? mk<T>(b[3].y - b[3].x, -(b[3].x + b[3].y)) : mk<T>(-(b[3].x + b[3].y), b[3].x - b[3].y);
    const cx<T> b2 = rot<DIR>(b[2]);
    const cx<T> s02 = add(b[0], b2), d02 = sub(b[0], b2);
    const cx<T> r13 = add(r1, r3), e13 = rot<DIR>(sub(r1, r3));
    v[1] = mk<T>(fma(h, r13.x, s02.x), fma(h, r13.y, s02.y));
    v[5] = mk<T>(fma(-h, r13.x, s02.x), fma(-h, r13.y, s02.y));
    v[3] = mk<T>(fma(h, e13.x, d02.x), fma(h, e13.y, d02.y));
    v[7] = mk<T>(fma(-h, e13.x, d02.x), fma(-h, e13.y, d02.y));
  } else {
    // b[r] *= W8^r (forward W8 = (1 - i)/sqrt2, inverse its conjugate)
    b[1] = DIR < 0 ? mk<T>(h * (b[1].x + b[1].y), h * (b[1].y - b[1].x))
                   : mk<T>(h * (b[1].x - b[1].y), h * (b[1].y + b[1].x));
    b[2] = rot<DIR>(b[2]);
    b[3] = DIR < 0 ? mk<T>(h * (b[3].y - b[3].x), -h * (b[3].x + b[3].y))
                   : mk<T>(-h * (b[3].x + b[3].y), h * (b[3].x - b[3].y));
    Dft<T, 4, DIR>::run(b);
#pragma unroll
    for (int q = 0; q < 4; ++q) v[2 * q + 1] = b[q];
  }
#pragma unroll
  for (int q = 0; q < 4; ++q) v[2 * q] = a[q];
}

// FP32 butterflies on Blackwell's packed FP32 instructions.  A float2 complex value is one
// register pair and FADD2 / FFMA2 / FMUL2 apply one operation to both halves, so an
// untwiddled complex add or subtract is one instruction instead of two.  A product with
// +-i swaps the halves; it is folded into an FFMA2 with a sign pair (x*1 + a and x*-1 + a
// round exactly as a + x and a - x do), so every result is the scalar form's, bit for bit.
#ifndef FF_PACKED_F32
#define FF_PACKED_F32 1
#endif
#if FF_PACKED_F32  // sm_100 and later (this library builds for sm_103a only)
namespace pk {
__device__ __forceinline__ float2 add(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 sub(float2 a, float2 b) { return __ffma2_rn(b, make_float2(-1.f, -1.f), a); }
__device__ __forceinline__ float2 swp(float2 a) { return make_float2(a.y, a.x); }
// a + rot<DIR>(b) and a - rot<DIR>(b); rot is -i (DIR < 0: (b.y, -b.x)) or +i ((-b.y, b.x))
template <int DIR> __device__ __forceinline__ float2 add_rot(float2 a, float2 b) {
  return __ffma2_rn(swp(b), DIR < 0 ? make_float2(1.f, -1.f) : make_float2(-1.f, 1.f), a);
}
template <int DIR> __device__ __forceinline__ float2 sub_rot(float2 a, float2 b) {
  return __ffma2_rn(swp(b), DIR < 0 ? make_float2(-1.f, 1.f) : make_float2(1.f, -1.f), a);
}
}  // namespace pk

template <int DIR> struct Dft<float, 2, DIR> {
  static __device__ __forceinline__ void run(float2* v) {
    const float2 a = v[0], b = v[1];
    v[0] = pk::add(a, b);
    v[1] = pk::sub(a, b);
  }
};

// v[2] enters multiplied by rot<DIR> when rot2 (the radix-8 butterfly's b[2] * W8^2)
template <int DIR, bool ROT2 = false> __device__ __forceinline__ void dft4_packed(float2* v) {
  const float2 s02 = ROT2 ? pk::add_rot<DIR>(v[0], v[2]) : pk::add(v[0], v[2]);
  const float2 d02 = ROT2 ? pk::sub_rot<DIR>(v[0], v[2]) : pk::sub(v[0], v[2]);
  const float2 s13 = pk::add(v[1], v[3]);
  const float2 x = pk::sub(v[1], v[3]);  // d13 = rot<DIR>(x)
  v[0] = pk::add(s02, s13);
  v[2] = pk::sub(s02, s13);
  v[1] = pk::add_rot<DIR>(d02, x);
  v[3] = pk::sub_rot<DIR>(d02, x);
}

template <int DIR> struct Dft<float, 4, DIR> {
  static __device__ __forceinline__ void run(float2* v) { dft4_packed<DIR>(v); }
};

template <int DIR> struct Dft<float, 8, DIR> {
  static __device__ __forceinline__ void run(float2* v) {
    const float h = float(FF_SQRT1_2);
    float2 a[4], b[4];
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      a[r] = pk::add(v[r], v[r + 4]);
      b[r] = pk::sub(v[r], v[r + 4]);
    }
    // b[1] *= W8 = (1 -+ i)/sqrt2: (b + rot(b)) h; b[3] *= W8^3 = -(1 +- i)/sqrt2: (b + rot'(b)) (-h)
    b[1] = __fmul2_rn(pk::add_rot<DIR>(b[1], b[1]), make_float2(h, h));
    b[3] = __fmul2_rn(pk::add_rot<-DIR>(b[3], b[3]), make_float2(-h, -h));
    dft4_packed<DIR>(a);
    dft4_packed<DIR, true>(b);  // b[2] *= W8^2 = rot<DIR>, folded into its first adds
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      v[2 * q] = a[q];
      v[2 * q + 1] = b[q];
    }
  }
};
#endif

template <typename T, int DIR> struct Dft<T, 3, DIR> {
  static __device__ __forceinline__ void run(cx<T>* v) {
    const T s = T(FF_SQRT3_2);
    cx<T> t = add(v[1], v[2]);
    cx<T> m = sub(v[0], scl(t, T(0.5)));
    cx<T> d = rot<DIR>(scl(sub(v[1], v[2]), s));
    v[0] = add(v[0], t);
    v[1] = add(m, d);
    v[2] = sub(m, d);
  }
};

template <typename T, int DIR> struct Dft<T, 5, DIR> {
  static __device__ __forceinline__ void run(cx<T>* v) {
    const T c1 = T(FF_C5_1), c2 = T(FF_C5_2), s1 = T(FF_S5_1), s2 = T(FF_S5_2);
    cx<T> t1 = add(v[1], v[4]), t2 = add(v[2], v[3]);
    cx<T> t3 = sub(v[1], v[4]), t4 = sub(v[2], v[3]);
    cx<T> a1 = mk<T>(v[0].x + c1 * t1.x + c2 * t2.x, v[0].y + c1 * t1.y + c2 * t2.y);
    cx<T> a2 = mk<T>(v[0].x + c2 * t1.x + c1 * t2.x, v[0].y + c2 * t1.y + c1 * t2.y);
    cx<T> b1 = rot<DIR>(mk<T>(s1 * t3.x + s2 * t4.x, s1 * t3.y + s2 * t4.y));
    cx<T> b2 = rot<DIR>(mk<T>(s2 * t3.x - s1 * t4.x, s2 * t3.y - s1 * t4.y));
    v[0] = add(v[0], add(t1, t2));
    v[1] = add(a1, b1);
    v[4] = sub(a1, b1);
    v[2] = add(a2, b2);
    v[3] = sub(a2, b2);
  }
};

// ---------------------------------------------------------------------------------------
// shared-memory addressing of a tile of lines
// ---------------------------------------------------------------------------------------
// Interleaved tile: element j of line ln at j*tl + ln.  Used by the strided-axis passes,
// whose tiles are tl adjacent columns; consecutive threads touch consecutive addresses.
struct AddrTile {
  int tl;
  __device__ __forceinline__ int operator()(int ln, int j) const { return j * tl + ln; }
  __device__ __forceinline__ void map(int b, int nb, int& ln, int& j) const {
    ln = b % tl;
    j = b / tl;
  }
};

// Line-major tile with one padding slot every 2^sh elements (bank-conflict relief for
// the power-of-two strides of the early Stockham stages).  Used by the row passes.
struct AddrRows {
  int stride;  // padded line length
  int sh;
  __device__ __forceinline__ int operator()(int ln, int j) const { return ln * stride + j + (j >> sh); }
  __device__ __forceinline__ void map(int b, int nb, int& ln, int& j) const {
    ln = b / nb;
    j = b - ln * nb;
  }
};

__host__ __device__ inline int rows_pad_shift(int elem_bytes) { return elem_bytes == 16 ? 3 : 4; }
__host__ __device__ inline int rows_stride(int n, int elem_bytes) {
  int sh = rows_pad_shift(elem_bytes);
  return n + (n >> sh) + 1;
}

// ---------------------------------------------------------------------------------------
// one Stockham stage
// ---------------------------------------------------------------------------------------
template <typename T, int R, int DIR, class A>
__device__ __forceinline__ void fft_stage(const cx<T>* __restrict__ src, cx<T>* __restrict__ dst,
                                          const cx<T>* __restrict__ tw, int n, int Ns, int nlines, A addr,
                                          int tid, int nth) {
  const int nb = n / R;
  const int tws = n / (Ns * R);
  const int total = nlines * nb;
  for (int b = tid; b < total; b += nth) {
    int ln, j;
    addr.map(b, nb, ln, j);
    cx<T> v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) v[r] = src[addr(ln, j + r * nb)];
    const int k = j % Ns;
    if constexpr (R == 8 && sizeof(T) == 8 && FF_TWIDDLE_FMA) {
      // FP64: the twiddle products inside the butterfly's first layer (Dft8Tw)
      if (Ns > 1) {
        cx<T> w[8];
#pragma unroll
        for (int r = 1; r < 8; ++r) w[r] = __ldg(&tw[k * r * tws]);
        Dft8Tw<T, DIR>::run(v, w);
      } else {
        Dft<T, 8, DIR>::run(v);
      }
    } else {
      if (Ns > 1) {
#pragma unroll
        for (int r = 1; r < R; ++r) {
          cx<T> w = __ldg(&tw[k * r * tws]);
          v[r] = DIR < 0 ? cmul(v[r], w) : cmulc(v[r], w);
        }
      }
      Dft<T, R, DIR>::run(v);
    }
    const int ob = (j - k) * R + k;
#pragma unroll
    for (int r = 0; r < R; ++r) dst[addr(ln, ob + r * Ns)] = v[r];
  }
}

// Any radix p <= FF_MAX_GENERIC_RADIX (odd primes without a dedicated butterfly): a direct
// O(p^2) DFT using the same length-n twiddle table, W_p^{e} = W_n^{e n/p}.
template <typename T, int DIR, class A>
__device__ void fft_stage_generic(const cx<T>* __restrict__ src, cx<T>* __restrict__ dst,
                                  const cx<T>* __restrict__ tw, int n, int Ns, int p, int nlines, A addr,
                                  int tid, int nth) {
  const int nb = n / p;
  const int tws = n / (Ns * p);
  const int total = nlines * nb;
  for (int b = tid; b < total; b += nth) {
    int ln, j;
    addr.map(b, nb, ln, j);
    cx<T> v[FF_MAX_GENERIC_RADIX];
    const int k = j % Ns;
    for (int r = 0; r < p; ++r) {
      cx<T> x = src[addr(ln, j + r * nb)];
      if (Ns > 1 && r > 0) {
        cx<T> w = __ldg(&tw[k * r * tws]);
        x = DIR < 0 ? cmul(x, w) : cmulc(x, w);
      }
      v[r] = x;
    }
    const int ob = (j - k) * p + k;
    for (int q = 0; q < p; ++q) {
      cx<T> acc = v[0];
      for (int r = 1; r < p; ++r) {
        cx<T> w = __ldg(&tw[((r * q) % p) * nb]);
        acc = add(acc, DIR < 0 ? cmul(v[r], w) : cmulc(v[r], w));
      }
      dst[addr(ln, ob + q * Ns)] = acc;
    }
  }
}

// Run every stage of plan P on the tile in buffer a (b is the second buffer).  The caller
// has filled a and synchronised; on return the result is in the returned buffer and the
// CTA is synchronised.
template <typename T, int DIR, class A>
__device__ cx<T>* fft_lines(cx<T>* a, cx<T>* b, const cx<T>* __restrict__ tw, const LinePlan& P, int nlines,
                            A addr) {
  const int tid = threadIdx.x, nth = blockDim.x;
  int Ns = 1;
  for (int s = 0; s < P.nst; ++s) {
    const int R = P.radix[s];
    switch (R) {
      case 8: fft_stage<T, 8, DIR>(a, b, tw, P.n, Ns, nlines, addr, tid, nth); break;
      case 4: fft_stage<T, 4, DIR>(a, b, tw, P.n, Ns, nlines, addr, tid, nth); break;
      case 2: fft_stage<T, 2, DIR>(a, b, tw, P.n, Ns, nlines, addr, tid, nth); break;
      case 3: fft_stage<T, 3, DIR>(a, b, tw, P.n, Ns, nlines, addr, tid, nth); break;
      case 5: fft_stage<T, 5, DIR>(a, b, tw, P.n, Ns, nlines, addr, tid, nth); break;
      default: fft_stage_generic<T, DIR>(a, b, tw, P.n, Ns, R, nlines, addr, tid, nth); break;
    }
    __syncthreads();
    cx<T>* t = a;
    a = b;
    b = t;
    Ns *= R;
  }
  return a;
}

// ---------------------------------------------------------------------------------------
// real <-> half-length complex packing (x[2m] + i x[2m+1] = z[m], N = 2h)
// ---------------------------------------------------------------------------------------
// Forward: from Z = FFT_h(z) produce X[k] and X[h-k] of the length-N real transform,
//   E = (Z[k] + conj Z[h-k]) / 2,  W O = -(i/2) W_N^k (Z[k] - conj Z[h-k]),
//   X[k] = E + W O,  X[h-k] = conj(E - W O).
template <typename T> __device__ __forceinline__ void r2c_pair(cx<T> zk, cx<T> zhk, cx<T> w, cx<T>& xk, cx<T>& xhk) {
  cx<T> b = conj(zhk);
  cx<T> e = scl(add(zk, b), T(0.5));
  cx<T> wo = cmul(mul_mi(scl(sub(zk, b), T(0.5))), w);
  xk = add(e, wo);
  xhk = conj(sub(e, wo));
}

// X[k] of r2c_pair when Z was computed from the signal scaled by 1/2: E and W O without
// their halvings.  Halving is exact, so the result is r2c_pair's bit for bit.
template <typename T> __device__ __forceinline__ cx<T> r2c_first_prescaled(cx<T> zk, cx<T> zhk, cx<T> w) {
  const cx<T> b = conj(zhk);
  return add(add(zk, b), cmul(mul_mi(sub(zk, b)), w));
}
// the same with the twiddle product and its add as two FMA chains (FP64, FP64-pipe bound):
// 8 instead of 10 operations, rounded differently within the FFT's error
template <typename T> __device__ __forceinline__ cx<T> r2c_first_prescaled_fma(cx<T> zk, cx<T> zhk, cx<T> w) {
  const cx<T> b = conj(zhk);
  const cx<T> e = add(zk, b), m = mul_mi(sub(zk, b));
  return mk<T>(fma(m.x, w.x, fma(-m.y, w.y, e.x)), fma(m.x, w.y, fma(m.y, w.x, e.y)));
}

// C2R packing of the pair (k, H-k) from X[k], X[H-k] and W = W_N^k: A = X[k] + conj X[H-k],
// D = X[k] - conj X[H-k], Z[k] = A + i D conj(W) and Z[H-k] = conj(2A - Z[k]) (= conj(A) +
// i conj(D conj(W))), the product and its add as two FMA chains: 10 instead of 12 FP64
// operations
template <typename T>
__device__ __forceinline__ void c2r_pair_fma(cx<T> xk, cx<T> xh, cx<T> w, cx<T>& zk, cx<T>& zh) {
  const cx<T> b = conj(xh);
  const cx<T> a = add(xk, b), d = sub(xk, b);
  zk = mk<T>(fma(d.x, w.y, fma(-d.y, w.x, a.x)), fma(d.x, w.x, fma(d.y, w.y, a.y)));
  zh = mk<T>(fma(T(2), a.x, -zk.x), fma(T(-2), a.y, zk.y));
}

// Inverse: 2 Z[k] = (X[k] + conj X[h-k]) + i conj(W_N^k) (X[k] - conj X[h-k]); the
// unnormalised length-h inverse of 2Z is N times the packed real signal.  At k = 0 only
// the real parts of X[0] and X[h] enter, the projection onto real signals that FFTW's
// and pocketfft's c2r make: a half spectrum whose kr = 0 column is not Hermitian (the
// asymmetric 2/3 mask keeps l = -n/3 but not +n/3) then inverts to the real part of
// the complex field it represents.
template <typename T> __device__ __forceinline__ cx<T> c2r_pre(cx<T> xk, cx<T> xhk, cx<T> w, int k) {
  if (k == 0) return mk<T>(xk.x + xhk.x, xk.x - xhk.x);
  cx<T> b = conj(xhk);
  return add(add(xk, b), mul_i(cmulc(sub(xk, b), w)));
}

}  // namespace ff
