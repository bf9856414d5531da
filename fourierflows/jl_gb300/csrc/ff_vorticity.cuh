// Fused 2D vorticity nonlinear term and time-stepper substeps (device side).
//
// One evaluation of N = -J(psi, zeta) = -(d/dx (u zeta) + d/dy (v zeta)) on the rfft
// half spectrum (nkr, ny) is three passes, each reading and writing HBM once:
//
//   A  column pass, per tile of kept kr columns and per field f in {u, v, zeta}:
//      gather zeta_hat with the 2/3 mask, form u_hat = i l zeta_hat / K^2,
//      v_hat = -i kr zeta_hat / K^2 or zeta_hat, inverse FFT along y  -> W[f]
//   B  row pass, per y row: three C2R transforms along x (half-length packing), the
//      products u zeta and v zeta in physical space, two R2C transforms  -> Q[0..1]
//   C  column pass, per tile of kr columns: forward FFTs along y of Q[0..1],
//      N_hat = -(i kr Q0 + i l Q1) with the output mask, then the stepper's substep
//      combination (the "epilogue") on the same tile.
//
// Only the kept columns kr < nkd (nkd = first aliased column) are carried through
// W and Q: the aliased modes of the input are zero after masking and those of the
// output are zeroed, so they are never transformed.  Physical-space fields never
// reach HBM.
//
// Every kernel walks a work list of (problem, tile) items over an array of problem
// descriptors, so one launch serves a single grid or an ensemble of grids of
// different sizes (grid-stride over the list: a persistent launch).
#pragma once

#include "ff_fft.cuh"
#include "ff_regfft.cuh"

// Register pass A: fields per work item, 3 (u, v, zeta of a column tile together) or 1
// (one work item per field: fewer registers, for FP64)
#ifndef FF_A_FIELDS_F32
#define FF_A_FIELDS_F32 3
#endif
#ifndef FF_A_FIELDS_F64
#define FF_A_FIELDS_F64 1
#endif
// Register path: pass C also runs the next substep's pass A (1) or pass A runs apart (0)
#ifndef FF_FUSE_A_F32
#define FF_FUSE_A_F32 1
#endif
#ifndef FF_FUSE_A_F64
#define FF_FUSE_A_F64 0
#endif

namespace ff {

template <typename T> struct AFields;
template <> struct AFields<float> { static constexpr int value = FF_A_FIELDS_F32; };
template <> struct AFields<double> { static constexpr int value = FF_A_FIELDS_F64; };
template <typename T> struct FuseA;
template <> struct FuseA<float> { static constexpr bool value = FF_FUSE_A_F32 != 0; };
template <> struct FuseA<double> { static constexpr bool value = FF_FUSE_A_F64 != 0; };

enum Epilogue {
  EPI_N = 0,      // n1 = N (the bare calcN!)
  EPI_ETD1 = 1,   // n1 = N; s1 = eh sol + zc N
  EPI_ETD2 = 2,   // n2 = N; s2 = eh sol + zc N
  EPI_ETD3 = 3,   // n3 = N; s2 = eh s1 + zc (2N - n1)
  EPI_ETD4 = 4,   // sol = [f](eL sol + al n1 + 2 be (n2 + n3) + ga N)
  EPI_RK1 = 5,    // n1 = N + L sol; s1 = sol + c n1
  EPI_RK2 = 6,    // n2 = N + L s1;  s1 = sol + c n2
  EPI_RK3 = 7,    // n3 = N + L s1;  s1 = sol + c n3
  EPI_RK4 = 8,    // sol = [f](sol + c (n1 + 2 n2 + 2 n3 + (N + L s1)))
  EPI_LS = 9,     // r = N + L sol; s1 = (first ? dt r : A s1 + dt r); sol = [f](sol + B s1)
};

template <typename T> struct VortProb {
  int nx, ny, nkr, nkd;  // nkd: kept kr columns [0, nkd)
  int la, lb;            // aliased l rows [la, lb)
  int nkp, pad0;         // row pitch of W and Q: nkd rounded up to 16 bytes
  T scale2;              // 1 / (nx ny)^2, applied to each physical product (generic path)
  LinePlan Px, Py;       // length nx/2 and ny
  const cx<T>* twx;
  const cx<T>* twy;
  const cx<T>* rtw;      // packing twiddles, nx/2 + 1
  const T* kr;           // nkr
  const T* l;            // ny
  const T* invK;         // nkr * ny, 1/K^2 with the mean mode 0
  // register path: kr (nkr) and l (ny) times the product scale scale2 / 2, a power of two
  // there, for the velocities of pass A, so that pass B's products u zeta and v zeta come
  // out scaled without a multiply of their own (bit for bit the products scaled after)
  const T* krs;
  const T* ls;
  cx<T>* W;              // 3 * nkp * ny
  cx<T>* Q;              // 2 * nkp * ny
  // stepper state (nkr * ny each)
  cx<T>* sol;
  cx<T>* s1;
  cx<T>* s2;
  cx<T>* n1;
  cx<T>* n2;
  cx<T>* n3;
  const T* L;   // linear operator (RK4 / LSRK54)
  const T* eL;  // ETDRK4: exp(L dt), exp(L dt / 2), zeta, alpha, beta, Gamma
  const T* eh;
  const T* zc;
  const T* al;
  const T* be;
  const T* ga;
  const T* filter;
  unsigned* cnt;  // pass C split by field: an arrival counter per kept column tile
};

struct WorkItem {
  int prob, tile, field, pad;
};

// per-launch scalars of the epilogue
template <typename T> struct EpiScalars {
  T c;      // dt/2, dt, dt/6 (RK); A (LS)
  T b;      // B (LS)
  T dt;     // dt (LS)
  int first;
  int use_filter;
};

// ---------------------------------------------------------------------------------------
// pass A
// ---------------------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(512) k_vort_a(const VortProb<T>* __restrict__ probs,
                                                const WorkItem* __restrict__ work, int nwork, int tl,
                                                const cx<T>* const* __restrict__ inputs) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  for (int w = blockIdx.x; w < nwork; w += gridDim.x) {
    const WorkItem it = work[w];
    const VortProb<T>& P = probs[it.prob];
    const cx<T>* zh = inputs[it.prob];
    const int ny = P.ny, nkr = P.nkr, nkd = P.nkd, la = P.la, lb = P.lb, f = it.field;
    const AddrTile ad{tl};
    cx<T>* A = reinterpret_cast<cx<T>*>(smem_raw);
    cx<T>* B = A + tl * ny;
    const int c0 = it.tile * tl;
    for (int idx = threadIdx.x; idx < tl * ny; idx += blockDim.x) {
      const int ln = idx % tl, j = idx / tl, c = c0 + ln;
      cx<T> v = czero<T>();
      if (c < nkd && (j < la || j >= lb)) {
        const int64_t e = (int64_t)c + (int64_t)j * nkr;
        const cx<T> z = zh[e];
        if (f == 0) v = mul_i(scl(z, P.l[j] * P.invK[e]));
        else if (f == 1) v = mul_mi(scl(z, P.kr[c] * P.invK[e]));
        else v = z;
      }
      A[ad(ln, j)] = v;
    }
    __syncthreads();
    const cx<T>* R = fft_lines<T, 1>(A, B, P.twy, P.Py, tl, ad);
    cx<T>* Wf = P.W + (int64_t)f * P.nkp * ny;
    for (int idx = threadIdx.x; idx < tl * ny; idx += blockDim.x) {
      const int ln = idx % tl, j = idx / tl, c = c0 + ln;
      if (c < nkd) Wf[c + (int64_t)j * P.nkp] = R[ad(ln, j)];
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------------------
// pass B
// ---------------------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(512) k_vort_b(const VortProb<T>* __restrict__ probs,
                                                const WorkItem* __restrict__ work, int nwork, int tlr) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  for (int w = blockIdx.x; w < nwork; w += gridDim.x) {
    const WorkItem it = work[w];
    const VortProb<T>& P = probs[it.prob];
    const int nx = P.nx, ny = P.ny, nkd = P.nkd, h = nx / 2;
    const AddrRows ad{rows_stride(h, sizeof(cx<T>)), rows_pad_shift(sizeof(cx<T>))};
    const int bufsz = tlr * ad.stride;
    cx<T>* b0 = reinterpret_cast<cx<T>*>(smem_raw);
    cx<T>* b[4] = {b0, b0 + bufsz, b0 + 2 * bufsz, b0 + 3 * bufsz};
    const int row0 = it.tile * tlr;
    const int64_t fstride = (int64_t)P.nkp * ny;
    // gather the three y-transformed fields and pack them for the C2R transforms
    for (int idx = threadIdx.x; idx < 3 * tlr * h; idx += blockDim.x) {
      const int f = idx / (tlr * h);
      const int r = idx - f * tlr * h;
      const int ln = r / h, k = r - ln * h;
      const int j = row0 + ln;
      cx<T> v = czero<T>();
      if (j < ny) {
        const cx<T>* src = P.W + f * fstride + (int64_t)j * P.nkp;
        const cx<T> xk = k < nkd ? src[k] : czero<T>();
        const cx<T> xh = (h - k) < nkd ? src[h - k] : czero<T>();
        v = c2r_pre<T>(xk, xh, __ldg(&P.rtw[k]), k);
      }
      b[f][ad(ln, k)] = v;
    }
    __syncthreads();
    cx<T>* spare = b[3];
    cx<T>* r[3];
    for (int f = 0; f < 3; ++f) {
      r[f] = fft_lines<T, 1>(b[f], spare, P.twx, P.Px, tlr, ad);
      if (r[f] == spare) spare = b[f];
    }
    // products in physical space (packed real pairs), normalisation folded in
    const T s2 = P.scale2;
    for (int idx = threadIdx.x; idx < tlr * h; idx += blockDim.x) {
      const int ln = idx / h, m = idx - ln * h;
      const int a = ad(ln, m);
      const cx<T> u = r[0][a], v = r[1][a], z = r[2][a];
      r[0][a] = mk<T>(u.x * z.x * s2, u.y * z.y * s2);
      r[1][a] = mk<T>(v.x * z.x * s2, v.y * z.y * s2);
    }
    __syncthreads();
    const cx<T>* q0 = fft_lines<T, -1>(r[0], spare, P.twx, P.Px, tlr, ad);
    const cx<T>* q1 = fft_lines<T, -1>(r[1], r[2], P.twx, P.Px, tlr, ad);
    // unpack the kept columns of the two real transforms
    for (int idx = threadIdx.x; idx < tlr * nkd; idx += blockDim.x) {
      const int ln = idx / nkd, k = idx - ln * nkd;
      const int j = row0 + ln;
      if (j >= ny) continue;
      cx<T> x0, x1;
      if (k == 0 || k == h) {
        const cx<T> z0 = q0[ad(ln, 0)], z1 = q1[ad(ln, 0)];
        x0 = k == 0 ? mk<T>(z0.x + z0.y, T(0)) : mk<T>(z0.x - z0.y, T(0));
        x1 = k == 0 ? mk<T>(z1.x + z1.y, T(0)) : mk<T>(z1.x - z1.y, T(0));
      } else {
        const cx<T> w = __ldg(&P.rtw[k]);
        cx<T> dummy;
        r2c_pair<T>(q0[ad(ln, k)], q0[ad(ln, h - k)], w, x0, dummy);
        r2c_pair<T>(q1[ad(ln, k)], q1[ad(ln, h - k)], w, x1, dummy);
      }
      P.Q[(int64_t)j * P.nkp + k] = x0;
      P.Q[fstride + (int64_t)j * P.nkp + k] = x1;
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------------------
// pass C
// ---------------------------------------------------------------------------------------
template <typename T> __device__ __forceinline__ cx<T> rmul(const T* c, int64_t e, cx<T> v) { return scl(v, c[e]); }

template <typename T, int EPI>
__device__ __forceinline__ void epilogue(const VortProb<T>& P, const EpiScalars<T>& S, int64_t e, cx<T> N) {
  if (EPI == EPI_N) {
    P.n1[e] = N;
  } else if (EPI == EPI_ETD1) {
    P.n1[e] = N;
    P.s1[e] = add(rmul(P.eh, e, P.sol[e]), rmul(P.zc, e, N));
  } else if (EPI == EPI_ETD2) {
    P.n2[e] = N;
    P.s2[e] = add(rmul(P.eh, e, P.sol[e]), rmul(P.zc, e, N));
  } else if (EPI == EPI_ETD3) {
    P.n3[e] = N;
    P.s2[e] = add(rmul(P.eh, e, P.s1[e]), rmul(P.zc, e, sub(scl(N, T(2)), P.n1[e])));
  } else if (EPI == EPI_ETD4) {
    cx<T> v = add(rmul(P.eL, e, P.sol[e]), rmul(P.al, e, P.n1[e]));
    v = add(v, scl(rmul(P.be, e, add(P.n2[e], P.n3[e])), T(2)));
    v = add(v, rmul(P.ga, e, N));
    if (S.use_filter) v = scl(v, P.filter[e]);
    P.sol[e] = v;
  } else if (EPI == EPI_RK1) {
    const cx<T> s = P.sol[e];
    const cx<T> r = add(N, rmul(P.L, e, s));
    P.n1[e] = r;
    P.s1[e] = add(s, scl(r, S.c));
  } else if (EPI == EPI_RK2 || EPI == EPI_RK3) {
    const cx<T> r = add(N, rmul(P.L, e, P.s1[e]));
    if (EPI == EPI_RK2) P.n2[e] = r;
    else P.n3[e] = r;
    P.s1[e] = add(P.sol[e], scl(r, S.c));
  } else if (EPI == EPI_RK4) {
    const cx<T> r4 = add(N, rmul(P.L, e, P.s1[e]));
    const cx<T> acc = add(add(add(P.n1[e], scl(P.n2[e], T(2))), scl(P.n3[e], T(2))), r4);
    cx<T> v = add(P.sol[e], scl(acc, S.c));
    if (S.use_filter) v = scl(v, P.filter[e]);
    P.sol[e] = v;
  } else if (EPI == EPI_LS) {
    const cx<T> s = P.sol[e];
    const cx<T> r = add(N, rmul(P.L, e, s));
    const cx<T> q = S.first ? scl(r, S.dt) : add(scl(P.s1[e], S.c), scl(r, S.dt));
    P.s1[e] = q;
    cx<T> v = add(s, scl(q, S.b));
    if (S.use_filter) v = scl(v, P.filter[e]);
    P.sol[e] = v;
  }
}

// The epilogue split into its loads and its arithmetic, so that a thread can issue the
// loads of several elements before the first store: the output arrays may alias the
// inputs as far as the compiler knows, so element by element every load would wait for
// the previous element's stores (one memory round trip per element).
template <typename T> struct EpiIn {
  cx<T> x, n1, n2, n3;     // sol or s1, and the stored nonlinear terms
  T a, b, c, d, fl;        // coefficients (by epilogue) and the filter
};

// live: false on the aliased l rows of kept columns under ETDRK4, where N is zero and the
// intermediates are never read: only what the last substep's expL sol [f] needs is loaded.
// FUSED (ETDRK4 with pass C running the next substep's pass A): the intermediate states
// go to the next pass A in registers, so sol1 and sol2 are never stored; substep 3 rebuilds
// sol1 = e_half sol + zeta n1 from sol and n1, the same operands substep 1 combined.
template <typename T, int EPI, bool FUSED = false>
__device__ __forceinline__ EpiIn<T> epi_load(const VortProb<T>& P, const EpiScalars<T>& S, int64_t e,
                                             bool live = true) {
  EpiIn<T> in;
  in.x = in.n1 = in.n2 = in.n3 = czero<T>();
  in.a = in.b = in.c = in.d = in.fl = T(0);
  if (!live && EPI >= EPI_ETD1 && EPI <= EPI_RK4) {
    if (EPI == EPI_ETD4 || EPI == EPI_RK4) {
      in.x = P.sol[e];
      in.a = EPI == EPI_ETD4 ? P.eL[e] : P.L[e];
      if (S.use_filter) in.fl = P.filter[e];
    }
    return in;
  }
  // ETDRK4 substeps 1-3 only read these arrays (read-only loads, which may move ahead of
  // the shared-memory traffic of the transforms)
  if (EPI == EPI_ETD1 || EPI == EPI_ETD2) {
    in.x = __ldg(P.sol + e);
    in.a = __ldg(P.eh + e);
    in.b = __ldg(P.zc + e);
  } else if (EPI == EPI_ETD3) {
    in.x = FUSED ? __ldg(P.sol + e) : __ldg(P.s1 + e);
    in.n1 = __ldg(P.n1 + e);
    in.a = __ldg(P.eh + e);
    in.b = __ldg(P.zc + e);
  } else if (EPI == EPI_ETD4) {
    // sol is rewritten by this pass; N1..N3 and the coefficients are only read
    in.x = P.sol[e];
    in.n1 = __ldg(P.n1 + e);
    in.n2 = __ldg(P.n2 + e);
    in.n3 = __ldg(P.n3 + e);
    in.a = __ldg(P.eL + e);
    in.b = __ldg(P.al + e);
    in.c = __ldg(P.be + e);
    in.d = __ldg(P.ga + e);
  } else if (EPI == EPI_RK1 || EPI == EPI_LS) {
    // RK1 writes only N1 and the stage state; an LSRK54 stage rewrites sol and S2
    in.x = EPI == EPI_RK1 ? __ldg(P.sol + e) : P.sol[e];
    in.a = __ldg(P.L + e);
    if (EPI == EPI_LS && !S.first) in.n1 = P.s1[e];
  } else if (EPI == EPI_RK2 || EPI == EPI_RK3) {
    in.x = P.s1[e];  // rewritten by this pass
    in.n1 = __ldg(P.sol + e);
    in.a = __ldg(P.L + e);
  } else if (EPI == EPI_RK4) {
    // sol is rewritten by this pass; the stage state, N1..N3 and L are only read
    in.x = __ldg(P.s1 + e);
    in.n1 = __ldg(P.n1 + e);
    in.n2 = __ldg(P.n2 + e);
    in.n3 = __ldg(P.n3 + e);
    in.a = __ldg(P.L + e);
  }
  if ((EPI == EPI_ETD4 || EPI == EPI_RK4 || EPI == EPI_LS) && S.use_filter) in.fl = __ldg(P.filter + e);
  return in;
}

// the same arithmetic, in the same order, as epilogue<T, EPI>; returns the value stored
// to the array the next substep transforms (s1, s2 or sol; zero for the last substeps)
template <typename T, int EPI, bool FUSED = false>
__device__ __forceinline__ cx<T> epi_store(const VortProb<T>& P, const EpiScalars<T>& S, int64_t e, cx<T> N,
                                           const EpiIn<T>& in, bool live = true) {
  cx<T> next = czero<T>();
  if (!live) {
    if ((EPI >= EPI_ETD1 && EPI <= EPI_ETD3) || (EPI >= EPI_RK1 && EPI <= EPI_RK3)) return next;  // never read
    if (EPI == EPI_RK4) {
      // the four RK4 stages of a mode with N = 0, in the order the substeps take them
      const T half = S.dt / T(2);
      const cx<T> n1 = scl(in.x, in.a);
      cx<T> s1 = add(in.x, scl(n1, half));
      const cx<T> n2 = scl(s1, in.a);
      s1 = add(in.x, scl(n2, half));
      const cx<T> n3 = scl(s1, in.a);
      s1 = add(in.x, scl(n3, S.dt));
      const cx<T> r4 = scl(s1, in.a);
      const cx<T> acc = add(add(add(n1, scl(n2, T(2))), scl(n3, T(2))), r4);
      cx<T> v = add(in.x, scl(acc, S.c));
      if (S.use_filter) v = scl(v, in.fl);
      P.sol[e] = v;
      return next;
    }
  }
  if (EPI == EPI_N) {
    P.n1[e] = N;
  } else if (EPI == EPI_ETD1 || EPI == EPI_ETD2) {
    (EPI == EPI_ETD1 ? P.n1 : P.n2)[e] = N;
    next = add(scl(in.x, in.a), scl(N, in.b));
    if (!FUSED) (EPI == EPI_ETD1 ? P.s1 : P.s2)[e] = next;
  } else if (EPI == EPI_ETD3) {
    P.n3[e] = N;
    const cx<T> x1 = FUSED ? add(scl(in.x, in.a), scl(in.n1, in.b)) : in.x;  // sol1
    next = add(scl(x1, in.a), scl(sub(scl(N, T(2)), in.n1), in.b));
    if (!FUSED) P.s2[e] = next;
  } else if (EPI == EPI_ETD4) {
    cx<T> v = add(scl(in.x, in.a), scl(in.n1, in.b));
    v = add(v, scl(scl(add(in.n2, in.n3), in.c), T(2)));
    v = add(v, scl(N, in.d));
    if (S.use_filter) v = scl(v, in.fl);
    P.sol[e] = v;
  } else if (EPI == EPI_RK1) {
    const cx<T> r = add(N, scl(in.x, in.a));
    P.n1[e] = r;
    next = add(in.x, scl(r, S.c));
    P.s1[e] = next;
  } else if (EPI == EPI_RK2 || EPI == EPI_RK3) {
    const cx<T> r = add(N, scl(in.x, in.a));
    (EPI == EPI_RK2 ? P.n2 : P.n3)[e] = r;
    next = add(in.n1, scl(r, S.c));
    P.s1[e] = next;
  } else if (EPI == EPI_RK4) {
    const cx<T> r4 = add(N, scl(in.x, in.a));
    const cx<T> acc = add(add(add(in.n1, scl(in.n2, T(2))), scl(in.n3, T(2))), r4);
    cx<T> v = add(P.sol[e], scl(acc, S.c));
    if (S.use_filter) v = scl(v, in.fl);
    P.sol[e] = v;
  } else if (EPI == EPI_LS) {
    const cx<T> r = add(N, scl(in.x, in.a));
    const cx<T> q = S.first ? scl(r, S.dt) : add(scl(in.n1, S.c), scl(r, S.dt));
    P.s1[e] = q;
    cx<T> v = add(in.x, scl(q, S.b));
    if (S.use_filter) v = scl(v, in.fl);
    P.sol[e] = v;
    next = v;
  }
  return next;
}

// elements per batch of loads: fewer for the epilogues with many input arrays and in FP64
template <typename T, int EPI> struct EpiBatch {
  static constexpr int value =
      EPI == EPI_LS ? 1 : ((EPI == EPI_ETD4 || EPI == EPI_RK4) ? 4 : 8) / (sizeof(T) == 8 ? 2 : 1);
};

template <typename T, int EPI>
__global__ void __launch_bounds__(512) k_vort_c(const VortProb<T>* __restrict__ probs,
                                                const WorkItem* __restrict__ work, int nwork, int tl,
                                                EpiScalars<T> S) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  for (int w = blockIdx.x; w < nwork; w += gridDim.x) {
    const WorkItem it = work[w];
    const VortProb<T>& P = probs[it.prob];
    const int ny = P.ny, nkr = P.nkr, nkd = P.nkd, la = P.la, lb = P.lb;
    const int c0 = it.tile * tl;
    if (c0 < nkd) {
      // two fields as 2*tl interleaved lines: line ln = field * tl + column
      const int nl = 2 * tl;
      const AddrTile ad{nl};
      cx<T>* A = reinterpret_cast<cx<T>*>(smem_raw);
      cx<T>* B = A + nl * ny;
      const int64_t fstride = (int64_t)P.nkp * ny;
      for (int idx = threadIdx.x; idx < nl * ny; idx += blockDim.x) {
        const int ln = idx % nl, j = idx / nl;
        const int f = ln / tl, c = c0 + (ln - f * tl);
        A[ad(ln, j)] = c < nkd ? P.Q[f * fstride + c + (int64_t)j * P.nkp] : czero<T>();
      }
      __syncthreads();
      const cx<T>* R = fft_lines<T, -1>(A, B, P.twy, P.Py, nl, ad);
      for (int idx = threadIdx.x; idx < tl * ny; idx += blockDim.x) {
        const int ln = idx % tl, j = idx / tl, c = c0 + ln;
        if (c >= nkr) continue;
        cx<T> N = czero<T>();
        if (c < nkd && (j < la || j >= lb)) {
          const cx<T> qa = R[ad(ln, j)], qb = R[ad(ln + tl, j)];
          // N = -(i kr qa + i l qb)
          N = mul_mi(add(scl(qa, P.kr[c]), scl(qb, P.l[j])));
        }
        epilogue<T, EPI>(P, S, (int64_t)c + (int64_t)j * nkr, N);
      }
      __syncthreads();
    } else {
      // aliased columns: N = 0, only the linear part of the substep
      for (int idx = threadIdx.x; idx < tl * ny; idx += blockDim.x) {
        const int ln = idx % tl, j = idx / tl, c = c0 + ln;
        if (c < nkr) epilogue<T, EPI>(P, S, (int64_t)c + (int64_t)j * nkr, czero<T>());
      }
    }
  }
}

// =======================================================================================
// register-resident passes for power-of-two lengths (ff_regfft.cuh)
// =======================================================================================
// A CTA of nt threads (a power of two) holds nt*8 elements: tl = nt*8/N lines of length
// N.  Columns map thread -> (t, ln) with the line fastest, so every load and store of a
// warp touches tl consecutive columns of (32/tl) rows; rows map thread -> (ln, t).
// Loads go straight from HBM to registers and results straight back; shared memory
// holds only the exchanges between stages.

// All three fields of a column tile in one work item: zeta_hat, 1/K^2 and l are read
// once, and the three inverse transforms share twiddles, exchanges and barriers.
template <typename T, int NY>
__device__ __forceinline__ void vort_a_reg3(const VortProb<T>& P, const cx<T>* __restrict__ zh, int tile,
                                            cx<T>* smem) {
  constexpr int PP = NY / 8;
  const int tl = blockDim.x / PP;
  const int ln = threadIdx.x & (tl - 1), t = threadIdx.x / tl;
  const int c = tile * tl + ln;
  const int nkr = P.nkr, nkd = P.nkd, la = P.la, lb = P.lb;
  const T kc = c < nkd ? P.krs[c] : T(0);
  cx<T> v[3][8];
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    const int j = t + q * PP;
    cx<T> s = czero<T>();
    T ik = T(0), lj = T(0);
    if (c < nkd && (j < la || j >= lb)) {
      const int e = c + j * nkr;
      s = zh[e];
      ik = P.invK[e];
      lj = P.ls[j];
    }
    v[0][q] = mul_i(scl(s, lj * ik));   // u_hat = i l zeta_hat / K^2 (scaled)
    v[1][q] = mul_mi(scl(s, kc * ik));  // v_hat = -i kr zeta_hat / K^2 (scaled)
    v[2][q] = s;
  }
  const int bsz = (NY + NY / 8) * tl;
  cx<T>* const buf[3] = {smem, smem + bsz, smem + 2 * bsz};
  regfft<T, 3, NY, 1>(v, t, P.twy, buf, XCol{tl, ln});
  if (c < nkd) {
    const int fs = P.nkp * P.ny;
    cx<T>* Wc = P.W + c;
#pragma unroll
    for (int f = 0; f < 3; ++f)
#pragma unroll
      for (int q = 0; q < 8; ++q) Wc[f * fs + (t + q * PP) * P.nkp] = v[f][q];
  }
}

template <typename T, int NY>
__device__ __forceinline__ void vort_a_reg(const VortProb<T>& P, const cx<T>* __restrict__ zh, int tile, int f,
                                           cx<T>* smem) {
  constexpr int PP = NY / 8;
  const int tl = blockDim.x / PP;
  const int ln = threadIdx.x & (tl - 1), t = threadIdx.x / tl;
  const int c = tile * tl + ln;
  const int nkr = P.nkr, nkd = P.nkd, la = P.la, lb = P.lb;
  cx<T> v[1][8];
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    const int j = t + q * PP;
    cx<T> z = czero<T>();
    if (c < nkd && (j < la || j >= lb)) {
      const int e = c + j * nkr;
      const cx<T> s = zh[e];
      if (f == 0) z = mul_i(scl(s, P.ls[j] * P.invK[e]));
      else if (f == 1) z = mul_mi(scl(s, P.krs[c] * P.invK[e]));
      else z = s;
    }
    v[0][q] = z;
  }
  cx<T>* const buf[1] = {smem};
  regfft<T, 1, NY, 1>(v, t, P.twy, buf, XCol{tl, ln});
  if (c < nkd) {
    cx<T>* Wf = P.W + f * P.nkp * P.ny + c;
#pragma unroll
    for (int q = 0; q < 8; ++q) Wf[(t + q * PP) * P.nkp] = v[0][q];
  }
}

// Loads go straight from W (an L2 prefetch one item ahead, see k_vort_b_r) into
// registers; shared memory holds only the exchanges.
template <typename T, int H>
__device__ __forceinline__ void vort_b_reg(const VortProb<T>& P, int tile, cx<T>* smem) {
  constexpr int PP = H / 8;
  constexpr int SH = sizeof(T) == 8 ? 3 : 4;
  constexpr int STRIDE = H + (H >> SH) + 1;
  const int rows = blockDim.x / PP;
  const int ln = threadIdx.x / PP, t = threadIdx.x & (PP - 1);
  const int j = tile * rows + ln;
  const int ny = P.ny, nkd = P.nkd, nkp = P.nkp;
  const int fstride = nkp * ny;
  const int bufsz = rows * STRIDE;
  cx<T>* const buf3[3] = {smem, smem + bufsz, smem + 2 * bufsz};
  const XRow xr{ln * STRIDE, SH};
  // C2R packing by pairs: for k = t + q PP, q < 4, A = X[k] + conj X[H-k] and
  // P = (X[k] - conj X[H-k]) conj(W^k) give both Z[k] = A + i P (this thread's slot q) and
  // Z[H-k] = conj(A) + i conj(P) (slot 7-q of thread PP-t), since X[H-k] + conj X[k] =
  // conj(A) and W^(H-k) = -conj(W^k).  Partner values go through shared memory; Z[0] and
  // the self-paired Z[H/2] are formed directly.
  cx<T> v[3][8];
  if constexpr (sizeof(T) == 4) {
    // FP32: every load of the row first, then the packing.  (Loads placed after the
    // shared-memory stores of the previous field wait behind them: one memory round trip
    // per field and pair, and this latency-bound pass took 19% longer.)
    cx<T> xa[3][4], xb[3][4], wk[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) wk[q] = __ldg(&P.rtw[t + q * PP]);
#pragma unroll
    for (int f = 0; f < 3; ++f) {
      const cx<T>* src = P.W + f * fstride + j * nkp;
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int k = t + q * PP;
        xa[f][q] = (j < ny && k < nkd) ? src[k] : czero<T>();
        xb[f][q] = (j < ny && (H - k) < nkd) ? src[H - k] : czero<T>();
      }
    }
#pragma unroll
    for (int f = 0; f < 3; ++f) {
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int k = t + q * PP;
        cx<T> zk = czero<T>(), zh = czero<T>();
        if (j < ny) {
          const cx<T> xk = xa[f][q], xh = xb[f][q];
          if (k == 0) {
            zk = c2r_pre<T>(xk, xh, wk[0], 0);
          } else {
            const cx<T> b = conj(xh);
            const cx<T> a = add(xk, b);
            const cx<T> pp = cmulc(sub(xk, b), wk[q]);
            zk = add(a, mul_i(pp));
            zh = mk<T>(a.x + pp.y, pp.x - a.y);
          }
        }
        v[f][q] = zk;
        if (k != 0) buf3[f][xr(H - k)] = zh;
      }
      if (t == 0) {
        const cx<T> xm = (j < ny && H / 2 < nkd) ? P.W[f * fstride + j * nkp + H / 2] : czero<T>();
        buf3[f][xr(H / 2)] = j < ny ? c2r_pre<T>(xm, xm, __ldg(&P.rtw[H / 2]), H / 2) : czero<T>();
      }
    }
  } else {
    // FP64: too few registers to hold the row; read-only global loads (W is not written
    // during this pass), which the compiler may move ahead of the shared-memory stores
#pragma unroll
    for (int f = 0; f < 3; ++f) {
      const cx<T>* src = P.W + f * fstride + j * nkp;
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int k = t + q * PP;
        cx<T> zk = czero<T>(), zh = czero<T>();
        if (j < ny) {
          const cx<T> xk = k < nkd ? __ldg(src + k) : czero<T>();
          const cx<T> xh = (H - k) < nkd ? __ldg(src + H - k) : czero<T>();
          if (k == 0) {
            zk = c2r_pre<T>(xk, xh, __ldg(&P.rtw[0]), 0);
          } else if constexpr (FF_TWIDDLE_FMA) {
            c2r_pair_fma<T>(xk, xh, __ldg(&P.rtw[k]), zk, zh);
          } else {
            const cx<T> b = conj(xh);
            const cx<T> a = add(xk, b);
            const cx<T> pp = cmulc(sub(xk, b), __ldg(&P.rtw[k]));
            zk = add(a, mul_i(pp));
            zh = mk<T>(a.x + pp.y, pp.x - a.y);
          }
        }
        v[f][q] = zk;
        if (k != 0) buf3[f][xr(H - k)] = zh;
      }
      if (t == 0) {
        const cx<T> xm = (j < ny && H / 2 < nkd) ? __ldg(src + H / 2) : czero<T>();
        buf3[f][xr(H / 2)] = j < ny ? c2r_pre<T>(xm, xm, __ldg(&P.rtw[H / 2]), H / 2) : czero<T>();
      }
    }
  }
  __syncthreads();
#pragma unroll
  for (int f = 0; f < 3; ++f)
#pragma unroll
    for (int q = 4; q < 8; ++q) v[f][q] = buf3[f][xr(t + q * PP)];
  __syncthreads();
  regfft<T, 3, H, 1>(v, t, P.twx, buf3, xr);
  // products u zeta and v zeta in physical space (packed real pairs).  u and v arrive
  // scaled by scale2 / 2 (pass A's krs and ls): the normalisation and the unpack's two
  // halvings, a power of two, so the products are those scaled afterwards bit for bit
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    const cx<T> z = v[2][q];
    v[0][q] = mk<T>(v[0][q].x * z.x, v[0][q].y * z.y);
    v[1][q] = mk<T>(v[1][q].x * z.x, v[1][q].y * z.y);
  }
  cx<T>(&p)[2][8] = *reinterpret_cast<cx<T>(*)[2][8]>(&v[0][0]);
  regfft<T, 2, H, -1>(p, t, P.twx, buf3, xr);
  // unpack X[k] = E + W O needs Z[H - k], held by another thread: one more exchange
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    buf3[0][xr(t + q * PP)] = p[0][q];
    buf3[1][xr(t + q * PP)] = p[1][q];
  }
  __syncthreads();
  if constexpr (sizeof(T) == 4) {
    // FP32: every unpacked value first, then the stores (a load placed after a store to Q
    // would wait behind it)
    if (j < ny) {
      cx<T>* q0 = P.Q + j * P.nkp;
      cx<T>* q1 = q0 + fstride;
      cx<T> x0[8], x1[8];
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const int k = t + q * PP;
        if (k == 0) {
          const cx<T> z0 = p[0][0], z1 = p[1][0];
          x0[q] = mk<T>((z0.x + z0.y) * T(2), T(0));
          x1[q] = mk<T>((z1.x + z1.y) * T(2), T(0));
        } else {
          const cx<T> w = __ldg(&P.rtw[k < nkd ? k : 0]);
          x0[q] = r2c_first_prescaled<T>(p[0][q], buf3[0][xr(H - k)], w);
          x1[q] = r2c_first_prescaled<T>(p[1][q], buf3[1][xr(H - k)], w);
        }
      }
      if (t == 0 && nkd > H) {  // no dealiasing: the Nyquist column too
        const cx<T> z0 = p[0][0], z1 = p[1][0];
        q0[H] = mk<T>((z0.x - z0.y) * T(2), T(0));
        q1[H] = mk<T>((z1.x - z1.y) * T(2), T(0));
      }
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const int k = t + q * PP;
        if (k < nkd) {
          q0[k] = x0[q];
          q1[k] = x1[q];
        }
      }
    }
    __syncthreads();
    return;
  }
  if (j < ny) {
    cx<T>* q0 = P.Q + j * P.nkp;
    cx<T>* q1 = q0 + fstride;
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const int k = t + q * PP;
      if (k >= nkd) continue;
      cx<T> x0, x1;
      if (k == 0) {  // Z is half the packed transform here: double X[0] (and X[H]) back
        const cx<T> z0 = p[0][0], z1 = p[1][0];
        x0 = mk<T>((z0.x + z0.y) * T(2), T(0));
        x1 = mk<T>((z1.x + z1.y) * T(2), T(0));
        if (nkd > H) {  // no dealiasing: the Nyquist column too
          q0[H] = mk<T>((z0.x - z0.y) * T(2), T(0));
          q1[H] = mk<T>((z1.x - z1.y) * T(2), T(0));
        }
      } else {
        const cx<T> w = __ldg(&P.rtw[k]);
        if constexpr (sizeof(T) == 8 && FF_TWIDDLE_FMA) {
          x0 = r2c_first_prescaled_fma<T>(p[0][q], buf3[0][xr(H - k)], w);
          x1 = r2c_first_prescaled_fma<T>(p[1][q], buf3[1][xr(H - k)], w);
        } else {
          x0 = r2c_first_prescaled<T>(p[0][q], buf3[0][xr(H - k)], w);
          x1 = r2c_first_prescaled<T>(p[1][q], buf3[1][xr(H - k)], w);
        }
      }
      // global-space stores: the shared-memory loads of the next pair need not wait
      __stcg(q0 + k, x0);
      __stcg(q1 + k, x1);
    }
  }
  __syncthreads();
}

// epilogue of thread t's eight elements (rows t + q NY/8) of column c: the loads of a
// batch of elements first, then their arithmetic and stores
// Under ETDRK4 and RK4 the aliased modes (c >= nkd or an aliased l row) are "dead": N is
// zero there, the substeps' intermediates are never read there, and the last substep
// advances them by the linear part alone.
template <typename T, int NY, int EPI, bool FUSED = false>
__device__ __forceinline__ void epilogue_col(const VortProb<T>& P, const EpiScalars<T>& S, int c, int t,
                                             const cx<T> (&N)[8], cx<T> (&next)[8]) {
  const bool col_live = c < P.nkd;
  constexpr int PP = NY / 8, QB = EpiBatch<T, EPI>::value;
#pragma unroll
  for (int q0 = 0; q0 < 8; q0 += QB) {
    EpiIn<T> in[QB];
#pragma unroll
    for (int b = 0; b < QB; ++b) {
      const int j = t + (q0 + b) * PP;
      in[b] = epi_load<T, EPI, FUSED>(P, S, c + (int64_t)j * P.nkr, col_live && (j < P.la || j >= P.lb));
    }
#pragma unroll
    for (int b = 0; b < QB; ++b) {
      const int j = t + (q0 + b) * PP;
      next[q0 + b] = epi_store<T, EPI, FUSED>(P, S, c + (int64_t)j * P.nkr, N[q0 + b], in[b],
                                       col_live && (j < P.la || j >= P.lb));
    }
  }
}

// Pass A of the next substep on values a thread already holds: x[q] is the next
// substep's input at row t + q NY/8 of column c (the epilogue's output), so the fused
// column pass skips reading it back.  Must be called by the whole CTA.
template <typename T, int NY>
__device__ __forceinline__ void a_from_regs(const VortProb<T>& P, int c, int t, int tl, int ln, const cx<T> (&x)[8],
                                            cx<T>* smem) {
  constexpr int PP = NY / 8;
  const int nkr = P.nkr, nkd = P.nkd, la = P.la, lb = P.lb;
  const T kc = c < nkd ? P.krs[c] : T(0);
  const int bsz = (NY + NY / 8) * tl;
  const int fs = P.nkp * P.ny;
  cx<T>* Wc = P.W + c;
  if (AFields<T>::value == 3) {
    cx<T> v[3][8];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const int j = t + q * PP;
      cx<T> z = czero<T>();
      T ik = T(0), lj = T(0);
      if (c < nkd && (j < la || j >= lb)) {
        z = x[q];
        ik = __ldg(P.invK + c + j * nkr);
        lj = __ldg(P.ls + j);
      }
      v[0][q] = mul_i(scl(z, lj * ik));
      v[1][q] = mul_mi(scl(z, kc * ik));
      v[2][q] = z;
    }
    cx<T>* const buf[3] = {smem, smem + bsz, smem + 2 * bsz};
    regfft<T, 3, NY, 1>(v, t, P.twy, buf, XCol{tl, ln});
    if (c < nkd) {
#pragma unroll
      for (int f = 0; f < 3; ++f)
#pragma unroll
        for (int q = 0; q < 8; ++q) Wc[f * fs + (t + q * PP) * P.nkp] = v[f][q];
    }
  } else {
#pragma unroll 1
    for (int f = 0; f < 3; ++f) {
      cx<T> v[1][8];
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const int j = t + q * PP;
        cx<T> z = czero<T>();
        if (c < nkd && (j < la || j >= lb)) {
          const T ik = P.invK[c + j * nkr];
          z = f == 0 ? mul_i(scl(x[q], P.ls[j] * ik)) : f == 1 ? mul_mi(scl(x[q], kc * ik)) : x[q];
        }
        v[0][q] = z;
      }
      cx<T>* const buf[1] = {smem};
      regfft<T, 1, NY, 1>(v, t, P.twy, buf, XCol{tl, ln});
      if (c < nkd) {
#pragma unroll
        for (int q = 0; q < 8; ++q) Wc[f * fs + (t + q * PP) * P.nkp] = v[0][q];
      }
    }
  }
}

// Pass C split by field: work item (tile, f) transforms field f of the tile's kept
// columns.  The first of the two items to finish leaves its transform F_f in its Q
// columns; the second (an atomic arrival count per tile tells them apart, and resets it)
// forms N = -i (kr F_0 + l F_1) from its own transform and the other's, by one formula
// whichever field came second, and runs the epilogue.  Nothing waits: twice as many items
// as column tiles balance a grid that has only a few kept columns per SM.
template <typename T, int NY, int EPI>
__device__ __forceinline__ void vort_c_split(const VortProb<T>& P, const EpiScalars<T>& S, int tile, int f,
                                             cx<T>* smem) {
  constexpr int PP = NY / 8;
  const int tl = blockDim.x / PP;
  const int ln = threadIdx.x & (tl - 1), t = threadIdx.x / tl;
  const int c = tile * tl + ln;
  const int nkd = P.nkd, la = P.la, lb = P.lb;
  const int fstride = P.nkp * P.ny;
  __shared__ unsigned s_arrived;
  cx<T> v[1][8];
  cx<T>* const mine = P.Q + f * fstride + c;
  // L2 loads: the columns are rewritten below and read back by the other item
#pragma unroll
  for (int q = 0; q < 8; ++q) v[0][q] = c < nkd ? __ldcg(mine + (t + q * PP) * P.nkp) : czero<T>();
  cx<T>* const buf[1] = {smem};
  regfft<T, 1, NY, -1>(v, t, P.twy, buf, XCol{tl, ln});
  if (c < nkd) {
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const int j = t + q * PP;
      if (j < la || j >= lb) __stcg(mine + j * P.nkp, v[0][q]);
    }
  }
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) {
    s_arrived = atomicInc(P.cnt + tile, 1u);  // 0 -> 1 for the first, 1 -> 0 for the second
    __threadfence();
  }
  __syncthreads();
  if (s_arrived == 0) return;
  const cx<T>* const other = P.Q + (1 - f) * fstride + c;
  cx<T> N[8], next[8];
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    const int j = t + q * PP;
    N[q] = czero<T>();
    if (c < nkd && (j < la || j >= lb)) {
      const cx<T> o = __ldcg(other + j * P.nkp);
      const cx<T> f0 = f == 0 ? v[0][q] : o, f1 = f == 0 ? o : v[0][q];
      N[q] = mul_mi(add(scl(f0, P.kr[c]), scl(f1, P.l[j])));
    }
  }
  if (c < P.nkr) epilogue_col<T, NY, EPI>(P, S, c, t, N, next);
}

// FUSE: also run the next substep's pass A on the new state of this column tile
template <typename T, int NY, int EPI, bool FUSE>
__device__ __forceinline__ void vort_c_reg(const VortProb<T>& P, const EpiScalars<T>& S, int tile, cx<T>* smem) {
  constexpr int PP = NY / 8;
  const int tl = blockDim.x / PP;
  const int ln = threadIdx.x & (tl - 1), t = threadIdx.x / tl;
  const int c0 = tile * tl, c = c0 + ln;
  const int nkr = P.nkr, nkd = P.nkd, la = P.la, lb = P.lb, ny = P.ny;
  if (c0 < nkd) {
    cx<T> v[2][8];
    const cx<T>* qsrc = P.Q + c;
    const int fstride = P.nkp * ny;
#pragma unroll
    for (int f = 0; f < 2; ++f)
#pragma unroll
      for (int q = 0; q < 8; ++q)
        v[f][q] = c < nkd ? qsrc[f * fstride + (t + q * PP) * P.nkp] : czero<T>();
    cx<T>* const buf2[2] = {smem, smem + (NY + NY / 8) * tl};
    regfft<T, 2, NY, -1>(v, t, P.twy, buf2, XCol{tl, ln});
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const int j = t + q * PP;
      cx<T> N = czero<T>();
      if (c < nkd && (j < la || j >= lb)) N = mul_mi(add(scl(v[0][q], P.kr[c]), scl(v[1][q], P.l[j])));
      v[0][q] = N;
      v[1][q] = czero<T>();
    }
    // ETDRK4 substeps 1-3 with the next pass A fused: sol1 / sol2 stay in registers
    constexpr bool kFusedEtd = FUSE && (EPI == EPI_ETD1 || EPI == EPI_ETD2 || EPI == EPI_ETD3);
    if (c < nkr) epilogue_col<T, NY, EPI, kFusedEtd>(P, S, c, t, v[0], v[1]);
    if (FUSE) a_from_regs<T, NY>(P, c, t, tl, ln, v[1], smem);
  } else if (c < nkr) {
    // aliased kr columns (substeps 1-3 of ETDRK4 and RK4 do not visit these tiles: their
    // work list is the prefix of kept tiles)
    cx<T> N[8], next[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) N[q] = czero<T>();
    epilogue_col<T, NY, EPI>(P, S, c, t, N, next);
  }
}

// Register budgets of the register-path kernels: max threads per CTA and the minimum
// number of resident CTAs per SM the compiler must fit
#ifndef FF_LB_A_MIN_F32
#define FF_LB_A_MIN_F32 (FF_A_FIELDS_F32 == 3 ? 1 : 3)
#endif
#ifndef FF_LB_B_MIN_F32
#define FF_LB_B_MIN_F32 2
#endif
#ifndef FF_LB_C_MIN_F32
#define FF_LB_C_MIN_F32 1
#endif
#ifndef FF_LB_A_MIN_F64
#define FF_LB_A_MIN_F64 (FF_A_FIELDS_F64 == 3 ? 1 : 2)
#endif
#ifndef FF_LB_B_MIN_F64
#define FF_LB_B_MIN_F64 2
#endif
#ifndef FF_LB_C_MIN_F64
#define FF_LB_C_MIN_F64 1
#endif
// the final substeps (ETDRK4 / RK4 updates) read four state arrays and up to five
// coefficient arrays in the epilogue: their own budget
#ifndef FF_LB_C4_MIN_F32
#define FF_LB_C4_MIN_F32 FF_LB_C_MIN_F32
#endif
#ifndef FF_LB_C4_MIN_F64
#define FF_LB_C4_MIN_F64 FF_LB_C_MIN_F64
#endif
template <typename T> struct RegBudget;  // minimum resident CTAs per SM by precision
template <> struct RegBudget<float> {
  static constexpr int A = FF_LB_A_MIN_F32, B = FF_LB_B_MIN_F32, C = FF_LB_C_MIN_F32, C4 = FF_LB_C4_MIN_F32;
};
template <> struct RegBudget<double> {
  static constexpr int A = FF_LB_A_MIN_F64, B = FF_LB_B_MIN_F64, C = FF_LB_C_MIN_F64, C4 = FF_LB_C4_MIN_F64;
};
#define FF_LB_A 512, RegBudget<T>::A
// pass B's largest CTA (threads; a power of two is used up to this bound)
#ifndef FF_LB_B_THREADS
#define FF_LB_B_THREADS 256
#endif
#define FF_LB_B FF_LB_B_THREADS, RegBudget<T>::B
#define FF_LB_C 512, ((EPI == EPI_ETD4 || EPI == EPI_RK4) ? RegBudget<T>::C4 : RegBudget<T>::C)
// the split pass C: CTAs of at most FF_SPLIT_C_THREADS threads (one 1024-row column or
// less), FF_SPLIT_C_MIN of them resident per SM
#ifndef FF_SPLIT_C_THREADS
#define FF_SPLIT_C_THREADS 128
#endif
#ifndef FF_SPLIT_C_MIN
#define FF_SPLIT_C_MIN 4
#endif
#define FF_LB_C_SPLIT FF_SPLIT_C_THREADS, FF_SPLIT_C_MIN

#define FF_REG_CASES(X) X(16) X(32) X(64) X(128) X(256) X(512) X(1024) X(2048) X(4096)
#define FF_REG_CASES_B(X) X(16) X(32) X(64) X(128) X(256) X(512) X(1024) X(2048)

template <typename T>
__global__ void __launch_bounds__(FF_LB_A) k_vort_a_r(const VortProb<T>* __restrict__ probs,
                                                  const WorkItem* __restrict__ work, int nwork,
                                                  const cx<T>* const* __restrict__ inputs) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cx<T>* smem = reinterpret_cast<cx<T>*>(smem_raw);
  for (int w = blockIdx.x; w < nwork; w += gridDim.x) {
    const WorkItem it = work[w];
    const VortProb<T>& P = probs[it.prob];
    const cx<T>* zh = inputs[it.prob];
    switch (P.ny) {
#define FF_A_CASE(N) \
  case N:                                                 \
    if (AFields<T>::value == 3) vort_a_reg3<T, N>(P, zh, it.tile, smem); \
    else vort_a_reg<T, N>(P, zh, it.tile, it.field, smem); \
    break;
      FF_REG_CASES(FF_A_CASE)
#undef FF_A_CASE
      default: break;
    }
    __syncthreads();
  }
}

// every line of the next item's three field-row blocks, into L2
template <typename T> __device__ __forceinline__ void prefetch_b(const VortProb<T>& P, const WorkItem& it) {
  const int rows = blockDim.x * 8 / (P.nx / 2), j0 = it.tile * rows;
  const int nr = min(rows, P.ny - j0);
  if (nr <= 0) return;
  const int fstride = P.nkp * P.ny;
  for (int f = 0; f < 3; ++f)
    prefetch_lines(P.W + f * fstride + j0 * P.nkp, nr * P.nkp, threadIdx.x, blockDim.x);
}

// Pass B, persistent over row blocks; each item's rows are prefetched into L2 one item
// ahead.  (Staging the rows through shared memory with cp.async one item ahead measured
// 23% slower, a bulk-copy pipeline 5%, and a form holding one field besides zeta in
// registers at a time 10%, at 32 x 1024^2 FP32.)
template <typename T>
__global__ void __launch_bounds__(FF_LB_B) k_vort_b_r(const VortProb<T>* __restrict__ probs,
                                                  const WorkItem* __restrict__ work, int nwork) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cx<T>* smem = reinterpret_cast<cx<T>*>(smem_raw);
  for (int w = blockIdx.x; w < nwork; w += gridDim.x) {
    const WorkItem it = work[w];
    const VortProb<T>& P = probs[it.prob];
    if (w + (int)gridDim.x < nwork) {
      const WorkItem nxt = work[w + gridDim.x];
      prefetch_b(probs[nxt.prob], nxt);
    }
    switch (P.nx / 2) {
#define FF_B_CASE(N) \
  case N: vort_b_reg<T, N>(P, it.tile, smem); break;
      FF_REG_CASES_B(FF_B_CASE)
#undef FF_B_CASE
      default: break;
    }
  }
}

// SPLIT: pass C split by field (vort_c_split) on the kept column tiles; the work list
// then holds two items, fields 0 and 1, per kept tile
template <typename T, int EPI, bool FUSE>
__global__ void __launch_bounds__(FF_LB_C) k_vort_c_r(const VortProb<T>* __restrict__ probs,
                                                  const WorkItem* __restrict__ work, int nwork, EpiScalars<T> S) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cx<T>* smem = reinterpret_cast<cx<T>*>(smem_raw);
  for (int w = blockIdx.x; w < nwork; w += gridDim.x) {
    const WorkItem it = work[w];
    const VortProb<T>& P = probs[it.prob];
    switch (P.ny) {
#define FF_C_CASE(N) \
  case N: vort_c_reg<T, N, EPI, FUSE>(P, S, it.tile, smem); break;
      FF_REG_CASES(FF_C_CASE)
#undef FF_C_CASE
      default: break;
    }
    __syncthreads();
  }
}

// Pass C split by field (vort_c_split) on the kept column tiles, whose work list holds two
// items, fields 0 and 1, per kept tile; aliased tiles run the plain epilogue.  Its own
// kernel, with a smaller CTA bound than the plain pass C so that more CTAs are resident
// (columns of up to 8 FF_SPLIT_C_THREADS rows).
template <typename T, int EPI>
__global__ void __launch_bounds__(FF_LB_C_SPLIT) k_vort_c_rs(const VortProb<T>* __restrict__ probs,
                                                         const WorkItem* __restrict__ work, int nwork,
                                                         EpiScalars<T> S) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cx<T>* smem = reinterpret_cast<cx<T>*>(smem_raw);
  for (int w = blockIdx.x; w < nwork; w += gridDim.x) {
    const WorkItem it = work[w];
    const VortProb<T>& P = probs[it.prob];
    const bool split = it.tile * (int)(blockDim.x * 8 / P.ny) < P.nkd;
    switch (P.ny) {
#define FF_C_CASE(N)                                                       \
  case N:                                                                  \
    if constexpr (N / 8 <= FF_SPLIT_C_THREADS) {                           \
      if (split) vort_c_split<T, N, EPI>(P, S, it.tile, it.field, smem);   \
      else vort_c_reg<T, N, EPI, false>(P, S, it.tile, smem);              \
    }                                                                      \
    break;
      FF_REG_CASES(FF_C_CASE)
#undef FF_C_CASE
      default: break;
    }
    __syncthreads();
  }
}

}  // namespace ff
