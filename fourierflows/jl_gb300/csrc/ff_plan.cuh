// Internal plan machinery shared by the generic transforms (ff_plan.cu) and the fused
// physics passes (ff_vorticity.cu): factorisation, twiddle tables, launch geometry.
#pragma once

#include <vector>

#include "ff_fft.cuh"

namespace ff {

// Split n into stage radices (8s first, then 4/2, then 3, 5 and other primes <= 31).
// Returns false when n has a prime factor above FF_MAX_GENERIC_RADIX.
bool factorize(int n, LinePlan& P);

// tw[e] = exp(-2 pi i e / n), e in [0, n), rounded from long-double values; host copy.
// W_n^e for e < n, then (power-of-two n, 16..4096) the register FFT's stage-major twiddles
void host_twiddles(int n, std::vector<double>& re_im);
// W_N^k for k in [0, N/2]: the packing twiddles of a length-N real transform.
void host_real_twiddles(int N, std::vector<double>& re_im);  // 2 (N/2 + 1) doubles

// Upload a twiddle table (2*count doubles) as double2 or float2 to a new device buffer.
int upload_table(const std::vector<double>& re_im, int prec, void** dev);

// Raise the dynamic shared-memory limit of a kernel once per device when needed.
int ensure_smem(const void* func, size_t bytes);

// Launch geometry of a strided-axis (column) pass and of a contiguous (row) pass.
struct ColGeom {
  int tl, nth;
  size_t smem;
};
struct RowGeom {
  int tlr, nth;
  size_t smem;
};
ColGeom col_geom(int n, int prec, int tl_hint = 0);
RowGeom row_geom(int h, int prec);

// Generic passes (launchers; sizes in elements).
template <typename T>
int launch_r2c_rows(const T* in, cx<T>* out, int64_t nrows, int nx, const LinePlan& P, const cx<T>* tw,
                    const cx<T>* rtw, cudaStream_t s);
template <typename T>
int launch_c2r_rows(const cx<T>* in, T* out, int64_t nrows, int nx, const LinePlan& P, const cx<T>* tw,
                    const cx<T>* rtw, T scale, cudaStream_t s);
template <typename T, int DIR>
int launch_c2c_rows(const cx<T>* in, cx<T>* out, int64_t nrows, int n, const LinePlan& P, const cx<T>* tw,
                    T scale, cudaStream_t s);
template <typename T, int DIR>
int launch_cols(const cx<T>* in, cx<T>* out, int64_t ncols, int n, int64_t stride, int64_t nouter,
                int64_t outer_stride, const LinePlan& P, const cx<T>* tw, T scale, cudaStream_t s);

// Register-resident passes for power-of-two lengths (ff_plan_reg.cu): rows of nx/2 <= 2048
// complex values (FP32 real transforms), lines of n <= 4096 (complex rows and columns, both
// precisions).  The launchers above route to them when the length qualifies, unless
// FF_PLAN_GENERIC=1.
bool reg_rows_ok(int h);
bool reg_line_ok(int n);
bool plan_generic_forced();
template <typename T>
int launch_r2c_rows_reg(const T* in, cx<T>* out, int64_t nrows, int nx, const cx<T>* tw, const cx<T>* rtw,
                        cudaStream_t s);
template <typename T>
int launch_c2r_rows_reg(const cx<T>* in, T* out, int64_t nrows, int nx, const cx<T>* tw, const cx<T>* rtw, T scale,
                        cudaStream_t s);
template <typename T, int DIR>
int launch_c2c_rows_reg(const cx<T>* in, cx<T>* out, int64_t nrows, int n, const cx<T>* tw, T scale,
                        cudaStream_t s);
template <typename T, int DIR>
int launch_cols_reg(const cx<T>* in, cx<T>* out, int64_t ncols, int n, int64_t stride, int64_t nouter,
                    int64_t outer_stride, const cx<T>* tw, T scale, cudaStream_t s);

}  // namespace ff
