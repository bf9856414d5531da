// Library-wide C ABI pieces: version, per-thread error messages, device queries.
#include <stdarg.h>
#include <string.h>

#include <mutex>

#include "ff_common.cuh"

namespace ff {

static thread_local char g_err[512] = "";

void set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}

int cuda_status(cudaError_t e, const char* what) {
  set_error("%s: %s (%s)", what, cudaGetErrorString(e), cudaGetErrorName(e));
  return e == cudaErrorMemoryAllocation ? FF_ERR_ALLOC : FF_ERR_CUDA;
}

int sm_count() {
  int dev = 0, n = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 152;
  if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) return 152;
  return n;
}

int elementwise_grid(int64_t n, int threads) {
  // enough CTAs to cover the SMs several times; every kernel is grid-stride
  const int64_t need = ceil_div(n, threads);
  const int64_t cap = (int64_t)sm_count() * 8;
  int64_t g = need < cap ? need : cap;
  return (int)(g < 1 ? 1 : g);
}

}  // namespace ff

extern "C" {

int ff_version(void) { return (0 << 16) | (1 << 8) | 0; }

int ff_last_error(char* buf, size_t len) {
  if (!buf || len == 0) return FF_ERR_ARG;
  strncpy(buf, ff::g_err, len - 1);
  buf[len - 1] = 0;
  return FF_OK;
}

}  // extern "C"
