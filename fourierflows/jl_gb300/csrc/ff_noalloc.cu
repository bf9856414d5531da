// ff_parsevalsum2_noalloc: the Parseval sum of ff_parsevalsum2 without any device
// allocation, for callers that cannot call cudaMalloc -- typically host programs whose
// device memory is owned by another allocator (a pooling allocator that has reserved the
// GPU, as the memory pools of CUDA.jl or PyTorch do, or an embedded code with a fixed
// memory budget).  The caller passes the input and a device output; the only scratch,
// one FP64 partial sum per CTA, is the file-scope array below, which every GPU that loads
// this library holds until the process exits.
//
// Two launches: each CTA reduces its own chunk of FF_NOALLOC_CHUNK modes into one slot
// of the scratch array, then one CTA adds the used slots in order (deterministic).  Every
// slot that the second launch reads was written by the first launch of the same call, so
// nothing needs clearing between calls; but all calls share the array, so calls that
// overlap on the GPU (different streams, or different host threads) race on it.
#include <cuda.h>  // CUcontext / CUresult types only: driver calls go through the runtime's entry points

#include <mutex>

#include "ff_common.cuh"
#include "ff_ctx_cache.h"

#define FF_NOALLOC_THREADS 256
#define FF_NOALLOC_CHUNK 8192                           // modes per CTA
#define FF_NOALLOC_MAX_SLOTS 4096                       // 32 KiB of FP64 partials
#define FF_NOALLOC_MAX_MODES ((int64_t)FF_NOALLOC_MAX_SLOTS * FF_NOALLOC_CHUNK)  // 33,554,432

static __device__ __align__(256) double g_noalloc_partials[FF_NOALLOC_MAX_SLOTS];

namespace {

__device__ __forceinline__ double noalloc_block_sum(double v) {
  __shared__ double sh[FF_NOALLOC_THREADS / 32];
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

// CTA b sums |uh|^2 (rows 1..n0-2 twice when rfft_form) over modes [b*CHUNK, (b+1)*CHUNK)
template <typename T>
__global__ void k_noalloc_partial(const ff::cx<T>* __restrict__ uh, int64_t n0, int64_t total, int rfft_form,
                                  double* __restrict__ slots) {
  const int64_t begin = (int64_t)blockIdx.x * FF_NOALLOC_CHUNK;
  int64_t end = begin + FF_NOALLOC_CHUNK;
  if (end > total) end = total;
  double acc = 0.0;
  for (int64_t i = begin + threadIdx.x; i < end; i += blockDim.x) {
    const ff::cx<T> u = uh[i];
    const double v = (double)u.x * (double)u.x + (double)u.y * (double)u.y;
    const int64_t i0 = i % n0;
    acc += (rfft_form && i0 > 0 && i0 < n0 - 1) ? 2.0 * v : v;
  }
  acc = noalloc_block_sum(acc);
  if (threadIdx.x == 0) slots[blockIdx.x] = acc;
}

__global__ void k_noalloc_finish(const double* __restrict__ slots, int nslots, double norm, double* out) {
  double acc = 0.0;
  for (int i = threadIdx.x; i < nslots; i += blockDim.x) acc += slots[i];
  acc = noalloc_block_sum(acc);
  if (threadIdx.x == 0) *out = acc * norm;
}

// The current context's unique ID (cuCtxGetId), through driver entry points that the
// runtime hands out, so the library does not link libcuda itself.  False when no context
// is current yet or the driver has no context IDs.
bool current_context_id(unsigned long long* id) {
  using GetCurrent = CUresult (*)(CUcontext*);
  using GetId = CUresult (*)(CUcontext, unsigned long long*);
  static GetCurrent get_cur = nullptr;
  static GetId get_id = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_cur = (GetCurrent)p;
    p = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_id = (GetId)p;
  });
  if (!get_cur || !get_id) return false;
  CUcontext ctx = nullptr;
  if (get_cur(&ctx) != CUDA_SUCCESS || !ctx) return false;
  return get_id(ctx, id) == CUDA_SUCCESS;
}

int fetch_scratch(void** p) {
  const cudaError_t e = cudaGetSymbolAddress(p, g_noalloc_partials);
  return e == cudaSuccess ? 0 : (int)e;
}

// Device address of g_noalloc_partials in the current context.  In host code the symbol
// names a host-side stand-in, never the device array itself.  The address is cached per
// context ID: after a device reset (or a re-created primary context) the new context has
// a new ID and the address is looked up again, in that context.
double* scratch_address(int* status) {
  static ff::CtxAddressCache<64> cache;
  unsigned long long id = 0;
  void* p = nullptr;
  if (!current_context_id(&id)) {
    // no current context yet (the runtime makes the primary context current lazily, and
    // this lookup does so) or no context IDs: look the address up directly
    if (const int e = fetch_scratch(&p)) {
      *status = ff::cuda_status((cudaError_t)e, "ff_parsevalsum2_noalloc: cudaGetSymbolAddress");
      return nullptr;
    }
    if (current_context_id(&id)) cache.get(id, &p, [p](void** q) { *q = p; return 0; });
    *status = FF_OK;
    return (double*)p;
  }
  if (const int e = cache.get(id, &p, fetch_scratch)) {
    *status = ff::cuda_status((cudaError_t)e, "ff_parsevalsum2_noalloc: cudaGetSymbolAddress");
    return nullptr;
  }
  *status = FF_OK;
  return (double*)p;
}

}  // namespace

extern "C" int ff_parsevalsum2_noalloc(int prec, const void* uh, int64_t n0, int64_t nrest, int rfft_form,
                                       double norm, double* out, void* stream) {
  FF_CHECK_ARG(uh && out, "ff_parsevalsum2_noalloc: null input or output");
  FF_CHECK_ARG(prec == FF_F64 || prec == FF_F32, "ff_parsevalsum2_noalloc: bad precision %d", prec);
  FF_CHECK_ARG(n0 >= 1 && nrest >= 1, "ff_parsevalsum2_noalloc: sizes must be positive");
  FF_CHECK_ARG(nrest <= FF_NOALLOC_MAX_MODES / n0,
               "ff_parsevalsum2_noalloc: %lld x %lld modes exceed the maximum of %lld (%d KiB static scratch)",
               (long long)n0, (long long)nrest, (long long)FF_NOALLOC_MAX_MODES,
               (int)(FF_NOALLOC_MAX_SLOTS * sizeof(double) / 1024));
  int st = FF_OK;
  double* slots = scratch_address(&st);
  if (!slots) return st;
  const int64_t total = n0 * nrest;
  const int nslots = (int)((total + FF_NOALLOC_CHUNK - 1) / FF_NOALLOC_CHUNK);
  auto s = (cudaStream_t)stream;
  if (prec == FF_F64)
    k_noalloc_partial<double><<<nslots, FF_NOALLOC_THREADS, 0, s>>>((const double2*)uh, n0, total, rfft_form, slots);
  else
    k_noalloc_partial<float><<<nslots, FF_NOALLOC_THREADS, 0, s>>>((const float2*)uh, n0, total, rfft_form, slots);
  FF_LAUNCHED("ff_parsevalsum2_noalloc: partial sums");
  k_noalloc_finish<<<1, FF_NOALLOC_THREADS, 0, s>>>(slots, nslots, norm, out);
  FF_LAUNCHED("ff_parsevalsum2_noalloc: final sum");
  return FF_OK;
}
