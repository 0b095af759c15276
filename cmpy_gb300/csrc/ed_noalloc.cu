// Allocation-free variant of ed_tridiag_lowest.
//
// ed_tridiag_lowest takes the 5*m doubles of inverse-iteration scratch from cudaMallocAsync.
// Some callers cannot allocate device memory at the point where they need the ground state
// of a Lanczos tridiagonal matrix: hosts whose device memory belongs to their own allocator
// (a framework's caching allocator or a fixed pool that a library must not bypass), plugin
// hosts that forbid libraries from allocating, and latency-critical loops where the
// allocator's bookkeeping or an implicit synchronisation is not acceptable. For them,
// ed_tridiag_lowest_noalloc takes its scratch from a fixed array that is part of this
// library's device image (ED_NOALLOC_MAX_M * 5 doubles = 160 KB), present on every GPU that
// loads the library until the process exits.
//
// The array's name in host code is only a host-side stand-in, not a device address, so the
// address is obtained with cudaGetSymbolAddress (with the device current) and passed to the
// kernel. That set-up happens in the first call on each device (and again after the device's
// context was replaced, e.g. after cudaDeviceReset: the cache is keyed on the context), so
// that first call should come before any stream capture on the device; later calls make no
// call that a stream capture forbids and can be captured into a CUDA graph. Every call shares the
// array: calls that overlap on the GPU (different streams without ordering) race on it. The
// kernel rebuilds every scratch value it reads, so nothing has to be cleared between calls.
#include <cuda.h>

#include <mutex>

#include "ed_common.cuh"
#include "ed_tridiag.cuh"

#define ED_NOALLOC_MAX_M 4096

namespace ed {

static __device__ __align__(256) double g_tridiag_scratch[5 * ED_NOALLOC_MAX_M];

static std::mutex g_scratch_mutex;
struct ScratchSlot {
  void* ctx;    // the context the address belongs to
  double* ptr;  // device address of g_tridiag_scratch in that context
};
static ScratchSlot g_scratch[64] = {};

// the calling thread's current driver context (the runtime makes the device's primary context
// current on first use); fetched through the runtime's driver entry-point query, so the
// library does not link libcuda
static ed_status current_context(void** out) {
  using GetCurrent = CUresult (*)(CUcontext*);
  static GetCurrent fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (GetCurrent)f;
  });
  if (!fn) return fail(ED_ERR_CUDA, "cuCtxGetCurrent is not available");
  CUcontext c = nullptr;
  if (fn(&c) != CUDA_SUCCESS) return fail(ED_ERR_CUDA, "cuCtxGetCurrent failed");
  *out = (void*)c;
  return ED_OK;
}

// device address of g_tridiag_scratch on the current device (looked up on first use per
// device and context)
static ed_status scratch_address(double** out) {
  int dev = 0;
  ED_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return fail(ED_ERR_INVALID_ARG, "device index out of range");
  void* ctx = nullptr;
  ED_TRY(current_context(&ctx));
  if (!ctx) {
    // no context on this thread yet: make the device's primary context current (only then:
    // cudaFree is not allowed while a stream of the device is being captured, and a thread
    // that captures already has its context current)
    ED_CUDA(cudaFree(nullptr));
    ED_TRY(current_context(&ctx));
    if (!ctx) return fail(ED_ERR_CUDA, "no current context on the device");
  }
  std::lock_guard<std::mutex> lock(g_scratch_mutex);
  if (!g_scratch[dev].ptr || g_scratch[dev].ctx != ctx) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_tridiag_scratch);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_tridiag_scratch)");
    g_scratch[dev] = ScratchSlot{ctx, (double*)p};
  }
  *out = g_scratch[dev].ptr;
  return ED_OK;
}

__global__ void k_tridiag_noalloc(const double* alpha, const double* beta, int m, double* value, double* vec,
                                  double* work) {
  const double e = tridiag_lowest_block<512>(alpha, beta, m, vec, work);
  if (threadIdx.x == 0) *value = e;
}

}  // namespace ed

using namespace ed;

extern "C" {

ED_API ed_status ed_tridiag_lowest_noalloc(const double* d_alpha, const double* d_beta, int m, double* d_value,
                                           double* d_vec, ed_stream_t stream) {
  if (m < 1) return fail(ED_ERR_INVALID_ARG, "m must be >= 1");
  if (m > ED_NOALLOC_MAX_M)  // the same limit and status as ed_tridiag_lowest
    return fail(ED_ERR_INVALID_ARG, "ed_tridiag_lowest_noalloc: m exceeds the static scratch (max 4096)");
  if (!d_alpha || !d_beta || !d_value) return fail(ED_ERR_INVALID_ARG, "null argument");
  double* work = nullptr;
  ED_TRY(scratch_address(&work));
  k_tridiag_noalloc<<<1, 256, 0, as_stream(stream)>>>(d_alpha, d_beta, m, d_value, d_vec, work);
  ED_CHECK_LAUNCH("k_tridiag_noalloc");
  return ED_OK;
}

}  // extern "C"
