// Allocation-free variant of ed_tridiag_lowest.
//
// ed_tridiag_lowest takes the 5*m doubles of inverse-iteration scratch from cudaMallocAsync.
// Some callers cannot allocate device memory at the point where they need the ground state
// of a Lanczos tridiagonal matrix: code that runs while one of their streams is being
// captured into a CUDA graph (allocation calls are not allowed then), or hosts whose device
// memory belongs to their own allocator and must not see allocations from a library. For
// them, ed_tridiag_lowest_noalloc takes its scratch from a fixed array that is part of this
// library's device image (ED_NOALLOC_MAX_M * 5 doubles = 160 KB), present on every GPU that
// loads the library until the process exits.
//
// The array's name in host code is only a host-side stand-in, not a device address, so the
// address is obtained once per device with cudaGetSymbolAddress (with that device current)
// and passed to the kernel. That set-up happens in the first call on each device, which
// therefore must come before any stream capture on that device. Every call shares the array:
// calls that overlap on the GPU (different streams without ordering) race on it. The kernel
// rebuilds every scratch value it reads, so nothing has to be cleared between calls.
#include <mutex>

#include "ed_common.cuh"
#include "ed_tridiag.cuh"

#define ED_NOALLOC_MAX_M 4096

namespace ed {

static __device__ __align__(256) double g_tridiag_scratch[5 * ED_NOALLOC_MAX_M];

static std::mutex g_scratch_mutex;
static double* g_scratch_ptr[64] = {};

// device address of g_tridiag_scratch on the current device (set-up on first use)
static ed_status scratch_address(double** out) {
  int dev = 0;
  ED_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return fail(ED_ERR_INVALID_ARG, "device index out of range");
  std::lock_guard<std::mutex> lock(g_scratch_mutex);
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_tridiag_scratch);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_tridiag_scratch)");
    g_scratch_ptr[dev] = (double*)p;
  }
  *out = g_scratch_ptr[dev];
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
  if (m > ED_NOALLOC_MAX_M)
    return fail(ED_ERR_TOO_LARGE, "ed_tridiag_lowest_noalloc: m exceeds the static scratch (max 4096)");
  if (!d_alpha || !d_beta || !d_value) return fail(ED_ERR_INVALID_ARG, "null argument");
  double* work = nullptr;
  ED_TRY(scratch_address(&work));
  k_tridiag_noalloc<<<1, 256, 0, as_stream(stream)>>>(d_alpha, d_beta, m, d_value, d_vec, work);
  ED_CHECK_LAUNCH("k_tridiag_noalloc");
  return ED_OK;
}

}  // extern "C"
