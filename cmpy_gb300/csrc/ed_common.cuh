// Shared device/host helpers of libcmpy_ed.so: status handling, the per-device context
// (binomial table, status word), bit helpers and deterministic block reductions.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <string>

#include "../../include/cmpy_ed.h"

#define ED_MAX_SITES 62
#define ED_MAX_BONDS 128

namespace ed {

// ---- host-side error plumbing --------------------------------------------------------
void set_error(const std::string& msg);
ed_status fail(ed_status st, const std::string& msg);
ed_status cuda_fail(cudaError_t e, const char* what);

#define ED_CUDA(call)                                        \
  do {                                                       \
    cudaError_t _e = (call);                                 \
    if (_e != cudaSuccess) return ::ed::cuda_fail(_e, #call); \
  } while (0)

// Checks the launch(es) just issued and adds n to the library's kernel-launch counter
// (ed_launch_count); every kernel launch of the library passes through one of these.
void count_launches(uint64_t n);
#define ED_CHECK_LAUNCH_N(name, n)                            \
  do {                                                        \
    ::ed::count_launches(n);                                  \
    cudaError_t _e = cudaGetLastError();                      \
    if (_e != cudaSuccess) return ::ed::cuda_fail(_e, name);  \
  } while (0)
#define ED_CHECK_LAUNCH(name) ED_CHECK_LAUNCH_N(name, 1)

#define ED_TRY(expr)                   \
  do {                                 \
    ed_status _s = (expr);             \
    if (_s != ED_OK) return _s;        \
  } while (0)

inline cudaStream_t as_stream(ed_stream_t s) { return reinterpret_cast<cudaStream_t>(s); }

// ---- per-device context ----------------------------------------------------------------
// Binomial table C(n,k), n,k in [0,64), row-major [n*64+k], on the current device.
struct DeviceContext {
  int device = -1;
  int num_sms = 0;
  int smem_optin = 0;  // largest shared memory (static + dynamic) one CTA may opt in to
  uint64_t* d_binom = nullptr;
  int* d_status = nullptr;  // device status word (first error code a kernel records)
};
// Returns the context of the current device, creating it on first use (synchronous then).
ed_status device_context(DeviceContext** out);
uint64_t host_binomial(int n, int k);

// Device status codes recorded by kernel bounds checks.
enum DeviceStatus : int { DEV_OK = 0, DEV_BOUNDS = 1, DEV_TIMEOUT = 2, DEV_NONFINITE = 3 };

__device__ __forceinline__ void record_status(int* status, int code) {
  if (status) atomicCAS(status, 0, code);
}

// ---- bit helpers (reference: cmpy/operators.py:226-299) ----------------------------------
__device__ __forceinline__ uint64_t binom(const uint64_t* __restrict__ tab, int n, int k) {
  return (k < 0 || k > n) ? 0ull : __ldg(tab + n * 64 + k);
}

// rank of s among the ascending states with the same popcount (colex rank):
// sum over set bits p_1<p_2<... of C(p_k, k).
__device__ __forceinline__ int64_t colex_rank(const uint64_t* __restrict__ tab, uint64_t s) {
  int64_t r = 0;
  int k = 1;
  while (s) {
    int p = __ffsll((long long)s) - 1;
    r += (int64_t)binom(tab, p, k);
    s &= s - 1;
    ++k;
  }
  return r;
}

// weighted_element (cmpy/operators.py:226-250): sequential ascending-site FP64 sum.
__device__ __forceinline__ double weighted_element(uint64_t state, const double* values, int n) {
  double v = 0.0;
  for (int i = 0; i < n; ++i)
    if (state & (1ull << i)) v = __dadd_rn(v, values[i]);
  return v;
}

// (-1)^(bits of state strictly between site1 and site2 that lie below `width`)
// — _hopping_sign + bit_count(number, width) of cmpy/operators.py:253-273,425-433.
__device__ __host__ __forceinline__ int hop_sign(uint64_t state, int width, int site1, int site2) {
  uint64_t mask = 0;
  if (site2 - site1 > 1) mask = ((1ull << site2) - 1) & ~((1ull << (site1 + 1)) - 1);
  uint64_t wmask = width >= 64 ? ~0ull : ((width <= 0) ? 0ull : ((1ull << width) - 1));
#ifdef __CUDA_ARCH__
  int c = __popcll(state & mask & wmask);
#else
  int c = __builtin_popcountll(state & mask & wmask);
#endif
  return (c & 1) ? -1 : 1;
}

// bisect_left (cmpy/operators.py:276-299) over a sorted array.
__device__ __forceinline__ int64_t bisect_left(const uint64_t* __restrict__ a, int64_t n, uint64_t x) {
  int64_t lo = 0, hi = n;
  while (lo < hi) {
    int64_t mid = (lo + hi) >> 1;
    if (a[mid] < x) lo = mid + 1; else hi = mid;
  }
  return lo;
}

// ---- deterministic block reduction -------------------------------------------------------
template <int NT>
__device__ __forceinline__ double block_sum(double v, double* smem /*[NT/32]*/) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) smem[w] = v;
  __syncthreads();
  double r = 0.0;
  if (w == 0) {
    r = (l < NT / 32) ? smem[l] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) r += __shfl_xor_sync(0xffffffffu, r, o);
  }
  return r;  // valid in thread 0
}

inline int grid_for(int64_t n, int threads, int cap) {
  int64_t b = (n + threads - 1) / threads;
  if (b < 1) b = 1;
  if (b > cap) b = cap;
  return (int)b;
}

}  // namespace ed
