// Library runtime (errors, per-device context) and the sector basis kernels:
// enumeration and ranking of spin-sector bitstrings with the combinatorial number system.
// Replaces Basis.generate_states/get_states/init (cmpy/basis.py:644-676) and the bisect
// lookups of cmpy/operators.py:276-299.
#include <atomic>
#include <mutex>
#include <string>
#include <vector>

#include "ed_common.cuh"

namespace ed {

static thread_local std::string g_last_error;
static std::atomic<uint64_t> g_launches{0};

void count_launches(uint64_t n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

void set_error(const std::string& msg) { g_last_error = msg; }

ed_status fail(ed_status st, const std::string& msg) {
  g_last_error = msg;
  return st;
}

ed_status cuda_fail(cudaError_t e, const char* what) {
  g_last_error = std::string(what) + ": " + cudaGetErrorString(e);
  // A non-sticky error (bad launch configuration, invalid attribute) stays in the runtime's
  // per-thread error slot and would be reported again by the next launch check: clear it.
  (void)cudaGetLastError();
  return ED_ERR_CUDA;
}

uint64_t host_binomial(int n, int k) {
  if (n < 0 || k < 0 || k > n || n > 63) return 0;
  if (k > n - k) k = n - k;
  unsigned __int128 r = 1;
  for (int i = 1; i <= k; ++i) r = r * (unsigned)(n - k + i) / (unsigned)i;
  return (uint64_t)r;
}

static std::mutex g_ctx_mutex;
static std::vector<DeviceContext*> g_ctx;

ed_status device_context(DeviceContext** out) {
  int dev = 0;
  ED_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lock(g_ctx_mutex);
  if ((int)g_ctx.size() <= dev) g_ctx.resize(dev + 1, nullptr);
  if (!g_ctx[dev]) {
    DeviceContext* c = new DeviceContext();
    c->device = dev;
    cudaError_t e = cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&c->smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (e != cudaSuccess) { delete c; return cuda_fail(e, "cudaDeviceGetAttribute"); }
    std::vector<uint64_t> tab(64 * 64);
    for (int n = 0; n < 64; ++n)
      for (int k = 0; k < 64; ++k) tab[n * 64 + k] = host_binomial(n, k);
    e = cudaMalloc(&c->d_binom, tab.size() * sizeof(uint64_t));
    if (e == cudaSuccess) e = cudaMemcpy(c->d_binom, tab.data(), tab.size() * sizeof(uint64_t), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMalloc(&c->d_status, sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(c->d_status, 0, sizeof(int));
    if (e != cudaSuccess) {
      if (c->d_binom) cudaFree(c->d_binom);
      delete c;
      return cuda_fail(e, "device_context");
    }
    g_ctx[dev] = c;
  }
  *out = g_ctx[dev];
  return ED_OK;
}

// Unranks r into the r-th ascending bitstring of popcount n (colex order).
__device__ __forceinline__ uint64_t colex_unrank(const uint64_t* __restrict__ tab, int n_sites, int n, uint64_t r) {
  uint64_t s = 0;
  int p = n_sites - 1;
  for (int k = n; k >= 1; --k) {
    while (p >= k - 1 && binom(tab, p, k) > r) --p;  // largest p with C(p,k) <= r
    s |= 1ull << p;
    r -= binom(tab, p, k);
    --p;
  }
  return s;
}

__global__ void k_enumerate(const uint64_t* __restrict__ tab, int n_sites, int n, int64_t count,
                            uint64_t* __restrict__ out) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < count; r += stride)
    out[r] = (n < 0) ? (uint64_t)r : colex_unrank(tab, n_sites, n, (uint64_t)r);
}

__global__ void k_rank(const uint64_t* __restrict__ tab, const uint64_t* __restrict__ states, int64_t count,
                       int64_t* __restrict__ ranks) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < count; i += stride)
    ranks[i] = colex_rank(tab, states[i]);
}

// Used by plan creation (ed_plan.cu).
ed_status enumerate_into(int n_sites, int n, uint64_t* d_out, cudaStream_t s) {
  DeviceContext* ctx;
  ED_TRY(device_context(&ctx));
  const int64_t count = ed_sector_size(n_sites, n);
  if (count <= 0) return ED_OK;
  k_enumerate<<<grid_for(count, 256, ctx->num_sms * 8), 256, 0, s>>>(ctx->d_binom, n_sites, n, count, d_out);
  ED_CHECK_LAUNCH("k_enumerate");
  return ED_OK;
}

}  // namespace ed

using namespace ed;

extern "C" {

ED_API const char* ed_status_string(int status) {
  switch (status) {
    case ED_OK: return "ok";
    case ED_ERR_INVALID_ARG: return "invalid argument";
    case ED_ERR_CUDA: return "CUDA error";
    case ED_ERR_TIMEOUT: return "device wait timed out";
    case ED_ERR_NONFINITE: return "non-finite input";
    case ED_ERR_TOO_LARGE: return "dimension too large";
    case ED_ERR_ZERO_VECTOR: return "zero start vector";
    case ED_ERR_DEVICE: return "device bounds check failed";
    case ED_ERR_NOT_FOUND: return "sector does not exist";
    default: return "unknown status";
  }
}

ED_API const char* ed_last_error(void) { return g_last_error.c_str(); }

ED_API int ed_version(void) { return 100; }

ED_API uint64_t ed_launch_count(void) { return g_launches.load(std::memory_order_relaxed); }

ED_API int64_t ed_binomial(int n, int k) {
  uint64_t v = host_binomial(n, k);
  return v > (uint64_t)INT64_MAX ? -1 : (int64_t)v;
}

ED_API int64_t ed_sector_size(int n_sites, int n) {
  if (n_sites < 0 || n_sites > ED_MAX_SITES) return 0;
  if (n < 0) return (int64_t)1 << n_sites;
  if (n > n_sites) return 0;
  return ed_binomial(n_sites, n);
}

ED_API ed_status ed_enumerate(int n_sites, int n, uint64_t* d_out, int64_t capacity, ed_stream_t stream) {
  if (n_sites < 0 || n_sites > ED_MAX_SITES) return fail(ED_ERR_INVALID_ARG, "ed_enumerate: n_sites must be in [0, 62]");
  if (n > n_sites) return fail(ED_ERR_INVALID_ARG, "ed_enumerate: n > n_sites");
  const int64_t count = ed_sector_size(n_sites, n);
  if (count > capacity) return fail(ED_ERR_INVALID_ARG, "ed_enumerate: capacity smaller than the sector");
  if (count > 0 && !d_out) return fail(ED_ERR_INVALID_ARG, "ed_enumerate: null output");
  return enumerate_into(n_sites, n, d_out, as_stream(stream));
}

ED_API ed_status ed_rank(const uint64_t* d_states, int64_t count, int64_t* d_ranks, ed_stream_t stream) {
  if (count < 0) return fail(ED_ERR_INVALID_ARG, "ed_rank: negative count");
  if (count == 0) return ED_OK;
  if (!d_states || !d_ranks) return fail(ED_ERR_INVALID_ARG, "ed_rank: null pointer");
  DeviceContext* ctx;
  ED_TRY(device_context(&ctx));
  k_rank<<<grid_for(count, 256, ctx->num_sms * 8), 256, 0, as_stream(stream)>>>(ctx->d_binom, d_states, count, d_ranks);
  ED_CHECK_LAUNCH("k_rank");
  return ED_OK;
}

}  // extern "C"
