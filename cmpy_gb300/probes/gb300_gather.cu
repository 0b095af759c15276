// Gather-throughput probe: W[u, c] = sum_{e<8} X[nbr[u][e], c] over a 3432 x 3432 int64 array
// (94 MB, L2-resident after the first pass). All indices in range: nbr < NU, c < ND.
#include <cstdio>
#include <cstdint>
#include <vector>
#include <cuda_runtime.h>
#define CK(x) do { cudaError_t e = (x); if (e != cudaSuccess) { printf("CUDA %s line %d\n", cudaGetErrorString(e), __LINE__); return 1; } } while (0)
constexpr int NU = 3432, ND = 3432, K = 8;

// A: lane-contiguous 8-byte loads, 8 in flight, R rows per CTA iteration
template <int R>
__global__ void kA(const int64_t* __restrict__ X, const int* __restrict__ nbr, int64_t* __restrict__ W) {
  for (int u0 = blockIdx.x * R; u0 < NU; u0 += gridDim.x * R) {
    for (int c = threadIdx.x; c < ND; c += blockDim.x) {
      int64_t h[R];
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const int u = min(u0 + r, NU - 1);
        int64_t v[K];
#pragma unroll
        for (int e = 0; e < K; ++e) v[e] = __ldg(X + (int64_t)__ldg(nbr + u * K + e) * ND + c);
        h[r] = 0;
#pragma unroll
        for (int e = 0; e < K; ++e) h[r] += v[e];
      }
#pragma unroll
      for (int r = 0; r < R; ++r) if (u0 + r < NU) W[(int64_t)(u0 + r) * ND + c] = h[r];
    }
  }
}
// B: 16-byte loads (two adjacent columns per lane)
__global__ void kB(const int64_t* __restrict__ X, const int* __restrict__ nbr, int64_t* __restrict__ W) {
  for (int u = blockIdx.x; u < NU; u += gridDim.x) {
    for (int p = threadIdx.x; p < ND / 2; p += blockDim.x) {
      longlong2 v[K];
#pragma unroll
      for (int e = 0; e < K; ++e) v[e] = __ldg((const longlong2*)(X + (int64_t)__ldg(nbr + u * K + e) * ND) + p);
      int64_t a = 0, b = 0;
#pragma unroll
      for (int e = 0; e < K; ++e) { a += v[e].x; b += v[e].y; }
      ((longlong2*)(W + (int64_t)u * ND))[p] = make_longlong2(a, b);
    }
  }
}
// C: bulk copies of the 8 neighbour rows of one target row (column chunk) into shared memory,
// then a shared-memory sum. Chunk = CH columns; one CTA per SM; double buffered.
constexpr int CH = 512;  // columns per chunk (4 KB per row chunk)
__device__ __forceinline__ unsigned su32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }
__global__ void kC(const int64_t* __restrict__ X, const int* __restrict__ nbr, int64_t* __restrict__ W, int* flag) {
  extern __shared__ __align__(128) unsigned char sm[];
  int64_t* buf = (int64_t*)sm;                 // [2][K][CH]
  uint64_t* bar = (uint64_t*)(sm + 2 * K * CH * 8);
  const int nchunks = (ND + CH - 1) / CH;      // last chunk partial: ND % CH = 360 -> 2880 B (multiple of 16)
  const int ntask = NU * nchunks;
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(su32(bar)));
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(su32(bar + 1)));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  auto issue = [&](int t, int s) {
    const int u = t / nchunks, ch = t % nchunks;
    const int c0 = ch * CH, n = min(CH, ND - c0);
    const unsigned bytes = n * 8;
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" :: "r"(su32(bar + s)), "r"(bytes * K) : "memory");
    for (int e = 0; e < K; ++e)
      asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                   :: "r"(su32(buf + (s * K + e) * CH)), "l"(X + (int64_t)nbr[u * K + e] * ND + c0), "r"(bytes), "r"(su32(bar + s)) : "memory");
  };
  int k = 0;
  unsigned par[2] = {0, 0};
  int t = blockIdx.x;
  if (t < ntask && threadIdx.x == 0) issue(t, 0);
  for (; t < ntask; t += gridDim.x, ++k) {
    const int s = k & 1;
    const int tn = t + gridDim.x;
    if (tn < ntask && threadIdx.x == 0) issue(tn, s ^ 1);
    unsigned ok = 0;
    for (long it = 0; it < (1L << 22) && !ok; ++it)
      asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}" : "=r"(ok) : "r"(su32(bar + s)), "r"(par[s]) : "memory");
    if (!ok) { atomicExch(flag, 1); }
    par[s] ^= 1;
    const int u = t / nchunks, ch = t % nchunks;
    const int c0 = ch * CH, n = min(CH, ND - c0);
    for (int c = threadIdx.x; c < n; c += blockDim.x) {
      int64_t h = 0;
#pragma unroll
      for (int e = 0; e < K; ++e) h += buf[(s * K + e) * CH + c];
      W[(int64_t)u * ND + c0 + c] = h;
    }
    __syncthreads();
  }
}

template <class F>
float timeit(F f, int reps) {
  cudaEvent_t a, b; cudaEventCreate(&a); cudaEventCreate(&b);
  f(); cudaDeviceSynchronize();
  cudaEventRecord(a);
  for (int i = 0; i < reps; ++i) f();
  cudaEventRecord(b); cudaEventSynchronize(b);
  float ms; cudaEventElapsedTime(&ms, a, b); return ms / reps;
}

int main() {
  int sms = 0; cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0);
  std::vector<int> h(NU * K);
  uint64_t s = 12345;
  for (auto& x : h) { s = s * 6364136223846793005ull + 1442695040888963407ull; x = (int)((s >> 33) % NU); }
  int64_t *X, *W; int *nbr, *flag;
  CK(cudaMalloc(&X, (size_t)NU * ND * 8)); CK(cudaMalloc(&W, (size_t)NU * ND * 8));
  CK(cudaMalloc(&nbr, h.size() * 4)); CK(cudaMalloc(&flag, 4));
  CK(cudaMemcpy(nbr, h.data(), h.size() * 4, cudaMemcpyHostToDevice));
  CK(cudaMemset(X, 1, (size_t)NU * ND * 8)); CK(cudaMemset(flag, 0, 4));
  const double bytes = (double)NU * ND * 8 * K;
  auto rep = [&](const char* name, float ms) {
    printf("%-34s %8.1f us   gather %7.1f GB/s  (%.2f B/clk/SM at 2.07 GHz)\n", name, ms * 1e3, bytes / (ms * 1e-3) / 1e9,
           bytes / (ms * 1e-3) / sms / 2.07e9);
  };
  for (int th : {256, 512, 864, 1024}) {
    for (int ctas : {1, 2, 4}) {
      if (th * ctas > 2048) continue;
      char name[64]; snprintf(name, 64, "A R=1 %4d thr x %d CTA/SM", th, ctas);
      rep(name, timeit([&] { kA<1><<<sms * ctas, th>>>(X, nbr, W); }, 10));
    }
  }
  rep("A R=2 864 thr x 1", timeit([&] { kA<2><<<sms, 864>>>(X, nbr, W); }, 10));
  rep("A R=2 512 thr x 2", timeit([&] { kA<2><<<sms * 2, 512>>>(X, nbr, W); }, 10));
  for (int th : {256, 512, 1024}) for (int ctas : {1, 2, 4}) {
    if (th * ctas > 2048) continue;
    char name[64]; snprintf(name, 64, "B 16B %4d thr x %d CTA/SM", th, ctas);
    rep(name, timeit([&] { kB<<<sms * ctas, th>>>(X, nbr, W); }, 10));
  }
  const size_t smemC = 2 * K * CH * 8 + 16;
  CK(cudaFuncSetAttribute(kC, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smemC));
  for (int ctas : {1, 2, 3}) {
    char name[64]; snprintf(name, 64, "C bulk 512 thr x %d CTA/SM", ctas);
    rep(name, timeit([&] { kC<<<sms * ctas, 512, smemC>>>(X, nbr, W, flag); }, 10));
  }
  CK(cudaGetLastError()); CK(cudaDeviceSynchronize());
  int hf = 0; CK(cudaMemcpy(&hf, flag, 4, cudaMemcpyDeviceToHost));
  printf("bulk wait timeouts: %d\n", hf);
  return 0;
}
