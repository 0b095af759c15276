// Throughput microbenchmarks for the arithmetic pipes that an FP64 sparse matvec can use.
// Every kernel: grid-stride free, fixed trip count, independent accumulator chains, result
// written to out[tid] so nothing is dead code. All indices < blocks*threads = size of out.
#include <cstdio>
#include <cstdint>
#include <cuda_runtime.h>

#define CK(x) do { cudaError_t e = (x); if (e != cudaSuccess) { printf("CUDA %s at %d\n", cudaGetErrorString(e), __LINE__); return 1; } } while (0)

constexpr int ITERS = 4096;
constexpr int CH = 8;

__global__ void k_dfma(double* out, double b, double c) {
  double a[CH];
  for (int i = 0; i < CH; ++i) a[i] = threadIdx.x * 1e-9 + i;
  for (int it = 0; it < ITERS; ++it)
#pragma unroll
    for (int i = 0; i < CH; ++i) a[i] = fma(a[i], b, c);
  double s = 0; for (int i = 0; i < CH; ++i) s += a[i];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}
__global__ void k_dadd(double* out, double b, double c) {
  double a[CH];
  for (int i = 0; i < CH; ++i) a[i] = threadIdx.x * 1e-9 + i;
  for (int it = 0; it < ITERS; ++it)
#pragma unroll
    for (int i = 0; i < CH; ++i) a[i] = a[i] + b;
  double s = 0; for (int i = 0; i < CH; ++i) s += a[i];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s + c;
}
__global__ void k_ffma(double* out, float b, float c) {
  float a[CH];
  for (int i = 0; i < CH; ++i) a[i] = threadIdx.x * 1e-9f + i;
  for (int it = 0; it < ITERS; ++it)
#pragma unroll
    for (int i = 0; i < CH; ++i) a[i] = fmaf(a[i], b, c);
  float s = 0; for (int i = 0; i < CH; ++i) s += a[i];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}
__global__ void k_iadd64(double* out, long long b, long long c) {
  long long a[CH];
  for (int i = 0; i < CH; ++i) a[i] = threadIdx.x + i * 977;
  for (int it = 0; it < ITERS; ++it)
#pragma unroll
    for (int i = 0; i < CH; ++i) a[i] = a[i] + (b ^ (long long)it);
  long long s = 0; for (int i = 0; i < CH; ++i) s += a[i];
  out[blockIdx.x * blockDim.x + threadIdx.x] = (double)(s + c);
}
__global__ void k_iadd32(double* out, int b, int c) {
  int a[CH];
  for (int i = 0; i < CH; ++i) a[i] = threadIdx.x + i * 977;
  for (int it = 0; it < ITERS; ++it)
#pragma unroll
    for (int i = 0; i < CH; ++i) a[i] = a[i] + (b ^ it);
  int s = 0; for (int i = 0; i < CH; ++i) s += a[i];
  out[blockIdx.x * blockDim.x + threadIdx.x] = (double)(s + c);
}
__global__ void k_imad32(double* out, int b, int c) {
  int a[CH];
  for (int i = 0; i < CH; ++i) a[i] = threadIdx.x + i * 977;
  for (int it = 0; it < ITERS; ++it)
#pragma unroll
    for (int i = 0; i < CH; ++i) a[i] = a[i] * b + c;
  int s = 0; for (int i = 0; i < CH; ++i) s += a[i];
  out[blockIdx.x * blockDim.x + threadIdx.x] = (double)s;
}
__global__ void k_mul64hi(double* out, unsigned long long b, unsigned long long c) {
  unsigned long long a[CH];
  for (int i = 0; i < CH; ++i) a[i] = threadIdx.x * 0x9E3779B97F4A7C15ull + i;
  for (int it = 0; it < ITERS; ++it)
#pragma unroll
    for (int i = 0; i < CH; ++i) a[i] = __umul64hi(a[i], b) + c;
  unsigned long long s = 0; for (int i = 0; i < CH; ++i) s += a[i];
  out[blockIdx.x * blockDim.x + threadIdx.x] = (double)s;
}
__global__ void k_cvt_s64_f64(double* out, long long b, double c) {
  // int64 -> f64 conversion chain: a = (double)(ia) ; ia = bits-ish update via integer op
  long long ia[CH];
  double acc[CH];
  for (int i = 0; i < CH; ++i) { ia[i] = threadIdx.x + i; acc[i] = 0; }
  for (int it = 0; it < ITERS; ++it)
#pragma unroll
    for (int i = 0; i < CH; ++i) { double d = __ll2double_rn(ia[i]); ia[i] += b ^ __double_as_longlong(d); }
  double s = 0; for (int i = 0; i < CH; ++i) s += acc[i] + (double)ia[i];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s + c;
}
__global__ void k_cvt_f64_s64(double* out, double b, long long c) {
  double a[CH];
  long long acc[CH];
  for (int i = 0; i < CH; ++i) { a[i] = threadIdx.x + i + 0.5; acc[i] = 0; }
  for (int it = 0; it < ITERS; ++it)
#pragma unroll
    for (int i = 0; i < CH; ++i) { acc[i] ^= __double2ll_rn(a[i]); a[i] = __longlong_as_double(__double_as_longlong(a[i]) + 1); }
  long long s = 0; for (int i = 0; i < CH; ++i) s += acc[i];
  out[blockIdx.x * blockDim.x + threadIdx.x] = (double)(s + c);
}
__global__ void k_popc64(double* out, unsigned long long b, int c) {
  unsigned long long a[CH]; int acc[CH];
  for (int i = 0; i < CH; ++i) { a[i] = threadIdx.x * 0x9E3779B97F4A7C15ull + i; acc[i] = 0; }
  for (int it = 0; it < ITERS; ++it)
#pragma unroll
    for (int i = 0; i < CH; ++i) { acc[i] += __popcll(a[i]); a[i] = (a[i] ^ b) + acc[i]; }
  int s = 0; for (int i = 0; i < CH; ++i) s += acc[i];
  out[blockIdx.x * blockDim.x + threadIdx.x] = (double)(s + c);
}
__global__ void k_mul128(double* out, long long b, long long c) {
  long long lo[CH], hi[CH];
  for (int i = 0; i < CH; ++i) { lo[i] = threadIdx.x * 0x9E3779B97F4A7C1ll + i; hi[i] = 0; }
  for (int it = 0; it < ITERS; ++it)
#pragma unroll
    for (int i = 0; i < CH; ++i) { long long l = lo[i] * b; long long h = __mul64hi(lo[i], b); lo[i] = l + c; hi[i] += h; }
  long long s = 0; for (int i = 0; i < CH; ++i) s += lo[i] + hi[i];
  out[blockIdx.x * blockDim.x + threadIdx.x] = (double)s;
}
// streaming copy for HBM bandwidth; n doubles, grid-stride
__global__ void k_copy(const double2* __restrict__ a, double2* __restrict__ b, size_t n2) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n2; i += (size_t)gridDim.x * blockDim.x) b[i] = a[i];
}
// L2 read bandwidth: repeatedly read a buffer of m double2 (fits in L2)
__global__ void k_l2read(const double2* __restrict__ a, size_t m2, int reps, double* out) {
  long long si = 0;
  for (int r = 0; r < reps; ++r)
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < m2; i += (size_t)gridDim.x * blockDim.x) {
      double2 v = __ldcg(a + i); si ^= __double_as_longlong(v.x) + __double_as_longlong(v.y);
    }
  out[blockIdx.x * blockDim.x + threadIdx.x] = (double)si;
}

template <class F>
float timeit(F f) {
  cudaEvent_t e0, e1; cudaEventCreate(&e0); cudaEventCreate(&e1);
  f(); cudaDeviceSynchronize();
  cudaEventRecord(e0); f(); cudaEventRecord(e1); cudaEventSynchronize(e1);
  float ms; cudaEventElapsedTime(&ms, e0, e1); return ms;
}

int main() {
  cudaDeviceProp p; CK(cudaGetDeviceProperties(&p, 0));
  int clk = 0; cudaDeviceGetAttribute(&clk, cudaDevAttrClockRate, 0);
  printf("device %s SMs %d cc %d.%d clock %d kHz L2 %d B smem/blk optin %zu\n", p.name, p.multiProcessorCount, p.major, p.minor, clk, p.l2CacheSize, p.sharedMemPerBlockOptin);
  const int blocks = p.multiProcessorCount * 8, threads = 256;
  double* out; CK(cudaMalloc(&out, sizeof(double) * blocks * threads));
  const double ops = (double)blocks * threads * ITERS * CH;
  auto rep = [&](const char* name, float ms) {
    double gops = ops / (ms * 1e-3) / 1e9;
    printf("%-14s %8.3f ms  %10.1f Gop/s  %7.2f op/clk/SM (at %d MHz)\n", name, ms, gops, gops * 1e9 / p.multiProcessorCount / (clk * 1e3), clk / 1000);
  };
  rep("dfma", timeit([&] { k_dfma<<<blocks, threads>>>(out, 1.0000001, 1e-9); }));
  rep("dadd", timeit([&] { k_dadd<<<blocks, threads>>>(out, 1.0000001, 1e-9); }));
  rep("ffma", timeit([&] { k_ffma<<<blocks, threads>>>(out, 1.0000001f, 1e-9f); }));
  rep("iadd32", timeit([&] { k_iadd32<<<blocks, threads>>>(out, 12345, 7); }));
  rep("iadd64", timeit([&] { k_iadd64<<<blocks, threads>>>(out, 1234567890123ll, 7); }));
  rep("imad32", timeit([&] { k_imad32<<<blocks, threads>>>(out, 12345, 7); }));
  rep("umul64hi", timeit([&] { k_mul64hi<<<blocks, threads>>>(out, 0x9E3779B97F4A7C15ull, 7); }));
  rep("cvt_s64->f64", timeit([&] { k_cvt_s64_f64<<<blocks, threads>>>(out, 1234567ll, 0.5); }));
  rep("cvt_f64->s64", timeit([&] { k_cvt_f64_s64<<<blocks, threads>>>(out, 0.5, 7); }));
  rep("mul64x64->128", timeit([&] { k_mul128<<<blocks, threads>>>(out, 0x1234567890ll, 7); }));
  rep("popc64", timeit([&] { k_popc64<<<blocks, threads>>>(out, 0x5555ull, 7); }));
  CK(cudaGetLastError());
  // HBM copy, 2 GiB each way
  size_t n2 = (size_t)1 << 27;  // double2 count = 2 GiB
  double2 *a, *b; CK(cudaMalloc(&a, n2 * 16)); CK(cudaMalloc(&b, n2 * 16));
  CK(cudaMemset(a, 0, n2 * 16));
  float ms = timeit([&] { k_copy<<<p.multiProcessorCount * 16, 512>>>(a, b, n2); });
  printf("hbm copy       %8.3f ms  %10.1f GB/s (read+write)\n", ms, 2.0 * n2 * 16 / (ms * 1e-3) / 1e9);
  for (size_t mb : {16, 48, 96}) {
    size_t m2 = mb * (1 << 20) / 16; int reps = 20;
    double* o2; CK(cudaMalloc(&o2, sizeof(double) * p.multiProcessorCount * 8 * 512));
    ms = timeit([&] { k_l2read<<<p.multiProcessorCount * 8, 512>>>(a, m2, reps, o2); });
    printf("l2 read %3zu MB %8.3f ms  %10.1f GB/s\n", mb, ms, (double)reps * m2 * 16 / (ms * 1e-3) / 1e9);
    cudaFree(o2);
  }
  CK(cudaGetLastError());
  CK(cudaDeviceSynchronize());
  return 0;
}
