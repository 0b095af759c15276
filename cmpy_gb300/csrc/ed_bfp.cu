// Block-fixed-point (BFP) Lanczos for fermionic sectors with one hopping magnitude.
//
// Why: on GB300 the FP64 pipe issues ~1.6 operations per clock per SM (measured), about 60x
// fewer than INT32 adds, while a Hubbard matvec needs ~16 FP64 operations per 16 bytes of
// HBM traffic — an FP64 matvec would run at <10% of HBM bandwidth. Here a Lanczos vector is
// stored as int64 mantissas with one power-of-two exponent per vector (value = m * 2^e):
//   * matvec: W = diag_int * X + t_int * sum(+-X_nbr) — exact int64 arithmetic;
//   * alpha, norms: exact 128-bit integer dot products, reduced to FP64 per thread;
//   * three-term update: 128-bit fixed-point products with one rounding per element;
//   * FP64 only for the scalars (alpha, beta, the tridiagonal solve).
// The vector stored for step k is the unnormalised residual r_k (||r_k|| = beta_k), so the
// normalisation 1/beta_k is folded into the scalar coefficients and needs no pass of its own.
// Per Lanczos step: one matvec kernel (+ alpha) and one update kernel (+ norm) — 48 B/element.
//
// Reductions are deterministic (fixed grid, per-block partials, last-block sum in block order).
#include <algorithm>
#include <atomic>
#include <cmath>
#include <vector>

#include "ed_lzcheck.cuh"
#include "ed_plan.cuh"
#include "ed_stripe_tables.h"
#include "ed_sweep_tables.h"
#include "ed_tridiag.cuh"

namespace ed {

// ---- 128-bit helpers ------------------------------------------------------------------------
struct I128 {
  uint64_t lo;
  int64_t hi;
};

__device__ __forceinline__ I128 mul_s64(int64_t a, int64_t b) {
  I128 r;
  r.lo = (uint64_t)a * (uint64_t)b;
  r.hi = __mul64hi(a, b);
  return r;
}

__device__ __forceinline__ void add128(I128& acc, const I128& v) {
  asm("add.cc.u64 %0, %0, %2;\n\taddc.u64 %1, %1, %3;"
      : "+l"(acc.lo), "+l"(acc.hi)
      : "l"(v.lo), "l"(v.hi));
}

__device__ __forceinline__ double i128_to_double(const I128& v) {
  return fma((double)v.hi, 0x1.0p64, (double)v.lo);
}

// round-to-nearest arithmetic right shift of a 128-bit value by 1 <= s <= 63, result in int64
__device__ __forceinline__ int64_t shr128_round(I128 v, int s) {
  I128 h;
  h.lo = 1ull << (s - 1);
  h.hi = 0;
  add128(v, h);
  return (int64_t)((v.lo >> s) | ((uint64_t)v.hi << (64 - s)));
}

__device__ __forceinline__ unsigned long long uabs64(int64_t v) {
  return v < 0 ? (unsigned long long)(-v) : (unsigned long long)v;
}

// ---- shared per-solve state --------------------------------------------------------------------
struct BfpState {
  int stop;            // 0 running, 1 converged, 2 invariant subspace
  int steps;
  int status;
  int pad;
  // update coefficients for the current step (written by the matvec's last block)
  int64_t A_w, A_q, A_p;
  int SA;
  int ew;              // exponent of W
  unsigned long long maxw;
  double energy, residual, e_prev;
  unsigned int ticket[4];
};

struct BfpVecs {
  int64_t* R;          // vectors, slot stride D
  int32_t* eR;         // exponent per Lanczos index
  unsigned long long* maxR;  // max |mantissa| per Lanczos index
  int store;           // 1: slot k = index k; 0: ring of 3
  int64_t D;
  __host__ __device__ __forceinline__ int64_t* vec(int k) const { return R + (int64_t)(store ? k : (k % 3)) * D; }
};

__device__ void bfp_scalars_tail(BfpVecs v, int k, int F, int m_in, double t, unsigned long long m, double* alpha,
                                 const double* beta, BfpState* st);

// Lanczos-step scalars folded into the last CTA of the matvec (when `on`)
struct BfpFuse {
  BfpVecs v;
  int k, F, m_in, on;
  double* alpha;
  const double* beta;
};

constexpr int BT = 256;  // block size of the streaming kernels

template <int NT>
__device__ __forceinline__ unsigned long long block_max_u64(unsigned long long v, unsigned long long* sm) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) sm[w] = v;
  __syncthreads();
  unsigned long long r = 0;
  if (w == 0) {
    r = (l < NT / 32) ? sm[l] : 0ull;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) r = max(r, __shfl_xor_sync(0xffffffffu, r, o));
  }
  return r;
}

__device__ __forceinline__ bool bfp_last_block(unsigned int* ticket) {
  __shared__ bool am_last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) am_last = (atomicAdd(ticket, 1u) == gridDim.x - 1);
  __syncthreads();
  if (am_last) __threadfence();
  return am_last;
}

// ---- conversion FP64 <-> BFP ------------------------------------------------------------------
__global__ void k_maxabs_f64(const double* __restrict__ x, int64_t n, unsigned long long* out) {
  __shared__ unsigned long long sm[BT / 32];
  unsigned long long m = 0;
  for (int64_t i = blockIdx.x * (int64_t)BT + threadIdx.x; i < n; i += (int64_t)gridDim.x * BT) {
    const double v = x[i];
    unsigned long long b = (unsigned long long)__double_as_longlong(fabs(v));
    if (!isfinite(v)) b = 0x7FF0000000000000ull;
    m = max(m, b);
  }
  m = block_max_u64<BT>(m, sm);
  if (threadIdx.x == 0) atomicMax(out, m);
}

// xm = round(x * 2^-e) with e chosen so that max|xm| < 2^m_in
__global__ void k_f64_to_bfp(const double* __restrict__ x, int64_t n, const unsigned long long* maxbits, int m_in,
                             int64_t* __restrict__ xm, int32_t* e_out, unsigned long long* max_out) {
  const double mx = __longlong_as_double((long long)*maxbits);
  int e2 = 0;
  frexp(mx, &e2);  // mx < 2^e2
  const int e = e2 - m_in;
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    *e_out = e;
    *max_out = (unsigned long long)llrint(ldexp(mx, -e));
  }
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    xm[i] = llrint(ldexp(x[i], -e));
}

__global__ void k_bfp_to_f64(const int64_t* __restrict__ xm, const int32_t* e, int64_t n, double* __restrict__ x) {
  const int ee = *e;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    x[i] = ldexp((double)xm[i], ee);
}

// ||R||^2 (exact per thread) -> beta[k]; also used for the start vector
__global__ void k_bfp_norm(BfpVecs v, int k, double* partial, BfpState* st, double* beta) {
  __shared__ double sm[BT / 32];
  const int64_t* x = v.vec(k);
  I128 acc{0, 0};
  for (int64_t i = blockIdx.x * (int64_t)BT + threadIdx.x; i < v.D; i += (int64_t)gridDim.x * BT)
    add128(acc, mul_s64(x[i], x[i]));
  double s = block_sum<BT>(i128_to_double(acc), sm);
  if (threadIdx.x == 0) partial[blockIdx.x] = s;
  if (bfp_last_block(&st->ticket[0])) {
    double t = 0.0;
    for (int b = threadIdx.x; b < (int)gridDim.x; b += BT) t += ((volatile double*)partial)[b];
    t = block_sum<BT>(t, sm);
    if (threadIdx.x == 0) {
      beta[k] = ldexp(sqrt(t), v.eR[k]);
      st->ticket[0] = 0;
    }
  }
}

// ---- the matvec ----------------------------------------------------------------------------------
struct BfpHubArgs {
  int64_t nu, nd;
  const int32_t* up_off; const int32_t* up_npos; const int32_t* up_idx;
  const uint16_t* dn_tab; int max_dn;
  const uint64_t* up_states; const uint64_t* dn_states;
  const int32_t* e_up; const int32_t* e_dn;
  int u_uniform; int32_t u0; int32_t u[ED_MAX_SITES + 2];
  int32_t t_int; int F;
  // diagonal mode 1 (arbitrary FP64 energies): int64 fixed point, shift = Fd - F
  const int64_t* e_up_fx; const int64_t* e_dn_fx;
  int64_t u0_fx; int64_t u_fx[ED_MAX_SITES + 2];
  int dshift;
};

__device__ __forceinline__ int32_t bfp_uterm(const BfpHubArgs& a, uint64_t both) {
  if (a.u_uniform) return a.u0 * __popcll(both);
  int32_t v = 0;
  while (both) {
    v += a.u[__ffsll((long long)both) - 1];
    both &= both - 1;
  }
  return v;
}

__device__ __forceinline__ int64_t bfp_uterm64(const BfpHubArgs& a, uint64_t both) {
  if (a.u_uniform) return a.u0_fx * (int64_t)__popcll(both);
  int64_t v = 0;
  while (both) {
    v += a.u_fx[__ffsll((long long)both) - 1];
    both &= both - 1;
  }
  return v;
}

// diagonal term D(x) of one element in units of the output grid
template <bool DIAG64>
__device__ __forceinline__ int64_t bfp_diag_term(const BfpHubArgs& a, int64_t row_e32, int64_t row_e64,
                                                 uint64_t su, int64_t d, int64_t x) {
  const uint64_t both = su & __ldg(a.dn_states + d);
  if (!DIAG64) {
    const int32_t dg = (int32_t)row_e32 + __ldg(a.e_dn + d) + bfp_uterm(a, both);
    return (int64_t)dg * x;
  } else {
    const int64_t dg = row_e64 + __ldg(a.e_dn_fx + d) + bfp_uterm64(a, both);
    return shr128_round(mul_s64(dg, x), a.dshift);
  }
}

// One CTA per target up-row (grid-stride). The row is staged in shared memory with its
// negation (dn-hop gathers pick the signed slot), up-neighbour rows stream from global.
// Epilogue: exact alpha partial <X, W> and max|W|. When x_scale != null the kernel is the
// public ed_matvec_fixed (no Lanczos scalars).
template <int NT, bool VEC2, bool DIAG64>
__global__ void __launch_bounds__(NT) k_bfp_hub_matvec(BfpHubArgs a, const int64_t* __restrict__ X,
                                                      int64_t* __restrict__ W, double* partial,
                                                      unsigned long long* partial_max, BfpState* st) {
  if (st && *(volatile int*)&st->stop) return;
  extern __shared__ int64_t xs[];  // [2*nd + 1]
  __shared__ double smd[NT / 32];
  __shared__ unsigned long long smu[NT / 32];
  const int64_t nd = a.nd;
  if (threadIdx.x == 0) xs[2 * nd] = 0;
  I128 dot{0, 0};
  unsigned long long mx = 0;
  for (int64_t row = blockIdx.x; row < a.nu; row += gridDim.x) {
    const int64_t* xrow = X + row * nd;
    for (int64_t d = threadIdx.x; d < nd; d += NT) {
      const int64_t v = __ldg(xrow + d);
      xs[d] = v;
      xs[nd + d] = -v;
    }
    __syncthreads();
    const int32_t o0 = __ldg(a.up_off + row), o1 = __ldg(a.up_off + row + 1);
    const int32_t op = o0 + __ldg(a.up_npos + row);
    const uint64_t su = __ldg(a.up_states + row);
    const int64_t eu = DIAG64 ? 0 : (int64_t)__ldg(a.e_up + row);
    const int64_t eu64 = DIAG64 ? __ldg(a.e_up_fx + row) : 0;
    if (VEC2) {
      for (int64_t d = 2 * threadIdx.x; d < nd; d += 2 * NT) {
        int64_t h0 = 0, h1 = 0;
        for (int32_t e = o0; e < op; ++e) {
          const longlong2 v = __ldg((const longlong2*)(X + (int64_t)__ldg(a.up_idx + e) * nd + d));
          h0 += v.x;
          h1 += v.y;
        }
        for (int32_t e = op; e < o1; ++e) {
          const longlong2 v = __ldg((const longlong2*)(X + (int64_t)__ldg(a.up_idx + e) * nd + d));
          h0 -= v.x;
          h1 -= v.y;
        }
        const uint32_t* tab = (const uint32_t*)a.dn_tab;
        for (int e = 0; e < a.max_dn; ++e) {
          const uint32_t sl = __ldg(tab + ((int64_t)e * nd + d) / 2);
          h0 += xs[sl & 0xFFFFu];
          h1 += xs[sl >> 16];
        }
        const int64_t x0 = xs[d], x1 = xs[d + 1];
        const int64_t w0 = (int64_t)a.t_int * h0 + bfp_diag_term<DIAG64>(a, eu, eu64, su, d, x0);
        const int64_t w1 = (int64_t)a.t_int * h1 + bfp_diag_term<DIAG64>(a, eu, eu64, su, d + 1, x1);
        *(longlong2*)(W + row * nd + d) = make_longlong2(w0, w1);
        add128(dot, mul_s64(x0, w0));
        add128(dot, mul_s64(x1, w1));
        mx = max(mx, max(uabs64(w0), uabs64(w1)));
      }
    } else {
      for (int64_t d = threadIdx.x; d < nd; d += NT) {
        int64_t h = 0;
        for (int32_t e = o0; e < op; ++e) h += __ldg(X + (int64_t)__ldg(a.up_idx + e) * nd + d);
        for (int32_t e = op; e < o1; ++e) h -= __ldg(X + (int64_t)__ldg(a.up_idx + e) * nd + d);
        for (int e = 0; e < a.max_dn; ++e) h += xs[__ldg(a.dn_tab + (int64_t)e * nd + d)];
        const int64_t x0 = xs[d];
        const int64_t w0 = (int64_t)a.t_int * h + bfp_diag_term<DIAG64>(a, eu, eu64, su, d, x0);
        W[row * nd + d] = w0;
        add128(dot, mul_s64(x0, w0));
        mx = max(mx, uabs64(w0));
      }
    }
    __syncthreads();
  }
  if (!partial) return;
  const double s = block_sum<NT>(i128_to_double(dot), smd);
  const unsigned long long m = block_max_u64<NT>(mx, smu);
  if (threadIdx.x == 0) {
    partial[blockIdx.x] = s;
    partial_max[blockIdx.x] = m;
  }
}

// ---- matvec v2: one 1024-thread CTA per SM, dn table resident in shared memory ----------------
// Each CTA keeps the whole dn slot table (max_dn x nd/2 packed slot pairs) in shared memory for
// its lifetime and processes MR target rows per iteration, so each table word serves MR rows.
// The input X is read with an L2 evict_last policy (every row is re-read by ~8 target rows) and
// W is written with evict_first, so the streaming output does not push X out of L2.
constexpr int MV2_NT = 1024;
constexpr int MV2_R = 2;
// the kernel's static shared memory (two warp-partial arrays) plus slack
constexpr size_t MV2_STATIC_SMEM = 2 * (MV2_NT / 32) * 8 + 512;

__device__ __forceinline__ uint64_t policy_evict_last() {
  uint64_t p;
  asm("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
  return p;
}
__device__ __forceinline__ uint64_t policy_evict_first() {
  uint64_t p;
  asm("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
  return p;
}
__device__ __forceinline__ longlong2 ld2_keep(const int64_t* p, uint64_t pol) {
  longlong2 v;
  asm volatile("ld.global.nc.L2::cache_hint.v2.s64 {%0, %1}, [%2], %3;"
               : "=l"(v.x), "=l"(v.y)
               : "l"(p), "l"(pol));
  return v;
}
__device__ __forceinline__ void st2_stream(int64_t* p, int64_t a, int64_t b, uint64_t pol) {
  asm volatile("st.global.L2::cache_hint.v2.s64 [%0], {%1, %2}, %3;" ::"l"(p), "l"(a), "l"(b), "l"(pol) : "memory");
}

template <bool DIAG64>
__global__ void __launch_bounds__(MV2_NT, 1) k_bfp_hub_matvec2(BfpHubArgs a, const int64_t* __restrict__ X,
                                                              int64_t* __restrict__ W, double* partial,
                                                              unsigned long long* partial_max, BfpState* st) {
  if (st && *(volatile int*)&st->stop) return;
  extern __shared__ int64_t smem[];
  __shared__ double smd[MV2_NT / 32];
  __shared__ unsigned long long smu[MV2_NT / 32];
  const int64_t nd = a.nd;
  const int np = (int)(nd / 2);                       // column pairs
  const int xstride = (int)(2 * nd + 2);              // +/- row copy and a zero slot, 16-byte aligned
  int64_t* xs = smem;                                 // [MV2_R][xstride]
  uint32_t* tab = (uint32_t*)(smem + MV2_R * xstride);  // [max_dn][np]
  const uint32_t* gtab = (const uint32_t*)a.dn_tab;
  for (int i = threadIdx.x; i < a.max_dn * np; i += MV2_NT) tab[i] = __ldg(gtab + i);
  for (int r = threadIdx.x; r < MV2_R; r += MV2_NT) { xs[r * xstride + 2 * nd] = 0; xs[r * xstride + 2 * nd + 1] = 0; }
  const uint64_t keep = policy_evict_last(), stream = policy_evict_first();
  I128 dot{0, 0};
  unsigned long long mx = 0;
  for (int64_t row0 = (int64_t)blockIdx.x * MV2_R; row0 < a.nu; row0 += (int64_t)gridDim.x * MV2_R) {
    const int nr = (int)min((int64_t)MV2_R, a.nu - row0);
    __syncthreads();
    for (int r = 0; r < nr; ++r) {
      const int64_t* xrow = X + (row0 + r) * nd;
      int64_t* xr = xs + r * xstride;
      for (int p = threadIdx.x; p < np; p += MV2_NT) {
        const longlong2 v = ld2_keep(xrow + 2 * p, keep);
        *(longlong2*)(xr + 2 * p) = v;
        *(longlong2*)(xr + nd + 2 * p) = make_longlong2(-v.x, -v.y);
      }
    }
    __syncthreads();
    int32_t o0[MV2_R], o1[MV2_R], op[MV2_R];
    uint64_t su[MV2_R];
    int64_t eu[MV2_R], eu64[MV2_R];
#pragma unroll
    for (int r = 0; r < MV2_R; ++r) {
      const int64_t row = r < nr ? row0 + r : row0;
      o0[r] = __ldg(a.up_off + row);
      o1[r] = r < nr ? __ldg(a.up_off + row + 1) : o0[r];
      op[r] = r < nr ? o0[r] + __ldg(a.up_npos + row) : o0[r];
      su[r] = __ldg(a.up_states + row);
      eu[r] = DIAG64 ? 0 : (int64_t)__ldg(a.e_up + row);
      eu64[r] = DIAG64 ? __ldg(a.e_up_fx + row) : 0;
    }
    for (int p = threadIdx.x; p < np; p += MV2_NT) {
      const int64_t d = 2 * p;
      int64_t h0[MV2_R], h1[MV2_R];
#pragma unroll
      for (int r = 0; r < MV2_R; ++r) {
        h0[r] = 0;
        h1[r] = 0;
        // four independent row loads in flight per iteration (memory-level parallelism)
        int32_t e = o0[r];
        for (; e + 4 <= op[r]; e += 4) {
          longlong2 v[4];
#pragma unroll
          for (int q = 0; q < 4; ++q) v[q] = ld2_keep(X + (int64_t)__ldg(a.up_idx + e + q) * nd + d, keep);
#pragma unroll
          for (int q = 0; q < 4; ++q) { h0[r] += v[q].x; h1[r] += v[q].y; }
        }
        for (; e < op[r]; ++e) {
          const longlong2 v = ld2_keep(X + (int64_t)__ldg(a.up_idx + e) * nd + d, keep);
          h0[r] += v.x;
          h1[r] += v.y;
        }
        for (; e + 4 <= o1[r]; e += 4) {
          longlong2 v[4];
#pragma unroll
          for (int q = 0; q < 4; ++q) v[q] = ld2_keep(X + (int64_t)__ldg(a.up_idx + e + q) * nd + d, keep);
#pragma unroll
          for (int q = 0; q < 4; ++q) { h0[r] -= v[q].x; h1[r] -= v[q].y; }
        }
        for (; e < o1[r]; ++e) {
          const longlong2 v = ld2_keep(X + (int64_t)__ldg(a.up_idx + e) * nd + d, keep);
          h0[r] -= v.x;
          h1[r] -= v.y;
        }
      }
      for (int e = 0; e < a.max_dn; ++e) {
        const uint32_t sl = tab[e * np + p];
        const int s0 = (int)(sl & 0xFFFFu), s1 = (int)(sl >> 16);
#pragma unroll
        for (int r = 0; r < MV2_R; ++r) {
          h0[r] += xs[r * xstride + s0];
          h1[r] += xs[r * xstride + s1];
        }
      }
#pragma unroll
      for (int r = 0; r < MV2_R; ++r) {
        if (r < nr) {
          const int64_t x0 = xs[r * xstride + d], x1 = xs[r * xstride + d + 1];
          const int64_t w0 = (int64_t)a.t_int * h0[r] + bfp_diag_term<DIAG64>(a, eu[r], eu64[r], su[r], d, x0);
          const int64_t w1 = (int64_t)a.t_int * h1[r] + bfp_diag_term<DIAG64>(a, eu[r], eu64[r], su[r], d + 1, x1);
          st2_stream(W + (row0 + r) * nd + d, w0, w1, stream);
          add128(dot, mul_s64(x0, w0));
          add128(dot, mul_s64(x1, w1));
          mx = max(mx, max(uabs64(w0), uabs64(w1)));
        }
      }
    }
  }
  if (!partial) return;
  const double s = block_sum<MV2_NT>(i128_to_double(dot), smd);
  const unsigned long long m = block_max_u64<MV2_NT>(mx, smu);
  if (threadIdx.x == 0) {
    partial[blockIdx.x] = s;
    partial_max[blockIdx.x] = m;
  }
}

// ---- matvec v3: bulk-copied rows, interleaved row pair, bond-major dn gathers -------------------
// One persistent CTA per SM walks groups of MV3_R = 2 target rows. A bulk copy (cp.async.bulk,
// completion on an mbarrier) brings the two rows of the NEXT group into a landing buffer while
// the CTA computes the current group from an interleaved copy xs2[c] = (row0[c], row1[c]), so one
// 16-byte shared load gathers a dn partner for both rows. Each thread owns columns
// c = tid + j*blockDim (lane-contiguous), so the gathers of one bond read nearly contiguous
// partner columns; one 32-bit table word holds the partner slots of two bonds.
// Up-neighbour rows stream from L2 (coalesced 8-byte loads, evict_last policy), eight loads in
// flight per thread; the neighbour lists are padded to multiples of 8 with the target row itself
// and the padding is subtracted once (exact integer arithmetic).
constexpr int MV3_R = 2;
constexpr int MV3_MAXNT = 896;  // 28 warps: up to 72 registers per thread with one CTA per SM
constexpr size_t MV3_STATIC_SMEM = 2 * (MV3_MAXNT / 32) * 8 + 512;
constexpr long MV3_WAIT_LIMIT = 1L << 22;  // bounded mbarrier polls before giving up

struct Mv3Layout {
  int lstride;  // int32 per staged up-list of one row: + segment, - segment, each padded to 4
  size_t raw_off, xs_off, tab_off, lst_off, cnt_off, bar_off, total;
};

__host__ __device__ inline Mv3Layout mv3_layout(int64_t nd, int n_b2, int max_up) {
  auto al = [](size_t v) { return (v + 127) & ~(size_t)127; };
  Mv3Layout L;
  L.lstride = ((max_up + 3) & ~3) + 4;
  // xs2 first: its base is the (constant) start of dynamic shared memory, so a gather address
  // is the table's byte offset plus an immediate
  L.xs_off = 0;                                                    // [nd + 1][MV3_R] interleaved
  L.raw_off = al(L.xs_off + (size_t)(nd + 1) * MV3_R * 8);         // [MV3_R][nd] landing rows
  L.tab_off = al(L.raw_off + (size_t)MV3_R * nd * 8);              // [n_b2][nd] slot pairs
  L.lst_off = al(L.tab_off + (size_t)n_b2 * nd * 4);               // [2][MV3_R][lstride]
  L.cnt_off = al(L.lst_off + (size_t)2 * MV3_R * L.lstride * 4);   // [2][MV3_R][4]
  L.bar_off = al(L.cnt_off + (size_t)2 * MV3_R * 4 * 4);
  L.total = L.bar_off + 8;
  return L;
}

__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// bounded wait for phase `parity` of an mbarrier; false when the limit ran out
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, unsigned parity) {
  for (long it = 0; it < MV3_WAIT_LIMIT; ++it)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}
// non-blocking test of an mbarrier phase
__device__ __forceinline__ bool mbar_test(uint64_t* bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// at most `limit` tests with a short sleep between them; false when the limit ran out
__device__ __forceinline__ bool mbar_wait_polls(uint64_t* bar, unsigned parity, long limit) {
  for (long it = 0; it < limit; ++it) {
    if (mbar_test(bar, parity)) return true;
    __nanosleep(32);
  }
  return false;
}

// global -> shared bulk copy (16-byte aligned, size a multiple of 16), completes on `bar`
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, unsigned bytes, uint64_t* bar, uint64_t pol) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1], %2, [%3], %4;" ::
          "r"(smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar)), "l"(pol)
      : "memory");
}
// read-only data (X is not written while the kernel runs), so the asm is not volatile: the
// compiler may batch these loads
__device__ __forceinline__ int64_t ld_keep(const int64_t* p, uint64_t pol) {
  int64_t v;
  asm("ld.global.nc.L2::cache_hint.s64 %0, [%1], %2;" : "=l"(v) : "l"(p), "l"(pol));
  return v;
}
__device__ __forceinline__ void st_stream(int64_t* p, int64_t v, uint64_t pol) {
  asm volatile("st.global.L2::cache_hint.s64 [%0], %1, %2;" ::"l"(p), "l"(v), "l"(pol) : "memory");
}

// block reductions for a runtime block size (a multiple of 32, at most MV3_MAXNT)
__device__ __forceinline__ double block_sum_rt(double v, double* sm) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = blockDim.x >> 5;
  __syncthreads();
  if (l == 0) sm[w] = v;
  __syncthreads();
  double r = 0.0;
  if (w == 0) {
    r = (l < nw) ? sm[l] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) r += __shfl_xor_sync(0xffffffffu, r, o);
  }
  return r;
}
__device__ __forceinline__ unsigned long long block_max_rt(unsigned long long v, unsigned long long* sm) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = blockDim.x >> 5;
  __syncthreads();
  if (l == 0) sm[w] = v;
  __syncthreads();
  unsigned long long r = 0;
  if (w == 0) {
    r = (l < nw) ? sm[l] : 0ull;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) r = max(r, __shfl_xor_sync(0xffffffffu, r, o));
  }
  return r;
}

// diagonal term of one element with the column's data already loaded
template <bool DIAG64>
__device__ __forceinline__ int64_t bfp_diag_col(const BfpHubArgs& a, int64_t row_e32, int64_t row_e64, uint64_t su,
                                                uint64_t sd, int32_t ed32, int64_t ed64, int64_t x) {
  const uint64_t both = su & sd;
  if (!DIAG64) {
    const int32_t dg = (int32_t)row_e32 + ed32 + bfp_uterm(a, both);
    return (int64_t)dg * x;
  } else {
    const int64_t dg = row_e64 + ed64 + bfp_uterm64(a, both);
    return shr128_round(mul_s64(dg, x), a.dshift);
  }
}

__device__ __forceinline__ longlong2 ld2_keep_nv(const int64_t* p, uint64_t pol) {
  longlong2 v;
  asm("ld.global.nc.L2::cache_hint.v2.s64 {%0, %1}, [%2], %3;" : "=l"(v.x), "=l"(v.y) : "l"(p), "l"(pol));
  return v;
}
// four 16-byte row loads (two adjacent columns) of the list entries lst[0..4), summed
__device__ __forceinline__ longlong2 sum4x2(const int64_t* xc, const int32_t* lst, uint64_t pol) {
  const int4 i = *(const int4*)lst;
  const longlong2 v0 = ld2_keep_nv(xc + i.x, pol), v1 = ld2_keep_nv(xc + i.y, pol), v2 = ld2_keep_nv(xc + i.z, pol),
                  v3 = ld2_keep_nv(xc + i.w, pol);
  return make_longlong2((v0.x + v1.x) + (v2.x + v3.x), (v0.y + v1.y) + (v2.y + v3.y));
}
// 64-bit warp shuffle
__device__ __forceinline__ int64_t shfl64(int64_t v, int src) {
  return (int64_t)__shfl_sync(0xffffffffu, (long long)v, src);
}

// the bulk copies of one row group (thread 0 of the v3 matvec; kept out of line so that the
// copy set-up does not take registers from the gather loops)
template <bool UPW>
__device__ __noinline__ void mv3_stage(int64_t g, int s, int64_t nu, int64_t nd, int lstride, const int64_t* X,
                                       const int32_t* up_lst, const int32_t* up_cnt, int64_t* raw, int32_t* lst,
                                       int32_t* cnt, uint64_t* bar) {
  const uint64_t keep = policy_evict_last();
  const int64_t u0 = g * MV3_R;
  const int nr = (int)min((int64_t)MV3_R, nu - u0);
  const unsigned row_bytes = (unsigned)(nd * 8);
  const unsigned lbytes = (unsigned)(MV3_R * lstride * 4), cbytes = (unsigned)(MV3_R * 4 * 4);
  // order this CTA's earlier generic-proxy reads of the buffers before the async-proxy writes
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  mbar_expect_tx(bar, row_bytes * nr + (UPW ? 0u : lbytes + cbytes));
  for (int r = 0; r < nr; ++r) bulk_g2s(raw + (size_t)r * nd, X + (u0 + r) * nd, row_bytes, bar, keep);
  if (!UPW) {
    bulk_g2s(lst + (size_t)s * MV3_R * lstride, up_lst + u0 * lstride, lbytes, bar, keep);
    bulk_g2s(cnt + (size_t)s * MV3_R * 4, up_cnt + u0 * 4, cbytes, bar, keep);
  }
}

// UPW: the up-neighbour sums were written into W by k_bfp_up_panels (two-pass H·v); the kernel
// reads them instead of gathering and overwrites W with the result (each element read, then
// written, by the same thread)
template <bool DIAG64, bool UPW, bool CMP = false>
__global__ void __launch_bounds__(MV3_MAXNT, 1)
    k_bfp_hub_matvec3(BfpHubArgs a, const uint32_t* __restrict__ btab2, int n_b2, int n_b2pos,
                      const uint16_t* __restrict__ chunk_cnt, int max_up,
                      const int32_t* __restrict__ up_lst, const int32_t* __restrict__ up_cnt,
                      const int64_t* __restrict__ X, int64_t* W, double* partial,
                      unsigned long long* partial_max, BfpState* st, int* status, BfpFuse fz, long wait_limit) {
  if (st && *(volatile int*)&st->stop) return;
  extern __shared__ __align__(128) unsigned char sm3[];
  __shared__ double smd[MV3_MAXNT / 32];
  __shared__ unsigned long long smu[MV3_MAXNT / 32];
  // element offsets in 32 bits: the kernel is chosen only for dim < 2^31 and nd < 4096
  const int nd = (int)a.nd, nu = (int)a.nu;
  const Mv3Layout L = mv3_layout(nd, n_b2, max_up);
  int64_t* raw = (int64_t*)(sm3 + L.raw_off);          // [MV3_R][nd]
  longlong2* xs2 = (longlong2*)(sm3 + L.xs_off);       // [nd + 1]
  uint32_t* tab = (uint32_t*)(sm3 + L.tab_off);        // [n_b2][nd]
  int32_t* lst = (int32_t*)(sm3 + L.lst_off);          // [2][MV3_R][lstride]
  int32_t* cnt = (int32_t*)(sm3 + L.cnt_off);          // [2][MV3_R][4]: + len, - len, pad correction
  uint64_t* bar = (uint64_t*)(sm3 + L.bar_off);
  const int tid = threadIdx.x, nt = blockDim.x;
  const int ngroups = (nu + MV3_R - 1) / MV3_R;
  const uint64_t keep = policy_evict_last(), stream = policy_evict_first();

  // stage group g from thread 0: bulk copies of its rows into `raw` and of its precomputed
  // padded up-lists and counts (rows u0, u0 + 1; row nu is an empty list) into list buffer s.
  // Everything lands on one mbarrier phase; no other thread waits on global loads here.
  auto stage = [&](int g, int s) {
    if (tid == 0) mv3_stage<UPW>(g, s, nu, nd, L.lstride, X, up_lst, up_cnt, raw, lst, cnt, bar);
  };

  // one-time set-up: the table, the zero slot pair, the barrier
  {
    for (int i = tid; i < n_b2 * nd; i += nt) tab[i] = __ldg(btab2 + i);
    if (tid == 0) {
      xs2[nd] = make_longlong2(0, 0);
      mbar_init(bar, 1);
      asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
  }
  bool pending = false;  // a bulk copy into `raw` has been issued and not yet waited for
  unsigned par = 0u;     // parity of the barrier's next phase completion
  if ((int)blockIdx.x < ngroups) {
    stage(blockIdx.x, 0);
    pending = true;
  }
  __syncthreads();

  I128 dot{0, 0};
  unsigned long long mx = 0;
  bool bad = false;
  int k = 0;
  const int lane = tid & 31, warp = tid >> 5, nwarp = nt >> 5;
  for (int g = blockIdx.x; g < ngroups; g += gridDim.x, ++k) {
    const int s = k & 1;
    const int row0 = g * MV3_R;
    const int nr = min(MV3_R, nu - row0);
    if (mbar_wait_polls(bar, par, wait_limit)) {
      pending = false;
      par ^= 1u;
    } else {
      bad = true;
    }
    if (__syncthreads_or(bad)) {
      bad = true;
      break;
    }
    // interleave the landed rows (a missing second row reads as zeros)
    for (int c = tid; c < nd; c += nt) xs2[c] = make_longlong2(raw[c], nr > 1 ? raw[nd + c] : 0);
    __syncthreads();  // xs2 complete; raw free for the next group's copy
    const int gn = g + gridDim.x;
    if (gn < ngroups) {
      stage(gn, s ^ 1);  // list buffer s^1 was released by the barrier that ended step k-1
      pending = true;
    }
    const int32_t* l0 = lst + (s * MV3_R + 0) * L.lstride;
    const int32_t* l1 = lst + (s * MV3_R + 1) * L.lstride;
    const int32_t cp0 = UPW ? 0 : cnt[(s * MV3_R + 0) * 4 + 0], cn0 = UPW ? 0 : cnt[(s * MV3_R + 0) * 4 + 1];
    const int32_t cp1 = UPW ? 0 : cnt[(s * MV3_R + 1) * 4 + 0], cn1 = UPW ? 0 : cnt[(s * MV3_R + 1) * 4 + 1];
    const int32_t corr0 = UPW ? 0 : cnt[(s * MV3_R + 0) * 4 + 2], corr1 = UPW ? 0 : cnt[(s * MV3_R + 1) * 4 + 2];
    const int row1 = row0 + (nr > 1 ? 1 : 0);
    const uint64_t su0 = __ldg(a.up_states + row0), su1 = __ldg(a.up_states + row1);
    const int64_t eu0 = DIAG64 ? 0 : (int64_t)__ldg(a.e_up + row0);
    const int64_t eu1 = DIAG64 ? 0 : (int64_t)__ldg(a.e_up + row1);
    const int64_t ef0 = DIAG64 ? __ldg(a.e_up_fx + row0) : 0;
    const int64_t ef1 = DIAG64 ? __ldg(a.e_up_fx + row1) : 0;
    // element offset of the group's first row (the second row, o0 + nd, is touched only when nr > 1)
    const int o0 = row0 * nd;
    const int n0 = cp0 + cn0, n1 = cp1 + cn1, nmax = max(n0, n1);
    // warps take 64-column chunks; lane l owns columns base + l and base + 32 + l
    for (int base = warp * 64; base < nd; base += nwarp * 64) {
      // dn table rows of this chunk: + pairs [0, np), - pairs [np, ne) (variant 7: per chunk)
      int np = n_b2pos, ne = n_b2;
      if (CMP) {
        const uint32_t cc = __ldg(chunk_cnt + (base >> 6));
        np = (int)(cc & 0xffu);
        ne = np + (int)(cc >> 8);
      }
      // the chunk's per-column data, requested early
      const int c_lo = min(base + lane, nd - 1), c_hi = min(base + 32 + lane, nd - 1);
      const uint64_t sd_lo = __ldg(a.dn_states + c_lo), sd_hi = __ldg(a.dn_states + c_hi);
      const int32_t e32_lo = DIAG64 ? 0 : __ldg(a.e_dn + c_lo), e32_hi = DIAG64 ? 0 : __ldg(a.e_dn + c_hi);
      const int64_t e64_lo = DIAG64 ? __ldg(a.e_dn_fx + c_lo) : 0, e64_hi = DIAG64 ? __ldg(a.e_dn_fx + c_hi) : 0;
      int64_t up_lo[2], up_hi[2];
      if (UPW) {
        // the up-neighbour sums of the two rows, written by the panel pass
        up_lo[0] = W[o0 + c_lo];
        up_hi[0] = W[o0 + c_hi];
        up_lo[1] = nr > 1 ? W[o0 + nd + c_lo] : 0;
        up_hi[1] = nr > 1 ? W[o0 + nd + c_hi] : 0;
      } else {
      // up neighbours in pair layout: lane l loads columns base + 2l, base + 2l + 1 (16 bytes)
      const int64_t* xc = X + min(base + 2 * lane, nd - 2);  // out-of-range lanes load a valid pair, unused
      longlong2 u0 = make_longlong2(0, 0), u1 = make_longlong2(0, 0);
      for (int e = 0; e < nmax; e += 4) {
        if (e < n0) {
          const longlong2 t = sum4x2(xc, l0 + e, keep);
          if (e < cp0) { u0.x += t.x; u0.y += t.y; } else { u0.x -= t.x; u0.y -= t.y; }
        }
        if (e < n1) {
          const longlong2 t = sum4x2(xc, l1 + e, keep);
          if (e < cp1) { u1.x += t.x; u1.y += t.y; } else { u1.x -= t.x; u1.y -= t.y; }
        }
      }
      // to the lane-contiguous layout: column base + l sits in lane l/2 (element l&1),
      // column base + 32 + l in lane 16 + l/2
      const bool odd = lane & 1;
      {
        const int s_lo = lane >> 1, s_hi = 16 + (lane >> 1);
        const int64_t a0 = shfl64(u0.x, s_lo), b0 = shfl64(u0.y, s_lo), a1 = shfl64(u1.x, s_lo), b1 = shfl64(u1.y, s_lo);
        const int64_t c0 = shfl64(u0.x, s_hi), d0 = shfl64(u0.y, s_hi), c1 = shfl64(u1.x, s_hi), d1 = shfl64(u1.y, s_hi);
        up_lo[0] = odd ? b0 : a0;
        up_lo[1] = odd ? b1 : a1;
        up_hi[0] = odd ? d0 : c0;
        up_hi[1] = odd ? d1 : c1;
      }
      }
#pragma unroll
      for (int half = 0; half < 2; ++half) {
        const int c = base + 32 * half + lane;
        if (c >= nd) continue;
        const longlong2 xo = xs2[c];
        int64_t h0 = (int64_t)corr0 * xo.x + (half ? up_hi[0] : up_lo[0]);
        int64_t h1 = (int64_t)corr1 * xo.y + (half ? up_hi[1] : up_lo[1]);
        // dn neighbours: two bonds per table word (byte offsets into xs2), + rows then - rows;
        // offset 16*nd reads zeros
        const uint32_t* tc = tab + c;
        for (int p = 0; p < np; ++p) {
          const uint32_t w = tc[p * nd];
          const longlong2 va = *(const longlong2*)((const char*)xs2 + (w & 0xffffu));
          const longlong2 vb = *(const longlong2*)((const char*)xs2 + (w >> 16));
          h0 += va.x + vb.x;
          h1 += va.y + vb.y;
        }
        for (int p = np; p < ne; ++p) {
          const uint32_t w = tc[p * nd];
          const longlong2 va = *(const longlong2*)((const char*)xs2 + (w & 0xffffu));
          const longlong2 vb = *(const longlong2*)((const char*)xs2 + (w >> 16));
          h0 -= va.x + vb.x;
          h1 -= va.y + vb.y;
        }
        const uint64_t sd = half ? sd_hi : sd_lo;
        const int32_t ed32 = half ? e32_hi : e32_lo;
        const int64_t ed64 = half ? e64_hi : e64_lo;
        {
          const int64_t w0 = (int64_t)a.t_int * h0 + bfp_diag_col<DIAG64>(a, eu0, ef0, su0, sd, ed32, ed64, xo.x);
          st_stream(W + (o0 + c), w0, stream);
          add128(dot, mul_s64(xo.x, w0));
          mx = max(mx, uabs64(w0));
        }
        if (nr > 1) {
          const int64_t w1 = (int64_t)a.t_int * h1 + bfp_diag_col<DIAG64>(a, eu1, ef1, su1, sd, ed32, ed64, xo.y);
          st_stream(W + (o0 + nd + c), w1, stream);
          add128(dot, mul_s64(xo.y, w1));
          mx = max(mx, uabs64(w1));
        }
      }
    }
    __syncthreads();  // xs2 and list buffer s free
  }
  if (bad) {
    // a wait ran out: record it, let a copy still in flight land (bounded), leave
    if (tid == 0) {
      record_status(status, DEV_TIMEOUT);
      if (st) *(volatile int*)&st->stop = 3;  // later kernels of the solve return at once
      if (pending) (void)mbar_wait_bounded(bar, par);
    }
    __syncthreads();
    return;
  }
  if (!partial) return;
  const double sdot = block_sum_rt(i128_to_double(dot), smd);
  const unsigned long long m = block_max_rt(mx, smu);
  if (tid == 0) {
    partial[blockIdx.x] = sdot;
    partial_max[blockIdx.x] = m;
  }
  if (fz.on && st && bfp_last_block(&st->ticket[2])) {
    // the last CTA to finish reduces the partials in CTA order and sets the step's scalars
    double t = 0.0;
    unsigned long long mm = 0;
    for (int b = tid; b < (int)gridDim.x; b += nt) {
      t += ((volatile double*)partial)[b];
      mm = max(mm, ((volatile unsigned long long*)partial_max)[b]);
    }
    t = block_sum_rt(t, smd);
    mm = block_max_rt(mm, smu);
    if (tid == 0) {
      bfp_scalars_tail(fz.v, fz.k, fz.F, fz.m_in, t, mm, fz.alpha, fz.beta, st);
      st->ticket[2] = 0;
    }
  }
}

#include "ed_sweep.cuh"
#include "ed_stripe.cuh"

// ---- two-pass H·v, pass 1: up-neighbour sums by column panels ---------------------------------
// The up-hop part of H·v, W[u, c] = sum_{u'} (+-) X[u', c], is a sparse-times-dense product. A
// CTA loads a panel of MV_PW = 4 columns of ALL rows (nu x 32 bytes) into shared memory once and
// forms the sums of every row from there, so each element of X crosses from L2 once instead of
// once per up-neighbour (7.5 times at 14 sites). Two CTAs per SM: one loads while the other sums.
// The dn/diagonal pass (k_bfp_hub_matvec3<., true>) then finishes W in place.
constexpr int MV_PW = 4;
constexpr int UP_NT = 512;

__global__ void __launch_bounds__(UP_NT, 2)
    k_bfp_up_panels(const int32_t* __restrict__ up_off, const int32_t* __restrict__ up_npos,
                    const int32_t* __restrict__ up_idx, int64_t nu, int64_t nd, const int64_t* __restrict__ X,
                    int64_t* __restrict__ W, const BfpState* st) {
  if (st && *(const volatile int*)&st->stop) return;
  extern __shared__ __align__(16) longlong2 pan[];  // [nu][2]: columns c0..c0+3 of every row
  const int64_t npan = nd / MV_PW;
  for (int64_t pnl = blockIdx.x; pnl < npan; pnl += gridDim.x) {
    const int64_t c0 = pnl * MV_PW;
    // load the panel: two 16-byte loads per row, four rows per thread in flight
    for (int64_t u = threadIdx.x; u < nu; u += 4 * UP_NT) {
      longlong2 v[8];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int64_t uu = min(u + q * UP_NT, nu - 1);
        const longlong2* src = (const longlong2*)(X + uu * nd + c0);
        v[2 * q] = __ldg(src);
        v[2 * q + 1] = __ldg(src + 1);
      }
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int64_t uu = u + q * UP_NT;
        if (uu < nu) {
          pan[2 * uu] = v[2 * q];
          pan[2 * uu + 1] = v[2 * q + 1];
        }
      }
    }
    __syncthreads();
    for (int64_t u = threadIdx.x; u < nu; u += UP_NT) {
      const int32_t o0 = __ldg(up_off + u), o1 = __ldg(up_off + u + 1), op = o0 + __ldg(up_npos + u);
      longlong2 a = make_longlong2(0, 0), b = make_longlong2(0, 0);
      for (int32_t e = o0; e < op; ++e) {
        const int32_t n = __ldg(up_idx + e);
        const longlong2 x0 = pan[2 * n], x1 = pan[2 * n + 1];
        a.x += x0.x; a.y += x0.y; b.x += x1.x; b.y += x1.y;
      }
      for (int32_t e = op; e < o1; ++e) {
        const int32_t n = __ldg(up_idx + e);
        const longlong2 x0 = pan[2 * n], x1 = pan[2 * n + 1];
        a.x -= x0.x; a.y -= x0.y; b.x -= x1.x; b.y -= x1.y;
      }
      longlong2* dst = (longlong2*)(W + u * nd + c0);
      dst[0] = a;
      dst[1] = b;
    }
    __syncthreads();  // the panel buffer is reloaded next
  }
}

// Lanczos scalars after the matvec of step k (single block, runs after the matvec):
//   alpha_k = <R_k, W> / beta_k^2 ;  R_{k+1} = c_w W + c_q R_k + c_p R_{k-1}
//   c_w = 1/beta_k, c_q = -alpha_k/beta_k, c_p = -beta_k/beta_{k-1}
__global__ void k_bfp_scalars(BfpVecs v, int k, int F, int m_in, const double* partial,
                              const unsigned long long* partial_max, int nparts, double* alpha, const double* beta,
                              BfpState* st) {
  if (*(volatile int*)&st->stop) return;
  __shared__ double sm[BT / 32];
  __shared__ unsigned long long smu[BT / 32];
  double t = 0.0;
  unsigned long long m = 0;
  for (int b = threadIdx.x; b < nparts; b += BT) {
    t += partial[b];
    m = max(m, partial_max[b]);
  }
  t = block_sum<BT>(t, sm);
  m = block_max_u64<BT>(m, smu);
  if (threadIdx.x != 0) return;
  bfp_scalars_tail(v, k, F, m_in, t, m, alpha, beta, st);
}

// alpha_k and the update coefficients from the reduced <R_k, W> (t, mantissa units) and
// max|W| (m); one thread
__device__ void bfp_scalars_tail(BfpVecs v, int k, int F, int m_in, double t, unsigned long long m, double* alpha,
                                 const double* beta, BfpState* st) {
  const int ek = v.eR[k];
  const int ew = ek - F;
  const double bk = beta[k];
  const double a = ldexp(t, ek + ew) / (bk * bk);
  alpha[k] = a;
  const double cw = 1.0 / bk, cq = -a / bk;
  const double cp = (k > 0) ? -bk / beta[k - 1] : 0.0;
  const int ep = (k > 0) ? v.eR[k - 1] : 0;
  const double mw = (double)m, mq = (double)v.maxR[k], mp = (k > 0) ? (double)v.maxR[k - 1] : 0.0;
  const double B = fabs(cw) * ldexp(mw, ew) + fabs(cq) * ldexp(mq, ek) + fabs(cp) * ldexp(mp, ep);
  int eb = 0;
  frexp(B > 0.0 ? B : 1.0, &eb);
  const int er = eb - m_in;  // B * 2^-er < 2^m_in
  const double gw = ldexp(cw, ew - er), gq = ldexp(cq, ek - er), gp = ldexp(cp, ep - er);
  const double gm = fmax(fabs(gw), fmax(fabs(gq), fabs(gp)));
  int eg = 0;
  frexp(gm > 0.0 ? gm : 1.0, &eg);  // gm < 2^eg
  const int SA = min(60, 60 - eg);
  st->A_w = llrint(ldexp(gw, SA));
  st->A_q = llrint(ldexp(gq, SA));
  st->A_p = llrint(ldexp(gp, SA));
  st->SA = SA;
  st->ew = ew;
  st->maxw = m;
  v.eR[k + 1] = er;
}

// one element of the three-term update, with the running exact norm and max
__device__ __forceinline__ int64_t bfp_upd1(int64_t Aw, int64_t Aq, int64_t Ap, int SA, int64_t w, int64_t q,
                                            int64_t pv, I128& nrm, unsigned long long& mx) {
  I128 s = mul_s64(Aw, w);
  add128(s, mul_s64(Aq, q));
  add128(s, mul_s64(Ap, pv));
  const int64_t r = shr128_round(s, SA);
  // r^2 = |r|^2: the unsigned square (|r| < 2^63) needs no sign corrections of the high word
  const unsigned long long ur = uabs64(r);
  I128 sq;
  sq.lo = ur * ur;
  sq.hi = (int64_t)__umul64hi(ur, ur);
  add128(nrm, sq);
  mx = max(mx, ur);
  return r;
}
__device__ __forceinline__ longlong2 ld2_stream(const int64_t* p, uint64_t pol) {
  longlong2 v;
  asm volatile("ld.global.nc.L2::cache_hint.v2.s64 {%0, %1}, [%2], %3;" : "=l"(v.x), "=l"(v.y) : "l"(p), "l"(pol));
  return v;
}
__device__ __forceinline__ void st2_keep(int64_t* p, int64_t a, int64_t b, uint64_t pol) {
  asm volatile("st.global.L2::cache_hint.v2.s64 [%0], {%1, %2}, %3;" ::"l"(p), "l"(a), "l"(b), "l"(pol) : "memory");
}

// R_{k+1} = round((A_w W + A_q R_k + A_p R_{k-1}) / 2^SA); ||R_{k+1}||^2 and max -> beta[k+1].
// VEC (D even, 16-byte aligned vectors): element pairs, two pairs per thread in flight; the
// inputs are read with an L2 evict_first policy and R_{k+1} is written with evict_last, so the
// next matvec finds its input in L2.
template <bool VEC>
__global__ void __launch_bounds__(BT, 4) k_bfp_update(BfpVecs v, int k, const int64_t* __restrict__ W, double* partial,
                                                   unsigned long long* partial_max, double* beta,
                                                   const double* alpha, BfpState* st, int final_k) {
  if (*(volatile int*)&st->stop) return;
  __shared__ double sm[BT / 32];
  __shared__ unsigned long long smu[BT / 32];
  const int64_t Aw = st->A_w, Aq = st->A_q, Ap = k > 0 ? st->A_p : 0;
  const int SA = st->SA;
  const int64_t* __restrict__ rq = v.vec(k);
  // k = 0: no R_{k-1}; read R_k again with a zero coefficient (keeps the loop branch-free)
  const int64_t* __restrict__ rp = k > 0 ? v.vec(k - 1) : rq;
  int64_t* __restrict__ rn = v.vec(k + 1);
  I128 nrm{0, 0};
  unsigned long long mx = 0;
  if (VEC) {
    const uint64_t first = policy_evict_first(), last = policy_evict_last();
    const int64_t P = v.D >> 1, stride = (int64_t)gridDim.x * BT;
    int64_t i = blockIdx.x * (int64_t)BT + threadIdx.x;
    for (; i + stride < P; i += 2 * stride) {
      const int64_t j0 = 2 * i, j1 = 2 * (i + stride);
      const longlong2 w0 = ld2_stream(W + j0, first), w1 = ld2_stream(W + j1, first);
      const longlong2 q0 = ld2_stream(rq + j0, first), q1 = ld2_stream(rq + j1, first);
      const longlong2 p0 = ld2_stream(rp + j0, first), p1 = ld2_stream(rp + j1, first);
      const int64_t a0 = bfp_upd1(Aw, Aq, Ap, SA, w0.x, q0.x, p0.x, nrm, mx);
      const int64_t a1 = bfp_upd1(Aw, Aq, Ap, SA, w0.y, q0.y, p0.y, nrm, mx);
      const int64_t b0 = bfp_upd1(Aw, Aq, Ap, SA, w1.x, q1.x, p1.x, nrm, mx);
      const int64_t b1 = bfp_upd1(Aw, Aq, Ap, SA, w1.y, q1.y, p1.y, nrm, mx);
      st2_keep(rn + j0, a0, a1, last);
      st2_keep(rn + j1, b0, b1, last);
    }
    for (; i < P; i += stride) {
      const int64_t j0 = 2 * i;
      const longlong2 w0 = ld2_stream(W + j0, first), q0 = ld2_stream(rq + j0, first), p0 = ld2_stream(rp + j0, first);
      const int64_t a0 = bfp_upd1(Aw, Aq, Ap, SA, w0.x, q0.x, p0.x, nrm, mx);
      const int64_t a1 = bfp_upd1(Aw, Aq, Ap, SA, w0.y, q0.y, p0.y, nrm, mx);
      st2_keep(rn + j0, a0, a1, last);
    }
  } else {
    for (int64_t i = blockIdx.x * (int64_t)BT + threadIdx.x; i < v.D; i += (int64_t)gridDim.x * BT)
      rn[i] = bfp_upd1(Aw, Aq, Ap, SA, W[i], rq[i], rp[i], nrm, mx);
  }
  const double s = block_sum<BT>(i128_to_double(nrm), sm);
  const unsigned long long m = block_max_u64<BT>(mx, smu);
  if (threadIdx.x == 0) {
    partial[blockIdx.x] = s;
    partial_max[blockIdx.x] = m;
  }
  if (bfp_last_block(&st->ticket[1])) {
    double t = 0.0;
    unsigned long long mm = 0;
    for (int b = threadIdx.x; b < (int)gridDim.x; b += BT) {
      t += ((volatile double*)partial)[b];
      mm = max(mm, ((volatile unsigned long long*)partial_max)[b]);
    }
    t = block_sum<BT>(t, sm);
    mm = block_max_u64<BT>(mm, smu);
    if (threadIdx.x == 0) {
      const double bn = ldexp(sqrt(t), v.eR[k + 1]);
      beta[k + 1] = bn;
      v.maxR[k + 1] = mm;
      // invariant subspace: the new residual vanishes relative to the scale of T
      // (beta[0] holds the start-vector norm, not an entry of T)
      const double scale = fabs(alpha[k]) + (k > 0 ? beta[k] : 0.0) + 1e-300;
      if (!(bn > 1e-13 * scale) || mm == 0) {
        st->steps = k + 1;
        st->stop = 2;
      }
      (void)final_k;
      st->ticket[1] = 0;
    }
  }
}

// ---- Ritz vector ------------------------------------------------------------------------------------
// psi = sum_k C_k R_k * 2^-SC (C_k and SC from the host: see bfp_lanczos)
// (pu, pd non-null: the vectors are in the renumbered basis of the sweep or the stripe matvec
// and psi is scattered back to the original order, nd = num_dn)
template <bool PAIRS>
__global__ void __launch_bounds__(256) k_bfp_ritz(const BfpVecs v, const int64_t* __restrict__ C, const int* SCp,
                                                  const BfpState* st, double* __restrict__ out,
                                                  const int32_t* __restrict__ pu, const int32_t* __restrict__ pd,
                                                  int64_t nd) {
  const int m = st->steps;
  const int SC = *SCp;
  const uint64_t first = policy_evict_first();  // every stored element is read once
  auto put = [&](int64_t i, const I128& acc) {
    int64_t o = i;
    if (pu) {
      const int64_t r = i / nd, c = i - r * nd;
      o = (int64_t)__ldg(pu + r) * nd + __ldg(pd + c);
    }
    out[o] = ldexp(i128_to_double(acc), -SC);
  };
  if (PAIRS) {
    // two adjacent elements per thread (16-byte loads; D even, store 16-byte aligned) and four
    // Krylov vectors per loop step: 64 bytes of independent loads in flight per thread
    const int64_t npairs = v.D >> 1;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < npairs; q += (int64_t)gridDim.x * blockDim.x) {
      const int64_t* base = v.R + 2 * q;
      I128 a0{0, 0}, a1{0, 0};
      int k = 0;
      for (; k + 4 <= m; k += 4) {
        const longlong2 x0 = ld2_stream(base + (int64_t)k * v.D, first);
        const longlong2 x1 = ld2_stream(base + (int64_t)(k + 1) * v.D, first);
        const longlong2 x2 = ld2_stream(base + (int64_t)(k + 2) * v.D, first);
        const longlong2 x3 = ld2_stream(base + (int64_t)(k + 3) * v.D, first);
        const int64_t c0 = __ldg(C + k), c1 = __ldg(C + k + 1), c2 = __ldg(C + k + 2), c3 = __ldg(C + k + 3);
        add128(a0, mul_s64(c0, x0.x));
        add128(a1, mul_s64(c0, x0.y));
        add128(a0, mul_s64(c1, x1.x));
        add128(a1, mul_s64(c1, x1.y));
        add128(a0, mul_s64(c2, x2.x));
        add128(a1, mul_s64(c2, x2.y));
        add128(a0, mul_s64(c3, x3.x));
        add128(a1, mul_s64(c3, x3.y));
      }
      for (; k < m; ++k) {
        const longlong2 x = ld2_stream(base + (int64_t)k * v.D, first);
        const int64_t c = __ldg(C + k);
        add128(a0, mul_s64(c, x.x));
        add128(a1, mul_s64(c, x.y));
      }
      put(2 * q, a0);
      put(2 * q + 1, a1);
    }
  } else {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < v.D; i += (int64_t)gridDim.x * blockDim.x) {
      I128 acc{0, 0};
      for (int k = 0; k < m; ++k) add128(acc, mul_s64(C[k], v.vec(k)[i]));
      put(i, acc);
    }
  }
}

// Ritz coefficients C_k = round(c_k / beta_k * 2^(e_k + SC)) of the final eigenvector c (one
// block): one SC for all k with |C_k| < 2^62 - 10 bits of headroom for the sum over k
__global__ void k_bfp_ritz_coef(const double* __restrict__ c, const double* __restrict__ beta,
                                const int32_t* __restrict__ eR, const TriResult* tr, int64_t* C, int* SCp) {
  __shared__ unsigned long long sm[BT / 32];
  __shared__ int sc_s;
  const int m = tr->m_final;
  unsigned long long gb = 0;  // max |c_k / beta_k * 2^e_k| as bits (non-negative doubles order as integers)
  for (int k = threadIdx.x; k < m; k += BT)
    gb = max(gb, (unsigned long long)__double_as_longlong(fabs(ldexp(c[k] / beta[k], eR[k]))));
  gb = block_max_u64<BT>(gb, sm);
  if (threadIdx.x == 0) {
    const double gm = __longlong_as_double((long long)gb);
    int eg = 0;
    frexp(gm > 0.0 ? gm : 1.0, &eg);
    sc_s = 52 - eg;
    *SCp = sc_s;
  }
  __syncthreads();
  for (int k = threadIdx.x; k < m; k += BT) C[k] = llrint(ldexp(c[k] / beta[k], eR[k] + sc_s));
}

// ---- tables ---------------------------------------------------------------------------------------------

static bool is_int_scaled(double v, int F, int64_t lim) {
  const double s = std::ldexp(v, F);
  return std::isfinite(s) && s == std::floor(s) && std::fabs(s) < (double)lim;
}

// shared memory of the two sweep passes for rings of r chunks
static size_t sweep_smem_up(int r) {
  return (size_t)r * (SW_CH * SW_W * 8 + 8) + (size_t)SW_LR * (SW_CH * SW_LST * 2 + 8);
}
static size_t sweep_smem_dn(int r) {
  return (size_t)SW_W * ((size_t)r * SW_CH + 1) * 8 + (size_t)SW_W * (SW_CH + 1) * 8 + (size_t)r * 8 +
         (size_t)SW_LR * (SW_CH * SW_LST * 2 + 8);
}

// device copy of a host array (at least 8 bytes allocated)
static ed_status dev_upload(void** dst, const void* src, size_t bytes, cudaStream_t s) {
  ED_CUDA(cudaMalloc(dst, std::max<size_t>(bytes, 8)));
  if (bytes) ED_CUDA(cudaMemcpyAsync(*dst, src, bytes, cudaMemcpyHostToDevice, s));
  return ED_OK;
}

// device copies of both species' diagonal data (states and per-state energies of the plan's
// diagonal mode) in a renumbered order (pu, pd: new -> old); synchronous
static ed_status upload_renumbered_diag(const ed_plan_s* p, const BfpTables& B, const std::vector<int32_t>& pu,
                                        const std::vector<int32_t>& pd, const std::vector<int32_t>& eui,
                                        const std::vector<int32_t>& edi, const std::vector<int64_t>& euf,
                                        const std::vector<int64_t>& edf, uint64_t** s_up, uint64_t** s_dn,
                                        int32_t** e_up, int32_t** e_dn, int64_t** f_up, int64_t** f_dn,
                                        cudaStream_t s) {
  const int64_t nu = p->num_up, nd = p->num_dn;
  std::vector<uint64_t> st_up(nu), st_dn(nd), sup(nu), sdn(nd);
  ED_CUDA(cudaMemcpyAsync(st_up.data(), p->up.states, nu * 8, cudaMemcpyDeviceToHost, s));
  ED_CUDA(cudaMemcpyAsync(st_dn.data(), p->dn.states, nd * 8, cudaMemcpyDeviceToHost, s));
  ED_CUDA(cudaStreamSynchronize(s));
  for (int64_t i = 0; i < nu; ++i) sup[i] = st_up[pu[i]];
  for (int64_t i = 0; i < nd; ++i) sdn[i] = st_dn[pd[i]];
  ED_TRY(dev_upload((void**)s_up, sup.data(), sup.size() * 8, s));
  ED_TRY(dev_upload((void**)s_dn, sdn.data(), sdn.size() * 8, s));
  if (!B.diag64) {
    std::vector<int32_t> a(nu), b(nd);
    for (int64_t i = 0; i < nu; ++i) a[i] = eui[pu[i]];
    for (int64_t i = 0; i < nd; ++i) b[i] = edi[pd[i]];
    ED_TRY(dev_upload((void**)e_up, a.data(), a.size() * 4, s));
    ED_TRY(dev_upload((void**)e_dn, b.data(), b.size() * 4, s));
    ED_CUDA(cudaStreamSynchronize(s));
  } else {
    std::vector<int64_t> a(nu), b(nd);
    for (int64_t i = 0; i < nu; ++i) a[i] = euf[pu[i]];
    for (int64_t i = 0; i < nd; ++i) b[i] = edf[pd[i]];
    ED_TRY(dev_upload((void**)f_up, a.data(), a.size() * 8, s));
    ED_TRY(dev_upload((void**)f_dn, b.data(), b.size() * 8, s));
    ED_CUDA(cudaStreamSynchronize(s));
  }
  return ED_OK;
}

// Tables of the stripe matvec (ed_stripe.cuh); leaves B.sp.on = 0 when the sector does not
// suit it (a target with more than 2 ST_PMAX - 2 hops, a stripe larger than one CTA's shared
// memory). CMPY_ED_STRIPE=0 disables it.
static ed_status build_stripe(ed_plan_s* p, BfpTables& B, const std::vector<int32_t>& uoff,
                              const std::vector<int32_t>& uidx, const std::vector<double>& ucoef,
                              const std::vector<int32_t>& doff, const std::vector<int32_t>& didx,
                              const std::vector<double>& dcoef, const std::vector<int32_t>& eui,
                              const std::vector<int32_t>& edi, const std::vector<int64_t>& euf,
                              const std::vector<int64_t>& edf, cudaStream_t s) {
  StripeTables& T = B.sp;
  T = StripeTables();
  const char* env = getenv("CMPY_ED_STRIPE");
  if (env && atoi(env) == 0) return ED_OK;
  const int64_t nu = p->num_up, nd = p->num_dn;
  // CTAs per SM: two when a stripe buffer fits in half of the SM's shared memory
  int per_sm = 0;
  ED_CUDA(cudaDeviceGetAttribute(&per_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, p->device));
  const size_t two = (size_t)per_sm / 2 - 1024 - 512, one = (size_t)p->ctx->smem_optin - 512;
  auto ctas = [&](int64_t n) { return stripe_smem(n) <= two ? 2 : (stripe_smem(n) <= one ? 1 : 0); };
  T.per_sm_up = ctas(nu);
  T.per_sm_dn = ctas(nd);
  if (T.per_sm_up == 0 || T.per_sm_dn == 0) return ED_OK;
  StripeSide su, sd;
  if (!stripe_order(nu, uoff, uidx, ucoef, &su) || !stripe_order(nd, doff, didx, dcoef, &sd)) return ED_OK;
  ED_TRY(upload_renumbered_diag(p, B, su.perm, sd.perm, eui, edi, euf, edf, &T.s_up, &T.s_dn, &T.e_up, &T.e_dn,
                                &T.f_up, &T.f_dn, s));
  ED_TRY(dev_upload((void**)&T.perm_up, su.perm.data(), su.perm.size() * 4, s));
  ED_TRY(dev_upload((void**)&T.perm_dn, sd.perm.data(), sd.perm.size() * 4, s));
  ED_TRY(dev_upload((void**)&T.lst_up, su.lst.data(), su.lst.size() * 4, s));
  ED_TRY(dev_upload((void**)&T.lst_dn, sd.lst.data(), sd.lst.size() * 4, s));
  ED_TRY(dev_upload((void**)&T.meta_up, su.meta.data(), su.meta.size() * 2, s));
  ED_TRY(dev_upload((void**)&T.meta_dn, sd.meta.data(), sd.meta.size() * 2, s));
  ED_CUDA(cudaStreamSynchronize(s));
  T.pmax_up = su.pmax;
  T.pmax_dn = sd.pmax;
  // L2 policies (bit set = evict_last): pass 1 X loads, pass 1 S stores, pass 2 X loads, pass 2
  // W stores
  const char* pe = getenv("CMPY_ED_STRIPE_POL");
  T.pol = pe ? atoi(pe) : 0b1010;
  T.on = 1;
  return ED_OK;
}

static void free_stripe(StripeTables& T) {
  cudaFree(T.perm_up); cudaFree(T.perm_dn); cudaFree(T.lst_up); cudaFree(T.lst_dn);
  cudaFree(T.meta_up); cudaFree(T.meta_dn); cudaFree(T.s_up); cudaFree(T.s_dn);
  cudaFree(T.e_up); cudaFree(T.e_dn); cudaFree(T.f_up); cudaFree(T.f_dn);
  T = StripeTables();
}

// Tables of variant 7 (k_bfp_hub_matvec3 with the dn states renumbered by hop count): the dn
// order of stripe_order, and per renumbered column its + then - partners as byte offsets 16*j
// of the interleaved row pair, two per word; every column of a 64-column chunk has the chunk's
// largest + and - pair counts (padded with the zero slot 16*nd). CMPY_ED_DNC=0 disables it.
static ed_status build_dncompact(ed_plan_s* p, BfpTables& B, const std::vector<int32_t>& doff,
                                 const std::vector<int32_t>& didx, const std::vector<double>& dcoef,
                                 const std::vector<int32_t>& edi, const std::vector<int64_t>& edf, cudaStream_t s) {
  DnCompactTables& T = B.dc;
  T = DnCompactTables();
  const char* env = getenv("CMPY_ED_DNC");
  if (env && atoi(env) == 0) return ED_OK;
  const int64_t nu = p->num_up, nd = p->num_dn;
  if (nd < 2 || nd % 2 || nd >= 4096) return ED_OK;  // the single-pass kernel's limits
  StripeSide sd;
  if (!stripe_order(nd, doff, didx, dcoef, &sd)) return ED_OK;
  std::vector<int32_t> inv(nd);
  for (int64_t i = 0; i < nd; ++i) inv[sd.perm[i]] = (int32_t)i;
  const int64_t nchunk = (nd + 63) / 64;
  std::vector<std::vector<uint32_t>> pos(nd), neg(nd);
  for (int64_t i = 0; i < nd; ++i) {
    const int64_t v = sd.perm[i];
    for (int32_t k = doff[v]; k < doff[v + 1]; ++k) {
      if (dcoef[k] == 0.0) continue;
      (dcoef[k] > 0.0 ? pos[i] : neg[i]).push_back(16u * (uint32_t)inv[didx[k]]);
    }
  }
  std::vector<uint16_t> chunk(nchunk);
  int rows = 0;
  for (int64_t c = 0; c < nchunk; ++c) {
    int pp = 0, pn = 0;
    for (int64_t i = c * 64; i < std::min<int64_t>(nd, (c + 1) * 64); ++i) {
      pp = std::max(pp, (int)(pos[i].size() + 1) / 2);
      pn = std::max(pn, (int)(neg[i].size() + 1) / 2);
    }
    chunk[c] = (uint16_t)(pp | (pn << 8));
    rows = std::max(rows, pp + pn);
  }
  rows = std::max(rows, 1);
  if (mv3_layout(nd, rows, B.max_up).total + MV3_STATIC_SMEM > (size_t)p->ctx->smem_optin) return ED_OK;
  const uint32_t zero = 16u * (uint32_t)nd;
  std::vector<uint32_t> tab((size_t)rows * nd, zero | (zero << 16));
  for (int64_t i = 0; i < nd; ++i) {
    const int pp = chunk[i / 64] & 0xff;
    auto put = [&](const std::vector<uint32_t>& lst, int row0) {
      for (size_t e = 0; e < lst.size(); e += 2) {
        const uint32_t lo = lst[e], hi = e + 1 < lst.size() ? lst[e + 1] : zero;
        tab[(size_t)(row0 + e / 2) * nd + i] = lo | (hi << 16);
      }
    };
    put(pos[i], 0);
    put(neg[i], pp);
  }
  std::vector<int32_t> ident(nu);
  for (int64_t i = 0; i < nu; ++i) ident[i] = (int32_t)i;
  std::vector<uint64_t> st_dn(nd), sdn(nd);
  ED_CUDA(cudaMemcpyAsync(st_dn.data(), p->dn.states, nd * 8, cudaMemcpyDeviceToHost, s));
  ED_CUDA(cudaStreamSynchronize(s));
  for (int64_t i = 0; i < nd; ++i) sdn[i] = st_dn[sd.perm[i]];
  ED_TRY(dev_upload((void**)&T.tab, tab.data(), tab.size() * 4, s));
  ED_TRY(dev_upload((void**)&T.chunk, chunk.data(), chunk.size() * 2, s));
  ED_TRY(dev_upload((void**)&T.perm_up, ident.data(), ident.size() * 4, s));
  ED_TRY(dev_upload((void**)&T.perm_dn, sd.perm.data(), sd.perm.size() * 4, s));
  ED_TRY(dev_upload((void**)&T.s_dn, sdn.data(), sdn.size() * 8, s));
  if (!B.diag64) {
    std::vector<int32_t> b(nd);
    for (int64_t i = 0; i < nd; ++i) b[i] = edi[sd.perm[i]];
    ED_TRY(dev_upload((void**)&T.e_dn, b.data(), b.size() * 4, s));
    ED_CUDA(cudaStreamSynchronize(s));
  } else {
    std::vector<int64_t> b(nd);
    for (int64_t i = 0; i < nd; ++i) b[i] = edf[sd.perm[i]];
    ED_TRY(dev_upload((void**)&T.f_dn, b.data(), b.size() * 8, s));
    ED_CUDA(cudaStreamSynchronize(s));
  }
  T.rows = rows;
  T.on = 1;
  return ED_OK;
}

static void free_dncompact(DnCompactTables& T) {
  cudaFree(T.tab); cudaFree(T.chunk); cudaFree(T.perm_up); cudaFree(T.perm_dn);
  cudaFree(T.s_dn); cudaFree(T.e_dn); cudaFree(T.f_dn);
  T = DnCompactTables();
}

// Tables of the banded two-pass matvec (ed_sweep.cuh); leaves B.sw.on = 0 when the sector does
// not suit it (odd num_dn: the 16-byte row-piece copies of pass 1 need even rows; a target with more than
// 15 hops; a band wider than the shared memory). CMPY_ED_SWEEP=0 disables it.
static ed_status build_sweep(ed_plan_s* p, BfpTables& B, const std::vector<int32_t>& uoff,
                             const std::vector<int32_t>& uidx, const std::vector<double>& ucoef,
                             const std::vector<int32_t>& doff, const std::vector<int32_t>& didx,
                             const std::vector<double>& dcoef, const std::vector<int32_t>& eui,
                             const std::vector<int32_t>& edi, const std::vector<int64_t>& euf,
                             const std::vector<int64_t>& edf, cudaStream_t s) {
  SweepTables& W = B.sw;
  W = SweepTables();
  const char* env = getenv("CMPY_ED_SWEEP");
  if (env && atoi(env) == 0) return ED_OK;
  const int64_t nu = p->num_up, nd = p->num_dn;
  if (nu < 1 || nd < 2 || nd % 2) return ED_OK;
  SweepSide su, sd;
  if (!sweep_order(nu, uoff, uidx, ucoef, &su) || !sweep_order(nd, doff, didx, dcoef, &sd)) return ED_OK;
  // rings: as many chunks as one CTA per SM allows: the chunks beyond the band window are the
  // prefetch depth, and with two CTAs per SM the window left ~1-2 chunks of it (the passes
  // then waited on every chunk); CMPY_ED_SWEEP_CTAS=2 selects the two-per-SM rings
  int per_sm = 0;
  ED_CUDA(cudaDeviceGetAttribute(&per_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, p->device));
  const size_t two = (size_t)per_sm / 2 - 2048, one = (size_t)p->ctx->smem_optin - 1024;
  auto pick = [&](int need, int64_t nchunks, size_t (*smem)(int)) -> int {
    int r2 = 0, r1 = 0;
    while (smem(r2 + 1) <= two) ++r2;
    while (smem(r1 + 1) <= one) ++r1;
    static const int per = [] {
      const char* e = getenv("CMPY_ED_SWEEP_CTAS");
      return e ? atoi(e) : 1;
    }();
    const int r = (per == 2 && need <= r2) ? r2 : (need <= r1 ? r1 : 0);
    if (r == 0) return 0;
    return (int)std::min<int64_t>(std::max<int64_t>(need, std::min<int64_t>(r, nchunks)), 32767 / SW_CH);
  };
  const int ru = pick(su.need, (nu + SW_CH - 1) / SW_CH, sweep_smem_up);
  const int rd = pick(sd.need, (nd + SW_CH - 1) / SW_CH, sweep_smem_dn);
  if (ru < su.need || rd < sd.need || ru == 0 || rd == 0) return ED_OK;
  sweep_lists(nu, uoff, uidx, ucoef, ru, &su);
  sweep_lists(nd, doff, didx, dcoef, rd, &sd);
  ED_TRY(upload_renumbered_diag(p, B, su.perm, sd.perm, eui, edi, euf, edf, &W.s_up, &W.s_dn, &W.e_up, &W.e_dn,
                                &W.f_up, &W.f_dn, s));
  auto up = [&](auto** dst, const void* src, size_t bytes) { return dev_upload((void**)dst, src, bytes, s); };
  ED_TRY(up(&W.perm_up, su.perm.data(), su.perm.size() * 4));
  ED_TRY(up(&W.perm_dn, sd.perm.data(), sd.perm.size() * 4));
  ED_TRY(up(&W.lst_up, su.lst.data(), su.lst.size() * 2));
  ED_TRY(up(&W.lst_dn, sd.lst.data(), sd.lst.size() * 2));
  ED_TRY(up(&W.win_up, su.win.data(), su.win.size() * sizeof(int2)));
  ED_TRY(up(&W.win_dn, sd.win.data(), sd.win.size() * sizeof(int2)));
  ED_CUDA(cudaStreamSynchronize(s));
  W.ring_up = ru;
  W.ring_dn = rd;
  W.nblk_up = (int)su.win.size();
  W.nblk_dn = (int)sd.win.size();
  // L2 policies (bit set = evict_last): pass 1 X loads, pass 1 S stores, pass 2 X loads, pass 2
  // W stores; default keeps S for pass 2 and W for the update kernel
  const char* pe = getenv("CMPY_ED_SWEEP_POL");
  W.pol = pe ? atoi(pe) : 0b1010;
  W.on = 1;
  return ED_OK;
}

static void free_sweep(SweepTables& W) {
  cudaFree(W.perm_up); cudaFree(W.perm_dn); cudaFree(W.lst_up); cudaFree(W.lst_dn);
  cudaFree(W.win_up); cudaFree(W.win_dn); cudaFree(W.s_up); cudaFree(W.s_dn);
  cudaFree(W.e_up); cudaFree(W.e_dn); cudaFree(W.f_up); cudaFree(W.f_dn);
  W = SweepTables();
}

ed_status build_bfp(ed_plan_s* p, cudaStream_t s) {
  BfpTables& B = p->bfp;
  B = BfpTables();
  if (p->kind != 0 || p->dim == 0) return ED_OK;
  // one hopping magnitude
  double tmag = 0.0;
  for (double h : p->hop) {
    if (h == 0.0) continue;
    if (tmag == 0.0) tmag = std::fabs(h);
    else if (std::fabs(h) != tmag) return ED_OK;
  }
  if (p->num_dn * 2 + 1 > 65535) return ED_OK;  // 16-bit shared-memory slots
  if ((2 * p->num_dn + 1) * 8 > 200 * 1024) return ED_OK;
  // coefficients: per-state energies (exact FP64 sums), U and t as integers * 2^-F
  std::vector<double> eu(p->num_up), edn(p->num_dn);
  ED_CUDA(cudaMemcpyAsync(eu.data(), p->up.energy, p->num_up * sizeof(double), cudaMemcpyDeviceToHost, s));
  ED_CUDA(cudaMemcpyAsync(edn.data(), p->dn.energy, p->num_dn * sizeof(double), cudaMemcpyDeviceToHost, s));
  ED_CUDA(cudaStreamSynchronize(s));
  // mode 0: t, U and the state energies are integers * 2^-F (exact diagonal)
  int F = -1;
  for (int f = 0; f <= 40 && F < 0; ++f) {
    bool ok = is_int_scaled(tmag, f, 1 << 24);
    for (double v : p->u) ok = ok && is_int_scaled(v, f, 1 << 24);
    for (double v : eu) ok = ok && is_int_scaled(v, f, 1 << 28);
    for (double v : edn) ok = ok && is_int_scaled(v, f, 1 << 28);
    if (ok) F = f;
  }
  int diag64 = 0;
  if (F < 0) {
    // mode 1: only t needs to be dyadic; the diagonal is an int64 fixed-point product
    for (int f = 0; f <= 40 && F < 0; ++f)
      if (is_int_scaled(tmag, f, 1 << 24)) F = f;
    if (F < 0) return ED_OK;
    diag64 = 1;
  }
  // row tables (host copies of the FP64 tables)
  std::vector<int32_t> uoff(p->num_up + 1), uidx(p->up.nnz), doff(p->num_dn + 1), didx(p->dn.nnz);
  std::vector<double> ucoef(p->up.nnz), dcoef(p->dn.nnz);
  std::vector<int16_t> dbond(p->dn.nnz);
  ED_CUDA(cudaMemcpyAsync(uoff.data(), p->up.off, uoff.size() * 4, cudaMemcpyDeviceToHost, s));
  ED_CUDA(cudaMemcpyAsync(doff.data(), p->dn.off, doff.size() * 4, cudaMemcpyDeviceToHost, s));
  if (p->up.nnz) {
    ED_CUDA(cudaMemcpyAsync(uidx.data(), p->up.idx, uidx.size() * 4, cudaMemcpyDeviceToHost, s));
    ED_CUDA(cudaMemcpyAsync(ucoef.data(), p->up.coef, ucoef.size() * 8, cudaMemcpyDeviceToHost, s));
  }
  if (p->dn.nnz) {
    ED_CUDA(cudaMemcpyAsync(didx.data(), p->dn.idx, didx.size() * 4, cudaMemcpyDeviceToHost, s));
    ED_CUDA(cudaMemcpyAsync(dcoef.data(), p->dn.coef, dcoef.size() * 8, cudaMemcpyDeviceToHost, s));
    ED_CUDA(cudaMemcpyAsync(dbond.data(), p->dn.bond, dbond.size() * 2, cudaMemcpyDeviceToHost, s));
  }
  ED_CUDA(cudaStreamSynchronize(s));
  const int64_t nu = p->num_up, nd = p->num_dn;
  std::vector<int32_t> boff(nu + 1), bnpos(nu), bidx;
  bidx.reserve(p->up.nnz);
  int max_up = 0;
  for (int64_t r = 0; r < nu; ++r) {
    boff[r] = (int32_t)bidx.size();
    int npos = 0;
    for (int32_t k = uoff[r]; k < uoff[r + 1]; ++k)
      if (ucoef[k] > 0.0) { bidx.push_back(uidx[k]); ++npos; }
    for (int32_t k = uoff[r]; k < uoff[r + 1]; ++k)
      if (ucoef[k] < 0.0) bidx.push_back(uidx[k]);
    bnpos[r] = npos;
    max_up = std::max(max_up, (int)(bidx.size() - boff[r]));
  }
  boff[nu] = (int32_t)bidx.size();
  int max_dn = 0;
  for (int64_t c = 0; c < nd; ++c) {
    int n = 0;
    for (int32_t k = doff[c]; k < doff[c + 1]; ++k) n += (dcoef[k] != 0.0);
    max_dn = std::max(max_dn, n);
  }
  std::vector<uint16_t> tab((size_t)std::max(max_dn, 1) * nd, (uint16_t)(2 * nd));
  for (int64_t c = 0; c < nd; ++c) {
    int e = 0;
    for (int32_t k = doff[c]; k < doff[c + 1]; ++k) {
      if (dcoef[k] == 0.0) continue;
      tab[(size_t)e * nd + c] = (uint16_t)(dcoef[k] > 0.0 ? didx[k] : nd + didx[k]);
      ++e;
    }
  }
  // bond-major table: one row per (bond, sign) pair that occurs, + rows first, so that a warp
  // of consecutive columns gathers partners of one bond (nearly contiguous addresses)
  std::vector<int> brow(2 * ED_MAX_BONDS, -1);
  int n_bpos = 0, n_bt = 0;
  for (int sg = 0; sg < 2; ++sg) {
    for (size_t k = 0; k < dcoef.size(); ++k) {
      if (dcoef[k] == 0.0 || (dcoef[k] < 0.0) != (sg == 1)) continue;
      const int key = 2 * dbond[k] + sg;
      if (brow[key] < 0) brow[key] = n_bt++;
    }
    if (sg == 0) n_bpos = n_bt;
  }
  // renumber so that rows follow bond order within each sign class
  {
    int nxt = 0;
    for (int sg = 0; sg < 2; ++sg)
      for (int b = 0; b < ED_MAX_BONDS; ++b)
        if (brow[2 * b + sg] >= 0) brow[2 * b + sg] = nxt++;
  }
  // padded row numbers: + rows [0, pos_pad), - rows [pos_pad, pos_pad + neg_pad)
  const int pos_pad = n_bpos + (n_bpos & 1), n_neg = n_bt - n_bpos, neg_pad = n_neg + (n_neg & 1);
  const int n_rows = pos_pad + neg_pad;
  std::vector<uint16_t> btab((size_t)std::max(n_rows, 2) * nd, (uint16_t)nd);
  for (int64_t c = 0; c < nd; ++c)
    for (int32_t k = doff[c]; k < doff[c + 1]; ++k) {
      if (dcoef[k] == 0.0) continue;
      int row = brow[2 * dbond[k] + (dcoef[k] < 0.0 ? 1 : 0)];
      if (row >= n_bpos) row += pos_pad - n_bpos;
      btab[(size_t)row * nd + c] = (uint16_t)didx[k];
    }
  std::vector<uint32_t> btab2((size_t)std::max(n_rows / 2, 1) * nd);
  for (int pr = 0; pr < std::max(n_rows / 2, 1); ++pr)
    for (int64_t c = 0; c < nd; ++c)
      // byte offsets of the 16-byte interleaved row pair (slot * 16 < 2^16 needs nd < 4096; the
      // kernel that reads this table is only chosen then)
      btab2[(size_t)pr * nd + c] = ((uint32_t)btab[(size_t)(2 * pr) * nd + c] * 16u & 0xffffu) |
                                   (((uint32_t)btab[(size_t)(2 * pr + 1) * nd + c] * 16u & 0xffffu) << 16);
  // diagonal bound in units of 2^-F, and the overflow guard
  //   |W| <= (max|diag| 2^F + hops * t_int) * 2^m_in < 2^62
  B.u_uniform = p->fp.u_uniform;
  double max_eu = 0.0, max_ed = 0.0;
  for (double v : eu) max_eu = std::max(max_eu, std::fabs(v));
  for (double v : edn) max_ed = std::max(max_ed, std::fabs(v));
  std::vector<double> uabs;
  for (int i = 0; i < p->n_sites; ++i) uabs.push_back(std::fabs(p->u[i]));
  std::sort(uabs.rbegin(), uabs.rend());
  double usum = 0.0;
  for (int i = 0; i < std::min(p->n_up, p->n_dn) && i < (int)uabs.size(); ++i) usum += uabs[i];
  const double diag_max = max_eu + max_ed + usum;
  B.t_int = (int32_t)std::ldexp(tmag, F);
  const double bound = std::ldexp(diag_max, F) + (double)(max_up + max_dn) * B.t_int;
  int lb = 0;
  while (std::ldexp(1.0, lb) <= bound) ++lb;  // bound < 2^lb
  const int m_in = std::min(56, 62 - lb);
  if (m_in < 48) return ED_OK;
  std::vector<int32_t> eui, edi;
  std::vector<int64_t> euf, edf;
  if (!diag64) {
    eui.resize(nu);
    edi.resize(nd);
    for (int64_t i = 0; i < nu; ++i) eui[i] = (int32_t)std::ldexp(eu[i], F);
    for (int64_t i = 0; i < nd; ++i) edi[i] = (int32_t)std::ldexp(edn[i], F);
    for (int i = 0; i < p->n_sites; ++i) B.u_int[i] = (int32_t)std::ldexp(p->u[i], F);
    B.u0_int = p->n_sites ? B.u_int[0] : 0;
  } else {
    // diag_fx = diag * 2^Fd with |diag_fx| < 2^61; the product with X (<= 2^m_in) is 128-bit
    int ld = 0;
    while (std::ldexp(1.0, ld) <= diag_max) ++ld;
    B.Fd = 61 - ld;
    if (B.Fd - F < 1 || B.Fd - F > 63) return ED_OK;
    euf.resize(nu);
    edf.resize(nd);
    for (int64_t i = 0; i < nu; ++i) euf[i] = std::llrint(std::ldexp(eu[i], B.Fd));
    for (int64_t i = 0; i < nd; ++i) edf[i] = std::llrint(std::ldexp(edn[i], B.Fd));
    for (int i = 0; i < p->n_sites; ++i) B.u_fx[i] = std::llrint(std::ldexp(p->u[i], B.Fd));
    B.u0_fx = p->n_sites ? B.u_fx[0] : 0;
  }
  B.diag64 = diag64;
  B.F = F;
  B.m_in = m_in;
  B.max_dn = max_dn;
  B.vec2 = (nd % 2 == 0) ? 1 : 0;
  auto up = [&](auto** dst, const void* src, size_t bytes) -> ed_status {
    ED_CUDA(cudaMalloc((void**)dst, std::max<size_t>(bytes, 8)));
    if (bytes) ED_CUDA(cudaMemcpyAsync(*dst, src, bytes, cudaMemcpyHostToDevice, s));
    return ED_OK;
  };
  ED_TRY(up(&B.up_off, boff.data(), boff.size() * 4));
  ED_TRY(up(&B.up_npos, bnpos.data(), bnpos.size() * 4));
  ED_TRY(up(&B.up_idx, bidx.data(), bidx.size() * 4));
  ED_TRY(up(&B.dn_tab, tab.data(), tab.size() * 2));
  ED_TRY(up(&B.dn_btab2, btab2.data(), btab2.size() * 4));
  B.n_b2 = n_rows / 2;
  B.n_b2pos = pos_pad / 2;
  B.max_up = max_up;
  {
    // staged up lists of the v3 matvec (element offsets must fit int32: checked at variant
    // selection, dim < 2^31)
    const int ls = mv3_layout(nd, B.n_b2, max_up).lstride;
    std::vector<int32_t> lst((size_t)(nu + 1) * ls, 0), cnt((size_t)(nu + 1) * 4, 0);
    for (int64_t r = 0; r < nu; ++r) {
      const int32_t o0 = boff[r], n = boff[r + 1] - o0, np = bnpos[r];
      const int32_t cp = (np + 3) & ~3, cn = ((n - np) + 3) & ~3;
      const int32_t self = (int32_t)(r * nd);
      int32_t* L = lst.data() + (size_t)r * ls;
      for (int e = 0; e < ls; ++e) L[e] = self;
      for (int e = 0; e < np; ++e) L[e] = (int32_t)((int64_t)bidx[o0 + e] * nd);
      for (int e = 0; e < n - np; ++e) L[cp + e] = (int32_t)((int64_t)bidx[o0 + np + e] * nd);
      cnt[(size_t)r * 4 + 0] = cp;
      cnt[(size_t)r * 4 + 1] = cn;
      cnt[(size_t)r * 4 + 2] = (cn - (n - np)) - (cp - np);  // padding copies of the row, with sign
    }
    ED_TRY(up(&B.up_lst, lst.data(), lst.size() * 4));
    ED_TRY(up(&B.up_cnt, cnt.data(), cnt.size() * 4));
    B.up_lstride = ls;
  }
  if (!diag64) {
    ED_TRY(up(&B.e_up_int, eui.data(), eui.size() * 4));
    ED_TRY(up(&B.e_dn_int, edi.data(), edi.size() * 4));
  } else {
    ED_TRY(up(&B.e_up_fx, euf.data(), euf.size() * 8));
    ED_TRY(up(&B.e_dn_fx, edf.data(), edf.size() * 8));
  }
  ED_CUDA(cudaStreamSynchronize(s));
  ED_TRY(build_sweep(p, B, uoff, uidx, ucoef, doff, didx, dcoef, eui, edi, euf, edf, s));
  ED_TRY(build_stripe(p, B, uoff, uidx, ucoef, doff, didx, dcoef, eui, edi, euf, edf, s));
  ED_TRY(build_dncompact(p, B, doff, didx, dcoef, edi, edf, s));
  B.eligible = 1;
  return ED_OK;
}

void free_bfp(ed_plan_s* p) {
  BfpTables& B = p->bfp;
  cudaFree(B.up_off); cudaFree(B.up_npos); cudaFree(B.up_idx); cudaFree(B.dn_tab); cudaFree(B.dn_btab2);
  cudaFree(B.up_lst); cudaFree(B.up_cnt);
  cudaFree(B.e_up_int); cudaFree(B.e_dn_int); cudaFree(B.e_up_fx); cudaFree(B.e_dn_fx);
  free_sweep(B.sw);
  free_stripe(B.sp);
  free_dncompact(B.dc);
  B = BfpTables();
}

// first-wait limit of the bulk-copy matvecs (polls); 0 selects MV3_WAIT_LIMIT
// (-1: no test at all, the first wait gives up at once)
static long wait_limit(const ed_plan_s* p) {
  return p->bfp.wait_limit > 0 ? p->bfp.wait_limit : (p->bfp.wait_limit < 0 ? 0 : MV3_WAIT_LIMIT);
}

static BfpHubArgs bfp_args(const ed_plan_s* p) {
  const BfpTables& B = p->bfp;
  BfpHubArgs a;
  a.nu = p->num_up; a.nd = p->num_dn;
  a.up_off = B.up_off; a.up_npos = B.up_npos; a.up_idx = B.up_idx;
  a.dn_tab = B.dn_tab; a.max_dn = B.max_dn;
  a.up_states = p->up.states; a.dn_states = p->dn.states;
  a.e_up = B.e_up_int; a.e_dn = B.e_dn_int;
  a.u_uniform = B.u_uniform; a.u0 = B.u0_int;
  for (int i = 0; i < ED_MAX_SITES + 2; ++i) a.u[i] = B.u_int[i];
  a.t_int = B.t_int; a.F = B.F;
  a.e_up_fx = B.e_up_fx; a.e_dn_fx = B.e_dn_fx;
  a.u0_fx = B.u0_fx;
  for (int i = 0; i < ED_MAX_SITES + 2; ++i) a.u_fx[i] = B.u_fx[i];
  a.dshift = B.Fd - B.F;
  return a;
}

constexpr int MV_NT = 256;
constexpr size_t MV_SMEM_LIMIT = 200 * 1024;

static size_t v2_smem(const ed_plan_s* p) {
  const size_t xstride = 2 * p->num_dn + 2;
  return MV2_R * xstride * sizeof(int64_t) + (size_t)p->bfp.max_dn * (p->num_dn / 2) * sizeof(uint32_t);
}

static size_t v3_smem(const ed_plan_s* p, bool compact = false) {
  return mv3_layout(p->num_dn, compact ? p->bfp.dc.rows : p->bfp.n_b2, p->bfp.max_up).total;
}

// block size of v3: warps take 64-column chunks; the fewest chunks per warp that fit in
// MV3_MAXNT threads, then as few warps as carry them (3432 columns = 54 chunks -> 27 warps x 2)
static int v3_threads(const ed_plan_s* p) {
  const int64_t chunks = (p->num_dn + 63) / 64;
  const int64_t per = (chunks + MV3_MAXNT / 32 - 1) / (MV3_MAXNT / 32);
  const int64_t warps = (chunks + per - 1) / per;
  return (int)std::min<int64_t>(MV3_MAXNT, 32 * std::max<int64_t>(1, warps));
}

// matvec variant: 7 (the single-pass kernel, bulk-copied double-buffered rows, with the dn
// states renumbered by hop count and per-chunk dn lists) when its tables fit, else 3 (the same
// kernel in the sector's own order, bond-major dn table), else 5 (banded two-pass sweep in a
// renumbered basis, ed_sweep.cuh) when the plan has its tables, else 2 (resident slot table,
// one stage), else 1; 6 (two-pass stripes in a renumbered basis, ed_stripe.cuh), 5 and 3 when
// forced. Rows must have an even length (16-byte row copies). CMPY_ED_MATVEC=1..7 or
// ed_plan_set_matvec_variant forces a variant when possible.
static int matvec_variant(const ed_plan_s* p) {
  static int env_forced = -1;
  if (env_forced < 0) {
    const char* e = getenv("CMPY_ED_MATVEC");
    env_forced = e ? atoi(e) : 0;
  }
  const int forced = p->bfp.force_var > 0 ? p->bfp.force_var : env_forced;
  const size_t optin = (size_t)p->ctx->smem_optin;
  const bool v2_ok = p->bfp.vec2 && v2_smem(p) + MV2_STATIC_SMEM <= optin && p->num_up >= 1;
  // list entries are int32 element offsets u * nd: the vector must have fewer than 2^31 elements
  // (and the table holds 16-bit byte offsets: nd < 4096)
  const bool v3_ok = p->bfp.vec2 && p->bfp.dn_btab2 && p->bfp.up_lst && v3_smem(p) + MV3_STATIC_SMEM <= optin &&
                     p->num_up >= 1 &&
                     p->dim < ((int64_t)1 << 31) && p->num_dn < 4096;
  // two-pass (4): column panels of 4 (nd % 4 == 0), a panel of all rows in half the shared memory
  const bool v4_ok = v3_ok && p->num_dn % MV_PW == 0 && (size_t)p->num_up * MV_PW * 8 + 1024 <= optin / 2;
  const bool v5_ok = p->bfp.sw.on != 0;
  const bool v6_ok = p->bfp.sp.on != 0;
  const bool v7_ok = v3_ok && p->bfp.dc.on != 0;
  if (forced == 1) return 1;
  if (forced == 2) return v2_ok ? 2 : 1;
  if (forced == 3 && v3_ok) return 3;
  if (forced == 4 && v4_ok) return 4;  // measured slower than 3 on GB300 (kept for comparison)
  // the sweep (5) only when asked for, or where the single-pass kernel does not fit: on the
  // 14-site sectors it measured 0.75 ms per H*v against 0.19 ms for 3 (its pass walks one
  // stripe per CTA through the band and waits on every chunk)
  if (v5_ok && forced == 5) return 5;
  if (v6_ok && forced == 6) return 6;
  // 7 (the single-pass kernel with the dn states renumbered by hop count) is 2.8 % faster than
  // 3 on the 14-site sectors and bit-identical to it
  if (v7_ok && (forced == 0 || forced == 7)) return 7;
  if (v3_ok) return 3;
  if (v5_ok) return 5;
  return v2_ok ? 2 : 1;
}

// CTAs of the stripe passes (persistent, as many as the SMs hold)
static int stripe_grid(const ed_plan_s* p, int64_t nstripes, int per_sm) {
  return (int)std::min<int64_t>(nstripes, (int64_t)p->ctx->num_sms * per_sm);
}

// the renumbering of the plan's matvec: variants 5 and 6 keep Lanczos vectors in a renumbered
// basis (pu, pd: new -> old); false for the variants that work in the sector's own order
static bool matvec_perms(const ed_plan_s* p, const int32_t** pu, const int32_t** pd) {
  const int v = matvec_variant(p);
  *pu = *pd = nullptr;
  if (v == 5) {
    *pu = p->bfp.sw.perm_up;
    *pd = p->bfp.sw.perm_dn;
  } else if (v == 6) {
    *pu = p->bfp.sp.perm_up;
    *pd = p->bfp.sp.perm_dn;
  } else if (v == 7) {
    *pu = p->bfp.dc.perm_up;
    *pd = p->bfp.dc.perm_dn;
  }
  return *pu != nullptr;
}

static int bfp_matvec_grid(const ed_plan_s* p) {
  if (matvec_variant(p) == 5) return (int)((p->num_up + SW_W - 1) / SW_W);  // pass 2 writes the partials
  if (matvec_variant(p) == 6) return stripe_grid(p, (p->num_up + ST_K - 1) / ST_K, p->bfp.sp.per_sm_dn);
  if (matvec_variant(p) >= 3)
    return (int)std::min<int64_t>((p->num_up + MV3_R - 1) / MV3_R, (int64_t)p->ctx->num_sms);
  if (matvec_variant(p) == 2)
    return (int)std::min<int64_t>((p->num_up + MV2_R - 1) / MV2_R, (int64_t)p->ctx->num_sms);
  const size_t smem = (2 * p->num_dn + 1) * sizeof(int64_t);
  int per_sm = (int)std::max<size_t>(1, MV_SMEM_LIMIT / std::max<size_t>(smem, 1));
  per_sm = std::min(per_sm, 2048 / MV_NT);
  return (int)std::min<int64_t>(p->num_up, (int64_t)p->ctx->num_sms * per_sm);
}

template <bool DIAG64>
static ed_status launch_v2(const ed_plan_s* p, int g, const int64_t* X, int64_t* W, double* partial,
                           unsigned long long* partial_max, BfpState* st, cudaStream_t s) {
  static std::atomic<uint64_t> done{0};
  const uint64_t bit = 1ull << (p->device & 63);
  if (!(done.load() & bit)) {
    // the opt-in limit covers static + dynamic shared memory of the CTA
    cudaFuncAttributes fa;
    ED_CUDA(cudaFuncGetAttributes(&fa, k_bfp_hub_matvec2<DIAG64>));
    if (fa.sharedSizeBytes > MV2_STATIC_SMEM) return fail(ED_ERR_CUDA, "k_bfp_hub_matvec2: static shared memory above its bound");
    ED_CUDA(cudaFuncSetAttribute(k_bfp_hub_matvec2<DIAG64>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 p->ctx->smem_optin - (int)fa.sharedSizeBytes));
    done.fetch_or(bit);
  }
  k_bfp_hub_matvec2<DIAG64><<<g, MV2_NT, v2_smem(p), s>>>(bfp_args(p), X, W, partial, partial_max, st);
  ED_CHECK_LAUNCH("k_bfp_hub_matvec2");
  return ED_OK;
}

template <bool DIAG64, bool UPW>
static ed_status launch_v3(const ed_plan_s* p, int g, const int64_t* X, int64_t* W, double* partial,
                           unsigned long long* partial_max, BfpState* st, cudaStream_t s, const BfpFuse& fz,
                           bool compact = false) {
  static std::atomic<uint64_t> done{0};
  const uint64_t bit = 1ull << (p->device & 63);
  if (!(done.load() & bit)) {
    cudaFuncAttributes fa;
    ED_CUDA(cudaFuncGetAttributes(&fa, k_bfp_hub_matvec3<DIAG64, UPW>));
    if (fa.sharedSizeBytes > MV3_STATIC_SMEM) return fail(ED_ERR_CUDA, "k_bfp_hub_matvec3: static shared memory above its bound");
    ED_CUDA(cudaFuncSetAttribute(k_bfp_hub_matvec3<DIAG64, UPW>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 p->ctx->smem_optin - (int)fa.sharedSizeBytes));
    if (!UPW) {
      ED_CUDA(cudaFuncGetAttributes(&fa, k_bfp_hub_matvec3<DIAG64, UPW, true>));
      if (fa.sharedSizeBytes > MV3_STATIC_SMEM) return fail(ED_ERR_CUDA, "k_bfp_hub_matvec3: static shared memory above its bound");
      ED_CUDA(cudaFuncSetAttribute(k_bfp_hub_matvec3<DIAG64, UPW, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   p->ctx->smem_optin - (int)fa.sharedSizeBytes));
    }
    if (UPW) ED_CUDA(cudaFuncSetAttribute(k_bfp_up_panels, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          p->ctx->smem_optin / 2));
    done.fetch_or(bit);
  }
  const BfpTables& B = p->bfp;
  int* status = st ? &st->status : p->ctx->d_status;
  if (UPW) {
    const size_t psm = (size_t)p->num_up * MV_PW * 8;
    const int gp = (int)std::min<int64_t>(p->num_dn / MV_PW, (int64_t)p->ctx->num_sms * 2);
    k_bfp_up_panels<<<gp, UP_NT, psm, s>>>(B.up_off, B.up_npos, B.up_idx, p->num_up, p->num_dn, X, W, st);
    ED_CHECK_LAUNCH("k_bfp_up_panels");
  }
  if (compact && !UPW) {
    // variant 7: renumbered dn columns, per-chunk list lengths
    BfpHubArgs a = bfp_args(p);
    a.dn_states = B.dc.s_dn;
    a.e_dn = B.dc.e_dn;
    a.e_dn_fx = B.dc.f_dn;
    k_bfp_hub_matvec3<DIAG64, UPW, true><<<g, v3_threads(p), v3_smem(p, true), s>>>(
        a, B.dc.tab, B.dc.rows, 0, B.dc.chunk, B.max_up, B.up_lst, B.up_cnt, X, W, partial, partial_max, st, status,
        fz, wait_limit(p));
  } else {
    k_bfp_hub_matvec3<DIAG64, UPW><<<g, v3_threads(p), v3_smem(p), s>>>(
        bfp_args(p), B.dn_btab2, B.n_b2, B.n_b2pos, nullptr, B.max_up, B.up_lst, B.up_cnt, X, W, partial,
        partial_max, st, status, fz, wait_limit(p));
  }
  ED_CHECK_LAUNCH("k_bfp_hub_matvec3");
  return ED_OK;
}

// the two sweep passes on renumbered vectors: S = A X into W, then W = t (S + X B) + D X with
// the Lanczos partials (and the step's scalars when fz.on)
template <bool DIAG64>
static ed_status launch_sweep(const ed_plan_s* p, const int64_t* X, int64_t* W, double* partial,
                              unsigned long long* partial_max, BfpState* st, cudaStream_t s, const BfpFuse& fz) {
  static std::atomic<uint64_t> done{0};
  const uint64_t bit = 1ull << (p->device & 63);
  if (!(done.load() & bit)) {
    cudaFuncAttributes fa;
    ED_CUDA(cudaFuncGetAttributes(&fa, k_sweep_up));
    ED_CUDA(cudaFuncSetAttribute(k_sweep_up, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 p->ctx->smem_optin - (int)fa.sharedSizeBytes));
    ED_CUDA(cudaFuncGetAttributes(&fa, k_sweep_dn<DIAG64>));
    ED_CUDA(cudaFuncSetAttribute(k_sweep_dn<DIAG64>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 p->ctx->smem_optin - (int)fa.sharedSizeBytes));
    done.fetch_or(bit);
  }
  const SweepTables& w = p->bfp.sw;
  int* status = st ? &st->status : p->ctx->d_status;
  const int64_t nu = p->num_up, nd = p->num_dn;
  SweepArgs au{nu, nd, w.ring_up, w.nblk_up, w.lst_up, w.win_up, w.pol & 3, wait_limit(p)};
  k_sweep_up<<<(int)((nd + SW_W - 1) / SW_W), SW_NT, sweep_smem_up(w.ring_up), s>>>(au, X, W, st, status);
  SweepArgs ad{nu, nd, w.ring_dn, w.nblk_dn, w.lst_dn, w.win_dn, (w.pol >> 2) & 3, wait_limit(p)};
  const SweepDiag dg{w.s_up, w.s_dn, w.e_up, w.e_dn, w.f_up, w.f_dn};
  k_sweep_dn<DIAG64><<<(int)((nu + SW_W - 1) / SW_W), SW_NT, sweep_smem_dn(w.ring_dn), s>>>(
      bfp_args(p), ad, dg, X, W, partial, partial_max, st, status, fz);
  ED_CHECK_LAUNCH_N("sweep matvec", 2);
  return ED_OK;
}

// the two stripe passes on renumbered vectors: S = A X into W, then W = t (S + X B) + D X with
// the Lanczos partials (and the step's scalars when fz.on)
template <bool DIAG64>
static ed_status launch_stripe(const ed_plan_s* p, const int64_t* X, int64_t* W, double* partial,
                               unsigned long long* partial_max, BfpState* st, cudaStream_t s, const BfpFuse& fz) {
  static std::atomic<uint64_t> done{0};
  const uint64_t bit = 1ull << (p->device & 63);
  if (!(done.load() & bit)) {
    cudaFuncAttributes fa;
    ED_CUDA(cudaFuncGetAttributes(&fa, k_stripe_up));
    ED_CUDA(cudaFuncSetAttribute(k_stripe_up, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 p->ctx->smem_optin - (int)fa.sharedSizeBytes));
    ED_CUDA(cudaFuncSetAttribute(k_stripe_up, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
    ED_CUDA(cudaFuncGetAttributes(&fa, k_stripe_dn<DIAG64>));
    ED_CUDA(cudaFuncSetAttribute(k_stripe_dn<DIAG64>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 p->ctx->smem_optin - (int)fa.sharedSizeBytes));
    ED_CUDA(cudaFuncSetAttribute(k_stripe_dn<DIAG64>, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
    done.fetch_or(bit);
  }
  const StripeTables& T = p->bfp.sp;
  const int64_t nu = p->num_up, nd = p->num_dn;
  const StripeArgs au{nu, nd, T.lst_up, T.meta_up, T.pol & 3};
  k_stripe_up<<<stripe_grid(p, (nd + ST_K - 1) / ST_K, T.per_sm_up), ST_NT, stripe_smem(nu), s>>>(au, X, W, st);
  const StripeArgs ad{nu, nd, T.lst_dn, T.meta_dn, (T.pol >> 2) & 3};
  const StripeDiag dg{T.s_up, T.s_dn, T.e_up, T.e_dn, T.f_up, T.f_dn};
  k_stripe_dn<DIAG64><<<stripe_grid(p, (nu + ST_K - 1) / ST_K, T.per_sm_dn), ST_NT, stripe_smem(nd), s>>>(
      bfp_args(p), ad, dg, X, W, partial, partial_max, st, fz);
  ED_CHECK_LAUNCH_N("stripe matvec", 2);
  return ED_OK;
}

// opt-in to large dynamic shared memory once per (kernel variant, device)
template <bool VEC2, bool DIAG64>
static ed_status launch_variant(const ed_plan_s* p, size_t smem, int g, const int64_t* X, int64_t* W,
                                double* partial, unsigned long long* partial_max, BfpState* st, cudaStream_t s) {
  static std::atomic<uint64_t> done{0};
  const uint64_t bit = 1ull << (p->device & 63);
  if (!(done.load() & bit)) {
    ED_CUDA(cudaFuncSetAttribute(k_bfp_hub_matvec<MV_NT, VEC2, DIAG64>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)MV_SMEM_LIMIT));
    done.fetch_or(bit);
  }
  k_bfp_hub_matvec<MV_NT, VEC2, DIAG64><<<g, MV_NT, smem, s>>>(bfp_args(p), X, W, partial, partial_max, st);
  ED_CHECK_LAUNCH("k_bfp_hub_matvec");
  return ED_OK;
}

// fz (optional): the Lanczos step whose scalars the matvec may compute in its last CTA;
// *fused tells the caller whether it did (then no separate scalars kernel is needed)
static ed_status launch_bfp_matvec(const ed_plan_s* p, const int64_t* X, int64_t* W, double* partial,
                                   unsigned long long* partial_max, BfpState* st, cudaStream_t s,
                                   const BfpFuse* fz = nullptr, bool* fused = nullptr) {
  BfpFuse off{};
  off.on = 0;
  if (fused) *fused = false;
  const size_t smem = (2 * p->num_dn + 1) * sizeof(int64_t);
  const int g = bfp_matvec_grid(p);
  const bool d64 = p->bfp.diag64 != 0;
  // v2/v3 and the paired-column v1 move 16 bytes at a time (bulk row copies, v2 loads and
  // stores): they need 16-byte aligned X and W, always true for the Lanczos store; other
  // caller buffers take the one-column v1 kernel
  // (the stripe matvec checks its own alignment and keeps its renumbered basis)
  const bool aligned = (((uintptr_t)X | (uintptr_t)W) & 15) == 0;
  const int var = (aligned || matvec_variant(p) == 6) ? matvec_variant(p) : 1;
  if (var == 5) {
    // renumbered vectors (the callers that choose variant 5 convert in and out)
    const BfpFuse& f = (fz && partial && st) ? *fz : off;
    if (fused) *fused = f.on != 0;
    return p->bfp.diag64 ? launch_sweep<true>(p, X, W, partial, partial_max, st, s, f)
                         : launch_sweep<false>(p, X, W, partial, partial_max, st, s, f);
  }
  if (var == 6) {
    // renumbered vectors, as for variant 5
    const BfpFuse& f = (fz && partial && st) ? *fz : off;
    if (fused) *fused = f.on != 0;
    return p->bfp.diag64 ? launch_stripe<true>(p, X, W, partial, partial_max, st, s, f)
                         : launch_stripe<false>(p, X, W, partial, partial_max, st, s, f);
  }
  if (var == 7) {
    // renumbered dn columns, as for variants 5 and 6
    const BfpFuse& f = (fz && partial && st) ? *fz : off;
    if (fused) *fused = f.on != 0;
    return d64 ? launch_v3<true, false>(p, g, X, W, partial, partial_max, st, s, f, true)
               : launch_v3<false, false>(p, g, X, W, partial, partial_max, st, s, f, true);
  }
  if (var >= 3) {
    const BfpFuse& f = (fz && partial && st) ? *fz : off;
    if (fused) *fused = f.on != 0;
    if (var == 4)
      return d64 ? launch_v3<true, true>(p, g, X, W, partial, partial_max, st, s, f)
                 : launch_v3<false, true>(p, g, X, W, partial, partial_max, st, s, f);
    return d64 ? launch_v3<true, false>(p, g, X, W, partial, partial_max, st, s, f)
               : launch_v3<false, false>(p, g, X, W, partial, partial_max, st, s, f);
  }
  if (var == 2)
    return d64 ? launch_v2<true>(p, g, X, W, partial, partial_max, st, s)
               : launch_v2<false>(p, g, X, W, partial, partial_max, st, s);
  const bool v2 = p->bfp.vec2 != 0 && aligned;
  if (v2 && !d64) return launch_variant<true, false>(p, smem, g, X, W, partial, partial_max, st, s);
  if (v2 && d64) return launch_variant<true, true>(p, smem, g, X, W, partial, partial_max, st, s);
  if (!v2 && !d64) return launch_variant<false, false>(p, smem, g, X, W, partial, partial_max, st, s);
  return launch_variant<false, true>(p, smem, g, X, W, partial, partial_max, st, s);
}

// ---- the BFP Lanczos driver ----------------------------------------------------------------------
struct BfpLayout {
  size_t off_R, off_W, off_eR, off_maxR, off_part, off_partmax, off_c, off_C, off_work, off_state, off_misc, off_tri,
      total;
  int nslots, nparts;
};

static size_t al256(size_t x) { return (x + 255) & ~(size_t)255; }

static BfpLayout bfp_layout(const ed_plan_s* p, int K, bool store) {
  BfpLayout L;
  const int64_t D = p->dim;
  L.nslots = store ? K + 1 : 3;
  L.nparts = std::max(bfp_matvec_grid(p), p->ctx->num_sms * 8);
  size_t o = 0;
  L.off_R = o; o = al256(o + (size_t)L.nslots * D * 8);
  L.off_W = o; o = al256(o + (size_t)D * 8);
  L.off_eR = o; o = al256(o + (size_t)(K + 2) * 4);
  L.off_maxR = o; o = al256(o + (size_t)(K + 2) * 8);
  L.off_part = o; o = al256(o + (size_t)L.nparts * 8);
  L.off_partmax = o; o = al256(o + (size_t)L.nparts * 8);
  L.off_c = o; o = al256(o + (size_t)(K + 2) * 8);
  L.off_C = o; o = al256(o + (size_t)(K + 2) * 8);
  L.off_work = o; o = al256(o + (size_t)5 * (K + 2) * 8);
  L.off_state = o; o = al256(o + sizeof(BfpState));
  L.off_misc = o; o = al256(o + 64);
  L.off_tri = o; o = al256(o + sizeof(TriResult));
  L.total = o;
  return L;
}

size_t bfp_workspace_bytes(const ed_plan_s* p, int K, bool store) { return bfp_layout(p, K, store).total; }

struct BfpRun {
  BfpLayout L;
  BfpVecs v;
  int64_t* W;
  double *part, *c, *work;
  unsigned long long* partmax;
  int64_t* C;
  BfpState* st;
  int* misc;
  TriResult* tri;
};

static BfpRun bfp_bind(const ed_plan_s* p, void* work, int K, bool store) {
  BfpRun r;
  r.L = bfp_layout(p, K, store);
  char* b = (char*)work;
  r.v.R = (int64_t*)(b + r.L.off_R);
  r.v.eR = (int32_t*)(b + r.L.off_eR);
  r.v.maxR = (unsigned long long*)(b + r.L.off_maxR);
  r.v.store = store ? 1 : 0;
  r.v.D = p->dim;
  r.W = (int64_t*)(b + r.L.off_W);
  r.part = (double*)(b + r.L.off_part);
  r.partmax = (unsigned long long*)(b + r.L.off_partmax);
  r.c = (double*)(b + r.L.off_c);
  r.C = (int64_t*)(b + r.L.off_C);
  r.work = (double*)(b + r.L.off_work);
  r.st = (BfpState*)(b + r.L.off_state);
  r.misc = (int*)(b + r.L.off_misc);
  r.tri = (TriResult*)(b + r.L.off_tri);
  return r;
}

// start vector (FP64, device) -> R_0 in BFP, beta_0 = ||v0||
// (pu, pd non-null: the run's matvec works in a renumbered basis, R_0 is stored in it)
static ed_status bfp_start(const ed_plan_s* p, BfpRun& r, const double* v0, double* beta, cudaStream_t s,
                           const int32_t* pu, const int32_t* pd) {
  const int64_t D = p->dim;
  const int gs = grid_for(D, 256, p->ctx->num_sms * 8);
  unsigned long long* mxb = (unsigned long long*)(r.misc + 8);
  ED_CUDA(cudaMemsetAsync(mxb, 0, 8, s));
  k_maxabs_f64<<<gs, BT, 0, s>>>(v0, D, mxb);
  if (pu)
    k_f64_to_bfp_perm<<<gs, 256, 0, s>>>(v0, p->num_up, p->num_dn, pu, pd, mxb, p->bfp.m_in, r.v.vec(0), r.v.eR,
                                         r.v.maxR);
  else
    k_f64_to_bfp<<<gs, 256, 0, s>>>(v0, D, mxb, p->bfp.m_in, r.v.vec(0), r.v.eR, r.v.maxR);
  k_bfp_norm<<<r.L.nparts, BT, 0, s>>>(r.v, 0, r.part, r.st, beta);
  ED_CHECK_LAUNCH_N("bfp start", 3);
  unsigned long long hm = 0;
  ED_CUDA(cudaMemcpyAsync(&hm, mxb, 8, cudaMemcpyDeviceToHost, s));
  ED_CUDA(cudaStreamSynchronize(s));
  const double mx = *(double*)&hm;
  if (!std::isfinite(mx)) return fail(ED_ERR_NONFINITE, "start vector is not finite");
  if (mx == 0.0) return fail(ED_ERR_ZERO_VECTOR, "start vector has zero norm");
  return ED_OK;
}

// the update kernel of step k; the caller checks and counts the launch
static ed_status launch_update(const ed_plan_s* p, BfpRun& r, int k, double* alpha, double* beta, cudaStream_t s) {
  const bool vec = (p->dim % 2 == 0) && (((uintptr_t)r.v.R | (uintptr_t)r.W) & 15) == 0;
  // one wave: four 256-thread blocks per SM (64 registers), two element pairs per thread in
  // flight; small vectors take only the blocks that have elements (every block joins the
  // reduction of the norm, so idle blocks cost time)
  const int64_t per_block = (int64_t)BT * (vec ? 4 : 1);
  const int need = (int)std::max<int64_t>(1, std::min<int64_t>((p->dim + per_block - 1) / per_block, 1 << 30));
  const int g = std::min({r.L.nparts, p->ctx->num_sms * 4, need});
  if (vec)
    k_bfp_update<true><<<g, BT, 0, s>>>(r.v, k, r.W, r.part, r.partmax, beta, alpha, r.st, 0);
  else
    k_bfp_update<false><<<std::min(r.L.nparts, need), BT, 0, s>>>(r.v, k, r.W, r.part, r.partmax, beta, alpha,
                                                                  r.st, 0);
  return ED_OK;
}

// one Lanczos step k: matvec + scalars + update (3 launches)
static BfpFuse bfp_fuse(const ed_plan_s* p, const BfpRun& r, int k, double* alpha, const double* beta) {
  BfpFuse f;
  f.v = r.v;
  f.k = k;
  f.F = p->bfp.F;
  f.m_in = p->bfp.m_in;
  f.on = 1;
  f.alpha = alpha;
  f.beta = beta;
  return f;
}

static ed_status bfp_step(const ed_plan_s* p, BfpRun& r, int k, double* alpha, double* beta, cudaStream_t s) {
  const int gmv = bfp_matvec_grid(p);
  const BfpFuse fz = bfp_fuse(p, r, k, alpha, beta);
  bool fused = false;
  ED_TRY(launch_bfp_matvec(p, r.v.vec(k), r.W, r.part, r.partmax, r.st, s, &fz, &fused));
  if (!fused)
    k_bfp_scalars<<<1, BT, 0, s>>>(r.v, k, p->bfp.F, p->bfp.m_in, r.part, r.partmax, gmv, alpha, beta, r.st);
  ED_TRY(launch_update(p, r, k, alpha, beta, s));
  ED_CHECK_LAUNCH_N("bfp step", fused ? 1 : 2);
  return ED_OK;
}

}  // namespace ed

using namespace ed;

// Internal entry points used by ed_lanczos / ed_lanczos_coeffs (ed_lanczos.cu).
namespace ed {

ed_status bfp_lanczos(const ed_plan_s* p, const ed_lanczos_params* prm, const double* v0_dev, void* work,
                      double* alpha, double* beta, double* evec, ed_lanczos_result* res, cudaStream_t s,
                      double* v0_tmp /* FP64[D] scratch when v0 is generated */) {
  const int K = prm->max_steps;
  const int64_t D = p->dim;
  const bool store = prm->want_vector != 0;
  BfpRun r = bfp_bind(p, work, K, store);
  const int32_t *pu, *pd;
  (void)matvec_perms(p, &pu, &pd);
  ED_CUDA(cudaMemsetAsync(r.st, 0, sizeof(BfpState), s));
  ED_CUDA(cudaMemsetAsync(alpha, 0, K * sizeof(double), s));
  ED_CUDA(cudaMemsetAsync(beta, 0, (K + 1) * sizeof(double), s));
  ED_TRY(bfp_start(p, r, v0_dev, beta, s, pu, pd));
  const int Km = (int)std::min<int64_t>(K, D);
  std::vector<cudaEvent_t> ev;
  if (prm->profile) {
    ev.resize(2 * (size_t)Km);
    for (auto& e : ev) ED_CUDA(cudaEventCreate(&e));
  }
  // convergence tests on a side stream and the final eigenpair, on the device (ed_lzcheck.cuh)
  const bool checks = prm->check_every > 0 && prm->tol > 0.0;
  SideChecks chk;
  ED_TRY(chk.init(checks ? Km / prm->check_every + 1 : 0));
  ED_CUDA(cudaMemsetAsync(r.tri, 0, sizeof(TriResult), s));
  int launched = 0;
  for (int k = 0; k < Km; ++k) {
    if (checks && chk.stopped()) break;
    if (prm->profile) ED_CUDA(cudaEventRecord(ev[2 * k], s));
    const BfpFuse fz = bfp_fuse(p, r, k, alpha, beta);
    bool fused = false;
    ED_TRY(launch_bfp_matvec(p, r.v.vec(k), r.W, r.part, r.partmax, r.st, s, &fz, &fused));
    if (prm->profile) ED_CUDA(cudaEventRecord(ev[2 * k + 1], s));
    if (!fused)
      k_bfp_scalars<<<1, BT, 0, s>>>(r.v, k, p->bfp.F, p->bfp.m_in, r.part, r.partmax, bfp_matvec_grid(p), alpha,
                                     beta, r.st);
    ED_TRY(launch_update(p, r, k, alpha, beta, s));
    ED_CHECK_LAUNCH_N("bfp lanczos step", fused ? 1 : 2);
    launched = k + 1;
    if (checks && ((k + 1) % prm->check_every == 0) && k + 1 < Km)
      ED_TRY(chk.launch(s, alpha, beta, k + 1, prm->tol, &r.st->stop, &r.st->steps, r.tri, r.c, r.work));
  }
  ED_TRY(chk.join(s));
  k_tri_final<<<1, TRI_NT, 0, s>>>(alpha, beta, launched, &r.st->stop, &r.st->steps, r.tri, r.c, r.work);
  ED_CHECK_LAUNCH("k_tri_final");
  if (evec) {
    k_bfp_ritz_coef<<<1, BT, 0, s>>>(r.c, beta, r.v.eR, r.tri, r.C, r.misc);
    // (the stored vectors are 16-byte aligned when D is even: base 256-aligned, slots of D)
    if (D % 2 == 0)
      k_bfp_ritz<true><<<p->ctx->num_sms * 8, 256, 0, s>>>(r.v, r.C, r.misc, r.st, evec, pu, pd, p->num_dn);
    else
      k_bfp_ritz<false><<<grid_for(D, 256, p->ctx->num_sms * 8), 256, 0, s>>>(r.v, r.C, r.misc, r.st, evec, pu,
                                                                            pd, p->num_dn);
    ED_CHECK_LAUNCH_N("k_bfp_ritz", 2);
  }
  BfpState hs;
  TriResult ht;
  ED_CUDA(cudaMemcpyAsync(&hs, r.st, sizeof(BfpState), cudaMemcpyDeviceToHost, s));
  ED_CUDA(cudaMemcpyAsync(&ht, r.tri, sizeof(TriResult), cudaMemcpyDeviceToHost, s));
  ED_CUDA(cudaStreamSynchronize(s));
  if (hs.status == DEV_TIMEOUT) return fail(ED_ERR_TIMEOUT, "fixed-point matvec: a bounded wait for a row copy ran out");
  const int m = ht.m_final;
  res->energy = ht.energy;
  res->residual = ht.residual;
  res->steps = m;
  res->converged = hs.stop;
  res->status = hs.status;
  res->matvec_ms = 0.0;
  res->matvecs = 0;
  if (prm->profile) {
    for (int k = 0; k < m; ++k) {
      float ms = 0.f;
      ED_CUDA(cudaEventElapsedTime(&ms, ev[2 * k], ev[2 * k + 1]));
      res->matvec_ms += ms;
      res->matvecs += 1;
    }
    for (auto& e : ev) cudaEventDestroy(e);
  }
  (void)v0_tmp;
  return ED_OK;
}

// a coefficient run in three parts, so that several independent runs can interleave their
// steps on separate streams (bfp_lanczos_coeffs_multi)
struct BfpCoeffRun {
  const ed_plan_s* p;
  BfpRun r;
  double *alpha, *beta;
  int Km = 0;
  bool empty = false;  // zero start vector: an empty Krylov space
};

// memsets, the start vector's finiteness and zero test (synchronous on s), R_0 and beta_0
static ed_status bfp_coeffs_begin(const ed_plan_s* p, int K, const double* start, void* work, double* alpha,
                                  double* beta, cudaStream_t s, BfpCoeffRun* run) {
  const int64_t D = p->dim;
  run->p = p;
  run->r = bfp_bind(p, work, K, false);
  run->alpha = alpha;
  run->beta = beta;
  BfpRun& r = run->r;
  ED_CUDA(cudaMemsetAsync(r.st, 0, sizeof(BfpState), s));
  ED_CUDA(cudaMemsetAsync(alpha, 0, K * sizeof(double), s));
  ED_CUDA(cudaMemsetAsync(beta, 0, (K + 1) * sizeof(double), s));
  {
    const int gs = grid_for(D, 256, p->ctx->num_sms * 8);
    unsigned long long* mxb = (unsigned long long*)(r.misc + 8);
    ED_CUDA(cudaMemsetAsync(mxb, 0, 8, s));
    k_maxabs_f64<<<gs, BT, 0, s>>>(start, D, mxb);
    ED_CHECK_LAUNCH("k_maxabs_f64");
    unsigned long long hm = 0;
    ED_CUDA(cudaMemcpyAsync(&hm, mxb, 8, cudaMemcpyDeviceToHost, s));
    ED_CUDA(cudaStreamSynchronize(s));
    const double mx = *(double*)&hm;
    if (!std::isfinite(mx)) return fail(ED_ERR_NONFINITE, "start vector is not finite");
    if (mx == 0.0) {
      run->empty = true;
      return ED_OK;
    }
  }
  const int32_t *pu, *pd;
  (void)matvec_perms(p, &pu, &pd);
  ED_TRY(bfp_start(p, r, start, beta, s, pu, pd));
  run->Km = (int)std::min<int64_t>(K, D);
  return ED_OK;
}

// the run's steps and norm once its stream has finished (synchronous on s)
static ed_status bfp_coeffs_end(BfpCoeffRun& run, int* steps, double* norm, cudaStream_t s) {
  if (run.empty) {
    *steps = 0;
    *norm = 0.0;
    return ED_OK;
  }
  BfpState hs;
  double b0 = 0.0;
  ED_CUDA(cudaMemcpyAsync(&hs, run.r.st, sizeof(BfpState), cudaMemcpyDeviceToHost, s));
  ED_CUDA(cudaMemcpyAsync(&b0, run.beta, sizeof(double), cudaMemcpyDeviceToHost, s));
  ED_CUDA(cudaStreamSynchronize(s));
  if (hs.status == DEV_TIMEOUT) return fail(ED_ERR_TIMEOUT, "fixed-point matvec: a bounded wait for a row copy ran out");
  *steps = hs.stop ? hs.steps : run.Km;
  *norm = b0;
  // the continued fraction expects beta[0] = 0 and beta[k] the couplings
  ED_CUDA(cudaMemsetAsync(run.beta, 0, sizeof(double), s));
  ED_CUDA(cudaStreamSynchronize(s));
  return ED_OK;
}

ed_status bfp_lanczos_coeffs(const ed_plan_s* p, int K, const double* start, void* work, double* alpha,
                             double* beta, int* steps, double* norm, cudaStream_t s) {
  BfpCoeffRun run;
  ED_TRY(bfp_coeffs_begin(p, K, start, work, alpha, beta, s, &run));
  for (int k = 0; k < run.Km; ++k) ED_TRY(bfp_step(p, run.r, k, alpha, beta, s));
  return bfp_coeffs_end(run, steps, norm, s);
}

// n independent coefficient runs with interleaved steps: run i on its own stream, forked from
// and joined back into s. Each step of a run is two kernels that each fill the GPU for most
// of their time; interleaving lets one run's kernels start on the SMs that the other run's
// last partial round leaves idle. Results are those of the runs done one after another.
ed_status bfp_lanczos_coeffs_multi(int n, const ed_plan_s* const* plans, int K, const double* const* starts,
                                   void* const* works, double* const* alphas, double* const* betas, int* steps,
                                   double* norms, cudaStream_t s) {
  std::vector<cudaStream_t> ss(n, nullptr);
  std::vector<BfpCoeffRun> runs(n);
  cudaEvent_t fork = nullptr;
  ed_status st = ED_OK;
  auto cleanup = [&]() {
    for (auto& x : ss)
      if (x) cudaStreamDestroy(x);
    if (fork) cudaEventDestroy(fork);
  };
  auto check = [&](cudaError_t e, const char* what) {
    if (e != cudaSuccess && st == ED_OK) st = cuda_fail(e, what);
  };
  check(cudaEventCreateWithFlags(&fork, cudaEventDisableTiming), "cudaEventCreateWithFlags");
  if (st == ED_OK) check(cudaEventRecord(fork, s), "cudaEventRecord");
  for (int i = 0; i < n && st == ED_OK; ++i) {
    check(cudaStreamCreateWithFlags(&ss[i], cudaStreamNonBlocking), "cudaStreamCreateWithFlags");
    if (st == ED_OK) check(cudaStreamWaitEvent(ss[i], fork, 0), "cudaStreamWaitEvent");
    if (st == ED_OK) st = bfp_coeffs_begin(plans[i], K, starts[i], works[i], alphas[i], betas[i], ss[i], &runs[i]);
  }
  int kmax = 0;
  for (int i = 0; i < n && st == ED_OK; ++i) kmax = std::max(kmax, runs[i].Km);
  for (int k = 0; k < kmax && st == ED_OK; ++k)
    for (int i = 0; i < n && st == ED_OK; ++i)
      if (k < runs[i].Km) st = bfp_step(runs[i].p, runs[i].r, k, runs[i].alpha, runs[i].beta, ss[i]);
  for (int i = 0; i < n && st == ED_OK; ++i) st = bfp_coeffs_end(runs[i], &steps[i], &norms[i], ss[i]);
  if (st != ED_OK)
    for (auto& x : ss)
      if (x) cudaStreamSynchronize(x);  // nothing of a failed call stays in flight
  cleanup();
  return st;
}

}  // namespace ed

extern "C" {

ED_API ed_status ed_fixed_from_f64(const double* d_x, int64_t n, int m_bits, int64_t* d_xm, int32_t* h_exp,
                                   ed_stream_t stream) {
  if (n < 0 || m_bits < 1 || m_bits > 62) return fail(ED_ERR_INVALID_ARG, "bad n / m_bits");
  if (n == 0) { *h_exp = 0; return ED_OK; }
  if (!d_x || !d_xm || !h_exp) return fail(ED_ERR_INVALID_ARG, "null argument");
  DeviceContext* ctx;
  ED_TRY(device_context(&ctx));
  cudaStream_t s = as_stream(stream);
  unsigned long long* tmp = nullptr;
  ED_CUDA(cudaMallocAsync(&tmp, 32, s));
  ED_CUDA(cudaMemsetAsync(tmp, 0, 32, s));
  const int g = grid_for(n, 256, ctx->num_sms * 8);
  k_maxabs_f64<<<g, BT, 0, s>>>(d_x, n, tmp);
  k_f64_to_bfp<<<g, 256, 0, s>>>(d_x, n, tmp, m_bits, d_xm, (int32_t*)(tmp + 1), tmp + 2);
  ED_CHECK_LAUNCH_N("ed_fixed_from_f64", 2);
  unsigned long long h[3];
  ED_CUDA(cudaMemcpyAsync(h, tmp, 24, cudaMemcpyDeviceToHost, s));
  ED_CUDA(cudaStreamSynchronize(s));
  ED_CUDA(cudaFreeAsync(tmp, s));
  const double mx = *(double*)&h[0];
  if (!std::isfinite(mx)) return fail(ED_ERR_NONFINITE, "input is not finite");
  *h_exp = *(int32_t*)&h[1];
  return ED_OK;
}

ED_API ed_status ed_fixed_to_f64(const int64_t* d_xm, int64_t n, int32_t exp, double* d_x, ed_stream_t stream) {
  if (n < 0) return fail(ED_ERR_INVALID_ARG, "negative n");
  if (n == 0) return ED_OK;
  if (!d_xm || !d_x) return fail(ED_ERR_INVALID_ARG, "null argument");
  DeviceContext* ctx;
  ED_TRY(device_context(&ctx));
  cudaStream_t s = as_stream(stream);
  int32_t* e = nullptr;
  ED_CUDA(cudaMallocAsync(&e, 4, s));
  ED_CUDA(cudaMemcpyAsync(e, &exp, 4, cudaMemcpyHostToDevice, s));
  k_bfp_to_f64<<<grid_for(n, 256, ctx->num_sms * 8), 256, 0, s>>>(d_xm, e, n, d_x);
  ED_CHECK_LAUNCH("k_bfp_to_f64");
  ED_CUDA(cudaFreeAsync(e, s));
  ED_CUDA(cudaStreamSynchronize(s));
  return ED_OK;
}

ED_API ed_status ed_matvec_fixed(ed_plan p, const int64_t* d_xm, int32_t ex, int64_t* d_wm, int32_t* h_ew,
                                 int* h_m_in, ed_stream_t stream) {
  ED_TRY(check_plan(p));
  if (!p->bfp.eligible) return fail(ED_ERR_INVALID_ARG, "sector has no fixed-point matvec (needs one hopping magnitude and dyadic coefficients)");
  if (h_m_in) *h_m_in = p->bfp.m_in;
  if (h_ew) *h_ew = ex - p->bfp.F;
  if (p->dim == 0) return ED_OK;
  if (!d_xm || !d_wm) return fail(ED_ERR_INVALID_ARG, "null vector");
  if (d_xm == d_wm) return fail(ED_ERR_INVALID_ARG, "x and w must not alias");
  cudaStream_t s = as_stream(stream);
  const int32_t *pu, *pd;
  if (matvec_perms(p, &pu, &pd)) {
    // the matvec works in its renumbered basis: renumber x, apply, renumber back (through an
    // aligned scratch buffer, whatever the alignment of the caller's vectors)
    int64_t* tmp = nullptr;
    const int64_t off = (p->dim + 1) & ~(int64_t)1;  // W 16-byte aligned like X
    ED_CUDA(cudaMallocAsync((void**)&tmp, (size_t)(off + p->dim) * sizeof(int64_t), s));
    const int g = grid_for(p->dim, 256, p->ctx->num_sms * 8);
    k_sweep_permute<<<g, 256, 0, s>>>(d_xm, tmp, p->num_up, p->num_dn, pu, pd, 1);
    ED_CHECK_LAUNCH("k_sweep_permute");
    ed_status st = launch_bfp_matvec(p, tmp, tmp + off, nullptr, nullptr, nullptr, s);
    if (st == ED_OK) {
      k_sweep_permute<<<g, 256, 0, s>>>(tmp + off, d_wm, p->num_up, p->num_dn, pu, pd, 0);
      ED_CHECK_LAUNCH("k_sweep_permute");
    }
    ED_CUDA(cudaFreeAsync(tmp, s));
    return st;
  }
  return launch_bfp_matvec(p, d_xm, d_wm, nullptr, nullptr, nullptr, s);
}

ED_API ed_status ed_plan_set_wait_limit(ed_plan p, int64_t polls) {
  ED_TRY(check_plan(p));
  if (polls < -1) return fail(ED_ERR_INVALID_ARG, "polls must be >= -1");
  p->bfp.wait_limit = (long)polls;
  return ED_OK;
}

ED_API int ed_plan_matvec_variant(ed_plan p) { return (p && p->bfp.eligible) ? matvec_variant(p) : 0; }

ED_API ed_status ed_plan_set_matvec_variant(ed_plan p, int variant) {
  ED_TRY(check_plan(p));
  if (variant < 0 || variant > 7) return fail(ED_ERR_INVALID_ARG, "variant must be in [0, 7]");
  p->bfp.force_var = variant;
  return ED_OK;
}

ED_API int ed_plan_fixed_point(ed_plan p) { return (p && p->bfp.eligible) ? p->bfp.m_in : 0; }

}  // extern "C"
