// Two-pass fixed-point H·v on whole stripes ("stripe" matvec, variant 6), included by ed_bfp.cu
// inside namespace ed after ed_sweep.cuh (it uses their copy, store, diagonal and reduction
// helpers; the host tables are in ed_stripe_tables.h).
//
// With the vector viewed as X[u][d] (num_up x num_dn, up-major like the reference's
// idx = up * num_dn + dn), H x = t (A X + X B) + D∘X: A and B are the single-spin hop matrices
// (entries +-1), D the diagonal.
//
// * Pass 1 (k_stripe_up): a CTA copies a whole stripe of 4 columns of X (every row: 32 bytes
//   per row, 110 KB for 3432 rows, two CTAs per SM) into shared memory with async copies,
//   waits once, and forms S = A X for the stripe. Lane = target row; each hop partner is one
//   32-byte record, read as two 16-byte shared loads that give its four columns. S goes to
//   the output buffer.
// * Pass 2 (k_stripe_dn): a CTA copies 4 whole rows of X into shared memory as 32-byte column
//   records (element (r, d) in record d) and forms X B the same way (lane = target column),
//   then writes W = t (S + X B) + D X over S, with the exact <X, W> partials and max |W|; the
//   last CTA to finish computes the Lanczos step's scalars.
// * The states of each spin species are renumbered by their numbers of + and - hops, so the
//   32 targets of a warp share their list lengths (no padded gathers, no divergence). A
//   Lanczos run keeps its vectors in that basis: the start vector is gathered into it and the
//   Ritz vector scattered back. alpha and beta do not change: every dot product is an exact
//   integer sum per element.
// * In every other group of four records the two halves are swapped (stripe_slot), so the
//   first halves of random records fall on all eight 16-byte bank groups.
//
// Neither pass waits on a barrier or another CTA: each stripe's copies end with
// cp.async.wait_all. Traffic per H·v: X twice (8 B/element each), S written and read, W
// written: 40 B/element from DRAM when nothing stays in L2; algorithmic 16 B/element.
#pragma once

struct StripeArgs {
  int64_t nu, nd;
  const uint32_t* lst;    // hop list pairs of the targets of this pass, [pair][n]
  const uint16_t* meta;   // + pairs | - pairs << 8 per target
  int pol;                // L2 policies: bit 0 X loads, bit 1 S stores (pass 1) / W stores (pass 2)
};

// adds the two records of a list word (slot | slot << 16) to a0..a3
__device__ __forceinline__ void stripe_gather2(const unsigned char* sm, uint32_t w, int64_t& a0, int64_t& a1,
                                               int64_t& a2, int64_t& a3) {
  const uint32_t s0 = w & 0xffffu, s1 = w >> 16;
  const longlong2 p0 = *(const longlong2*)(sm + (s0 << 4));
  const longlong2 q0 = *(const longlong2*)(sm + ((s0 ^ 1u) << 4));
  const longlong2 p1 = *(const longlong2*)(sm + (s1 << 4));
  const longlong2 q1 = *(const longlong2*)(sm + ((s1 ^ 1u) << 4));
  a0 += p0.x + p1.x;
  a1 += p0.y + p1.y;
  a2 += q0.x + q1.x;
  a3 += q0.y + q1.y;
}

// sum over the hop list of target t (n targets): + pairs minus - pairs, four columns; every
// lane of the warp calls it (the loop bounds are the warp's largest list lengths)
__device__ __forceinline__ void stripe_hops(const unsigned char* sm, const StripeArgs& a, int64_t n, int64_t t,
                                            bool valid, int64_t r[ST_K]) {
  const uint32_t m = valid ? (uint32_t)__ldg(a.meta + t) : 0u;
  const int pp = (int)(m & 0xffu), pn = (int)(m >> 8);
  const int tmax = (int)__reduce_max_sync(0xffffffffu, (unsigned)(pp + pn));
  uint32_t wv[ST_PMAX];
#pragma unroll
  for (int p = 0; p < ST_PMAX; ++p) wv[p] = (p < pp + pn) ? __ldg(a.lst + (size_t)p * n + t) : 0u;
  int64_t a0 = 0, a1 = 0, a2 = 0, a3 = 0, b0 = 0, b1 = 0, b2 = 0, b3 = 0;
#pragma unroll
  for (int p = 0; p < ST_PMAX; ++p) {
    if (p < tmax && p < pp + pn) {
      if (p < pp) stripe_gather2(sm, wv[p], a0, a1, a2, a3);
      else stripe_gather2(sm, wv[p], b0, b1, b2, b3);
    }
  }
  r[0] = a0 - b0;
  r[1] = a1 - b1;
  r[2] = a2 - b2;
  r[3] = a3 - b3;
}

// a load of S that the compiler must not move out of its condition (S may end at the last
// row, and lanes past the last column would read beyond it)
__device__ __forceinline__ int64_t stripe_ld_s(const int64_t* p, uint64_t pol) {
  int64_t v;
  asm volatile("ld.global.nc.L2::cache_hint.s64 %0, [%1], %2;" : "=l"(v) : "l"(p), "l"(pol));
  return v;
}

// element j of record i
__device__ __forceinline__ int64_t* stripe_elem(unsigned char* sm, int64_t i, int j) {
  return (int64_t*)(sm + ((stripe_slot(i) ^ (uint32_t)(j >> 1)) << 4) + ((j & 1) << 3));
}

// shared memory of a pass over n targets (records 0..n-1 and the zero record n)
__host__ __device__ constexpr size_t stripe_smem(int64_t n) { return (size_t)(n + 1) * 32; }

// ---- pass 1: S = A X, 4-column stripes ---------------------------------------------------------
__global__ void __launch_bounds__(ST_NT, 2)
    k_stripe_up(StripeArgs a, const int64_t* __restrict__ X, int64_t* __restrict__ S, BfpState* st) {
  if (st && *(volatile int*)&st->stop) return;
  extern __shared__ __align__(128) unsigned char sm_stu[];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int64_t nu = a.nu, nd = a.nd;
  const int64_t nstripes = (nd + ST_K - 1) / ST_K;
  const uint64_t pol_x = sweep_policy(a.pol, 0), pol_s = sweep_policy(a.pol, 1);
  if (tid < ST_K) *stripe_elem(sm_stu, nu, tid) = 0;  // the zero record
  // 16-byte copies and stores need even rows and 16-byte aligned X and S (Lanczos vectors of
  // odd dimension alternate their alignment)
  const bool even = (nd & 1) == 0 && (((uintptr_t)X | (uintptr_t)S) & 15) == 0;
  for (int64_t sI = blockIdx.x; sI < nstripes; sI += gridDim.x) {
    const int64_t c0 = sI * ST_K;
    const int ncols = (int)min((int64_t)ST_K, nd - c0);
    if (even && ncols == ST_K) {
      // two 16-byte copies per row
      for (int64_t q = tid; q < 2 * nu; q += ST_NT) {
        const int64_t u = q >> 1;
        const uint32_t h = (uint32_t)(q & 1);
        cp_async16(sm_stu + ((stripe_slot(u) ^ h) << 4), X + u * nd + c0 + 2 * h, pol_x);
      }
    } else {
      for (int64_t q = tid; q < ST_K * nu; q += ST_NT) {
        const int64_t u = q >> 2;
        const int j = (int)(q & 3);
        int64_t* dst = stripe_elem(sm_stu, u, j);
        if (j < ncols) cp_async8(dst, X + u * nd + c0 + j, pol_x);
        else *dst = 0;
      }
    }
    cp_async_wait_all();
    __syncthreads();
    for (int64_t ub = (int64_t)warp * 32; ub < nu; ub += ST_NT) {
      const int64_t u = ub + lane;
      const bool valid = u < nu;
      int64_t r[ST_K];
      stripe_hops(sm_stu, a, nu, u, valid, r);
      if (valid) {
        int64_t* o = S + u * nd + c0;
        if (even && ncols == ST_K) {
          st2_stream(o, r[0], r[1], pol_s);
          st2_stream(o + 2, r[2], r[3], pol_s);
        } else {
#pragma unroll
          for (int j = 0; j < ST_K; ++j)
            if (j < ncols) st_stream(o + j, r[j], pol_s);
        }
      }
    }
    __syncthreads();  // the stripe buffer is free for the next copy
  }
}

// per-element diagonal data of pass 2 (renumbered tables)
struct StripeDiag {
  const uint64_t* s_up; const uint64_t* s_dn;
  const int32_t* e_up; const int32_t* e_dn;
  const int64_t* f_up; const int64_t* f_dn;
};

// ---- pass 2: W = t (S + X B) + D X, 4-row stripes, with the Lanczos partials -----------------------
template <bool DIAG64>
__global__ void __launch_bounds__(ST_NT, 2)
    k_stripe_dn(BfpHubArgs h, StripeArgs a, StripeDiag dg, const int64_t* __restrict__ X, int64_t* W,
                double* partial, unsigned long long* partial_max, BfpState* st, BfpFuse fz) {
  if (st && *(volatile int*)&st->stop) return;
  extern __shared__ __align__(128) unsigned char sm_std[];
  __shared__ double smd[ST_NT / 32];
  __shared__ unsigned long long smu[ST_NT / 32];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int64_t nu = a.nu, nd = a.nd;
  const int64_t nstripes = (nu + ST_K - 1) / ST_K;
  const uint64_t pol_x = sweep_policy(a.pol, 0), pol_w = sweep_policy(a.pol, 1), pol_s = policy_evict_first();
  if (tid < ST_K) *stripe_elem(sm_std, nd, tid) = 0;  // the zero record
  I128 dot{0, 0};
  unsigned long long mx = 0;
  for (int64_t sI = blockIdx.x; sI < nstripes; sI += gridDim.x) {
    const int64_t u0 = sI * ST_K;
    const int nrows = (int)min((int64_t)ST_K, nu - u0);
    for (int j = 0; j < ST_K; ++j) {
      for (int64_t d = tid; d < nd; d += ST_NT) {
        int64_t* dst = stripe_elem(sm_std, d, j);
        if (j < nrows) cp_async8(dst, X + (u0 + j) * nd + d, pol_x);
        else *dst = 0;
      }
    }
    cp_async_wait_all();
    __syncthreads();
    for (int64_t db = (int64_t)warp * 32; db < nd; db += ST_NT) {
      const int64_t d = db + lane;
      const bool valid = d < nd;
      // S of the four rows (written by pass 1), requested first
      int64_t sv[ST_K];
#pragma unroll
      for (int j = 0; j < ST_K; ++j) sv[j] = (valid && j < nrows) ? stripe_ld_s(W + (u0 + j) * nd + d, pol_s) : 0;
      const uint64_t sd = valid ? __ldg(dg.s_dn + d) : 0;
      const int64_t ed = !valid ? 0 : (DIAG64 ? __ldg(dg.f_dn + d) : (int64_t)__ldg(dg.e_dn + d));
      int64_t r[ST_K];
      stripe_hops(sm_std, a, nd, d, valid, r);
      if (!valid) continue;
      const uint32_t so = stripe_slot(d);
      const longlong2 x01 = *(const longlong2*)(sm_std + (so << 4));
      const longlong2 x23 = *(const longlong2*)(sm_std + ((so ^ 1u) << 4));
      const int64_t xv[ST_K] = {x01.x, x01.y, x23.x, x23.y};
#pragma unroll
      for (int j = 0; j < ST_K; ++j) {
        if (j >= nrows) break;
        const int64_t u = u0 + j;
        const uint64_t su = __ldg(dg.s_up + u);
        const int64_t eu = DIAG64 ? 0 : (int64_t)__ldg(dg.e_up + u);
        const int64_t ef = DIAG64 ? __ldg(dg.f_up + u) : 0;
        const int64_t ww = (int64_t)h.t_int * (sv[j] + r[j]) +
                           bfp_diag_col<DIAG64>(h, eu, ef, su, sd, DIAG64 ? 0 : (int32_t)ed, DIAG64 ? ed : 0, xv[j]);
        st_stream(W + u * nd + d, ww, pol_w);
        add128(dot, mul_s64(xv[j], ww));
        mx = max(mx, uabs64(ww));
      }
    }
    __syncthreads();  // the stripe buffer is free for the next copy
  }
  if (!partial) return;
  const double sdot = block_sum<ST_NT>(i128_to_double(dot), smd);
  const unsigned long long m = block_max_u64<ST_NT>(mx, smu);
  if (tid == 0) {
    partial[blockIdx.x] = sdot;
    partial_max[blockIdx.x] = m;
  }
  if (fz.on && st && bfp_last_block(&st->ticket[2])) {
    double t = 0.0;
    unsigned long long mm = 0;
    for (int b = tid; b < (int)gridDim.x; b += ST_NT) {
      t += ((volatile double*)partial)[b];
      mm = max(mm, ((volatile unsigned long long*)partial_max)[b]);
    }
    t = block_sum<ST_NT>(t, smd);
    mm = block_max_u64<ST_NT>(mm, smu);
    if (tid == 0) {
      bfp_scalars_tail(fz.v, fz.k, fz.F, fz.m_in, t, mm, fz.alpha, fz.beta, st);
      st->ticket[2] = 0;
    }
  }
}
