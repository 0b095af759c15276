// Banded two-pass fixed-point H·v ("sweep" matvec), included by ed_bfp.cu inside namespace ed
// (it uses that file's 128-bit, mbarrier and bulk-copy helpers; the host tables are in
// ed_sweep_tables.h).
//
// With the vector viewed as X[u][d] (num_up x num_dn, up-major like the reference's
// idx = up * num_dn + dn), H x = t (A X + X B) + D∘X: A and B are the single-spin hop matrices
// (entries +-1), D the diagonal. The single-pass kernels of ed_bfp.cu gather ~7.5 whole
// neighbour rows of X from L2 per target row (5x the vector per H·v crosses from L2), which
// makes them latency-bound. Here each pass reads X exactly once from memory:
//
// * The up and the dn states are renumbered in reverse Cuthill-McKee order of their hop graph.
//   That makes A and B banded (14 sites, 7 particles: bandwidth 1912 in ascending order, 369
//   renumbered). A Lanczos run keeps its vectors in the renumbered basis: the start vector is
//   gathered into it and the Ritz vector scattered back. alpha and beta do not change: every
//   dot product is an exact integer sum per element.
// * Pass 1 (k_sweep_up): one CTA per 16-column stripe of X walks down the rows in blocks of
//   32. A ring of row chunks (32 rows x 16 columns = 4 KB as 256 16-byte async copies, each
//   thread arriving on the chunk's mbarrier once its copy has landed) holds the band around
//   the current block; each chunk is copied once. A half-warp forms one target row's 16 sums
//   S = A X from its hop list (entries are precomputed ring offsets), lane = column, so a
//   gather reads one contiguous 128-byte ring row (one shared-memory wavefront). Output S goes to the W buffer.
// * Pass 2 (k_sweep_dn): one CTA per 16-row stripe walks along the columns in blocks of 32. A
//   ring of column chunks (16 rows x 32 columns, 8-byte async copies) is laid out with a row
//   stride of (ring columns + 1) elements, so the 16 rows of one column sit in 16 different
//   bank pairs: a half-warp (lane = row) gathers one dn partner for 16 rows in one wavefront.
//   The epilogue (one row per warp, consecutive columns per lane) reads S, adds the diagonal
//   term, writes W = t (S + X B) + D X in place, and forms the exact <X, W> partials and
//   max |W|; the last CTA to finish computes the Lanczos step's scalars.
//
// Traffic per H·v: X twice (8 B/element each), S written and read, W written: 40 B/element
// from DRAM when nothing stays in L2 (S and W share the buffer, so S can stay in L2 between
// the passes); algorithmic 16 B/element.
#pragma once

// ---- device helpers ------------------------------------------------------------------------------

__device__ __forceinline__ void cp_async8(void* dst, const void* src, uint64_t pol) {
  asm volatile("cp.async.ca.shared.global.L2::cache_hint [%0], [%1], 8, %2;" ::"r"(smem_u32(dst)), "l"(src), "l"(pol)
               : "memory");
}
__device__ __forceinline__ void cp_async16(void* dst, const void* src, uint64_t pol) {
  asm volatile("cp.async.cg.shared.global.L2::cache_hint [%0], [%1], 16, %2;" ::"r"(smem_u32(dst)), "l"(src), "l"(pol)
               : "memory");
}
// after a wait gave up: let copies that may still be in flight land before the CTA leaves
// (about 0.1 ms; a copy takes microseconds)
__device__ __forceinline__ void sweep_settle() {
  for (int i = 0; i < 3000; ++i) __nanosleep(32);
}
// arrive on `bar` once this thread's earlier cp.async copies have landed (no pending-count
// increment: the barrier is initialised with one arrival per thread)
__device__ __forceinline__ void cp_async_arrive(uint64_t* bar) {
  asm volatile("cp.async.mbarrier.arrive.noinc.shared::cta.b64 [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

static_assert(SW_NT >= SW_CH * SW_W / 2, "pass 1 copies a chunk as 16-byte pieces, one per thread");
static_assert(SW_NT == SW_CH * SW_W, "pass 2 copies a chunk as 8-byte elements, one per thread");

// L2 policy of the sweep's memory streams, by selector bit (1 = evict_last, 0 = evict_first)
__device__ __forceinline__ uint64_t sweep_policy(int sel, int bit) {
  return ((sel >> bit) & 1) ? policy_evict_last() : policy_evict_first();
}

// sum of one target's hop partners from a ring: base points at the target's column (pass 1:
// ring row r at base[r * STRIDE]) or row (pass 2: ring column r at base[r]); le is the hop list
// in shared memory (entries with positive sign first, entry 15 = count | positive count << 8)
template <int STRIDE>
__device__ __forceinline__ int64_t sweep_hops(const int64_t* __restrict__ base, const uint16_t* le) {
  const uint32_t cw = le[SW_LST - 1];
  const int cnt = (int)(cw & 0xffu), npos = (int)(cw >> 8);
  int64_t h0 = 0, h1 = 0, hn = 0;
  int e = 0;
  for (; e + 4 <= npos; e += 4) {  // four independent gathers in flight
    const uint2 pr = *(const uint2*)(le + e);
    h0 += base[(pr.x & 0xffffu) * STRIDE] + base[(pr.x >> 16) * STRIDE];
    h1 += base[(pr.y & 0xffffu) * STRIDE] + base[(pr.y >> 16) * STRIDE];
  }
  for (; e < npos; ++e) h0 += base[(uint32_t)le[e] * STRIDE];
  for (; e < cnt; ++e) hn += base[(uint32_t)le[e] * STRIDE];
  return (h0 + h1) - hn;
}

struct SweepArgs {
  int64_t nu, nd;
  int ring;              // ring capacity in chunks
  int nblk;              // target blocks
  const uint16_t* lst;   // hop lists of the targets of this pass
  const int2* win;       // per-block chunk windows
  int pol;               // policy selector: bit 0 X loads, bit 1 S stores (pass 1) / W stores (pass 2)
  long wait_limit;       // mbarrier tests before a first wait gives up
};

// hop lists of target blocks, staged through a small ring (SW_LR blocks of SW_CH lists, one
// 1 KB bulk copy each, issued SW_LR - 1 blocks ahead of their use)
constexpr int SW_LR = 4;
constexpr int SW_LBYTES = SW_CH * SW_LST * 2;

// bulk copy of the lists of target block b (of n targets) into list-ring slot `slot`
__device__ __forceinline__ void sweep_stage_lists(const uint16_t* lst, int64_t n, int64_t b, uint16_t* lring,
                                                  uint64_t* lbar, int slot) {
  const int64_t t0 = b * SW_CH;
  const unsigned bytes = (unsigned)(min((int64_t)SW_CH, n - t0) * SW_LST * 2);
  mbar_expect_tx(&lbar[slot], bytes);
  bulk_g2s(lring + (size_t)slot * SW_CH * SW_LST, lst + t0 * SW_LST, bytes, &lbar[slot], policy_evict_last());
}

// after a wait gave up (thread 0, every thread past cp.async.wait_all): the chunk arrivals
// those copies trigger and the staged list copies reach their barriers (bounded, the first
// wait that runs out ends the waiting), then a short pause for anything still in flight
__device__ __forceinline__ void sweep_drain(uint64_t* bar, uint64_t* lbar, int ring, int64_t ready, int64_t next,
                                            int slot_w, unsigned par_w, int lwaited, int lstaged) {
  bool ok = true;
  for (; ok && ready < next - 1; ++ready) {
    ok = mbar_wait_bounded(&bar[slot_w], par_w);
    if (++slot_w == ring) {
      slot_w = 0;
      par_w ^= 1u;
    }
  }
  for (int b = lwaited; ok && b < lstaged; ++b) ok = mbar_wait_bounded(&lbar[b % SW_LR], (unsigned)(b / SW_LR) & 1u);
  sweep_settle();
}

// ---- pass 1: S = A X, column stripes -----------------------------------------------------------
__global__ void __launch_bounds__(SW_NT, 2)
    k_sweep_up(SweepArgs a, const int64_t* __restrict__ X, int64_t* __restrict__ S, BfpState* st, int* status) {
  if (st && *(volatile int*)&st->stop) return;
  extern __shared__ __align__(128) unsigned char sm_up[];
  int64_t* ring = (int64_t*)sm_up;                                                 // [ring * SW_CH][SW_W]
  uint16_t* lring = (uint16_t*)(sm_up + (size_t)a.ring * SW_CH * SW_W * 8);       // [SW_LR][SW_CH][SW_LST]
  uint64_t* bar = (uint64_t*)((unsigned char*)lring + (size_t)SW_LR * SW_LBYTES);  // [ring]
  uint64_t* lbar = bar + a.ring;                                                   // [SW_LR]
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int64_t c0 = (int64_t)blockIdx.x * SW_W;
  const int ncols = (int)min((int64_t)SW_W, a.nd - c0);
  const int64_t nchunks = (a.nu + SW_CH - 1) / SW_CH;
  int lstaged = 0;   // list blocks staged (thread 0)
  int lwaited = 0;   // list blocks whose copy this thread has seen land
  if (tid == 0) {
    // one thread initialises every barrier: its fence makes exactly those inits visible to
    // the bulk copies (async proxy) that complete on them
    for (int i = 0; i < a.ring; ++i) mbar_init(&bar[i], SW_NT);  // chunk barriers: one arrival per thread
    for (int i = 0; i < SW_LR; ++i) mbar_init(&lbar[i], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    for (; lstaged < SW_LR && lstaged < a.nblk; ++lstaged) sweep_stage_lists(a.lst, a.nu, lstaged, lring, lbar, lstaged);
  }
  __syncthreads();
  const uint64_t pol_x = sweep_policy(a.pol, 0), pol_s = sweep_policy(a.pol, 1);
  int64_t next = 0;          // next chunk to issue
  int slot_i = 0;            // its ring slot
  int64_t ready = -1;        // chunks <= ready have landed (every thread waited for them)
  int slot_w = 0;
  unsigned par_w = 0;
  bool bad = false;
  const int col = lane & 15, half = lane >> 4;
  int2 w_next = __ldg(&a.win[0]);
  for (int j = 0; j < a.nblk; ++j) {
    const int2 w = w_next;
    if (j + 1 < a.nblk) w_next = __ldg(&a.win[j + 1]);  // one block ahead
    const int ls = j % SW_LR;
    {
      // refill: chunks up to (first chunk still needed) + ring - 1; their slots were last read
      // in blocks that every thread has finished (barrier at the end of the previous block).
      // A chunk is 32 rows x 16 columns: threads 0..255 copy 16 bytes each, then every thread
      // arrives on the chunk's barrier once its own copies have landed.
      const int64_t lim = min(nchunks - 1, (int64_t)w.x + a.ring - 1);
      const int crow = tid >> 3, cpart = tid & 7;
      for (; next <= lim; ++next) {
        const int64_t r = next * SW_CH + crow;
        if (tid < SW_CH * 8 && r < a.nu && 2 * cpart < ncols)
          cp_async16(ring + ((size_t)slot_i * SW_CH + crow) * SW_W + 2 * cpart, X + r * a.nd + c0 + 2 * cpart, pol_x);
        cp_async_arrive(&bar[slot_i]);
        if (++slot_i == a.ring) slot_i = 0;
      }
    }
    for (; ready < w.y && !bad; ++ready) {
      if (!mbar_wait_polls(&bar[slot_w], par_w, a.wait_limit)) {
        bad = true;
        break;
      }
      if (++slot_w == a.ring) {
        slot_w = 0;
        par_w ^= 1u;
      }
    }
    if (!bad) {
      if (mbar_wait_polls(&lbar[ls], (unsigned)(j / SW_LR) & 1u, a.wait_limit)) ++lwaited; else bad = true;
    }
    if (__syncthreads_or(bad)) {
      bad = true;
      break;
    }
    {
      // half-warp = one target row of the block, lane = column of the stripe
      const int ul = 2 * warp + half;
      const int64_t u = (int64_t)j * SW_CH + ul;
      if (u < a.nu) {
        const int64_t hsum = sweep_hops<SW_W>(ring + col, lring + ((size_t)ls * SW_CH + ul) * SW_LST);
        if (col < ncols) st_stream(S + u * a.nd + c0 + col, hsum, pol_s);
      }
    }
    __syncthreads();
    if (tid == 0 && j + SW_LR < a.nblk) {
      // the list slot of block j is free: stage block j + SW_LR into it
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      sweep_stage_lists(a.lst, a.nu, j + SW_LR, lring, lbar, ls);
      ++lstaged;
    }
  }
  if (bad) {
    // a wait ran out: record it, let every issued copy land (bounded), leave
    cp_async_wait_all();
    __syncthreads();
    if (tid == 0) {
      record_status(status, DEV_TIMEOUT);
      if (st) *(volatile int*)&st->stop = 3;
      sweep_drain(bar, lbar, a.ring, ready, next, slot_w, par_w, lwaited, lstaged);
    }
    __syncthreads();
    return;
  }
  cp_async_wait_all();
}

// per-row diagonal data of pass 2 (renumbered tables)
struct SweepDiag {
  const uint64_t* s_up; const uint64_t* s_dn;
  const int32_t* e_up; const int32_t* e_dn;
  const int64_t* f_up; const int64_t* f_dn;
};

// the epilogue's global inputs of one target column block, for one thread
struct SweepPre {
  int64_t s;         // S of the thread's row
  uint64_t sd;       // dn state
  int64_t ed;        // dn energy (int32 or fixed point)
};

template <bool DIAG64>
__device__ __forceinline__ SweepPre sweep_prefetch(const SweepDiag& dg, const int64_t* W, int64_t nd, int64_t u0,
                                                   int er, bool rv, int64_t j, int lane, int nblk, uint64_t pol) {
  SweepPre p{0, 0, 0};
  const int64_t d = j * SW_CH + lane;
  if (j < nblk && d < nd) {
    p.sd = __ldg(dg.s_dn + d);
    p.ed = DIAG64 ? __ldg(dg.f_dn + d) : (int64_t)__ldg(dg.e_dn + d);
    if (rv) p.s = ld_keep(W + (u0 + er) * nd + d, pol);
  }
  return p;
}

// ---- pass 2: W = t (S + X B) + D X, row stripes, with the Lanczos partials ---------------------
template <bool DIAG64>
__global__ void __launch_bounds__(SW_NT, 2)
    k_sweep_dn(BfpHubArgs h, SweepArgs a, SweepDiag dg, const int64_t* __restrict__ X, int64_t* W, double* partial,
               unsigned long long* partial_max, BfpState* st, int* status, BfpFuse fz) {
  if (st && *(volatile int*)&st->stop) return;
  extern __shared__ __align__(128) unsigned char sm_dn[];
  __shared__ double smd[SW_NT / 32];
  __shared__ unsigned long long smu[SW_NT / 32];
  const int RC = a.ring * SW_CH;       // ring columns
  const int RS = RC + 1;               // row stride (elements): 16 rows of a column in 16 bank pairs
  int64_t* win = (int64_t*)sm_dn;                                       // [SW_W][RS]
  int64_t* stage = win + (size_t)SW_W * RS;                             // [SW_W][SW_CH + 1]
  uint16_t* lring = (uint16_t*)(stage + (size_t)SW_W * (SW_CH + 1));   // [SW_LR][SW_CH][SW_LST]
  uint64_t* bar = (uint64_t*)((unsigned char*)lring + (size_t)SW_LR * SW_LBYTES);  // [ring]
  uint64_t* lbar = bar + a.ring;                                        // [SW_LR]
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int64_t u0 = (int64_t)blockIdx.x * SW_W;
  const int nrows = (int)min((int64_t)SW_W, a.nu - u0);
  const int64_t nchunks = (a.nd + SW_CH - 1) / SW_CH;
  int lstaged = 0;   // list blocks staged (thread 0)
  int lwaited = 0;   // list blocks whose copy this thread has seen land
  if (tid == 0) {
    // one thread initialises every barrier and fences its inits (see pass 1)
    for (int i = 0; i < a.ring; ++i) mbar_init(&bar[i], SW_NT);
    for (int i = 0; i < SW_LR; ++i) mbar_init(&lbar[i], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    for (; lstaged < SW_LR && lstaged < a.nblk; ++lstaged) sweep_stage_lists(a.lst, a.nd, lstaged, lring, lbar, lstaged);
  }
  __syncthreads();
  const uint64_t pol_x = sweep_policy(a.pol, 0), pol_w = sweep_policy(a.pol, 1), pol_s = policy_evict_first();
  // the epilogue row of this thread (= warp) and its diagonal data
  const int er = warp;
  const bool rv = er < nrows;
  const int64_t eu_row = rv ? u0 + er : u0;
  const uint64_t su = __ldg(dg.s_up + eu_row);
  const int64_t eu = DIAG64 ? 0 : (int64_t)__ldg(dg.e_up + eu_row);
  const int64_t ef = DIAG64 ? __ldg(dg.f_up + eu_row) : 0;
  int64_t next = 0;
  int slot_i = 0;
  int64_t ready = -1;
  int slot_w = 0;
  unsigned par_w = 0;
  int jslot = 0;   // ring slot of the current target block (block j is chunk j)
  bool bad = false;
  I128 dot{0, 0};
  unsigned long long mx = 0;
  const int rr = lane & 15, half = lane >> 4;
  // epilogue inputs two blocks ahead, the window one block ahead
  SweepPre pre0 = sweep_prefetch<DIAG64>(dg, W, a.nd, u0, er, rv, 0, lane, a.nblk, pol_s);
  SweepPre pre1 = sweep_prefetch<DIAG64>(dg, W, a.nd, u0, er, rv, 1, lane, a.nblk, pol_s);
  int2 w_next = __ldg(&a.win[0]);
  for (int j = 0; j < a.nblk; ++j) {
    const int2 w = w_next;
    if (j + 1 < a.nblk) w_next = __ldg(&a.win[j + 1]);
    const SweepPre cur = pre0;
    pre0 = pre1;
    pre1 = sweep_prefetch<DIAG64>(dg, W, a.nd, u0, er, rv, j + 2, lane, a.nblk, pol_s);
    const int ls = j % SW_LR;
    // refill (every thread copies two elements of each new chunk, then arrives)
    const int64_t lim = min(nchunks - 1, (int64_t)w.x + a.ring - 1);
    for (; next <= lim; ++next) {
      const int64_t cc0 = next * SW_CH;
      {
        const int r = tid >> 5, c = tid & 31;  // 16 rows x 32 columns: one element per thread
        if (r < nrows && cc0 + c < a.nd)
          cp_async8(win + (size_t)r * RS + slot_i * SW_CH + c, X + (u0 + r) * a.nd + cc0 + c, pol_x);
      }
      cp_async_arrive(&bar[slot_i]);
      if (++slot_i == a.ring) slot_i = 0;
    }
    for (; ready < w.y && !bad; ++ready) {
      if (!mbar_wait_polls(&bar[slot_w], par_w, a.wait_limit)) {
        bad = true;
        break;
      }
      if (++slot_w == a.ring) {
        slot_w = 0;
        par_w ^= 1u;
      }
    }
    if (!bad) {
      if (mbar_wait_polls(&lbar[ls], (unsigned)(j / SW_LR) & 1u, a.wait_limit)) ++lwaited; else bad = true;
    }
    if (__syncthreads_or(bad)) {
      bad = true;
      break;
    }
    // gather: half-warp = one target column of the block, lane = row of the stripe
    {
      const int cl = 2 * warp + half;
      const int64_t d = (int64_t)j * SW_CH + cl;
      const int64_t hsum =
          d < a.nd ? sweep_hops<1>(win + (size_t)rr * RS, lring + ((size_t)ls * SW_CH + cl) * SW_LST) : 0;
      stage[rr * (SW_CH + 1) + cl] = hsum;
    }
    __syncthreads();
    if (tid == 0 && j + SW_LR < a.nblk) {
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      sweep_stage_lists(a.lst, a.nd, j + SW_LR, lring, lbar, ls);
      ++lstaged;
    }
    // epilogue: row er (= warp), column j*32 + lane
    {
      const int64_t d = (int64_t)j * SW_CH + lane;
      if (d < a.nd && rv) {
        const int32_t ed32 = DIAG64 ? 0 : (int32_t)cur.ed;
        const int64_t ed64 = DIAG64 ? cur.ed : 0;
        const int64_t x = win[(size_t)er * RS + jslot * SW_CH + lane];
        const int64_t ww = (int64_t)h.t_int * (cur.s + stage[er * (SW_CH + 1) + lane]) +
                           bfp_diag_col<DIAG64>(h, eu, ef, su, cur.sd, ed32, ed64, x);
        st_stream(W + (u0 + er) * a.nd + d, ww, pol_w);
        add128(dot, mul_s64(x, ww));
        mx = max(mx, uabs64(ww));
      }
    }
    if (++jslot == a.ring) jslot = 0;
    __syncthreads();
  }
  if (bad) {
    cp_async_wait_all();  // every copy this thread issued has landed before the CTA leaves
    __syncthreads();
    if (tid == 0) {
      record_status(status, DEV_TIMEOUT);
      if (st) *(volatile int*)&st->stop = 3;
      sweep_drain(bar, lbar, a.ring, ready, next, slot_w, par_w, lwaited, lstaged);
    }
    __syncthreads();
    return;
  }
  cp_async_wait_all();
  if (!partial) return;
  const double sdot = block_sum<SW_NT>(i128_to_double(dot), smd);
  const unsigned long long m = block_max_u64<SW_NT>(mx, smu);
  if (tid == 0) {
    partial[blockIdx.x] = sdot;
    partial_max[blockIdx.x] = m;
  }
  if (fz.on && st && bfp_last_block(&st->ticket[2])) {
    double t = 0.0;
    unsigned long long mm = 0;
    for (int b = tid; b < (int)gridDim.x; b += SW_NT) {
      t += ((volatile double*)partial)[b];
      mm = max(mm, ((volatile unsigned long long*)partial_max)[b]);
    }
    t = block_sum<SW_NT>(t, smd);
    mm = block_max_u64<SW_NT>(mm, smu);
    if (tid == 0) {
      bfp_scalars_tail(fz.v, fz.k, fz.F, fz.m_in, t, mm, fz.alpha, fz.beta, st);
      st->ticket[2] = 0;
    }
  }
}

// ---- renumbering of whole vectors ----------------------------------------------------------------
// FP64 (original order) -> fixed point (renumbered order): xm[u'*nd + d'] = round(x[perm_up[u']*nd +
// perm_dn[d']] * 2^-e), e chosen as in k_f64_to_bfp
__global__ void k_f64_to_bfp_perm(const double* __restrict__ x, int64_t nu, int64_t nd, const int32_t* __restrict__ pu,
                                  const int32_t* __restrict__ pd, const unsigned long long* maxbits, int m_in,
                                  int64_t* __restrict__ xm, int32_t* e_out, unsigned long long* max_out) {
  const double mx = __longlong_as_double((long long)*maxbits);
  int e2 = 0;
  frexp(mx, &e2);
  const int e = e2 - m_in;
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    *e_out = e;
    *max_out = (unsigned long long)llrint(ldexp(mx, -e));
  }
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nu * nd; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = i / nd, c = i - r * nd;
    xm[i] = llrint(ldexp(x[(int64_t)__ldg(pu + r) * nd + __ldg(pd + c)], -e));
  }
}

// int64 vectors between the original (to_new = 0: dst renumbered, src original) and the
// renumbered order
__global__ void k_sweep_permute(const int64_t* __restrict__ src, int64_t* __restrict__ dst, int64_t nu, int64_t nd,
                                const int32_t* __restrict__ pu, const int32_t* __restrict__ pd, int to_new) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nu * nd; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = i / nd, c = i - r * nd;
    const int64_t o = (int64_t)__ldg(pu + r) * nd + __ldg(pd + c);
    if (to_new) dst[i] = src[o]; else dst[o] = src[i];
  }
}

