// Batched Lanczos: many independent sectors (all (n_up, n_dn) sectors of a model, or many
// disorder realisations) in ONE persistent launch. No reference counterpart — the reference
// loops over sectors on the host (cmpy/exactdiag.py:24-43, one ARPACK solve each).
//
// Each CTA pulls problems from a device work queue (largest dimension first) and runs the
// whole fixed-point Lanczos of that problem with block-level synchronisation only (scalars in
// shared memory, vectors in the CTA's own workspace slot); CTAs never wait on each other, so
// there is no grid-wide barrier. With want_vector the CTA replays the recurrence once — the
// integer arithmetic and the fixed-order reductions make the replay bit-identical — and
// accumulates the ground-state vector in 128-bit fixed point. The launch is asynchronous and
// allocation-free, so host sequences of batched launches can be captured in a CUDA graph.
//
// Vector arithmetic is the block-fixed-point scheme of ed_bfp.cu (int64 mantissas, one
// exponent per vector, exact integer matvec, 128-bit dot products).
//
// With a thread-block cluster of CS > 1 CTAs per problem, the cluster's CTAs split the
// elements of every vector loop (CTA rank r takes the r-th stripe of CS * NT) and exchange their
// block totals through distributed shared memory at the hardware cluster barrier; every CTA
// then holds the same totals and computes the same scalars, so all CTAs of a cluster take the
// same branches and reach the same barriers. The largest sectors, which bound the makespan of
// the work queue, thus run on CS SMs.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include <cooperative_groups.h>

#include "ed_plan.cuh"
#include "ed_tridiag.cuh"

namespace cg = cooperative_groups;

namespace ed {

namespace {

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
  asm("add.cc.u64 %0, %0, %2;\n\taddc.u64 %1, %1, %3;" : "+l"(acc.lo), "+l"(acc.hi) : "l"(v.lo), "l"(v.hi));
}
__device__ __forceinline__ double i128_to_double(const I128& v) { return fma((double)v.hi, 0x1.0p64, (double)v.lo); }
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
__device__ __forceinline__ uint64_t bsplitmix(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

}  // namespace

// one problem = one fixed-point sector (device pointers owned by its plan)
struct BatchProblem {
  int64_t nu, nd, D;
  const int32_t* up_off;
  const int32_t* up_npos;
  const int32_t* up_idx;
  const uint16_t* dn_tab;
  const uint64_t* up_states;
  const uint64_t* dn_states;
  const int32_t* e_up;
  const int32_t* e_dn;
  const int64_t* e_up_fx;
  const int64_t* e_dn_fx;
  int max_dn, diag64, dshift, F, m_in, u_uniform;
  int32_t t_int, u0;
  int64_t u0_fx;
  int32_t u[ED_MAX_SITES + 2];
  int64_t u_fx[ED_MAX_SITES + 2];
};

struct BatchOut {
  double* alpha;     // [n][K]
  double* beta;      // [n][K+1]; beta[p][0] = start norm, beta[p][k>0] couplings
  double* energy;    // [n]
  double* residual;  // [n]
  int32_t* steps;    // [n]
  double* vec;       // optional ground-state vectors: problem p at vec + vec_off[p]
  const int64_t* vec_off;
};

struct BatchWork {
  int64_t* slots;     // per CTA: Ra, Rb, W, acc_lo, acc_hi (each dmax)
  int64_t dmax;
  double* tri;        // per CTA: 6*(K+2) doubles (tridiagonal work + eigenvector)
  int32_t* exps;      // per CTA: K+2 exponents of R_k
  int64_t* coefs;     // per CTA: K+2 Ritz coefficients
  int* queue;
};

template <int NT>
struct BlockScratch {
  double d[NT / 32];
  unsigned long long u[NT / 32];
};

// block sum with the same (warp, lane) order every time: deterministic
template <int NT>
__device__ __forceinline__ double bsum(double v, BlockScratch<NT>& s) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) s.d[w] = v;
  __syncthreads();
  double r = 0.0;
  for (int i = 0; i < NT / 32; ++i) r += s.d[i];
  return r;
}

template <int NT>
__device__ __forceinline__ unsigned long long bmax(unsigned long long v, BlockScratch<NT>& s) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) s.u[w] = v;
  __syncthreads();
  unsigned long long r = 0;
  for (int i = 0; i < NT / 32; ++i) r = max(r, s.u[i]);
  return r;
}

// Cluster-wide (sum, max) of values held per thread: block totals first, then (CS > 1) the CS
// block totals through distributed shared memory, in rank order, so every CTA gets the same
// result. xd / xu: two exchange slots each (alternating with `ph`: a slot is rewritten only
// after a later cluster barrier, when every CTA has read it). The barrier (release / acquire
// at cluster scope) also orders the global-memory writes of the phase before it for all CTAs
// of the cluster.
struct ClusterXch {
  double* xd;
  unsigned long long* xu;
  int ph;
};

// block sum and max together: one shared-memory exchange (same order as bsum / bmax)
template <int NT>
__device__ __forceinline__ void bsummax(double& v, unsigned long long& m, BlockScratch<NT>& s) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    v += __shfl_xor_sync(0xffffffffu, v, o);
    m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
  }
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) {
    s.d[w] = v;
    s.u[w] = m;
  }
  __syncthreads();
  double r = 0.0;
  unsigned long long q = 0;
  for (int i = 0; i < NT / 32; ++i) {
    r += s.d[i];
    q = max(q, s.u[i]);
  }
  v = r;
  m = q;
}

template <int NT, int CS>
__device__ __forceinline__ void cred(double& sumv, unsigned long long& maxv, BlockScratch<NT>& s, ClusterXch& x) {
  bsummax<NT>(sumv, maxv, s);
  if constexpr (CS > 1) {
    cg::cluster_group cl = cg::this_cluster();
    if (threadIdx.x == 0) {
      x.xd[x.ph] = sumv;
      x.xu[x.ph] = maxv;
    }
    cl.sync();  // arrive.release / wait.acquire at cluster scope: orders shared and global writes
    double t = 0.0;
    unsigned long long m = 0;
#pragma unroll
    for (int q = 0; q < CS; ++q) {
      t += *cl.map_shared_rank(x.xd + x.ph, q);
      m = max(m, *cl.map_shared_rank(x.xu + x.ph, q));
    }
    sumv = t;
    maxv = m;
    x.ph ^= 1;
  }
}

// a cluster barrier with global-memory ordering (no-op for CS = 1 beyond the block barrier)
template <int CS>
__device__ __forceinline__ void csync() {
  if constexpr (CS > 1) {
    cg::this_cluster().sync();
  } else {
    __syncthreads();
  }
}

__device__ __forceinline__ double start_value(const double* start, int64_t i, uint64_t seed) {
  if (start) return start[i];
  return (double)(bsplitmix(seed * 0x100000001B3ull + (uint64_t)i) >> 11) * 0x1.0p-53 + 0x1.0p-54;
}

// R0 = round(v0 * 2^-e), max |R0| < 2^m_in; returns e, writes ||v0|| and max |R0|
// (elements i = rk * NT + tid, step CS * NT: this CTA's stripe)
template <int NT, int CS>
__device__ int batch_start(const BatchProblem& P, const double* start, int64_t* R0, uint64_t seed,
                           BlockScratch<NT>& s, ClusterXch& x, int rk, double* norm, unsigned long long* maxm) {
  unsigned long long mb = 0;
  bool finite = true;
  for (int64_t i = (int64_t)rk * NT + threadIdx.x; i < P.D; i += (int64_t)CS * NT) {
    const double v = start_value(start, i, seed);
    finite &= (bool)isfinite(v);
    mb = max(mb, (unsigned long long)__double_as_longlong(fabs(v)));
  }
  double dummy = 0.0;
  mb = finite ? mb : 0x7FF0000000000000ull;
  cred<NT, CS>(dummy, mb, s, x);
  const double mx = __longlong_as_double((long long)mb);
  if (!isfinite(mx) || mx == 0.0) {
    *norm = isfinite(mx) ? 0.0 : NAN;
    *maxm = 0;
    return 0;
  }
  int e2 = 0;
  frexp(mx, &e2);
  const int e = e2 - P.m_in;
  I128 acc{0, 0};
  unsigned long long mm = 0;
  for (int64_t i = (int64_t)rk * NT + threadIdx.x; i < P.D; i += (int64_t)CS * NT) {
    const int64_t r = llrint(ldexp(start_value(start, i, seed), -e));
    R0[i] = r;
    add128(acc, mul_s64(r, r));
    mm = max(mm, uabs64(r));
  }
  __syncthreads();
  double t = i128_to_double(acc);
  cred<NT, CS>(t, mm, s, x);
  *maxm = mm;
  *norm = ldexp(sqrt(t), e);
  return e;
}

// W = H X in integers on this CTA's stripe of rows; returns <X, W> (exact per thread, FP64
// across threads and CTAs), max |W|. X is read at every element (the hops reach other stripes).
template <int NT, int CS>
__device__ double batch_matvec(const BatchProblem& P, const int64_t* __restrict__ X, int64_t* __restrict__ W,
                               BlockScratch<NT>& s, ClusterXch& xc, int rk, unsigned long long* maxw) {
  I128 dot{0, 0};
  unsigned long long mx = 0;
  const int64_t nd = P.nd;
  for (int64_t i = (int64_t)rk * NT + threadIdx.x; i < P.D; i += (int64_t)CS * NT) {
    const int64_t u = i / nd, d = i - u * nd;
    const int64_t* xrow = X + u * nd;
    int64_t h = 0;
    const int32_t o0 = __ldg(P.up_off + u), o1 = __ldg(P.up_off + u + 1), op = o0 + __ldg(P.up_npos + u);
    for (int32_t e = o0; e < op; ++e) h += X[(int64_t)__ldg(P.up_idx + e) * nd + d];
    for (int32_t e = op; e < o1; ++e) h -= X[(int64_t)__ldg(P.up_idx + e) * nd + d];
    for (int e = 0; e < P.max_dn; ++e) {
      const int sl = __ldg(P.dn_tab + (int64_t)e * nd + d);
      if (sl < nd) h += xrow[sl];
      else if (sl < 2 * nd) h -= xrow[sl - nd];
    }
    const int64_t x = xrow[d];
    const uint64_t both = __ldg(P.up_states + u) & __ldg(P.dn_states + d);
    int64_t dterm;
    if (!P.diag64) {
      int32_t dg = __ldg(P.e_up + u) + __ldg(P.e_dn + d);
      if (P.u_uniform) dg += P.u0 * __popcll(both);
      else
        for (uint64_t b = both; b; b &= b - 1) dg += P.u[__ffsll((long long)b) - 1];
      dterm = (int64_t)dg * x;
    } else {
      int64_t dg = __ldg(P.e_up_fx + u) + __ldg(P.e_dn_fx + d);
      if (P.u_uniform) dg += P.u0_fx * (int64_t)__popcll(both);
      else
        for (uint64_t b = both; b; b &= b - 1) dg += P.u_fx[__ffsll((long long)b) - 1];
      dterm = shr128_round(mul_s64(dg, x), P.dshift);
    }
    const int64_t w = (int64_t)P.t_int * h + dterm;
    W[i] = w;
    add128(dot, mul_s64(x, w));
    mx = max(mx, uabs64(w));
  }
  __syncthreads();
  double t = i128_to_double(dot);
  cred<NT, CS>(t, mx, s, xc);
  *maxw = mx;
  return t;
}

struct StepCoef {
  int64_t Aw, Aq, Ap;
  int SA, er;
};

// R_{k+1} = W/b_k - (a_k/b_k) R_k - (b_k/b_{k-1}) R_{k-1} on a grid with max |R_{k+1}| < 2^m_in
__device__ StepCoef batch_coef(double a, double bk, double bkm1, int k, int ew, int ek, int ep, double mw, double mq,
                               double mp, int m_in) {
  const double cw = 1.0 / bk, cq = -a / bk, cp = (k > 0) ? -bk / bkm1 : 0.0;
  const double B = fabs(cw) * ldexp(mw, ew) + fabs(cq) * ldexp(mq, ek) + fabs(cp) * ldexp(mp, ep);
  int eb = 0;
  frexp(B > 0.0 ? B : 1.0, &eb);
  StepCoef c;
  c.er = eb - m_in;
  const double gw = ldexp(cw, ew - c.er), gq = ldexp(cq, ek - c.er), gp = ldexp(cp, ep - c.er);
  const double gm = fmax(fabs(gw), fmax(fabs(gq), fabs(gp)));
  int eg = 0;
  frexp(gm > 0.0 ? gm : 1.0, &eg);
  c.SA = min(60, 60 - eg);
  c.Aw = llrint(ldexp(gw, c.SA));
  c.Aq = llrint(ldexp(gq, c.SA));
  c.Ap = llrint(ldexp(gp, c.SA));
  return c;
}

// The Lanczos recurrence of one problem. Pass 1 (Ck == null) records alpha, beta and the
// exponent of every R_k and stops on convergence / invariant subspace; pass 2 replays
// exactly `m` steps and accumulates acc += Ck[k] * R_k. alpha / beta are this CTA's copies.
template <int NT, int CS>
__device__ void batch_recurrence(const BatchProblem& P, const double* start, uint64_t seed, int K, double tol,
                                 int check_every, int rk, int64_t* Ra, int64_t* Rb, int64_t* W, double* alpha,
                                 double* beta, double* c, double* work, int32_t* exps, int* m_io,
                                 const int64_t* Ck, uint64_t* acc_lo, int64_t* acc_hi) {
  __shared__ BlockScratch<NT> s;
  __shared__ int sh_stop, sh_m, sh_e0, sh_e1;
  __shared__ unsigned long long sh_m0, sh_m1;
  __shared__ StepCoef sh_c;
  __shared__ double xd[2];
  __shared__ unsigned long long xu[2];
  ClusterXch xc{xd, xu, 0};
  const bool pass2 = Ck != nullptr;
  double nrm = 0.0;
  unsigned long long mstart = 0;
  const int e_start = batch_start<NT, CS>(P, start, Ra, seed, s, xc, rk, &nrm, &mstart);
  if (threadIdx.x == 0) {
    sh_stop = 0;
    sh_m = 0;
    sh_e0 = 0;
    sh_e1 = e_start;
    sh_m0 = 0;
    sh_m1 = mstart;
    if (!pass2) {
      beta[0] = nrm;
      exps[0] = e_start;
    }
  }
  if (pass2)
    for (int64_t i = (int64_t)rk * NT + threadIdx.x; i < P.D; i += (int64_t)CS * NT) {
      acc_lo[i] = 0;
      acc_hi[i] = 0;
    }
  __syncthreads();
  if (!(nrm > 0.0)) {  // zero or non-finite start vector: empty Krylov space
    if (threadIdx.x == 0 && !pass2) *m_io = 0;
    csync<CS>();  // m is read by every thread (and nrm is the same in every CTA of the cluster)
    return;
  }
  const int Km = (int)min((int64_t)K, P.D);
  const int mlim = pass2 ? *m_io : Km;
  int64_t* Rk = Ra;
  int64_t* Rp = Rb;
  for (int k = 0; k < mlim; ++k) {
    if (pass2) {
      const int64_t C = Ck[k];
      for (int64_t i = (int64_t)rk * NT + threadIdx.x; i < P.D; i += (int64_t)CS * NT) {
        I128 v{acc_lo[i], acc_hi[i]};
        add128(v, mul_s64(C, Rk[i]));
        acc_lo[i] = v.lo;
        acc_hi[i] = v.hi;
      }
      if (k + 1 == mlim) break;
    }
    unsigned long long mw = 0;
    const double dot = batch_matvec<NT, CS>(P, Rk, W, s, xc, rk, &mw);
    if (threadIdx.x == 0) {
      const int ek = sh_e1, ew = ek - P.F;
      const double bk = beta[k];
      const double a = ldexp(dot, ek + ew) / (bk * bk);
      if (!pass2) alpha[k] = a;
      sh_c = batch_coef(a, bk, k > 0 ? beta[k - 1] : 1.0, k, ew, ek, sh_e0, (double)mw, (double)sh_m1, (double)sh_m0,
                        P.m_in);
    }
    __syncthreads();
    const StepCoef cf = sh_c;
    I128 nn{0, 0};
    unsigned long long mx = 0;
    for (int64_t i = (int64_t)rk * NT + threadIdx.x; i < P.D; i += (int64_t)CS * NT) {
      I128 t = mul_s64(cf.Aw, W[i]);
      add128(t, mul_s64(cf.Aq, Rk[i]));
      if (k > 0) add128(t, mul_s64(cf.Ap, Rp[i]));
      const int64_t r = shr128_round(t, cf.SA);
      Rp[i] = r;  // R_{k+1} overwrites R_{k-1}
      add128(nn, mul_s64(r, r));
      mx = max(mx, uabs64(r));
    }
    __syncthreads();
    // the cluster exchange also orders every CTA's R_{k+1} stripe before the next matvec
    double t2 = i128_to_double(nn);
    cred<NT, CS>(t2, mx, s, xc);
    if (threadIdx.x == 0) {
      const double bn = ldexp(sqrt(t2), cf.er);
      if (!pass2) {
        beta[k + 1] = bn;
        exps[k + 1] = cf.er;
        const double scale = fabs(alpha[k]) + (k > 0 ? beta[k] : 0.0) + 1e-300;
        if (!(bn > 1e-13 * scale) || mx == 0) {
          sh_stop = 2;
          sh_m = k + 1;
        }
      }
      sh_e0 = sh_e1;
      sh_e1 = cf.er;
      sh_m0 = sh_m1;
      sh_m1 = mx;
    }
    __syncthreads();
    int64_t* tmp = Rk;
    Rk = Rp;
    Rp = tmp;
    if (!pass2) {
      if (sh_stop) break;
      if (check_every > 0 && (k + 1) % check_every == 0 && k + 1 < Km) {
        // every CTA of the cluster solves the same tridiagonal (same data, same result)
        const double e = tridiag_lowest_block(alpha, beta, k + 1, c, work);
        if (threadIdx.x == 0) {
          const double res = fabs(beta[k + 1] * c[k]);
          if (res <= tol * fmax(1.0, fabs(e))) {
            sh_stop = 1;
            sh_m = k + 1;
          }
        }
        __syncthreads();
        if (sh_stop) break;
      }
    }
  }
  __syncthreads();
  if (!pass2 && threadIdx.x == 0) *m_io = sh_stop ? sh_m : Km;
  csync<CS>();  // the pass's last vector writes, ordered before what follows
}

template <int NT, int CS>
__global__ void __launch_bounds__(NT) k_batch_lanczos(const BatchProblem* __restrict__ probs,
                                                      const int* __restrict__ order, int n, int K, double tol,
                                                      int check_every, uint64_t seed,
                                                      const double* const* __restrict__ starts, int want_vector,
                                                      BatchOut out, BatchWork wk) {
  __shared__ int sh_p, sh_m, sh_sc;
  __shared__ BlockScratch<NT> s2;
  __shared__ double xd2[2];
  __shared__ unsigned long long xu2[2];
  const int rk = CS > 1 ? (int)(blockIdx.x % CS) : 0;
  const int64_t cid = blockIdx.x / CS;  // the cluster's vector slots
  int64_t* Ra = wk.slots + cid * 5 * wk.dmax;
  int64_t* Rb = Ra + wk.dmax;
  int64_t* W = Rb + wk.dmax;
  uint64_t* acc_lo = (uint64_t*)(W + wk.dmax);
  int64_t* acc_hi = (int64_t*)(acc_lo + wk.dmax);
  // this CTA's tridiagonal work, eigenvector and copies of alpha, beta
  double* work = wk.tri + (int64_t)blockIdx.x * 8 * (K + 2);
  double* c = work + 5 * (K + 2);
  double* al = c + (K + 2);
  double* be = al + (K + 2);
  int32_t* exps = wk.exps + (int64_t)blockIdx.x * (K + 2);
  int64_t* Ck = wk.coefs + (int64_t)blockIdx.x * (K + 2);
  while (true) {
    // rank 0 pulls the next problem; every CTA of the cluster reads it from rank 0
    if (threadIdx.x == 0 && rk == 0) sh_p = atomicAdd(wk.queue, 1);
    csync<CS>();
    int q;
    if constexpr (CS > 1) q = *cg::this_cluster().map_shared_rank(&sh_p, 0);
    else q = sh_p;
    csync<CS>();
    if (q >= n) break;
    const int p = order[q];
    const BatchProblem& P = probs[p];
    const double* start = starts ? starts[p] : nullptr;
    const uint64_t sd = seed + 0x9E37ull * (uint64_t)p;
    batch_recurrence<NT, CS>(P, start, sd, K, tol, check_every, rk, Ra, Rb, W, al, be, c, work, exps, &sh_m,
                             nullptr, nullptr, nullptr);
    const int m = sh_m;
    if (rk == 0) {
      double* alpha = out.alpha + (int64_t)p * K;
      double* beta = out.beta + (int64_t)p * (K + 1);
      for (int k = threadIdx.x; k < m; k += NT) alpha[k] = al[k];
      for (int k = threadIdx.x; k <= m; k += NT) beta[k] = be[k];
    }
    if (m == 0) {
      if (threadIdx.x == 0 && rk == 0) {
        out.energy[p] = NAN;
        out.residual[p] = 0.0;
        out.steps[p] = 0;
      }
      continue;
    }
    const double e = tridiag_lowest_block(al, be, m, c, work);
    if (threadIdx.x == 0 && rk == 0) {
      out.energy[p] = e;
      out.residual[p] = fabs(be[m] * c[m - 1]);
      out.steps[p] = m;
    }
    if (want_vector && out.vec) {
      // psi = sum_k (c_k / beta_k) R_k,  R_k = Rm_k 2^e_k:  C_k = round(c_k/beta_k 2^(e_k + SC))
      if (threadIdx.x == 0) {
        double gm = 0.0;
        for (int k = 0; k < m; ++k) gm = fmax(gm, fabs(ldexp(c[k] / be[k], exps[k])));
        int eg = 0;
        frexp(gm > 0.0 ? gm : 1.0, &eg);
        sh_sc = 52 - eg;
        for (int k = 0; k < m; ++k) Ck[k] = llrint(ldexp(c[k] / be[k], exps[k] + sh_sc));
      }
      __syncthreads();
      int mm = m;
      batch_recurrence<NT, CS>(P, start, sd, K, tol, check_every, rk, Ra, Rb, W, al, be, c, work, exps, &mm, Ck,
                               acc_lo, acc_hi);
      // normalise and write FP64
      double sq = 0.0;
      const int sc = sh_sc;
      for (int64_t i = (int64_t)rk * NT + threadIdx.x; i < P.D; i += (int64_t)CS * NT) {
        const double v = ldexp(i128_to_double(I128{acc_lo[i], acc_hi[i]}), -sc);
        sq = fma(v, v, sq);
      }
      ClusterXch xc{xd2, xu2, 0};
      unsigned long long dummy = 0;
      cred<NT, CS>(sq, dummy, s2, xc);
      const double inv = 1.0 / sqrt(sq);
      double* vo = out.vec + out.vec_off[p];
      for (int64_t i = (int64_t)rk * NT + threadIdx.x; i < P.D; i += (int64_t)CS * NT)
        vo[i] = ldexp(i128_to_double(I128{acc_lo[i], acc_hi[i]}), -sc) * inv;
    }
    csync<CS>();  // the cluster's slots are free for the next problem
  }
  csync<CS>();  // no CTA leaves while another may still read its shared memory
}

// G_p(z) += sign * norm_p^2 / (z' - a0 - b1^2 / (z' - a1 - ...)),  z' = sign*z + e0_p,
// norm_p = beta[p][0] (start norm), m_p = steps[p]; one thread per (problem, frequency)
__global__ void k_batch_cf(int n, int K, const double* __restrict__ alpha, const double* __restrict__ beta,
                           const int32_t* __restrict__ steps, const double* __restrict__ e0, int sign,
                           const double2* __restrict__ z, int64_t nz, double2* __restrict__ g) {
  const int64_t tot = (int64_t)n * nz;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < tot; t += (int64_t)gridDim.x * blockDim.x) {
    const int p = (int)(t / nz);
    const int64_t j = t - (int64_t)p * nz;
    const int m = steps[p];
    const double* a = alpha + (int64_t)p * K;
    const double* b = beta + (int64_t)p * (K + 1);
    double2 r = g[t];
    if (m > 0) {
      const double2 zi = z[j];
      const double zr = sign * zi.x + e0[p], zm = sign * zi.y;
      double tr = zr - a[m - 1], tm = zm;
      for (int l = m - 2; l >= 0; --l) {
        const double bb = b[l + 1] * b[l + 1];
        const double inv = bb / (tr * tr + tm * tm);
        tr = zr - a[l] - tr * inv;
        tm = zm + tm * inv;
      }
      const double inv = sign * b[0] * b[0] / (tr * tr + tm * tm);
      r.x += tr * inv;
      r.y -= tm * inv;
    }
    g[t] = r;
  }
}

}  // namespace ed

// ---- host side ---------------------------------------------------------------------------------

struct ed_batch_s {
  int device = -1;
  int n = 0;
  int64_t dmax = 0;
  ed::BatchProblem* d_probs = nullptr;
  int* d_order = nullptr;
  std::vector<int64_t> dims;
  ed::DeviceContext* ctx = nullptr;
  int tuned_threads = 0;
  int tuned_per_sm = 0;
  int tuned_cluster = 0;
};

namespace ed {

// the grid: clusters of cs CTAs, at most one cluster per problem and per_sm CTAs per SM
static int batch_grid(const ed_batch_s* b, int per_sm, int cs) {
  const int clusters = std::max(1, std::min(b->n, b->ctx->num_sms * per_sm / cs));
  return clusters * cs;
}

struct BatchLayout {
  size_t off_queue, off_slots, off_tri, off_exps, off_coefs, total;
};

static size_t al256b(size_t x) { return (x + 255) & ~(size_t)255; }

// vector slots per cluster; tridiagonal work, eigenvector, alpha/beta copies, exponents and
// Ritz coefficients per CTA
static BatchLayout batch_layout(const ed_batch_s* b, int K, int grid, int cs) {
  BatchLayout L;
  size_t o = 0;
  L.off_queue = o; o = al256b(o + 256);
  L.off_slots = o; o = al256b(o + (size_t)(grid / cs) * 5 * b->dmax * 8);
  L.off_tri = o; o = al256b(o + (size_t)grid * 8 * (K + 2) * 8);
  L.off_exps = o; o = al256b(o + (size_t)grid * (K + 2) * 4);
  L.off_coefs = o; o = al256b(o + (size_t)grid * (K + 2) * 8);
  L.total = o;
  return L;
}

static bool valid_config(int threads, int per_sm, int cs) {
  const bool t_ok = threads == 128 || threads == 256 || threads == 512 || threads == 1024;
  const bool c_ok = cs == 1 || ((cs == 2 || cs == 4 || cs == 8) && threads >= 512);
  return t_ok && c_ok && per_sm >= 1 && per_sm <= 16;
}

template <int NT, int CS>
static ed_status launch_batch(const ed_batch_s* b, int grid, int K, double tol, int check_every, uint64_t seed,
                              const double* const* starts, int want_vector, const BatchOut& out, const BatchWork& wk,
                              cudaStream_t s) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(NT);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = CS;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = CS > 1 ? 1 : 0;
  const cudaError_t e = cudaLaunchKernelEx(&cfg, k_batch_lanczos<NT, CS>, (const BatchProblem*)b->d_probs,
                                           (const int*)b->d_order, b->n, K, tol, check_every, seed, starts, want_vector,
                                           out, wk);
  if (e != cudaSuccess) return cuda_fail(e, "k_batch_lanczos");
  ED_CHECK_LAUNCH("k_batch_lanczos");
  return ED_OK;
}

static ed_status run_batch(const ed_batch_s* b, int threads, int per_sm, int cs, int K, double tol, int check_every,
                           uint64_t seed, const double* const* starts, int want_vector, void* work, size_t bytes,
                           const BatchOut& out, cudaStream_t s) {
  if (!valid_config(threads, per_sm, cs))
    return fail(ED_ERR_INVALID_ARG, "threads 128/256/512/1024; clusters of 2, 4 or 8 CTAs need 512 or 1024 threads");
  const int grid = batch_grid(b, per_sm, cs);
  const BatchLayout L = batch_layout(b, K, grid, cs);
  if (!work || bytes < L.total) return fail(ED_ERR_INVALID_ARG, "batch workspace too small (see ed_batch_workspace)");
  char* base = (char*)work;
  BatchWork wk;
  wk.queue = (int*)(base + L.off_queue);
  wk.slots = (int64_t*)(base + L.off_slots);
  wk.dmax = b->dmax;
  wk.tri = (double*)(base + L.off_tri);
  wk.exps = (int32_t*)(base + L.off_exps);
  wk.coefs = (int64_t*)(base + L.off_coefs);
  ED_CUDA(cudaMemsetAsync(wk.queue, 0, sizeof(int), s));
#define ED_BATCH_CASE(NT, CS) \
  if (threads == NT && cs == CS) return launch_batch<NT, CS>(b, grid, K, tol, check_every, seed, starts, want_vector, out, wk, s);
  ED_BATCH_CASE(128, 1)
  ED_BATCH_CASE(256, 1)
  ED_BATCH_CASE(512, 1)
  ED_BATCH_CASE(512, 2)
  ED_BATCH_CASE(512, 4)
  ED_BATCH_CASE(512, 8)
  ED_BATCH_CASE(1024, 1)
  ED_BATCH_CASE(1024, 2)
  ED_BATCH_CASE(1024, 4)
  ED_BATCH_CASE(1024, 8)
#undef ED_BATCH_CASE
  return fail(ED_ERR_INVALID_ARG, "unsupported launch configuration");
}

// how many clusters of cs CTAs of the NT-thread kernel the device can hold at once (0: none)
template <int NT, int CS>
static int clusters_for() {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(CS * 16);
  cfg.blockDim = dim3(NT);
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = CS;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  int n = 0;
  if (cudaOccupancyMaxActiveClusters(&n, k_batch_lanczos<NT, CS>, &cfg) != cudaSuccess) {
    (void)cudaGetLastError();
    return 0;
  }
  return n;
}

static int cluster_schedulable(int threads, int cs) {
  if (threads == 512 && cs == 2) return clusters_for<512, 2>();
  if (threads == 512 && cs == 4) return clusters_for<512, 4>();
  if (threads == 512 && cs == 8) return clusters_for<512, 8>();
  if (threads == 1024 && cs == 2) return clusters_for<1024, 2>();
  if (threads == 1024 && cs == 4) return clusters_for<1024, 4>();
  if (threads == 1024 && cs == 8) return clusters_for<1024, 8>();
  return 0;
}

static void default_config(const ed_batch_s* b, int* threads, int* per_sm, int* cs) {
  if (b->tuned_threads) {
    *threads = b->tuned_threads;
    *per_sm = b->tuned_per_sm;
    *cs = b->tuned_cluster;
    return;
  }
  *threads = 512;
  *per_sm = 2;
  *cs = 1;
}

}  // namespace ed

using namespace ed;

extern "C" {

ED_API ed_status ed_batch_create(const ed_plan* plans, int n, ed_batch* out) {
  if (!out) return fail(ED_ERR_INVALID_ARG, "null output");
  *out = nullptr;
  if (n < 1 || !plans) return fail(ED_ERR_INVALID_ARG, "need at least one plan");
  ed_batch_s* b = new ed_batch_s();
  ED_CUDA(cudaGetDevice(&b->device));
  ed_status st = device_context(&b->ctx);
  if (st != ED_OK) { delete b; return st; }
  std::vector<BatchProblem> hp(n);
  for (int i = 0; i < n; ++i) {
    const ed_plan_s* p = plans[i];
    if (!p || p->device != b->device) { delete b; return fail(ED_ERR_INVALID_ARG, "plans must be on the current device"); }
    if (p->kind != 0 || !p->bfp.eligible) {
      delete b;
      return fail(ED_ERR_INVALID_ARG, "batched Lanczos needs fixed-point sectors (ed_plan_fixed_point > 0)");
    }
    const BfpTables& B = p->bfp;
    BatchProblem& q = hp[i];
    memset(&q, 0, sizeof(q));
    q.nu = p->num_up; q.nd = p->num_dn; q.D = p->dim;
    q.up_off = B.up_off; q.up_npos = B.up_npos; q.up_idx = B.up_idx; q.dn_tab = B.dn_tab;
    q.up_states = p->up.states; q.dn_states = p->dn.states;
    q.e_up = B.e_up_int; q.e_dn = B.e_dn_int; q.e_up_fx = B.e_up_fx; q.e_dn_fx = B.e_dn_fx;
    q.max_dn = B.max_dn; q.diag64 = B.diag64; q.dshift = B.Fd - B.F; q.F = B.F; q.m_in = B.m_in;
    q.u_uniform = B.u_uniform; q.t_int = B.t_int; q.u0 = B.u0_int; q.u0_fx = B.u0_fx;
    for (int k = 0; k < ED_MAX_SITES + 2; ++k) { q.u[k] = B.u_int[k]; q.u_fx[k] = B.u_fx[k]; }
    b->dims.push_back(p->dim);
    b->dmax = std::max(b->dmax, p->dim);
  }
  b->n = n;
  // largest problems first (longest-processing-time order for the work queue)
  std::vector<int> order(n);
  for (int i = 0; i < n; ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](int a, int c) { return b->dims[a] > b->dims[c]; });
  cudaError_t e = cudaMalloc(&b->d_probs, n * sizeof(BatchProblem));
  if (e == cudaSuccess) e = cudaMemcpy(b->d_probs, hp.data(), n * sizeof(BatchProblem), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMalloc(&b->d_order, n * sizeof(int));
  if (e == cudaSuccess) e = cudaMemcpy(b->d_order, order.data(), n * sizeof(int), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    cudaFree(b->d_probs);
    cudaFree(b->d_order);
    delete b;
    return cuda_fail(e, "ed_batch_create");
  }
  b->n = n;
  *out = b;
  return ED_OK;
}

ED_API ed_status ed_batch_destroy(ed_batch b) {
  if (!b) return ED_OK;
  cudaFree(b->d_probs);
  cudaFree(b->d_order);
  delete b;
  return ED_OK;
}

ED_API ed_status ed_batch_workspace(ed_batch b, int max_steps, int threads, int ctas_per_sm, int cluster_size,
                                    size_t* bytes) {
  if (!b || !bytes) return fail(ED_ERR_INVALID_ARG, "null argument");
  if (max_steps < 1 || max_steps > 4096) return fail(ED_ERR_INVALID_ARG, "max_steps must be in [1, 4096]");
  int t = threads, ps = ctas_per_sm, cs = cluster_size;
  if (t <= 0 || ps <= 0) default_config(b, &t, &ps, &cs);
  if (cs <= 0) cs = 1;
  if (!valid_config(t, ps, cs)) return fail(ED_ERR_INVALID_ARG, "unsupported launch configuration");
  *bytes = batch_layout(b, max_steps, batch_grid(b, ps, cs), cs).total;
  return ED_OK;
}

ED_API ed_status ed_batch_lanczos(ed_batch b, int max_steps, double tol, int check_every, uint64_t seed,
                                  const double* const* d_starts, int want_vector, void* d_work, size_t work_bytes,
                                  double* d_alpha, double* d_beta, double* d_energy, double* d_residual,
                                  int32_t* d_steps, double* d_vecs, const int64_t* d_vec_offsets, int threads,
                                  int ctas_per_sm, int cluster_size, ed_stream_t stream) {
  if (!b) return fail(ED_ERR_INVALID_ARG, "null batch");
  if (max_steps < 1 || max_steps > 4096) return fail(ED_ERR_INVALID_ARG, "max_steps must be in [1, 4096]");
  if (!d_alpha || !d_beta || !d_energy || !d_residual || !d_steps)
    return fail(ED_ERR_INVALID_ARG, "null output array");
  if (want_vector && (!d_vecs || !d_vec_offsets)) return fail(ED_ERR_INVALID_ARG, "want_vector needs vectors");
  int dev = -1;
  ED_CUDA(cudaGetDevice(&dev));
  if (dev != b->device) return fail(ED_ERR_INVALID_ARG, "batch belongs to another device");
  int t = threads, ps = ctas_per_sm, cs = cluster_size;
  if (t <= 0 || ps <= 0) default_config(b, &t, &ps, &cs);
  if (cs <= 0) cs = 1;
  BatchOut out{d_alpha, d_beta, d_energy, d_residual, d_steps, d_vecs, d_vec_offsets};
  return run_batch(b, t, ps, cs, max_steps, tol, check_every, seed, d_starts, want_vector, d_work, work_bytes, out,
                   as_stream(stream));
}

// Autotuner: times the candidate (threads, CTAs per SM, cluster size) configurations on a short
// run (tune_steps Lanczos steps, no vector) and keeps the fastest for this batch. Cluster
// candidates the device cannot schedule (no active cluster) are skipped.
ED_API ed_status ed_batch_tune(ed_batch b, int tune_steps, void* d_work, size_t work_bytes, double* d_alpha,
                               double* d_beta, double* d_energy, double* d_residual, int32_t* d_steps,
                               int* h_threads, int* h_ctas_per_sm, int* h_cluster_size, float* h_ms,
                               ed_stream_t stream) {
  if (!b) return fail(ED_ERR_INVALID_ARG, "null batch");
  cudaStream_t s = as_stream(stream);
  const int cand[][3] = {{128, 4, 1}, {256, 2, 1},  {256, 4, 1},  {512, 1, 1},  {512, 2, 1},  {1024, 1, 1},
                         {512, 2, 2}, {1024, 1, 2}, {512, 2, 4},  {1024, 1, 4}, {512, 2, 8},  {1024, 1, 8}};
  float best = 1e30f;
  int bt = 0, bp = 0, bc = 0;
  cudaEvent_t e0, e1;
  ED_CUDA(cudaEventCreate(&e0));
  ED_CUDA(cudaEventCreate(&e1));
  BatchOut out{d_alpha, d_beta, d_energy, d_residual, d_steps, nullptr, nullptr};
  for (auto& c : cand) {
    const int grid = batch_grid(b, c[1], c[2]);
    const size_t need = batch_layout(b, tune_steps, grid, c[2]).total;
    if (need > work_bytes) continue;
    if (c[2] > 1 && cluster_schedulable(c[0], c[2]) < 1) continue;
    // warm once, then time
    ED_TRY(run_batch(b, c[0], c[1], c[2], tune_steps, 0.0, 0, 1, nullptr, 0, d_work, work_bytes, out, s));
    ED_CUDA(cudaEventRecord(e0, s));
    ED_TRY(run_batch(b, c[0], c[1], c[2], tune_steps, 0.0, 0, 1, nullptr, 0, d_work, work_bytes, out, s));
    ED_CUDA(cudaEventRecord(e1, s));
    ED_CUDA(cudaEventSynchronize(e1));
    float ms = 0.f;
    ED_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    if (ms < best) { best = ms; bt = c[0]; bp = c[1]; bc = c[2]; }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (!bt) return fail(ED_ERR_INVALID_ARG, "workspace too small for every tuning candidate");
  b->tuned_threads = bt;
  b->tuned_per_sm = bp;
  b->tuned_cluster = bc;
  if (h_threads) *h_threads = bt;
  if (h_ctas_per_sm) *h_ctas_per_sm = bp;
  if (h_cluster_size) *h_cluster_size = bc;
  if (h_ms) *h_ms = best;
  return ED_OK;
}

ED_API ed_status ed_batch_gf_continued_fraction(int n, int max_steps, const double* d_alpha, const double* d_beta,
                                                const int32_t* d_steps, const double* d_e0, int sign,
                                                const double* d_z, int64_t n_z, double* d_g, ed_stream_t stream) {
  if (n < 1 || n_z < 0) return fail(ED_ERR_INVALID_ARG, "bad sizes");
  if (sign != 1 && sign != -1) return fail(ED_ERR_INVALID_ARG, "sign must be +1 or -1");
  if (n_z == 0) return ED_OK;
  if (!d_alpha || !d_beta || !d_steps || !d_e0 || !d_z || !d_g) return fail(ED_ERR_INVALID_ARG, "null argument");
  DeviceContext* ctx;
  ED_TRY(device_context(&ctx));
  const int64_t tot = (int64_t)n * n_z;
  k_batch_cf<<<grid_for(tot, 128, ctx->num_sms * 16), 128, 0, as_stream(stream)>>>(
      n, max_steps, d_alpha, d_beta, d_steps, d_e0, sign, (const double2*)d_z, n_z, (double2*)d_g);
  ED_CHECK_LAUNCH("k_batch_cf");
  return ED_OK;
}

}  // extern "C"
