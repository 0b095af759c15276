// Device helpers shared by the adjoint kernels of one problem (ed_adjoint.cu) and of a batch
// of problems with one structure (ed_adjoint_batch.cu): the parameter term a^T (dH/dtheta) b
// of a fermionic plan and the deterministic last-block reductions of the taped Lanczos.
// Parameter layout: [eps_0..eps_{N-1}, U_0..U_{N-1}, t_0..t_{nb-1}], N <= 16, nb <= 32.
#pragma once

#include <algorithm>
#include <cmath>
#include <vector>

#include "ed_plan.cuh"
#include "ed_tridiag.cuh"

namespace ed {

constexpr int SW_SITES = 16;
constexpr int SW_BONDS = 32;
constexpr int SW_P = 2 * SW_SITES + SW_BONDS;
constexpr int SW_NT = 128;

struct SandwichArgs {
  const uint64_t* up_states; const uint64_t* dn_states;
  const int32_t* up_off; const int32_t* up_idx; const double* up_coef; const int16_t* up_bond;
  const int32_t* dn_off; const int32_t* dn_idx; const double* dn_coef; const int16_t* dn_bond;
  int64_t nu, nd;
};

// Row i's terms of a^T (dH/dtheta) b, added to the calling thread's accumulator column
// acc[p * SW_NT] (p in the packed order [eps(ns), U(ns), t(nb)]; the column lives in shared
// memory, so a term costs one add whatever the parameter count). The diagonal part (eps, U)
// depends on a_i b_i only; the hop part gathers b at the row's hop partners.
__device__ __forceinline__ void sandwich_diag_terms(const SandwichArgs& g, int ns, int64_t i, double pr, double* acc) {
  const int64_t u = i / g.nd, d = i - u * g.nd;
  const uint64_t su = g.up_states[u], sd = g.dn_states[d];
  for (uint64_t bits = su; bits; bits &= bits - 1) acc[(__ffsll((long long)bits) - 1) * SW_NT] += pr;
  for (uint64_t bits = sd; bits; bits &= bits - 1) acc[(__ffsll((long long)bits) - 1) * SW_NT] += pr;
  for (uint64_t bits = su & sd; bits; bits &= bits - 1) acc[(ns + __ffsll((long long)bits) - 1) * SW_NT] += pr;
}

__device__ __forceinline__ void sandwich_hop_terms(const SandwichArgs& g, int ns, int64_t i, double ai,
                                                   const double* __restrict__ b, double* acc) {
  const int64_t u = i / g.nd, d = i - u * g.nd;
  // the hop's sign (that of its coefficient) flips the sign bit of a_i: integer operations
  const long long ab = __double_as_longlong(ai);
  const long long sbit = (long long)0x8000000000000000ull;
  const int32_t u0 = g.up_off[u], u1 = g.up_off[u + 1];
  for (int32_t e = u0; e < u1; ++e) {
    const double as = __longlong_as_double(ab ^ (__double_as_longlong(g.up_coef[e]) & sbit));
    double* a = acc + (2 * ns + g.up_bond[e]) * SW_NT;
    *a = fma(as, b[(int64_t)g.up_idx[e] * g.nd + d], *a);
  }
  const int32_t d0 = g.dn_off[d], d1 = g.dn_off[d + 1];
  for (int32_t e = d0; e < d1; ++e) {
    const double as = __longlong_as_double(ab ^ (__double_as_longlong(g.dn_coef[e]) & sbit));
    double* a = acc + (2 * ns + g.dn_bond[e]) * SW_NT;
    *a = fma(as, b[u * g.nd + g.dn_idx[e]], *a);
  }
}

__device__ __forceinline__ void sandwich_row(const SandwichArgs& g, int ns, int64_t i, double ai, double bi,
                                             const double* __restrict__ b, double* acc) {
  sandwich_diag_terms(g, ns, i, ai * bi, acc);
  sandwich_hop_terms(g, ns, i, ai, b, acc);
}

__device__ __forceinline__ void sandwich_zero(double* sacc, int P) {
  for (int t = threadIdx.x; t < P * SW_NT; t += SW_NT) sacc[t] = 0.0;
  __syncthreads();
}

// the block's P sums (threads in a fixed order) into out_row[0..P), written or added
__device__ __forceinline__ void sandwich_block_out(const double* sacc, int P, double* out_row, bool accumulate) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  __syncthreads();
  for (int p = warp; p < P; p += SW_NT / 32) {
    double v = 0.0;
#pragma unroll
    for (int r = 0; r < SW_NT / 32; ++r) v += sacc[p * SW_NT + lane + 32 * r];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) out_row[p] = accumulate ? out_row[p] + v : v;
  }
}

constexpr int TP_NT = 256;

__device__ __forceinline__ bool tp_last_block(unsigned int* ticket) {
  __shared__ bool am_last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) am_last = (atomicAdd(ticket, 1u) == gridDim.x - 1);
  __syncthreads();
  if (am_last) __threadfence();
  return am_last;
}

// sum of row j of partial[j * nb + b] over b in block order (whole block; valid in thread 0)
__device__ __forceinline__ double tp_row_sum(const double* partial, int nb, double* sm) {
  double v = 0.0;
  for (int b = threadIdx.x; b < nb; b += TP_NT) v += ((volatile const double*)partial)[b];
  return block_sum<TP_NT>(v, sm);
}

// the residual of step k, element i (shared by the forward and the recompute)
__device__ __forceinline__ double tp_resid(double w, double a, double q, double b, const double* qp, int64_t i) {
  double x = fma(-a, q, w);
  if (qp) x = fma(-b, qp[i], x);
  return x;
}

inline SandwichArgs sandwich_args(const ed_plan_s* p) {
  return SandwichArgs{p->up.states, p->dn.states, p->up.off, p->up.idx, p->up.coef, p->up.bond,
                      p->dn.off, p->dn.idx, p->dn.coef, p->dn.bond, p->num_up, p->num_dn};
}

inline size_t sandwich_smem(int P) { return (size_t)P * SW_NT * sizeof(double); }



// ---- continued fraction and its adjoint, for one problem or a batch ------------------------
// G(z) = sign n2 / t_0, t_l = z' - alpha_l - beta_{l+1}^2 / t_{l+1}, t_{m-1} = z' - alpha_{m-1},
// z' = sign z + shift. For L = Re sum_z conj(gbar_z) G_z the adjoints follow the chain
// u_0 = dG/dt_0 = -sign n2 / t_0^2, u_{l+1} = u_l beta_{l+1}^2 / t_{l+1}^2:
//   dG/dalpha_l = -u_l, dG/dbeta_{l+1} = -2 u_l beta_{l+1} / t_{l+1}, dG/dshift = sum_l u_l,
//   dG/dn2 = sign / t_0.
// One thread per (frequency, problem); per-level block sums to partial rows [2m + 2][G] of the
// problem, the problem's last block sums them in block order.
constexpr int CFA_NT = 256;

__device__ __forceinline__ double2 c_mul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 c_div(double2 a, double2 b) {
  const double d = b.x * b.x + b.y * b.y;
  return make_double2((a.x * b.x + a.y * b.y) / d, (a.y * b.x - a.x * b.y) / d);
}

// problem b's scalars: arrays when given (batch), else the single values
struct CfaBatch {
  const double* alpha; int64_t ka;  // alpha[b * ka + l]
  const double* beta; int64_t kb;   // beta[b * kb + l]
  const int* m_arr; const double* n2_arr; const double* shift_arr;
  int m1; double n21, shift1;
  int sign;
  const double* gbar;               // [B][nz] interleaved complex
  double* abar; double* bbar;       // [B][ka], [B][kb]
  double* scal;                     // [B][2]: dL/dshift, dL/dn2
};

static __global__ void __launch_bounds__(CFA_NT) k_cf_adjoint(CfaBatch cb, const double2* __restrict__ z, int64_t nz,
                                                       double2* __restrict__ ts_all, int mmax, double* partial_all,
                                                       unsigned int* tickets) {
  __shared__ double sm[CFA_NT / 32];
  const int pb = blockIdx.y, G = gridDim.x;
  const int m = cb.m_arr ? cb.m_arr[pb] : cb.m1;
  if (m < 1) return;
  const double n2 = cb.n2_arr ? cb.n2_arr[pb] : cb.n21;
  const double shift = cb.shift_arr ? cb.shift_arr[pb] : cb.shift1;
  const int sign = cb.sign;
  const double* a = cb.alpha + (int64_t)pb * cb.ka;
  const double* b = cb.beta + (int64_t)pb * cb.kb;
  const double2* gbar = (const double2*)cb.gbar + (int64_t)pb * nz;
  double2* ts = ts_all + (int64_t)pb * mmax * nz;
  double* partial = partial_all + (int64_t)pb * (2 * mmax + 2) * G;
  const int64_t i = blockIdx.x * (int64_t)CFA_NT + threadIdx.x;
  const bool ok = i < nz;
  double2 cg = make_double2(0.0, 0.0), zp = make_double2(0.0, 0.0);
  if (ok) {
    cg = make_double2(gbar[i].x, -gbar[i].y);
    zp = make_double2(sign * z[i].x + shift, sign * z[i].y);
    double2 t = make_double2(zp.x - a[m - 1], zp.y);
    ts[(int64_t)(m - 1) * nz + i] = t;
    for (int l = m - 2; l >= 0; --l) {
      const double bb = b[l + 1] * b[l + 1];
      const double2 q = c_div(make_double2(bb, 0.0), t);
      t = make_double2(zp.x - a[l] - q.x, zp.y - q.y);
      ts[(int64_t)l * nz + i] = t;
    }
  }
  double2 t0 = ok ? ts[i] : make_double2(1.0, 0.0);
  double2 u = ok ? c_div(make_double2(-sign * n2, 0.0), c_mul(t0, t0)) : make_double2(0.0, 0.0);
  double2 dz = make_double2(0.0, 0.0);
  for (int l = 0; l < m; ++l) {
    dz.x += u.x;
    dz.y += u.y;
    const double ca = -(cg.x * u.x - cg.y * u.y);  // Re(cg * (-u))
    double cbv = 0.0;
    double2 t1 = make_double2(1.0, 0.0);
    if (l + 1 < m && ok) {
      t1 = ts[(int64_t)(l + 1) * nz + i];
      const double2 f = c_div(make_double2(-2.0 * b[l + 1], 0.0), t1);
      const double2 uf = c_mul(u, f);
      cbv = cg.x * uf.x - cg.y * uf.y;
    }
    const double sa = block_sum<CFA_NT>(ok ? ca : 0.0, sm);
    const double sbv = block_sum<CFA_NT>(cbv, sm);
    if (threadIdx.x == 0) {
      partial[(int64_t)l * G + blockIdx.x] = sa;
      partial[(int64_t)(m + l) * G + blockIdx.x] = sbv;
    }
    if (l + 1 < m && ok) {
      const double bb = b[l + 1] * b[l + 1];
      u = c_mul(u, c_div(make_double2(bb, 0.0), c_mul(t1, t1)));
    }
  }
  const double ce = ok ? cg.x * dz.x - cg.y * dz.y : 0.0;
  double cn = 0.0;
  if (ok) {
    const double2 f = c_div(make_double2((double)sign, 0.0), t0);
    cn = cg.x * f.x - cg.y * f.y;
  }
  const double se = block_sum<CFA_NT>(ce, sm);
  const double sn = block_sum<CFA_NT>(cn, sm);
  if (threadIdx.x == 0) {
    partial[(int64_t)(2 * m) * G + blockIdx.x] = se;
    partial[(int64_t)(2 * m + 1) * G + blockIdx.x] = sn;
  }
  if (!tp_last_block(&tickets[pb])) return;
  double* abar = cb.abar + (int64_t)pb * cb.ka;
  double* bbar = cb.bbar + (int64_t)pb * cb.kb;
  double* scal = cb.scal + 2 * (int64_t)pb;
  // one row per thread, blocks summed in order
  for (int r = threadIdx.x; r < 2 * m + 2; r += CFA_NT) {
    double t = 0.0;
    for (int bk = 0; bk < G; ++bk) t += ((volatile const double*)partial)[(int64_t)r * G + bk];
    if (r < m) abar[r] = t;
    else if (r < 2 * m) { if (r - m + 1 < m) bbar[r - m + 1] = t; }
    else if (r == 2 * m) scal[0] = t;
    else { scal[1] = t; bbar[0] = 2.0 * sqrt(n2) * t; }
  }
  if (threadIdx.x == 0) {
    bbar[m] = 0.0;
    tickets[pb] = 0;
  }
}

// B problems (m_max the largest m), scratch allocated stream-ordered
inline ed_status cf_adjoint_launch(const CfaBatch& cb, int B, int mmax, const double2* z, int64_t nz, cudaStream_t s) {
  const int G = (int)((nz + CFA_NT - 1) / CFA_NT);
  const size_t ts_bytes = (size_t)B * mmax * nz * sizeof(double2);
  const size_t part_bytes = (size_t)B * (2 * mmax + 2) * G * sizeof(double);
  char* buf = nullptr;
  ED_CUDA(cudaMallocAsync((void**)&buf, ts_bytes + part_bytes + (size_t)B * sizeof(unsigned int) + 256, s));
  unsigned int* tickets = (unsigned int*)(buf + ts_bytes + part_bytes);
  ED_CUDA(cudaMemsetAsync(tickets, 0, (size_t)B * sizeof(unsigned int), s));
  k_cf_adjoint<<<dim3(G, B), CFA_NT, 0, s>>>(cb, z, nz, (double2*)buf, mmax, (double*)(buf + ts_bytes), tickets);
  ED_CHECK_LAUNCH("k_cf_adjoint");
  ED_CUDA(cudaFreeAsync(buf, s));
  return ED_OK;
}

}  // namespace ed
