// Batched adjoint Green's function: B problems that share one plan's structure (sector, bonds,
// hopping signs) and differ in their parameters theta[b] = [eps(N), U(N), t(nb)]. Every vector
// is stored problem-major ([B][D]); one launch serves all B problems of a Lanczos step, so at
// the adjoint's sector sizes (D ~ 6e4, where one problem's kernels are latency-bound) the
// batch turns B chains of small launches into one chain of launches that fill the GPU.
//
// The arithmetic of problem b is that of the single-problem tape (ed_adjoint.cu): the same
// diagonal, the same order of the hop sums, the same explicit FMAs and reciprocals, so a batch
// reproduces B single-problem runs. The plan passed in is a structure plan: built with t = 1 on
// every bond (its coefficients are the fermionic signs); its eps and U are not used.
// No reference counterpart (the reference has no derivatives); the use is fitting Anderson bath
// parameters (cmpy/models/anderson.py:93-145) for many impurity models at once.
#include <algorithm>
#include <cmath>
#include <vector>

#include "ed_adjoint.cuh"
#include "ed_lzcheck.cuh"

namespace ed {

constexpr int BT_NT = 256;

struct BState {
  int* stop;    // [B] 0 running, 1 converged (host), 2 breakdown
  int* steps;   // [B] m at a breakdown
  int* m;       // [B] tape length (combine / reverse)
  unsigned int* ticket;  // [2][B]
};

// per-problem diagonal: (sum_{i in up} eps_i + sum_{i in dn} eps_i) + U-term, ascending sites,
// the arithmetic of the single-problem plan
__global__ void __launch_bounds__(BT_NT) k_bdiag(SandwichArgs g, int ns, int P, const double* __restrict__ theta,
                                                 double* __restrict__ diag) {
  __shared__ double eps[SW_SITES], uu[SW_SITES];
  __shared__ int uni;
  const int b = blockIdx.y;
  if (threadIdx.x < ns) {
    eps[threadIdx.x] = theta[(int64_t)b * P + threadIdx.x];
    uu[threadIdx.x] = theta[(int64_t)b * P + ns + threadIdx.x];
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    int u = 1;
    for (int j = 1; j < ns; ++j) u &= (uu[j] == uu[0]) ? 1 : 0;
    uni = u;
  }
  __syncthreads();
  const int64_t D = g.nu * g.nd;
  for (int64_t i = blockIdx.x * (int64_t)BT_NT + threadIdx.x; i < D; i += (int64_t)gridDim.x * BT_NT) {
    const int64_t u = i / g.nd, d = i - u * g.nd;
    const uint64_t su = g.up_states[u], sd = g.dn_states[d];
    const double eu = weighted_element(su, eps, ns), ed_ = weighted_element(sd, eps, ns);
    uint64_t both = su & sd;
    double ut;
    if (uni) {
      ut = (ns > 0 ? uu[0] : 0.0) * (double)__popcll(both);
    } else {
      ut = 0.0;
      while (both) {
        ut += uu[__ffsll((long long)both) - 1];
        both &= both - 1;
      }
    }
    diag[(int64_t)b * D + i] = eu + ed_ + ut;
  }
}

// hop coefficient of a problem: t with the sign bit of the structure plan's coefficient (the
// fermionic sign +-1.0), applied with integer operations (the FP64 pipe is the scarce one)
__device__ __forceinline__ double bhop(double sign, double t) {
  return __longlong_as_double(__double_as_longlong(t) ^ (__double_as_longlong(sign) & (long long)0x8000000000000000ull));
}

// problem b is skipped when mode 1: gate[b] != 0, mode 2: k >= gate[b]
__device__ __forceinline__ bool bskip(const int* gate, int mode, int k, int b) {
  if (mode == 1) return gate[b] != 0;
  if (mode == 2) return k >= gate[b];
  return false;
}

// y[b] = H_b x[b] for BMV_PB problems per CTA: one CTA per (up-row, group of problems), threads
// over the dn index. The hop lists are loaded once for the group and each problem keeps its
// own FMA chain (independent chains for the narrow FP64 pipe); per element and problem the
// diagonal term, then the up-hop list, then the dn-hop list, the single-problem order.
constexpr int BMV_PB = 4;

__global__ void __launch_bounds__(BT_NT) k_bmv(SandwichArgs g, int B, int P, int tofs, int nb,
                                               const double* __restrict__ theta, const double* __restrict__ diag,
                                               const double* __restrict__ x, double* __restrict__ y, const int* gate,
                                               int mode, int k) {
  const int b0 = blockIdx.y * BMV_PB;
  __shared__ double t[BMV_PB][SW_BONDS];
  __shared__ int live_s[BMV_PB];
  if (threadIdx.x < BMV_PB) {
    const int b = b0 + threadIdx.x;
    live_s[threadIdx.x] = (b < B && !bskip(gate, mode, k, b)) ? 1 : 0;
  }
  for (int q = threadIdx.x; q < BMV_PB * SW_BONDS; q += BT_NT) {
    const int pb = q / SW_BONDS, j = q - pb * SW_BONDS;
    t[pb][j] = (b0 + pb < B && j < nb) ? theta[(int64_t)(b0 + pb) * P + tofs + j] : 0.0;
  }
  __syncthreads();
  bool live[BMV_PB];
  int any = 0;
#pragma unroll
  for (int pb = 0; pb < BMV_PB; ++pb) {
    live[pb] = live_s[pb] != 0;
    any |= live_s[pb];
  }
  if (!any) return;
  const int64_t nd = g.nd, D = g.nu * nd;
  for (int64_t u = blockIdx.x; u < g.nu; u += gridDim.x) {
    const int32_t u0 = g.up_off[u], u1 = g.up_off[u + 1];
    for (int64_t d = threadIdx.x; d < nd; d += BT_NT) {
      const int64_t i = u * nd + d;
      double acc[BMV_PB];
#pragma unroll
      for (int pb = 0; pb < BMV_PB; ++pb)
        acc[pb] = live[pb] ? diag[(int64_t)(b0 + pb) * D + i] * x[(int64_t)(b0 + pb) * D + i] : 0.0;
      for (int32_t e = u0; e < u1; ++e) {
        const double sg = __ldg(g.up_coef + e);
        const int bd = __ldg(g.up_bond + e);
        const int64_t j = (int64_t)__ldg(g.up_idx + e) * nd + d;
#pragma unroll
        for (int pb = 0; pb < BMV_PB; ++pb)
          if (live[pb]) acc[pb] = fma(bhop(sg, t[pb][bd]), x[(int64_t)(b0 + pb) * D + j], acc[pb]);
      }
      const int32_t d0 = __ldg(g.dn_off + d), d1 = __ldg(g.dn_off + d + 1);
      for (int32_t e = d0; e < d1; ++e) {
        const double sg = __ldg(g.dn_coef + e);
        const int bd = __ldg(g.dn_bond + e);
        const int64_t j = u * nd + __ldg(g.dn_idx + e);
#pragma unroll
        for (int pb = 0; pb < BMV_PB; ++pb)
          if (live[pb]) acc[pb] = fma(bhop(sg, t[pb][bd]), x[(int64_t)(b0 + pb) * D + j], acc[pb]);
      }
#pragma unroll
      for (int pb = 0; pb < BMV_PB; ++pb)
        if (live[pb]) y[(int64_t)(b0 + pb) * D + i] = acc[pb];
    }
  }
}

// per-problem sum of row j of partial[(j * B + b) * G + blk] over blk in block order
__device__ __forceinline__ double bt_row_sum(const double* partial, int G, double* sm) {
  return tp_row_sum(partial, G, sm);
}

// res[b * rstride] = <a[b], c[b]> (and its sqrt -> rsq[b * qstride]); mode/gate as bskip
__global__ void __launch_bounds__(BT_NT) k_bt_dot(const double* __restrict__ a, const double* __restrict__ c, int64_t n,
                                                  double* partial, unsigned int* ticket, double* res, int64_t rstride,
                                                  double* rsq, int64_t qstride, const int* gate, int mode, int k) {
  const int b = blockIdx.y, G = gridDim.x;
  if (bskip(gate, mode, k, b)) return;
  __shared__ double sm[BT_NT / 32];
  const double* ab = a + (int64_t)b * n;
  const double* cb = c + (int64_t)b * n;
  double v = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)BT_NT + threadIdx.x; i < n; i += (int64_t)G * BT_NT) v = fma(ab[i], cb[i], v);
  v = block_sum<BT_NT>(v, sm);
  if (threadIdx.x == 0) partial[(int64_t)b * G + blockIdx.x] = v;
  if (tp_last_block(&ticket[b])) {
    const double s = bt_row_sum(partial + (int64_t)b * G, G, sm);
    if (threadIdx.x == 0) {
      res[b * rstride] = s;
      if (rsq) rsq[b * qstride] = sqrt(s);
      ticket[b] = 0;
    }
  }
}

// out[b] = v[b] * (1 / scale[b * sstride])
__global__ void k_bt_scale(const double* __restrict__ v, double* __restrict__ out, int64_t n, const double* scale,
                           int64_t sstride, const int* gate, int mode, int k) {
  const int b = blockIdx.y;
  if (bskip(gate, mode, k, b)) return;
  const double s = 1.0 / scale[b * sstride];
  const double* vb = v + (int64_t)b * n;
  double* ob = out + (int64_t)b * n;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    ob[i] = vb[i] * s;
}

// w[b] <- w - alpha_k q_k - beta_k q_{k-1}; beta_{k+1} = ||w||; breakdown as the single tape
__global__ void __launch_bounds__(BT_NT) k_bt_update(double* __restrict__ w, const double* __restrict__ q,
                                                     const double* __restrict__ qp, int64_t n, const double* alpha,
                                                     double* beta, int K, int k, double breakdown, double* partial,
                                                     BState bs) {
  const int b = blockIdx.y, G = gridDim.x;
  if (bs.stop[b]) return;
  __shared__ double sm[BT_NT / 32];
  const double a = alpha[(int64_t)b * K + k], bk = qp ? beta[(int64_t)b * (K + 1) + k] : 0.0;
  double* wb = w + (int64_t)b * n;
  const double* qb = q + (int64_t)b * n;
  const double* qpb = qp ? qp + (int64_t)b * n : nullptr;
  double v = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)BT_NT + threadIdx.x; i < n; i += (int64_t)G * BT_NT) {
    const double xv = tp_resid(wb[i], a, qb[i], bk, qpb, i);
    wb[i] = xv;
    v = fma(xv, xv, v);
  }
  v = block_sum<BT_NT>(v, sm);
  if (threadIdx.x == 0) partial[(int64_t)b * G + blockIdx.x] = v;
  unsigned int* tk = bs.ticket + gridDim.y;
  if (tp_last_block(&tk[b])) {
    const double s = bt_row_sum(partial + (int64_t)b * G, G, sm);
    if (threadIdx.x == 0) {
      const double bn = sqrt(s);
      beta[(int64_t)b * (K + 1) + k + 1] = bn;
      const double scale = fabs(a) + (k > 0 ? bk : 0.0);
      if (!(bn > breakdown * scale)) {
        bs.steps[b] = k + 1;
        bs.stop[b] = 2;
      }
      tk[b] = 0;
    }
  }
}

// checkpoint slot [2][B][n]: [q_{k-1} (zeros for k = 0), q_k]
__global__ void k_bt_ckpt(const double* __restrict__ q, const double* __restrict__ qp, double* __restrict__ dst,
                          int64_t n, const int* stop) {
  const int b = blockIdx.y, B = gridDim.y;
  if (stop[b]) return;
  const double* qb = q + (int64_t)b * n;
  const double* qpb = qp ? qp + (int64_t)b * n : nullptr;
  double* d0 = dst + (int64_t)b * n;
  double* d1 = dst + ((int64_t)B + b) * n;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    d0[i] = qpb ? qpb[i] : 0.0;
    d1[i] = qb[i];
  }
}

// q_{k+1}[b] recomputed from w_k = H q_k (problems with k + 1 >= m[b] skip); optionally
// y += coef[b][k+1] q_{k+1} and dots[b][k+1] = q_{k+1} . probe
__global__ void __launch_bounds__(BT_NT) k_bt_next(const double* __restrict__ w, const double* __restrict__ q,
                                                   const double* __restrict__ qp, int64_t n, const double* alpha,
                                                   const double* beta, int K, int k, double* __restrict__ out,
                                                   const double* coef, double* __restrict__ y,
                                                   const double* __restrict__ probe, double* partial, BState bs,
                                                   double* dots) {
  const int b = blockIdx.y, G = gridDim.x;
  if (k + 1 >= bs.m[b]) return;
  __shared__ double sm[BT_NT / 32];
  const double a = alpha[(int64_t)b * K + k], bk = qp ? beta[(int64_t)b * (K + 1) + k] : 0.0;
  const double s = 1.0 / beta[(int64_t)b * (K + 1) + k + 1];
  const double cy = y ? coef[(int64_t)b * K + k + 1] : 0.0;
  const int64_t o = (int64_t)b * n;
  const double* qpb = qp ? qp + o : nullptr;
  double v = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)BT_NT + threadIdx.x; i < n; i += (int64_t)G * BT_NT) {
    const double q1 = tp_resid(w[o + i], a, q[o + i], bk, qpb, i) * s;
    out[o + i] = q1;
    if (y) y[o + i] = fma(cy, q1, y[o + i]);
    if (probe) v = fma(q1, probe[o + i], v);
  }
  if (!probe) return;
  v = block_sum<BT_NT>(v, sm);
  if (threadIdx.x == 0) partial[(int64_t)b * G + blockIdx.x] = v;
  if (tp_last_block(&bs.ticket[b])) {
    const double t = bt_row_sum(partial + (int64_t)b * G, G, sm);
    if (threadIdx.x == 0) {
      dots[(int64_t)b * K + k + 1] = t;
      bs.ticket[b] = 0;
    }
  }
}

// segment start q_k[b] (k < m[b]): y += coef[b][k] q_k, dots[b][k] = q_k . probe
__global__ void __launch_bounds__(BT_NT) k_bt_acc(const double* __restrict__ q, int64_t n, int K, int k,
                                                  const double* coef, double* __restrict__ y,
                                                  const double* __restrict__ probe, double* partial, BState bs,
                                                  double* dots) {
  const int b = blockIdx.y, G = gridDim.x;
  if (k >= bs.m[b]) return;
  __shared__ double sm[BT_NT / 32];
  const double cy = y ? coef[(int64_t)b * K + k] : 0.0;
  const int64_t o = (int64_t)b * n;
  double v = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)BT_NT + threadIdx.x; i < n; i += (int64_t)G * BT_NT) {
    if (y) y[o + i] = fma(cy, q[o + i], y[o + i]);
    if (probe) v = fma(q[o + i], probe[o + i], v);
  }
  if (!probe) return;
  v = block_sum<BT_NT>(v, sm);
  if (threadIdx.x == 0) partial[(int64_t)b * G + blockIdx.x] = v;
  if (tp_last_block(&bs.ticket[b])) {
    const double t = bt_row_sum(partial + (int64_t)b * G, G, sm);
    if (threadIdx.x == 0) {
      dots[(int64_t)b * K + k] = t;
      bs.ticket[b] = 0;
    }
  }
}

// reverse step k, part 1, per problem with k + 1 < m[b] (the single tape's k_tp_radot);
// fin: k = -1, completes q_bar_0 and res[b] = q_bar_0 . q_0 for problems with m[b] >= 1
__global__ void __launch_bounds__(BT_NT) k_bt_radot(double* __restrict__ qb1, const double* __restrict__ tmp,
                                                    const double* __restrict__ ext, const double* ext_coef,
                                                    const double* __restrict__ q1, const double* __restrict__ q0,
                                                    const double* __restrict__ qm, int64_t n, const double* beta,
                                                    double* abar, double* bbar, int K, int k, double* partial,
                                                    BState bs, double* res) {
  const int b = blockIdx.y, B = gridDim.y, G = gridDim.x;
  const bool fin = res != nullptr;
  if (k + 1 >= bs.m[b]) return;
  __shared__ double sm[BT_NT / 32];
  const int64_t o = (int64_t)b * n;
  const double ce = ext ? ext_coef[(int64_t)b * K + k + 1] : 0.0;
  double d1 = 0.0, d2 = 0.0, d3 = 0.0, d4 = 0.0, d5 = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)BT_NT + threadIdx.x; i < n; i += (int64_t)G * BT_NT) {
    double v = qb1[o + i];
    if (tmp) v += tmp[o + i];
    if (ext) v = fma(ce, ext[o + i], v);
    qb1[o + i] = v;
    const double x1 = q1[o + i];
    d1 = fma(v, x1, d1);
    if (!fin) {
      const double x0 = q0[o + i], xm = qm ? qm[o + i] : 0.0;
      d2 = fma(v, x0, d2);
      d3 = fma(v, xm, d3);
      d4 = fma(x1, x0, d4);
      d5 = fma(x1, xm, d5);
    }
  }
  const int nd = fin ? 1 : 5;
  double dv[5] = {d1, d2, d3, d4, d5};
  for (int j = 0; j < nd; ++j) {
    const double s = block_sum<BT_NT>(dv[j], sm);
    if (threadIdx.x == 0) partial[((int64_t)j * B + b) * G + blockIdx.x] = s;
  }
  if (tp_last_block(&bs.ticket[b])) {
    double t[5];
    for (int j = 0; j < nd; ++j) t[j] = bt_row_sum(partial + ((int64_t)j * B + b) * G, G, sm);
    if (threadIdx.x == 0) {
      if (fin) {
        res[b] = t[0];
      } else {
        double* ab = abar + (int64_t)b * K;
        double* bb = bbar + (int64_t)b * (K + 1);
        const double bk1 = beta[(int64_t)b * (K + 1) + k + 1];
        const double bb1 = bb[k + 1] - t[0] / bk1;
        bb[k + 1] = bb1;
        ab[k] -= t[1] / bk1 + bb1 * t[3];
        if (k > 0) bb[k] -= t[2] / bk1 + bb1 * t[4];
      }
      bs.ticket[b] = 0;
    }
  }
}

// reverse step k, part 2, per problem with k < m[b] (the single tape's k_tp_rstep), fused with
// w_bar^T (dH_b/dtheta) q_k added to the block's row of psw[b][blk][SW_P]
__global__ void __launch_bounds__(SW_NT) k_bt_rstep(SandwichArgs g, int ns, int P, const double* __restrict__ qb1,
                                                    const double* __restrict__ q1, const double* __restrict__ q0,
                                                    const double* __restrict__ w0, double* __restrict__ qbk,
                                                    double* __restrict__ qbm, double* __restrict__ wbar,
                                                    const double* alpha, const double* beta, const double* abar,
                                                    const double* bbar, int K, int k, BState bs,
                                                    double* __restrict__ pracc, double* __restrict__ psw) {
  const int b = blockIdx.y;
  const int m = bs.m[b];
  if (k >= m) return;
  extern __shared__ double sacc[];  // [P][SW_NT]
  sandwich_zero(sacc, P);
  const bool has_next = k + 1 < m, first = k == m - 1;
  const double ak = alpha[(int64_t)b * K + k], ab = abar[(int64_t)b * K + k];
  const double inv = has_next ? 1.0 / beta[(int64_t)b * (K + 1) + k + 1] : 0.0;
  const double bb1 = has_next ? bbar[(int64_t)b * (K + 1) + k + 1] : 0.0;
  const double bk = k > 0 ? beta[(int64_t)b * (K + 1) + k] : 0.0;
  const int64_t D = g.nu * g.nd, o = (int64_t)b * D;
  const double* q0b = q0 + o;
  for (int64_t i = blockIdx.x * (int64_t)SW_NT + threadIdx.x; i < D; i += (int64_t)gridDim.x * SW_NT) {
    const double rb = has_next ? fma(bb1, q1[o + i], qb1[o + i] * inv) : 0.0;
    const double x0 = q0b[i];
    const double wb = fma(ab, x0, rb);
    qbk[o + i] = fma(ab, w0[o + i], fma(-ak, rb, first ? 0.0 : qbk[o + i]));
    if (qbm) qbm[o + i] = -bk * rb;
    wbar[o + i] = wb;
    // the hop part now, the diagonal part through sum_k w_bar_k q_k
    pracc[o + i] = fma(wb, x0, first ? 0.0 : pracc[o + i]);
    sandwich_hop_terms(g, ns, i, wb, q0b, sacc + threadIdx.x);
  }
  sandwich_block_out(sacc, P, psw + ((int64_t)b * gridDim.x + blockIdx.x) * SW_P, true);
}

// the diagonal (eps, U) part from pracc[b] = sum_k w_bar_k q_k (problems with m[b] >= 1)
__global__ void __launch_bounds__(SW_NT) k_bt_diag_terms(SandwichArgs g, int ns, int P, const double* __restrict__ pracc,
                                                         BState bs, double* __restrict__ psw) {
  const int b = blockIdx.y;
  if (bs.m[b] < 1) return;
  extern __shared__ double sacc[];  // [P][SW_NT]
  sandwich_zero(sacc, P);
  const int64_t D = g.nu * g.nd, o = (int64_t)b * D;
  for (int64_t i = blockIdx.x * (int64_t)SW_NT + threadIdx.x; i < D; i += (int64_t)gridDim.x * SW_NT)
    sandwich_diag_terms(g, ns, i, pracc[o + i], sacc + threadIdx.x);
  sandwich_block_out(sacc, P, psw + ((int64_t)b * gridDim.x + blockIdx.x) * SW_P, true);
}

// start_bar[b] = (q_bar_0 - (q_bar_0.q_0) q_0) / beta_0 + beta_bar_0 q_0   (m[b] >= 1)
__global__ void k_bt_startbar(const double* __restrict__ qb0, const double* __restrict__ q0, int64_t n,
                              const double* beta, const double* bbar, int K, const double* dres, BState bs,
                              double* __restrict__ out) {
  const int b = blockIdx.y;
  const int64_t o = (int64_t)b * n;
  if (bs.m[b] < 1) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
      out[o + i] = 0.0;
    return;
  }
  const double d = dres[b], ib = 1.0 / beta[(int64_t)b * (K + 1)], b0 = bbar[(int64_t)b * (K + 1)];
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[o + i] = fma(b0, q0[o + i], (qb0[o + i] - d * q0[o + i]) * ib);
}

// theta_bar[b][p] += sum_blk psw[b][blk][p]
__global__ void k_bt_param_reduce(const double* __restrict__ psw, int nblk, int P, double* __restrict__ out) {
  const int b = blockIdx.x, p = threadIdx.x;
  if (p >= P) return;
  double s = 0.0;
  for (int k = 0; k < nblk; ++k) s += psw[((int64_t)b * nblk + k) * SW_P + p];
  out[(int64_t)b * P + p] += s;
}

// G[b](z) (+)= sign n2_b / (z' - alpha_0 - beta_1^2 / (z' - ...)), z' = sign z + shift_b: the
// arithmetic of k_cf (single problem) for every problem with m[b] >= 1; one thread per (z, b)
__global__ void k_bcf(const double* __restrict__ alpha, int64_t ka, const double* __restrict__ beta, int64_t kb,
                      const int* __restrict__ m_arr, const double* __restrict__ n2_arr,
                      const double* __restrict__ shift_arr, int sign, const double2* __restrict__ z, int64_t nz,
                      double2* __restrict__ g) {
  const int pb = blockIdx.y;
  const int n = m_arr[pb];
  if (n < 1) return;
  const double* a = alpha + (int64_t)pb * ka;
  const double* bt = beta + (int64_t)pb * kb;
  const double norm2 = n2_arr[pb], shift = shift_arr[pb];
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nz; i += (int64_t)gridDim.x * blockDim.x) {
    const double2 zi = z[i];
    const double zr = sign * zi.x + shift, zm = sign * zi.y;
    double tr = zr - a[n - 1], tm = zm;
    for (int l = n - 2; l >= 0; --l) {
      const double bb = bt[l + 1] * bt[l + 1];
      const double inv = bb / (tr * tr + tm * tm);
      tr = zr - a[l] - tr * inv;
      tm = zm + tm * inv;
    }
    const double inv = sign * norm2 / (tr * tr + tm * tm);
    double2 r = make_double2(tr * inv, -tm * inv);
    double2* gi = g + (int64_t)pb * nz + i;
    r.x += gi->x;
    r.y += gi->y;
    *gi = r;
  }
}

}  // namespace ed

using namespace ed;

namespace {

struct BLayout {
  size_t off_tri = 0;
  int nvec, gx, nsw;
  size_t off_vec, off_part, off_psw, off_scal, off_int, total;
};

size_t bt_align(size_t x) { return (x + 255) & ~(size_t)255; }

BLayout blayout(const ed_plan_s* p, int B, int K, int c) {
  BLayout L;
  const int64_t D = p->dim;
  L.nvec = std::max(4, 2 * c + 6);
  // CTAs per problem of the streaming kernels: no more than one resident wave over all B
  // problems. Every CTA ends with one to five block sums in FP64 (the narrow pipe here), so at
  // large B fewer, longer CTAs cut that overhead (forward 97 -> 90 ms at B = 64, D = 63,504).
  // The parameter-term CTAs keep up to 64 per problem: with fewer the reverse sweep got slower.
  const int64_t wave = (int64_t)p->ctx->num_sms * (2048 / BT_NT);  // 256-thread CTAs at full occupancy
  L.gx = (int)std::max<int64_t>(
      1, std::min<int64_t>({(D + 4 * BT_NT - 1) / (4 * BT_NT), (int64_t)64, (wave + B - 1) / B}));
  L.nsw = (int)std::max<int64_t>(1, std::min<int64_t>((D + 4 * SW_NT - 1) / (4 * SW_NT), 64));
  size_t o = 0;
  L.off_vec = o; o = bt_align(o + (size_t)L.nvec * B * D * sizeof(double));
  L.off_part = o; o = bt_align(o + (size_t)5 * B * L.gx * sizeof(double));
  L.off_psw = o; o = bt_align(o + (size_t)B * L.nsw * SW_P * sizeof(double));
  // abar[B][K], bbar[B][K+1], n2 / res [B]
  L.off_scal = o; o = bt_align(o + (size_t)B * (2 * K + 2) * sizeof(double));
  // stop, steps, m [B]; tickets [2][B]
  L.off_int = o; o = bt_align(o + (size_t)5 * B * sizeof(int));
  // per problem: eigenvector and work of the device convergence tests, [B][6 (K + 2)]
  L.off_tri = o; o = bt_align(o + (size_t)B * 6 * (K + 2) * sizeof(double));
  L.total = o;
  return L;
}

ed_status bcheck(const ed_plan_s* p, int B, int K, int c) {
  if (p->kind != 0) return fail(ED_ERR_INVALID_ARG, "the batched tape needs a fermionic plan");
  if (p->dim < 1) return fail(ED_ERR_INVALID_ARG, "empty sector");
  if (B < 1 || B > 65535) return fail(ED_ERR_INVALID_ARG, "batch size must be in [1, 65535]");
  if (K < 1 || K > 4096) return fail(ED_ERR_INVALID_ARG, "max_steps must be in [1, 4096]");
  if (c < 1 || c > 256) return fail(ED_ERR_INVALID_ARG, "checkpoint spacing must be in [1, 256]");
  if (p->n_sites > SW_SITES || (int)p->hop.size() > SW_BONDS)
    return fail(ED_ERR_TOO_LARGE, "batched parameters support up to 16 sites and 32 bonds");
  return ED_OK;
}

BState bstate(const BLayout& L, char* base, int B) {
  int* ib = (int*)(base + L.off_int);
  return BState{ib, ib + B, ib + 2 * B, (unsigned int*)(ib + 3 * B)};
}

// y[b] = H_b x[b] with the gate of bskip
void launch_bmv(const ed_plan_s* p, int B, const double* theta, const double* diag, const double* x, double* y,
                const int* gate, int mode, int k, cudaStream_t s) {
  const int P = 2 * p->n_sites + (int)p->hop.size();
  const int gx = (int)std::min<int64_t>(p->num_up, 1024);
  k_bmv<<<dim3(gx, (B + BMV_PB - 1) / BMV_PB), BT_NT, 0, s>>>(sandwich_args(p), B, P, 2 * p->n_sites,
                                                               (int)p->hop.size(), theta, diag, x, y, gate, mode, k);
}

}  // namespace

extern "C" {

ED_API ed_status ed_batch_diag(ed_plan p, int B, const double* d_theta, double* d_diag, ed_stream_t stream) {
  ED_TRY(check_plan(p));
  ED_TRY(bcheck(p, B, 1, 1));
  if (!d_theta || !d_diag) return fail(ED_ERR_INVALID_ARG, "null argument");
  const int P = 2 * p->n_sites + (int)p->hop.size();
  const int gx = (int)std::max<int64_t>(1, std::min<int64_t>((p->dim + BT_NT - 1) / BT_NT, 256));
  k_bdiag<<<dim3(gx, B), BT_NT, 0, as_stream(stream)>>>(sandwich_args(p), p->n_sites, P, d_theta, d_diag);
  ED_CHECK_LAUNCH("k_bdiag");
  return ED_OK;
}

ED_API ed_status ed_batch_matvec_params(ed_plan p, int B, const double* d_theta, const double* d_diag,
                                        const double* d_x, double* d_y, ed_stream_t stream) {
  ED_TRY(check_plan(p));
  ED_TRY(bcheck(p, B, 1, 1));
  if (!d_theta || !d_diag || !d_x || !d_y) return fail(ED_ERR_INVALID_ARG, "null argument");
  launch_bmv(p, B, d_theta, d_diag, d_x, d_y, nullptr, 0, 0, as_stream(stream));
  ED_CHECK_LAUNCH("k_bmv");
  return ED_OK;
}

ED_API ed_status ed_batch_tape_workspace(ed_plan p, int B, int max_steps, int ckpt, size_t* bytes) {
  ED_TRY(check_plan(p));
  if (!bytes) return fail(ED_ERR_INVALID_ARG, "null argument");
  ED_TRY(bcheck(p, B, max_steps, ckpt));
  *bytes = blayout(p, B, max_steps, ckpt).total;
  return ED_OK;
}

ED_API ed_status ed_batch_lanczos_tape(ed_plan p, int B, const double* d_theta, const double* d_diag,
                                       const double* d_start, int max_steps, int ckpt, double tol, int check_every,
                                       double breakdown, void* d_work, size_t work_bytes, double* d_alpha,
                                       double* d_beta, double* d_ckpt, int* h_steps, ed_stream_t stream) {
  ED_TRY(check_plan(p));
  if (!d_theta || !d_diag || !d_start || !d_alpha || !d_beta || !d_ckpt || !h_steps)
    return fail(ED_ERR_INVALID_ARG, "null argument");
  ED_TRY(bcheck(p, B, max_steps, ckpt));
  const BLayout L = blayout(p, B, max_steps, ckpt);
  if (!d_work || work_bytes < L.total) return fail(ED_ERR_INVALID_ARG, "workspace too small (see ed_batch_tape_workspace)");
  const int64_t D = p->dim;
  const int K = max_steps, c = ckpt;
  cudaStream_t s = as_stream(stream);
  char* base = (char*)d_work;
  double* V = (double*)(base + L.off_vec);
  double* part = (double*)(base + L.off_part);
  double* n2 = (double*)(base + L.off_scal) + (size_t)B * (2 * K + 1);
  const BState bs = bstate(L, base, B);
  ED_CUDA(cudaMemsetAsync(base + L.off_int, 0, (size_t)5 * B * sizeof(int), s));
  ED_CUDA(cudaMemsetAsync(d_alpha, 0, (size_t)B * K * sizeof(double), s));
  ED_CUDA(cudaMemsetAsync(d_beta, 0, (size_t)B * (K + 1) * sizeof(double), s));
  const dim3 gv(L.gx, B);
  auto qv = [&](int k) -> double* { return V + (int64_t)(k % 3) * B * D; };
  double* w = V + (int64_t)3 * B * D;
  k_bt_dot<<<gv, BT_NT, 0, s>>>(d_start, d_start, D, part, bs.ticket, n2, 1, d_beta, K + 1, nullptr, 0, 0);
  ED_CHECK_LAUNCH("k_bt_dot");
  std::vector<double> hn2(B);
  ED_CUDA(cudaMemcpyAsync(hn2.data(), n2, B * sizeof(double), cudaMemcpyDeviceToHost, s));
  ED_CUDA(cudaStreamSynchronize(s));
  std::vector<int> hstop(B, 0), m_conv(B, 0);
  int live = 0;
  for (int b = 0; b < B; ++b) {
    if (!std::isfinite(hn2[b])) return fail(ED_ERR_NONFINITE, "a start vector is not finite");
    if (hn2[b] == 0.0) hstop[b] = 1; else ++live;
  }
  ED_CUDA(cudaMemcpyAsync(bs.stop, hstop.data(), B * sizeof(int), cudaMemcpyHostToDevice, s));
  k_bt_scale<<<gv, BT_NT, 0, s>>>(d_start, qv(0), D, d_beta, K + 1, bs.stop, 1, 0);
  ED_CHECK_LAUNCH("k_bt_scale");
  const int Km = (int)std::min<int64_t>(K, D);
  std::vector<int> hsteps(B, 0);
  // convergence tests of all live problems on a side stream, one block per problem, on the
  // device (ed_lzcheck.cuh); the host never waits for them
  const bool checks = check_every > 0 && tol > 0.0;
  SideChecks chk;
  ED_TRY(chk.init(checks ? Km / check_every + 1 : 0, B));
  double* tvec = (double*)(base + L.off_tri);
  const int ldw = K + 2;
  int k = 0;
  for (; k < Km && live > 0; ++k) {
    if (checks && chk.stopped()) break;
    double* q = qv(k);
    double* qp = k > 0 ? qv(k - 1) : nullptr;
    int nl = 4;
    if (k % c == 0) {
      k_bt_ckpt<<<gv, BT_NT, 0, s>>>(q, qp, d_ckpt + (int64_t)(k / c) * 2 * B * D, D, bs.stop);
      ++nl;
    }
    launch_bmv(p, B, d_theta, d_diag, q, w, bs.stop, 1, k, s);
    k_bt_dot<<<gv, BT_NT, 0, s>>>(q, w, D, part, bs.ticket, d_alpha + k, K, nullptr, 0, bs.stop, 1, k);
    k_bt_update<<<gv, BT_NT, 0, s>>>(w, q, qp, D, d_alpha, d_beta, K, k, breakdown, part, bs);
    k_bt_scale<<<gv, BT_NT, 0, s>>>(w, qv(k + 1), D, d_beta + k + 1, K + 1, bs.stop, 1, k);
    ED_CHECK_LAUNCH_N("ed_batch_lanczos_tape step", nl);
    if (checks && (k + 1) % check_every == 0 && k + 1 < Km) {
      const int kd = k + 1;
      ED_TRY(chk.launch(
          s,
          [&](cudaStream_t s2) {
            k_tri_check_batch<<<B, TRI_NT, 0, s2>>>(d_alpha, d_beta, K, kd, tol, bs.stop, bs.steps, tvec,
                                                     tvec + (size_t)B * ldw, ldw);
          },
          bs.stop));
    }
  }
  ED_TRY(chk.join(s));
  ED_CUDA(cudaMemcpyAsync(hstop.data(), bs.stop, B * sizeof(int), cudaMemcpyDeviceToHost, s));
  ED_CUDA(cudaMemcpyAsync(hsteps.data(), bs.steps, B * sizeof(int), cudaMemcpyDeviceToHost, s));
  ED_CUDA(cudaStreamSynchronize(s));
  for (int b = 0; b < B; ++b) {
    if (hn2[b] == 0.0) h_steps[b] = 0;
    else if (hstop[b]) h_steps[b] = hsteps[b];  // converged or invariant subspace
    else h_steps[b] = k;                         // every launched step ran for it
  }
  return ED_OK;
}

ED_API ed_status ed_batch_tape_combine(ed_plan p, int B, const double* d_theta, const double* d_diag, const int* h_m,
                                       int max_steps, int ckpt, const double* d_alpha, const double* d_beta,
                                       const double* d_ckpt, const double* d_coef, double* d_out,
                                       const double* d_probe, double* d_dots, void* d_work, size_t work_bytes,
                                       ed_stream_t stream) {
  ED_TRY(check_plan(p));
  if (!d_theta || !d_diag || !h_m || !d_alpha || !d_beta || !d_ckpt) return fail(ED_ERR_INVALID_ARG, "null argument");
  if ((d_out != nullptr) != (d_coef != nullptr) || (d_probe != nullptr) != (d_dots != nullptr))
    return fail(ED_ERR_INVALID_ARG, "d_out needs d_coef and d_probe needs d_dots");
  ED_TRY(bcheck(p, B, max_steps, ckpt));
  const BLayout L = blayout(p, B, max_steps, ckpt);
  if (!d_work || work_bytes < L.total) return fail(ED_ERR_INVALID_ARG, "workspace too small (see ed_batch_tape_workspace)");
  const int64_t D = p->dim;
  const int K = max_steps, c = ckpt;
  int mmax = 0;
  for (int b = 0; b < B; ++b) {
    if (h_m[b] < 0 || h_m[b] > K) return fail(ED_ERR_INVALID_ARG, "tape length outside [0, max_steps]");
    mmax = std::max(mmax, h_m[b]);
  }
  cudaStream_t s = as_stream(stream);
  char* base = (char*)d_work;
  double* V = (double*)(base + L.off_vec);
  double* part = (double*)(base + L.off_part);
  const BState bs = bstate(L, base, B);
  ED_CUDA(cudaMemsetAsync(base + L.off_int, 0, (size_t)5 * B * sizeof(int), s));
  ED_CUDA(cudaMemcpyAsync(bs.m, h_m, B * sizeof(int), cudaMemcpyHostToDevice, s));
  if (d_out) ED_CUDA(cudaMemsetAsync(d_out, 0, (size_t)B * D * sizeof(double), s));
  const dim3 gv(L.gx, B);
  double* w = V + (int64_t)3 * B * D;
  for (int s0 = 0; s0 < mmax; s0 += c) {
    const int s1 = std::min(s0 + c, mmax);
    const double* slot = d_ckpt + (int64_t)(s0 / c) * 2 * B * D;
    auto q = [&](int k) -> const double* {
      if (k == s0 - 1) return slot;
      if (k == s0) return slot + (int64_t)B * D;
      return V + (int64_t)((k - s0 - 1) % 3) * B * D;
    };
    k_bt_acc<<<gv, BT_NT, 0, s>>>(q(s0), D, K, s0, d_coef, d_out, d_probe, part, bs, d_dots);
    ED_CHECK_LAUNCH("k_bt_acc");
    for (int k = s0; k + 1 < s1; ++k) {
      launch_bmv(p, B, d_theta, d_diag, q(k), w, bs.m, 2, k + 1, s);
      k_bt_next<<<gv, BT_NT, 0, s>>>(w, q(k), k > 0 ? q(k - 1) : nullptr, D, d_alpha, d_beta, K, k,
                                     (double*)q(k + 1), d_coef, d_out, d_probe, part, bs, d_dots);
      ED_CHECK_LAUNCH_N("ed_batch_tape_combine step", 2);
    }
  }
  return ED_OK;
}

ED_API ed_status ed_batch_tape_reverse(ed_plan p, int B, const double* d_theta, const double* d_diag, const int* h_m,
                                       int max_steps, int ckpt, const double* d_alpha, const double* d_beta,
                                       const double* d_ckpt, const double* d_abar, const double* d_bbar,
                                       const double* d_ext_coef, const double* d_ext_vec, void* d_work,
                                       size_t work_bytes, double* d_theta_bar, double* d_start_bar,
                                       ed_stream_t stream) {
  ED_TRY(check_plan(p));
  if (!d_theta || !d_diag || !h_m || !d_alpha || !d_beta || !d_ckpt || !d_abar || !d_bbar || !d_theta_bar ||
      !d_start_bar)
    return fail(ED_ERR_INVALID_ARG, "null argument");
  if ((d_ext_coef != nullptr) != (d_ext_vec != nullptr))
    return fail(ED_ERR_INVALID_ARG, "d_ext_coef and d_ext_vec go together");
  ED_TRY(bcheck(p, B, max_steps, ckpt));
  const BLayout L = blayout(p, B, max_steps, ckpt);
  if (!d_work || work_bytes < L.total) return fail(ED_ERR_INVALID_ARG, "workspace too small (see ed_batch_tape_workspace)");
  const int64_t D = p->dim;
  const int K = max_steps, c = ckpt;
  int mmax = 0;
  for (int b = 0; b < B; ++b) {
    if (h_m[b] < 0 || h_m[b] > K) return fail(ED_ERR_INVALID_ARG, "tape length outside [0, max_steps]");
    mmax = std::max(mmax, h_m[b]);
  }
  cudaStream_t s = as_stream(stream);
  char* base = (char*)d_work;
  double* V = (double*)(base + L.off_vec);
  double* part = (double*)(base + L.off_part);
  double* psw = (double*)(base + L.off_psw);
  double* AB = (double*)(base + L.off_scal);   // [B][K]
  double* BB = AB + (size_t)B * K;             // [B][K+1]
  double* res = BB + (size_t)B * (K + 1);      // [B]
  const BState bs = bstate(L, base, B);
  const int64_t BD = (int64_t)B * D;
  double* Qs = V;                   // [c][B][D]
  double* Ws = V + (int64_t)c * BD; // [c][B][D]
  double* QB = V + (int64_t)2 * c * BD;
  double* wbar = QB + 3 * BD;
  double* tmp = wbar + BD;
  double* pracc = tmp + BD;  // [B][D]: sum_k w_bar_k q_k
  auto qb = [&](int k) -> double* { return QB + (int64_t)(k % 3) * BD; };
  const int P = 2 * p->n_sites + (int)p->hop.size();
  ED_CUDA(cudaFuncSetAttribute(k_bt_rstep, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sandwich_smem(SW_P)));
  ED_CUDA(cudaFuncSetAttribute(k_bt_diag_terms, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sandwich_smem(SW_P)));
  ED_CUDA(cudaMemsetAsync(base + L.off_int, 0, (size_t)5 * B * sizeof(int), s));
  ED_CUDA(cudaMemcpyAsync(bs.m, h_m, B * sizeof(int), cudaMemcpyHostToDevice, s));
  ED_CUDA(cudaMemsetAsync(psw, 0, (size_t)B * L.nsw * SW_P * sizeof(double), s));
  ED_CUDA(cudaMemcpyAsync(AB, d_abar, (size_t)B * K * sizeof(double), cudaMemcpyDeviceToDevice, s));
  ED_CUDA(cudaMemcpyAsync(BB, d_bbar, (size_t)B * (K + 1) * sizeof(double), cudaMemcpyDeviceToDevice, s));
  // problems with m = 0 have no tape: their q_bar_0 stays zero
  ED_CUDA(cudaMemsetAsync(qb(0), 0, BD * sizeof(double), s));
  const SandwichArgs g = sandwich_args(p);
  const dim3 gv(L.gx, B), gw(L.nsw, B);
  if (mmax > 0) {
    const int last_seg = ((mmax - 1) / c) * c;
    for (int s0 = last_seg; s0 >= 0; s0 -= c) {
      const int s1 = std::min(s0 + c, mmax);
      const double* slot = d_ckpt + (int64_t)(s0 / c) * 2 * BD;
      auto q = [&](int k) -> const double* {
        if (k == s0 - 1) return k >= 0 ? slot : nullptr;
        if (k == s0) return slot + BD;
        if (k == s1) return s1 < mmax ? d_ckpt + (int64_t)(s1 / c) * 2 * BD + BD : nullptr;
        return Qs + (int64_t)(k - s0 - 1) * BD;
      };
      for (int k = s0; k < s1; ++k) {
        launch_bmv(p, B, d_theta, d_diag, q(k), Ws + (int64_t)(k - s0) * BD, bs.m, 2, k, s);
        if (k + 1 < s1)
          k_bt_next<<<gv, BT_NT, 0, s>>>(Ws + (int64_t)(k - s0) * BD, q(k), k > 0 ? q(k - 1) : nullptr, D, d_alpha,
                                         d_beta, K, k, (double*)q(k + 1), nullptr, nullptr, nullptr, part, bs,
                                         nullptr);
        ED_CHECK_LAUNCH_N("ed_batch_tape_reverse replay", k + 1 < s1 ? 2 : 1);
      }
      for (int k = s1 - 1; k >= s0; --k) {
        // q_{k+1} exists for problems with k + 1 < m[b]; the last segment of the longest tape
        // has none (k + 1 = mmax), and the kernels skip every problem there
        const double* q1 = q(k + 1) ? q(k + 1) : q(k);
        k_bt_radot<<<gv, BT_NT, 0, s>>>(qb(k + 1), tmp, d_ext_vec, d_ext_coef, q1, q(k), k > 0 ? q(k - 1) : nullptr,
                                        D, d_beta, AB, BB, K, k, part, bs, nullptr);
        k_bt_rstep<<<gw, SW_NT, sandwich_smem(P), s>>>(g, p->n_sites, P, qb(k + 1), q1, q(k),
                                                      Ws + (int64_t)(k - s0) * BD, qb(k), k > 0 ? qb(k - 1) : nullptr,
                                                      wbar, d_alpha, d_beta, AB, BB, K, k, bs, pracc, psw);
        launch_bmv(p, B, d_theta, d_diag, wbar, tmp, bs.m, 2, k, s);
        ED_CHECK_LAUNCH_N("ed_batch_tape_reverse step", 3);
      }
    }
  }
  // q_bar_0 complete (problems with m >= 1), then the start vectors' adjoints
  const double* q0 = d_ckpt + BD;
  k_bt_radot<<<gv, BT_NT, 0, s>>>(qb(0), tmp, d_ext_vec, d_ext_coef, q0, nullptr, nullptr, D, d_beta, AB, BB, K, -1,
                                  part, bs, res);
  k_bt_startbar<<<gv, BT_NT, 0, s>>>(qb(0), q0, D, d_beta, BB, K, res, bs, d_start_bar);
  k_bt_diag_terms<<<gw, SW_NT, sandwich_smem(P), s>>>(g, p->n_sites, P, pracc, bs, psw);
  k_bt_param_reduce<<<B, SW_P, 0, s>>>(psw, L.nsw, P, d_theta_bar);
  ED_CHECK_LAUNCH_N("ed_batch_tape_reverse final", 4);
  return ED_OK;
}

ED_API ed_status ed_batch_cf(int B, const double* d_alpha, int64_t ka, const double* d_beta, int64_t kb,
                             const int* d_m, const double* d_n2, const double* d_shift, int sign, const double* d_z,
                             int64_t n_z, double* d_g, ed_stream_t stream) {
  if (B < 1 || B > 65535 || n_z < 0) return fail(ED_ERR_INVALID_ARG, "batch size or n_z out of range");
  if (sign != 1 && sign != -1) return fail(ED_ERR_INVALID_ARG, "sign must be +1 or -1");
  if (!d_alpha || !d_beta || !d_m || !d_n2 || !d_shift || !d_z || !d_g) return fail(ED_ERR_INVALID_ARG, "null argument");
  if (n_z == 0) return ED_OK;
  const int gx = (int)std::min<int64_t>((n_z + 127) / 128, 64);
  k_bcf<<<dim3(gx, B), 128, 0, as_stream(stream)>>>(d_alpha, ka, d_beta, kb, d_m, d_n2, d_shift, sign,
                                                   (const double2*)d_z, n_z, (double2*)d_g);
  ED_CHECK_LAUNCH("k_bcf");
  return ED_OK;
}

ED_API ed_status ed_batch_cf_adjoint(int B, const double* d_alpha, int64_t ka, const double* d_beta, int64_t kb,
                                     const int* d_m, int m_max, const double* d_n2, const double* d_shift, int sign,
                                     const double* d_z, int64_t n_z, const double* d_gbar, double* d_abar,
                                     double* d_bbar, double* d_scal, ed_stream_t stream) {
  if (B < 1 || B > 65535) return fail(ED_ERR_INVALID_ARG, "batch size must be in [1, 65535]");
  if (m_max < 1 || m_max > 4096 || m_max > ka || m_max + 1 > kb) return fail(ED_ERR_INVALID_ARG, "m_max out of range");
  if (n_z < 1 || n_z > (int64_t)CFA_NT * 65535) return fail(ED_ERR_INVALID_ARG, "n_z out of range");
  if (sign != 1 && sign != -1) return fail(ED_ERR_INVALID_ARG, "sign must be +1 or -1");
  if (!d_alpha || !d_beta || !d_m || !d_n2 || !d_shift || !d_z || !d_gbar || !d_abar || !d_bbar || !d_scal)
    return fail(ED_ERR_INVALID_ARG, "null argument");
  CfaBatch cb{d_alpha, ka, d_beta, kb, d_m, d_n2, d_shift, 0, 0.0, 0.0, sign, d_gbar, d_abar, d_bbar, d_scal};
  return cf_adjoint_launch(cb, B, m_max, (const double2*)d_z, n_z, as_stream(stream));
}

}  // extern "C"

