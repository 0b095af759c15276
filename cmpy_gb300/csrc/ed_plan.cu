// Plan creation (sector basis + per-spin hopping tables), the FP64 matrix-free matvec,
// dense and diagonal builders. Replaces AbstractManyBodyModel.hamilton_operator
// (cmpy/models/abc.py:242-256), HamiltonOperator._matvec/toarray/_trace
// (cmpy/operators.py:614-646) and AbstractSpinModel.hamilton_operator (abc.py:186-203).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "ed_plan.cuh"

namespace ed {

// ---------------------------------------------------------------------------------------
// table construction
// ---------------------------------------------------------------------------------------

struct BondList {
  int n;
  int width;
  int s1[128];
  int s2[128];
  double hop[128];
};

__global__ void k_state_energy(const uint64_t* __restrict__ states, int64_t n, FermionParams fp,
                               const double* __restrict__ eps, double* __restrict__ out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = weighted_element(states[i], eps, fp.n_sites);
}

__global__ void k_hop_count(const uint64_t* __restrict__ states, int64_t n, BondList bl, int32_t* __restrict__ cnt) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t s = states[i];
    int c = 0;
    for (int b = 0; b < bl.n; ++b) c += (int)(((s >> bl.s1[b]) ^ (s >> bl.s2[b])) & 1ull);
    cnt[i] = c;
  }
}

__global__ void k_hop_fill(const uint64_t* __restrict__ tab, const uint64_t* __restrict__ states, int64_t n,
                           BondList bl, const int32_t* __restrict__ off, int32_t* __restrict__ idx,
                           double* __restrict__ coef, int16_t* __restrict__ bond) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t s = states[i];
    int64_t o = off[i];
    for (int b = 0; b < bl.n; ++b) {
      if (((s >> bl.s1[b]) ^ (s >> bl.s2[b])) & 1ull) {
        const uint64_t t = s ^ (1ull << bl.s1[b]) ^ (1ull << bl.s2[b]);
        idx[o] = (int32_t)colex_rank(tab, t);
        const int sg = hop_sign(s, bl.width, bl.s1[b], bl.s2[b]);
        coef[o] = sg < 0 ? -bl.hop[b] : bl.hop[b];
        bond[o] = (int16_t)b;
        ++o;
      }
    }
  }
}

// Heisenberg tables (cmpy/models/heisenberg.py:19-40 with per-pair couplings).
struct PairList {
  int n;
  int p1[256];
  int p2[256];
  double j[256];
  double jz[256];
};
#define ED_MAX_PAIRS 256

__global__ void k_spin_count(const uint64_t* __restrict__ states, int64_t n, PairList pl, int32_t* __restrict__ cnt,
                             double* __restrict__ diag) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t s = states[i];
    double dg = 0.0;
    // count distinct flip targets (the two directions of a bond give the same target)
    uint64_t targets[64];
    int nt = 0;
    for (int p = 0; p < pl.n; ++p) {
      const int b1 = (int)((s >> pl.p1[p]) & 1ull), b2 = (int)((s >> pl.p2[p]) & 1ull);
      const double sign = (b1 == b2) ? 1.0 : -1.0;
      dg = __dadd_rn(dg, __dmul_rn(__dmul_rn(sign, 0.25), pl.jz[p]));
      if (b1 != b2) {
        const uint64_t t = s ^ (1ull << pl.p1[p]) ^ (1ull << pl.p2[p]);
        bool dup = false;
        for (int q = 0; q < nt; ++q) dup |= (targets[q] == t);
        if (!dup && nt < 64) targets[nt++] = t;
      }
    }
    cnt[i] = nt;
    diag[i] = dg;
  }
}

// full = 1: the sector is all 2^N states and a state's index is its value
__global__ void k_spin_fill(const uint64_t* __restrict__ tab, const uint64_t* __restrict__ states, int64_t n,
                            PairList pl, const int32_t* __restrict__ off, int32_t* __restrict__ idx,
                            double* __restrict__ coef, int full) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t s = states[i];
    const int64_t o0 = off[i];
    int nt = 0;
    uint64_t targets[64];
    for (int p = 0; p < pl.n; ++p) {
      const int b1 = (int)((s >> pl.p1[p]) & 1ull), b2 = (int)((s >> pl.p2[p]) & 1ull);
      if (b1 != b2) {
        const uint64_t t = s ^ (1ull << pl.p1[p]) ^ (1ull << pl.p2[p]);
        const double v = __dmul_rn(0.25, pl.j[p]) / 2.0;
        int q = 0;
        for (; q < nt; ++q) if (targets[q] == t) break;
        if (q < nt) {
          coef[o0 + q] = __dadd_rn(coef[o0 + q], v);
        } else if (nt < 64) {
          targets[nt] = t;
          idx[o0 + nt] = full ? (int32_t)t : (int32_t)colex_rank(tab, t);
          coef[o0 + nt] = v;
          ++nt;
        }
      }
    }
  }
}

__global__ void k_row_abs_max(const int32_t* __restrict__ off, const double* __restrict__ coef, int64_t n,
                              unsigned long long* __restrict__ out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int32_t k = off[i]; k < off[i + 1]; ++k) s += fabs(coef[k]);
    atomicMax(out, (unsigned long long)__double_as_longlong(s));
  }
}

static void free_table(SpinTable& t) {
  cudaFree(t.states); cudaFree(t.energy); cudaFree(t.off); cudaFree(t.idx); cudaFree(t.coef); cudaFree(t.bond);
  t = SpinTable();
}

static ed_status build_fermion_table(ed_plan_s* p, SpinTable& t, int n, cudaStream_t s) {
  t.n = ed_sector_size(p->n_sites, n);
  ED_CUDA(cudaMalloc(&t.states, std::max<int64_t>(t.n, 1) * sizeof(uint64_t)));
  ED_CUDA(cudaMalloc(&t.energy, std::max<int64_t>(t.n, 1) * sizeof(double)));
  ED_CUDA(cudaMalloc(&t.off, (t.n + 1) * sizeof(int32_t)));
  ED_TRY(enumerate_into(p->n_sites, n, t.states, s));
  double* d_eps = nullptr;
  ED_CUDA(cudaMallocAsync(&d_eps, (p->n_sites + 1) * sizeof(double), s));
  if (p->n_sites > 0)
    ED_CUDA(cudaMemcpyAsync(d_eps, p->eps.data(), p->n_sites * sizeof(double), cudaMemcpyHostToDevice, s));
  const int g = grid_for(t.n, 256, p->ctx->num_sms * 8);
  k_state_energy<<<g, 256, 0, s>>>(t.states, t.n, p->fp, d_eps, t.energy);
  ED_CHECK_LAUNCH("k_state_energy");
  ED_CUDA(cudaFreeAsync(d_eps, s));

  BondList bl;
  bl.n = (int)p->hop.size();
  bl.width = p->sign_width;
  for (int b = 0; b < bl.n; ++b) { bl.s1[b] = p->b1[b]; bl.s2[b] = p->b2[b]; bl.hop[b] = p->hop[b]; }
  int32_t* d_cnt = nullptr;
  ED_CUDA(cudaMallocAsync(&d_cnt, std::max<int64_t>(t.n, 1) * sizeof(int32_t), s));
  k_hop_count<<<g, 256, 0, s>>>(t.states, t.n, bl, d_cnt);
  ED_CHECK_LAUNCH("k_hop_count");
  std::vector<int32_t> cnt(t.n), off(t.n + 1, 0);
  if (t.n) ED_CUDA(cudaMemcpyAsync(cnt.data(), d_cnt, t.n * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
  ED_CUDA(cudaStreamSynchronize(s));
  ED_CUDA(cudaFreeAsync(d_cnt, s));
  int64_t acc = 0;
  for (int64_t i = 0; i < t.n; ++i) {
    off[i] = (int32_t)acc;
    acc += cnt[i];
    t.max_row = std::max(t.max_row, cnt[i]);
  }
  if (acc > INT32_MAX) return fail(ED_ERR_TOO_LARGE, "hopping table exceeds 2^31 entries");
  off[t.n] = (int32_t)acc;
  t.nnz = acc;
  ED_CUDA(cudaMemcpyAsync(t.off, off.data(), (t.n + 1) * sizeof(int32_t), cudaMemcpyHostToDevice, s));
  ED_CUDA(cudaMalloc(&t.idx, std::max<int64_t>(acc, 1) * sizeof(int32_t)));
  ED_CUDA(cudaMalloc(&t.coef, std::max<int64_t>(acc, 1) * sizeof(double)));
  ED_CUDA(cudaMalloc(&t.bond, std::max<int64_t>(acc, 1) * sizeof(int16_t)));
  k_hop_fill<<<g, 256, 0, s>>>(p->ctx->d_binom, t.states, t.n, bl, t.off, t.idx, t.coef, t.bond);
  ED_CHECK_LAUNCH("k_hop_fill");
  ED_CUDA(cudaStreamSynchronize(s));  // host `off` must outlive the copy
  return ED_OK;
}

static ed_status finish_bounds(ed_plan_s* p, cudaStream_t s) {
  // ||H||_inf bound from table row sums and the diagonal
  unsigned long long* d_m = nullptr;
  ED_CUDA(cudaMallocAsync(&d_m, 2 * sizeof(unsigned long long), s));
  ED_CUDA(cudaMemsetAsync(d_m, 0, 2 * sizeof(unsigned long long), s));
  uint64_t nl = 0;
  if (p->up.n) { k_row_abs_max<<<grid_for(p->up.n, 256, 1024), 256, 0, s>>>(p->up.off, p->up.coef, p->up.n, d_m); ++nl; }
  if (p->kind == 0 && p->dn.n) { k_row_abs_max<<<grid_for(p->dn.n, 256, 1024), 256, 0, s>>>(p->dn.off, p->dn.coef, p->dn.n, d_m + 1); ++nl; }
  ED_CHECK_LAUNCH_N("k_row_abs_max", nl);
  unsigned long long hm[2];
  ED_CUDA(cudaMemcpyAsync(hm, d_m, sizeof(hm), cudaMemcpyDeviceToHost, s));
  double diag_max = 0.0;
  if (p->kind == 0) {
    std::vector<double> eu(p->up.n), edn(p->dn.n);
    if (p->up.n) ED_CUDA(cudaMemcpyAsync(eu.data(), p->up.energy, p->up.n * sizeof(double), cudaMemcpyDeviceToHost, s));
    if (p->dn.n) ED_CUDA(cudaMemcpyAsync(edn.data(), p->dn.energy, p->dn.n * sizeof(double), cudaMemcpyDeviceToHost, s));
    ED_CUDA(cudaStreamSynchronize(s));
    double mu_ = 0, md = 0, su = 0;
    for (double v : eu) mu_ = std::max(mu_, std::fabs(v));
    for (double v : edn) md = std::max(md, std::fabs(v));
    for (double v : p->u) su += std::fabs(v);
    diag_max = mu_ + md + su;
  } else {
    std::vector<double> dg(p->dim);
    if (p->dim) ED_CUDA(cudaMemcpyAsync(dg.data(), p->spin_diag, p->dim * sizeof(double), cudaMemcpyDeviceToHost, s));
    ED_CUDA(cudaStreamSynchronize(s));
    for (double v : dg) diag_max = std::max(diag_max, std::fabs(v));
  }
  ED_CUDA(cudaFreeAsync(d_m, s));
  double h0, h1;
  memcpy(&h0, &hm[0], 8);
  memcpy(&h1, &hm[1], 8);
  p->hnorm_bound = diag_max + h0 + h1;
  ED_CUDA(cudaStreamSynchronize(s));
  return ED_OK;
}

ed_status check_plan(const ed_plan_s* p) {
  if (!p) return fail(ED_ERR_INVALID_ARG, "null plan");
  int dev = -1;
  ED_CUDA(cudaGetDevice(&dev));
  if (dev != p->device) return fail(ED_ERR_INVALID_ARG, "plan belongs to another device");
  return ED_OK;
}

// ---------------------------------------------------------------------------------------
// matvec, FP64: one CTA per target up-row, threads over the dn index.
//   y[u,d] = (E_up[u] + E_dn[d] + U(up_u & dn_d)) x[u,d]
//          + sum_{(u',c) in up-table[u]} c x[u',d] + sum_{(d',c) in dn-table[d]} c x[u,d']
// ---------------------------------------------------------------------------------------

struct HubArgs {
  const uint64_t* up_states; const double* e_up; const int32_t* up_off; const int32_t* up_idx; const double* up_coef;
  const uint64_t* dn_states; const double* e_dn; const int32_t* dn_off; const int32_t* dn_idx; const double* dn_coef;
  int64_t nu, nd;
};

__device__ __forceinline__ double u_term(const FermionParams& fp, uint64_t both) {
  if (fp.u_uniform) return fp.u0 * (double)__popcll(both);
  double v = 0.0;
  while (both) {
    const int i = __ffsll((long long)both) - 1;
    v += fp.u[i];
    both &= both - 1;
  }
  return v;
}

template <int NT>
__global__ void __launch_bounds__(NT) k_hub_matvec_f64(HubArgs a, FermionParams fp, const double* __restrict__ x,
                                                       double* __restrict__ y, int64_t nvec, int64_t ld,
                                                       const int* __restrict__ stop) {
  if (stop && *(volatile const int*)stop) return;
  const int64_t rows = a.nu * nvec;
  for (int64_t rv = blockIdx.x; rv < rows; rv += gridDim.x) {
    const int64_t v = rv / a.nu, u = rv - v * a.nu;
    const double* xv = x + v * ld;
    double* yv = y + v * ld;
    const uint64_t su = a.up_states[u];
    const double eu = a.e_up[u];
    const int32_t b0 = a.up_off[u], b1 = a.up_off[u + 1];
    const double* xrow = xv + u * a.nd;
    for (int64_t d = threadIdx.x; d < a.nd; d += NT) {
      const double diag = eu + a.e_dn[d] + u_term(fp, su & a.dn_states[d]);
      double acc = diag * xrow[d];
      for (int32_t k = b0; k < b1; ++k) acc = fma(__ldg(a.up_coef + k), xv[(int64_t)__ldg(a.up_idx + k) * a.nd + d], acc);
      const int32_t c0 = __ldg(a.dn_off + d), c1 = __ldg(a.dn_off + d + 1);
      for (int32_t k = c0; k < c1; ++k) acc = fma(__ldg(a.dn_coef + k), xrow[__ldg(a.dn_idx + k)], acc);
      yv[u * a.nd + d] = acc;
    }
  }
}

struct SpinArgs {
  const double* diag; const int32_t* off; const int32_t* idx; const double* coef; int64_t n;
};

__global__ void k_spin_matvec_f64(SpinArgs a, const double* __restrict__ x, double* __restrict__ y, int64_t nvec, int64_t ld,
                                  const int* __restrict__ stop) {
  if (stop && *(volatile const int*)stop) return;
  const int64_t tot = a.n * nvec;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < tot; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t v = t / a.n, i = t - v * a.n;
    const double* xv = x + v * ld;
    double acc = a.diag[i] * xv[i];
    for (int32_t k = a.off[i]; k < a.off[i + 1]; ++k) acc = fma(a.coef[k], xv[a.idx[k]], acc);
    y[v * ld + i] = acc;
  }
}

static HubArgs hub_args(const ed_plan_s* p) {
  HubArgs a;
  a.up_states = p->up.states; a.e_up = p->up.energy; a.up_off = p->up.off; a.up_idx = p->up.idx; a.up_coef = p->up.coef;
  a.dn_states = p->dn.states; a.e_dn = p->dn.energy; a.dn_off = p->dn.off; a.dn_idx = p->dn.idx; a.dn_coef = p->dn.coef;
  a.nu = p->num_up; a.nd = p->num_dn;
  return a;
}

ed_status matvec_f64(const ed_plan_s* p, const double* x, double* y, int64_t nvec, int64_t ld, cudaStream_t s,
                     const int* stop) {
  if (p->dim == 0 || nvec == 0) return ED_OK;
  if (p->kind == 0) {
    const int64_t rows = p->num_up * nvec;
    const int g = (int)std::min<int64_t>(rows, (int64_t)p->ctx->num_sms * 16);
    k_hub_matvec_f64<256><<<g, 256, 0, s>>>(hub_args(p), p->fp, x, y, nvec, ld, stop);
    ED_CHECK_LAUNCH("k_hub_matvec_f64");
  } else {
    SpinArgs a{p->spin_diag, p->up.off, p->up.idx, p->up.coef, p->dim};
    k_spin_matvec_f64<<<grid_for(p->dim * nvec, 256, p->ctx->num_sms * 16), 256, 0, s>>>(a, x, y, nvec, ld, stop);
    ED_CHECK_LAUNCH("k_spin_matvec_f64");
  }
  return ED_OK;
}

// ---------------------------------------------------------------------------------------
// dense / diagonal
// ---------------------------------------------------------------------------------------

// Diagonal in the reference's triplet order: onsite-up, onsite-dn, interaction, each added
// only when nonzero (cmpy/operators.py:305-422 skip exact zeros), starting from 0.0.
__device__ __forceinline__ double hub_diag_ref(const HubArgs& a, const FermionParams& fp, int64_t u, int64_t d) {
  double v = 0.0;
  const double eu = a.e_up[u], ed_ = a.e_dn[d];
  if (eu != 0.0 || isnan(eu)) v = __dadd_rn(v, eu);
  if (ed_ != 0.0 || isnan(ed_)) v = __dadd_rn(v, ed_);
  double ei = 0.0;
  uint64_t both = a.up_states[u] & a.dn_states[d];
  for (int i = 0; i < fp.n_sites; ++i)
    if (both & (1ull << i)) ei = __dadd_rn(ei, fp.u[i]);
  if (ei != 0.0 || isnan(ei)) v = __dadd_rn(v, ei);
  return v;
}

__global__ void k_hub_dense(HubArgs a, FermionParams fp, double* __restrict__ out, int64_t D) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < D; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t u = i / a.nd, d = i - u * a.nd;
    double* row = out + i * D;
    row[i] = hub_diag_ref(a, fp, u, d);
    for (int32_t k = a.up_off[u]; k < a.up_off[u + 1]; ++k) {
      const int64_t j = (int64_t)a.up_idx[k] * a.nd + d;
      row[j] = __dadd_rn(row[j], a.up_coef[k]);
    }
    for (int32_t k = a.dn_off[d]; k < a.dn_off[d + 1]; ++k) {
      const int64_t j = u * a.nd + a.dn_idx[k];
      row[j] = __dadd_rn(row[j], a.dn_coef[k]);
    }
  }
}

__global__ void k_hub_diag(HubArgs a, FermionParams fp, double* __restrict__ out, int64_t D) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < D; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t u = i / a.nd, d = i - u * a.nd;
    out[i] = hub_diag_ref(a, fp, u, d);
  }
}

__global__ void k_spin_dense(SpinArgs a, double* __restrict__ out, int64_t D) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < D; i += (int64_t)gridDim.x * blockDim.x) {
    double* row = out + i * D;
    row[i] = a.diag[i];
    for (int32_t k = a.off[i]; k < a.off[i + 1]; ++k) row[a.idx[k]] = __dadd_rn(row[a.idx[k]], a.coef[k]);
  }
}

}  // namespace ed

using namespace ed;

static ed_status validate_fermion(const ed_fermion_model* m, int n_up, int n_dn) {
  if (!m) return fail(ED_ERR_INVALID_ARG, "null model");
  if (m->n_sites < 0 || m->n_sites > 30) return fail(ED_ERR_INVALID_ARG, "n_sites must be in [0, 30] for a fermionic plan");
  if (n_up < 0 || n_up > m->n_sites || n_dn < 0 || n_dn > m->n_sites) return fail(ED_ERR_INVALID_ARG, "filling outside [0, n_sites]");
  if (m->n_bonds < 0 || m->n_bonds > ED_MAX_BONDS) return fail(ED_ERR_INVALID_ARG, "n_bonds must be in [0, 128]");
  if (m->n_sites > 0 && (!m->h_eps || !m->h_u)) return fail(ED_ERR_INVALID_ARG, "null eps/u");
  for (int i = 0; i < m->n_sites; ++i)
    if (!std::isfinite(m->h_eps[i]) || !std::isfinite(m->h_u[i])) return fail(ED_ERR_NONFINITE, "non-finite eps/u");
  for (int b = 0; b < m->n_bonds; ++b) {
    const int i = m->h_bond_site1[b], j = m->h_bond_site2[b];
    if (!(0 <= i && i < j && j < m->n_sites)) return fail(ED_ERR_INVALID_ARG, "bond sites must satisfy 0 <= site1 < site2 < n_sites");
    if (!std::isfinite(m->h_bond_hop[b])) return fail(ED_ERR_NONFINITE, "non-finite hopping");
  }
  return ED_OK;
}

extern "C" {

ED_API ed_status ed_plan_create_fermion(const ed_fermion_model* m, int n_up, int n_dn, ed_plan* out, ed_stream_t stream) {
  if (!out) return fail(ED_ERR_INVALID_ARG, "null output plan");
  *out = nullptr;
  ED_TRY(validate_fermion(m, n_up, n_dn));
  const int64_t nu = ed_sector_size(m->n_sites, n_up), nd = ed_sector_size(m->n_sites, n_dn);
  if (nu > INT32_MAX || nd > INT32_MAX) return fail(ED_ERR_TOO_LARGE, "spin sector too large");
  cudaStream_t s = as_stream(stream);
  ed_plan_s* p = new ed_plan_s();
  p->kind = 0;
  ED_CUDA(cudaGetDevice(&p->device));
  ed_status st = device_context(&p->ctx);
  if (st != ED_OK) { delete p; return st; }
  p->n_sites = m->n_sites; p->n_up = n_up; p->n_dn = n_dn;
  p->num_up = nu; p->num_dn = nd; p->dim = nu * nd;
  p->eps.assign(m->h_eps, m->h_eps + m->n_sites);
  p->u.assign(m->h_u, m->h_u + m->n_sites);
  for (int b = 0; b < m->n_bonds; ++b) {
    p->b1.push_back(m->h_bond_site1[b]); p->b2.push_back(m->h_bond_site2[b]); p->hop.push_back(m->h_bond_hop[b]);
  }
  p->sign_width = m->sign_width;
  p->fp.n_sites = m->n_sites;
  p->fp.u_uniform = 1;
  p->fp.u0 = m->n_sites ? m->h_u[0] : 0.0;
  for (int i = 0; i < ED_MAX_SITES + 2; ++i) p->fp.u[i] = 0.0;
  for (int i = 0; i < m->n_sites; ++i) {
    p->fp.u[i] = m->h_u[i];
    if (m->h_u[i] != p->fp.u0) p->fp.u_uniform = 0;
  }
  st = build_fermion_table(p, p->up, n_up, s);
  if (st == ED_OK) st = build_fermion_table(p, p->dn, n_dn, s);
  if (st == ED_OK) st = finish_bounds(p, s);
  if (st == ED_OK) st = build_bfp(p, s);
  if (st != ED_OK) { ed_plan_destroy(p); return st; }
  *out = p;
  return ED_OK;
}

ED_API ed_status ed_plan_create_spin(const ed_spin_model* m, int n_up, ed_plan* out, ed_stream_t stream) {
  if (!out) return fail(ED_ERR_INVALID_ARG, "null output plan");
  *out = nullptr;
  if (!m) return fail(ED_ERR_INVALID_ARG, "null model");
  if (m->n_sites < 0 || m->n_sites > ED_MAX_SITES) return fail(ED_ERR_INVALID_ARG, "n_sites out of range");
  if (n_up < -1 || n_up > m->n_sites) return fail(ED_ERR_INVALID_ARG, "n_up outside [-1, n_sites]");
  if (n_up < 0 && m->n_sites > 30) return fail(ED_ERR_TOO_LARGE, "full spin space limited to 30 sites");
  if (m->n_pairs < 0 || m->n_pairs > ED_MAX_PAIRS) return fail(ED_ERR_INVALID_ARG, "n_pairs must be in [0, 256]");
  for (int q = 0; q < m->n_pairs; ++q) {
    const int a = m->h_pos1[q], b = m->h_pos2[q];
    if (a < 0 || b < 0 || a >= m->n_sites || b >= m->n_sites || a == b) return fail(ED_ERR_INVALID_ARG, "pair sites out of range");
    if (!std::isfinite(m->h_j[q]) || !std::isfinite(m->h_jz[q])) return fail(ED_ERR_NONFINITE, "non-finite coupling");
  }
  const int64_t D = ed_sector_size(m->n_sites, n_up);
  if (D > INT32_MAX) return fail(ED_ERR_TOO_LARGE, "spin sector too large");
  cudaStream_t s = as_stream(stream);
  ed_plan_s* p = new ed_plan_s();
  p->kind = 1;
  ED_CUDA(cudaGetDevice(&p->device));
  ed_status st = device_context(&p->ctx);
  if (st != ED_OK) { delete p; return st; }
  p->n_sites = m->n_sites; p->n_up = n_up; p->n_dn = 0;
  p->num_up = D; p->num_dn = 1; p->dim = D;
  p->p1.assign(m->h_pos1, m->h_pos1 + m->n_pairs); p->p2.assign(m->h_pos2, m->h_pos2 + m->n_pairs);
  p->pj.assign(m->h_j, m->h_j + m->n_pairs); p->pjz.assign(m->h_jz, m->h_jz + m->n_pairs);
  PairList pl;
  pl.n = m->n_pairs;
  for (int q = 0; q < pl.n; ++q) { pl.p1[q] = m->h_pos1[q]; pl.p2[q] = m->h_pos2[q]; pl.j[q] = m->h_j[q]; pl.jz[q] = m->h_jz[q]; }
  SpinTable& t = p->up;
  t.n = D;
  auto run = [&]() -> ed_status {
    ED_CUDA(cudaMalloc(&t.states, std::max<int64_t>(D, 1) * sizeof(uint64_t)));
    ED_CUDA(cudaMalloc(&t.off, (D + 1) * sizeof(int32_t)));
    ED_CUDA(cudaMalloc(&p->spin_diag, std::max<int64_t>(D, 1) * sizeof(double)));
    ED_TRY(enumerate_into(m->n_sites, n_up, t.states, s));
    int32_t* d_cnt = nullptr;
    ED_CUDA(cudaMallocAsync(&d_cnt, std::max<int64_t>(D, 1) * sizeof(int32_t), s));
    const int g = grid_for(D, 128, p->ctx->num_sms * 8);
    k_spin_count<<<g, 128, 0, s>>>(t.states, D, pl, d_cnt, p->spin_diag);
    ED_CHECK_LAUNCH("k_spin_count");
    std::vector<int32_t> cnt(D), off(D + 1, 0);
    if (D) ED_CUDA(cudaMemcpyAsync(cnt.data(), d_cnt, D * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    ED_CUDA(cudaStreamSynchronize(s));
    ED_CUDA(cudaFreeAsync(d_cnt, s));
    int64_t acc = 0;
    for (int64_t i = 0; i < D; ++i) { off[i] = (int32_t)acc; acc += cnt[i]; t.max_row = std::max(t.max_row, cnt[i]); }
    if (acc > INT32_MAX) return fail(ED_ERR_TOO_LARGE, "spin table too large");
    off[D] = (int32_t)acc;
    t.nnz = acc;
    ED_CUDA(cudaMemcpyAsync(t.off, off.data(), (D + 1) * sizeof(int32_t), cudaMemcpyHostToDevice, s));
    ED_CUDA(cudaMalloc(&t.idx, std::max<int64_t>(acc, 1) * sizeof(int32_t)));
    ED_CUDA(cudaMalloc(&t.coef, std::max<int64_t>(acc, 1) * sizeof(double)));
    k_spin_fill<<<g, 128, 0, s>>>(p->ctx->d_binom, t.states, D, pl, t.off, t.idx, t.coef, n_up < 0 ? 1 : 0);
    ED_CHECK_LAUNCH("k_spin_fill");
    ED_CUDA(cudaStreamSynchronize(s));
    return finish_bounds(p, s);
  };
  st = run();
  if (st != ED_OK) { ed_plan_destroy(p); return st; }
  // triplets the reference emits: per state n_pairs diagonals plus one per differing pair
  *out = p;
  return ED_OK;
}

ED_API ed_status ed_plan_destroy(ed_plan p) {
  if (!p) return ED_OK;
  int prev = -1;
  cudaGetDevice(&prev);
  if (p->device >= 0 && prev != p->device) cudaSetDevice(p->device);
  free_table(p->up);
  free_table(p->dn);
  free_bfp(p);
  cudaFree(p->spin_diag);
  if (prev >= 0 && prev != p->device) cudaSetDevice(prev);
  delete p;
  return ED_OK;
}

ED_API ed_status ed_plan_get_info(ed_plan p, ed_plan_info* out) {
  if (!p || !out) return fail(ED_ERR_INVALID_ARG, "null argument");
  out->dim = p->dim; out->num_up = p->num_up; out->num_dn = p->num_dn;
  out->hop_up = p->up.nnz; out->hop_dn = p->dn.nnz;
  out->n_sites = p->n_sites; out->kind = p->kind; out->n_up = p->n_up; out->n_dn = p->n_dn;
  out->hnorm_bound = p->hnorm_bound;
  out->nnz = p->nnz;
  return ED_OK;
}

ED_API ed_status ed_plan_states(ed_plan p, const uint64_t** d_up, const uint64_t** d_dn) {
  if (!p) return fail(ED_ERR_INVALID_ARG, "null plan");
  if (d_up) *d_up = p->up.states;
  if (d_dn) *d_dn = p->kind == 0 ? p->dn.states : nullptr;
  return ED_OK;
}

ED_API ed_status ed_matvec(ed_plan p, const double* x, double* y, ed_stream_t stream) {
  ED_TRY(check_plan(p));
  if (p->dim && (!x || !y)) return fail(ED_ERR_INVALID_ARG, "null vector");
  if (x == y && p->dim) return fail(ED_ERR_INVALID_ARG, "x and y must not alias");
  return matvec_f64(p, x, y, 1, p->dim, as_stream(stream));
}

ED_API ed_status ed_matmat(ed_plan p, const double* x, double* y, int64_t nvec, int64_t ld, ed_stream_t stream) {
  ED_TRY(check_plan(p));
  if (nvec < 0 || ld < p->dim) return fail(ED_ERR_INVALID_ARG, "bad n_vec/ld");
  if (p->dim && nvec && (!x || !y)) return fail(ED_ERR_INVALID_ARG, "null vector");
  return matvec_f64(p, x, y, nvec, ld, as_stream(stream));
}

ED_API ed_status ed_dense(ed_plan p, double* out, ed_stream_t stream) {
  ED_TRY(check_plan(p));
  if (p->dim > 32768) return fail(ED_ERR_TOO_LARGE, "ed_dense: dimension above 32768");
  if (p->dim == 0) return ED_OK;
  if (!out) return fail(ED_ERR_INVALID_ARG, "null output");
  cudaStream_t s = as_stream(stream);
  ED_CUDA(cudaMemsetAsync(out, 0, (size_t)p->dim * p->dim * sizeof(double), s));
  if (p->kind == 0) {
    k_hub_dense<<<grid_for(p->dim, 128, 4096), 128, 0, s>>>(hub_args(p), p->fp, out, p->dim);
  } else {
    SpinArgs a{p->spin_diag, p->up.off, p->up.idx, p->up.coef, p->dim};
    k_spin_dense<<<grid_for(p->dim, 128, 4096), 128, 0, s>>>(a, out, p->dim);
  }
  ED_CHECK_LAUNCH("ed_dense");
  return ED_OK;
}

ED_API ed_status ed_diagonal(ed_plan p, double* out, ed_stream_t stream) {
  ED_TRY(check_plan(p));
  if (p->dim == 0) return ED_OK;
  if (!out) return fail(ED_ERR_INVALID_ARG, "null output");
  cudaStream_t s = as_stream(stream);
  if (p->kind == 0) {
    k_hub_diag<<<grid_for(p->dim, 256, 4096), 256, 0, s>>>(hub_args(p), p->fp, out, p->dim);
    ED_CHECK_LAUNCH("k_hub_diag");
  } else {
    ED_CUDA(cudaMemcpyAsync(out, p->spin_diag, p->dim * sizeof(double), cudaMemcpyDeviceToDevice, s));
  }
  return ED_OK;
}

}  // extern "C"
