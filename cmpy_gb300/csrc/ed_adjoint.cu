// Parameter derivatives of a fermionic Hamiltonian for the adjoint (reverse-mode) Green's
// function: out[theta] (+)= a^T (dH/dtheta) b for every model parameter theta at once,
//   theta = eps_j (dH = n_j_up + n_j_dn), U_j (dH = n_j_up n_j_dn), t_b (dH = hop of bond b
//   with its fermionic sign, i.e. the bond's matrix elements divided by t_b).
// No reference counterpart (the reference has no derivatives); the parameter meaning follows
// HubbardModel / SIAM (cmpy/models/hubbard.py:13-22, cmpy/models/anderson.py:147-158).
// Output layout: [eps_0..eps_{N-1}, U_0..U_{N-1}, t_0..t_{nb-1}], N <= 16, nb <= 32.
#include <algorithm>

#include "ed_plan.cuh"

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

__global__ void __launch_bounds__(SW_NT) k_sandwich(SandwichArgs g, const double* __restrict__ a,
                                                    const double* __restrict__ b, double* __restrict__ partial) {
  __shared__ double sm[SW_NT / 32];
  double eps[SW_SITES], uu[SW_SITES], hop[SW_BONDS];
#pragma unroll
  for (int j = 0; j < SW_SITES; ++j) { eps[j] = 0.0; uu[j] = 0.0; }
#pragma unroll
  for (int j = 0; j < SW_BONDS; ++j) hop[j] = 0.0;
  const int64_t D = g.nu * g.nd;
  for (int64_t i = blockIdx.x * (int64_t)SW_NT + threadIdx.x; i < D; i += (int64_t)gridDim.x * SW_NT) {
    const int64_t u = i / g.nd, d = i - u * g.nd;
    const double ai = a[i];
    const double ab = ai * b[i];
    const uint64_t su = g.up_states[u], sd = g.dn_states[d], both = su & sd;
#pragma unroll
    for (int j = 0; j < SW_SITES; ++j) {
      eps[j] = fma(ab, (double)(((su >> j) & 1ull) + ((sd >> j) & 1ull)), eps[j]);
      if ((both >> j) & 1ull) uu[j] += ab;
    }
    for (int32_t e = g.up_off[u]; e < g.up_off[u + 1]; ++e) {
      const double v = ai * copysign(1.0, g.up_coef[e]) * b[(int64_t)g.up_idx[e] * g.nd + d];
      const int bb = g.up_bond[e];
#pragma unroll
      for (int q = 0; q < SW_BONDS; ++q)
        if (q == bb) hop[q] += v;
    }
    for (int32_t e = g.dn_off[d]; e < g.dn_off[d + 1]; ++e) {
      const double v = ai * copysign(1.0, g.dn_coef[e]) * b[u * g.nd + g.dn_idx[e]];
      const int bb = g.dn_bond[e];
#pragma unroll
      for (int q = 0; q < SW_BONDS; ++q)
        if (q == bb) hop[q] += v;
    }
  }
  double* out = partial + (int64_t)blockIdx.x * SW_P;
#pragma unroll
  for (int j = 0; j < SW_SITES; ++j) {
    const double s = block_sum<SW_NT>(eps[j], sm);
    if (threadIdx.x == 0) out[j] = s;
    const double t = block_sum<SW_NT>(uu[j], sm);
    if (threadIdx.x == 0) out[SW_SITES + j] = t;
  }
#pragma unroll
  for (int q = 0; q < SW_BONDS; ++q) {
    const double s = block_sum<SW_NT>(hop[q], sm);
    if (threadIdx.x == 0) out[2 * SW_SITES + q] = s;
  }
}

// sum the block partials in block order and scatter into the packed parameter layout
__global__ void k_sandwich_reduce(const double* __restrict__ partial, int nblocks, int n_sites, int n_bonds,
                                  double* __restrict__ out, int accumulate) {
  const int q = threadIdx.x;
  if (q >= SW_P) return;
  double s = 0.0;
  for (int b = 0; b < nblocks; ++b) s += partial[(int64_t)b * SW_P + q];
  int dst = -1;
  if (q < SW_SITES) dst = q < n_sites ? q : -1;
  else if (q < 2 * SW_SITES) dst = (q - SW_SITES) < n_sites ? n_sites + (q - SW_SITES) : -1;
  else dst = (q - 2 * SW_SITES) < n_bonds ? 2 * n_sites + (q - 2 * SW_SITES) : -1;
  if (dst >= 0) out[dst] = accumulate ? out[dst] + s : s;
}

}  // namespace ed

using namespace ed;

extern "C" {

ED_API int ed_plan_num_params(ed_plan p) {
  if (!p || p->kind != 0) return 0;
  return 2 * p->n_sites + (int)p->hop.size();
}

ED_API ed_status ed_param_sandwich(ed_plan p, const double* d_a, const double* d_b, double* d_out, int accumulate,
                                   ed_stream_t stream) {
  ED_TRY(check_plan(p));
  if (p->kind != 0) return fail(ED_ERR_INVALID_ARG, "parameter derivatives need a fermionic plan");
  if (p->n_sites > SW_SITES || (int)p->hop.size() > SW_BONDS)
    return fail(ED_ERR_TOO_LARGE, "parameter derivatives support up to 16 sites and 32 bonds");
  if (!d_a || !d_b || !d_out) return fail(ED_ERR_INVALID_ARG, "null argument");
  cudaStream_t s = as_stream(stream);
  const int nb = (int)std::max<int64_t>(1, std::min<int64_t>((p->dim + SW_NT - 1) / SW_NT, (int64_t)p->ctx->num_sms * 2));
  double* partial = nullptr;
  ED_CUDA(cudaMallocAsync(&partial, (size_t)nb * SW_P * sizeof(double), s));
  SandwichArgs g{p->up.states, p->dn.states, p->up.off, p->up.idx, p->up.coef, p->up.bond,
                 p->dn.off, p->dn.idx, p->dn.coef, p->dn.bond, p->num_up, p->num_dn};
  k_sandwich<<<nb, SW_NT, 0, s>>>(g, d_a, d_b, partial);
  k_sandwich_reduce<<<1, 64, 0, s>>>(partial, nb, p->n_sites, (int)p->hop.size(), d_out, accumulate);
  ED_CHECK_LAUNCH_N("ed_param_sandwich", 2);
  ED_CUDA(cudaFreeAsync(partial, s));
  return ED_OK;
}

}  // extern "C"
