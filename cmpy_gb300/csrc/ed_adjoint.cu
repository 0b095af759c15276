// Parameter derivatives of a fermionic Hamiltonian for the adjoint (reverse-mode) Green's
// function: out[theta] (+)= a^T (dH/dtheta) b for every model parameter theta at once,
//   theta = eps_j (dH = n_j_up + n_j_dn), U_j (dH = n_j_up n_j_dn), t_b (dH = hop of bond b
//   with its fermionic sign, i.e. the bond's matrix elements divided by t_b).
// No reference counterpart (the reference has no derivatives); the parameter meaning follows
// HubbardModel / SIAM (cmpy/models/hubbard.py:13-22, cmpy/models/anderson.py:147-158).
// Output layout: [eps_0..eps_{N-1}, U_0..U_{N-1}, t_0..t_{nb-1}], N <= 16, nb <= 32.
#include <algorithm>
#include <cmath>
#include <vector>

#include "ed_adjoint.cuh"
#include "ed_lzcheck.cuh"

namespace ed {

__global__ void __launch_bounds__(SW_NT) k_sandwich(SandwichArgs g, int ns, int P, const double* __restrict__ a,
                                                    const double* __restrict__ b, double* __restrict__ partial) {
  extern __shared__ double sacc[];  // [P][SW_NT]
  sandwich_zero(sacc, P);
  const int64_t D = g.nu * g.nd;
  for (int64_t i = blockIdx.x * (int64_t)SW_NT + threadIdx.x; i < D; i += (int64_t)gridDim.x * SW_NT)
    sandwich_row(g, ns, i, a[i], b[i], b, sacc + threadIdx.x);
  sandwich_block_out(sacc, P, partial + (int64_t)blockIdx.x * SW_P, false);
}

// sum the block rows in block order: out[p] (+)= sum_b partial[b * SW_P + p]
__global__ void k_param_reduce(const double* __restrict__ partial, int nblocks, int P, double* __restrict__ out,
                               int accumulate) {
  const int p = threadIdx.x;
  if (p >= P) return;
  double s = 0.0;
  for (int b = 0; b < nblocks; ++b) s += partial[(int64_t)b * SW_P + p];
  out[p] = accumulate ? out[p] + s : s;
}


// ---- taped FP64 Lanczos, segment recompute and reverse sweep --------------------------------
// The forward is the plain three-term recurrence (no reorthogonalisation) of the reference's
// Lanczos coefficients (cmpy/exactdiag.py:324-365), normalised:
//   w = H q_k, alpha_k = q_k.w, r = w - alpha_k q_k - beta_k q_{k-1}, beta_{k+1} = ||r||,
//   q_{k+1} = r / beta_{k+1}.
// It keeps the scalars and the pair (q_{k-1}, q_k) for k = 0 (mod c). The segment recompute
// repeats the same floating-point operations (explicit FMAs, the same reciprocal), so every
// recomputed q_k equals the forward's bit for bit. The reverse sweep is the exact adjoint of
// those recurrences; the parameter gradient term w_bar^T (dH/dtheta) q_k of each step is fused
// into the step's elementwise kernel and accumulated per block across steps.
struct TapeState {
  int stop;   // 0 running, 1 converged, 2 breakdown (invariant subspace)
  int steps;  // m once stopped
  int pad[2];
  unsigned int ticket[4];
};

__device__ __forceinline__ bool tp_stopped(const int* stop) { return stop && *(volatile const int*)stop != 0; }

// *res = <a, b> (and sqrt -> *res_sqrt)
__global__ void __launch_bounds__(TP_NT) k_tp_dot(const double* __restrict__ a, const double* __restrict__ b,
                                                  int64_t n, double* partial, unsigned int* ticket, double* res,
                                                  double* res_sqrt, const int* stop) {
  if (tp_stopped(stop)) return;
  __shared__ double sm[TP_NT / 32];
  double v = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)TP_NT + threadIdx.x; i < n; i += (int64_t)gridDim.x * TP_NT)
    v = fma(a[i], b[i], v);
  v = block_sum<TP_NT>(v, sm);
  if (threadIdx.x == 0) partial[blockIdx.x] = v;
  if (tp_last_block(ticket)) {
    const double s = tp_row_sum(partial, gridDim.x, sm);
    if (threadIdx.x == 0) {
      *res = s;
      if (res_sqrt) *res_sqrt = sqrt(s);
      *ticket = 0;
    }
  }
}

// out = v * (1 / *scale)
__global__ void k_tp_scale(const double* __restrict__ v, double* __restrict__ out, int64_t n, const double* scale,
                           const int* stop) {
  if (tp_stopped(stop)) return;
  const double s = 1.0 / *scale;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = v[i] * s;
}

// w <- w - alpha_k q_k - beta_k q_{k-1}; beta_{k+1} = ||w||; breakdown when
// beta_{k+1} <= breakdown * (|alpha_k| + beta_k)
__global__ void __launch_bounds__(TP_NT) k_tp_update(double* __restrict__ w, const double* __restrict__ q,
                                                     const double* __restrict__ qp, int64_t n, const double* alpha,
                                                     double* beta, int k, double breakdown, double* partial,
                                                     TapeState* st) {
  if (tp_stopped(&st->stop)) return;
  __shared__ double sm[TP_NT / 32];
  const double a = alpha[k], b = qp ? beta[k] : 0.0;
  double v = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)TP_NT + threadIdx.x; i < n; i += (int64_t)gridDim.x * TP_NT) {
    const double x = tp_resid(w[i], a, q[i], b, qp, i);
    w[i] = x;
    v = fma(x, x, v);
  }
  v = block_sum<TP_NT>(v, sm);
  if (threadIdx.x == 0) partial[blockIdx.x] = v;
  if (tp_last_block(&st->ticket[1])) {
    const double s = tp_row_sum(partial, gridDim.x, sm);
    if (threadIdx.x == 0) {
      const double bn = sqrt(s);
      beta[k + 1] = bn;
      const double scale = fabs(a) + (k > 0 ? b : 0.0);
      if (!(bn > breakdown * scale)) { st->steps = k + 1; st->stop = 2; }
      st->ticket[1] = 0;
    }
  }
}

// checkpoint slot: [q_{k-1} (zeros for k = 0), q_k]
__global__ void k_tp_ckpt(const double* __restrict__ q, const double* __restrict__ qp, double* __restrict__ dst,
                          int64_t n, const int* stop) {
  if (tp_stopped(stop)) return;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    dst[i] = qp ? qp[i] : 0.0;
    dst[n + i] = q[i];
  }
}

// q_{k+1} recomputed from w_k = H q_k (w is not modified); optionally y += coef[k+1] q_{k+1} and
// dots[k+1] = q_{k+1} . probe
__global__ void __launch_bounds__(TP_NT) k_tp_next(const double* __restrict__ w, const double* __restrict__ q,
                                                   const double* __restrict__ qp, int64_t n, const double* alpha,
                                                   const double* beta, int k, double* __restrict__ out,
                                                   const double* coef, double* __restrict__ y,
                                                   const double* __restrict__ probe, double* partial,
                                                   unsigned int* ticket, double* dots) {
  __shared__ double sm[TP_NT / 32];
  const double a = alpha[k], b = qp ? beta[k] : 0.0, s = 1.0 / beta[k + 1];
  const double cy = y ? coef[k + 1] : 0.0;
  double v = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)TP_NT + threadIdx.x; i < n; i += (int64_t)gridDim.x * TP_NT) {
    const double q1 = tp_resid(w[i], a, q[i], b, qp, i) * s;
    out[i] = q1;
    if (y) y[i] = fma(cy, q1, y[i]);
    if (probe) v = fma(q1, probe[i], v);
  }
  if (!probe) return;
  v = block_sum<TP_NT>(v, sm);
  if (threadIdx.x == 0) partial[blockIdx.x] = v;
  if (tp_last_block(ticket)) {
    const double t = tp_row_sum(partial, gridDim.x, sm);
    if (threadIdx.x == 0) {
      dots[k + 1] = t;
      *ticket = 0;
    }
  }
}

// the checkpointed q_k of a segment start: y += coef[k] q_k, dots[k] = q_k . probe
__global__ void __launch_bounds__(TP_NT) k_tp_acc(const double* __restrict__ q, int64_t n, int k, const double* coef,
                                                  double* __restrict__ y, const double* __restrict__ probe,
                                                  double* partial, unsigned int* ticket, double* dots) {
  __shared__ double sm[TP_NT / 32];
  const double cy = y ? coef[k] : 0.0;
  double v = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)TP_NT + threadIdx.x; i < n; i += (int64_t)gridDim.x * TP_NT) {
    if (y) y[i] = fma(cy, q[i], y[i]);
    if (probe) v = fma(q[i], probe[i], v);
  }
  if (!probe) return;
  v = block_sum<TP_NT>(v, sm);
  if (threadIdx.x == 0) partial[blockIdx.x] = v;
  if (tp_last_block(ticket)) {
    const double t = tp_row_sum(partial, gridDim.x, sm);
    if (threadIdx.x == 0) {
      dots[k] = t;
      *ticket = 0;
    }
  }
}

// Reverse step k, part 1. q_bar_{k+1} is complete once H w_bar_{k+1} (tmp) and the external
// adjoint ext_coef[k+1] * ext are added; then, with r_bar = q_bar_{k+1}/beta_{k+1} +
// beta_bar_{k+1} q_{k+1} (beta_bar_{k+1} first updated by -q_bar_{k+1}.q_{k+1}/beta_{k+1}):
//   alpha_bar_k -= r_bar.q_k,  beta_bar_k -= r_bar.q_{k-1}
// from five dot products of one pass. final != 0: k = -1, only q_bar_0 is completed and
// res = q_bar_0 . q_0 (q1 = q_0).
__global__ void __launch_bounds__(TP_NT) k_tp_radot(double* __restrict__ qb1, const double* __restrict__ tmp,
                                                    const double* __restrict__ ext, const double* ext_coef,
                                                    const double* __restrict__ q1, const double* __restrict__ q0,
                                                    const double* __restrict__ qm, int64_t n, const double* beta,
                                                    double* abar, double* bbar, int k, double* partial,
                                                    unsigned int* ticket, double* res) {
  __shared__ double sm[TP_NT / 32];
  const int G = gridDim.x;
  const double ce = ext ? ext_coef[k + 1] : 0.0;
  const bool fin = res != nullptr;
  double d1 = 0.0, d2 = 0.0, d3 = 0.0, d4 = 0.0, d5 = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)TP_NT + threadIdx.x; i < n; i += (int64_t)gridDim.x * TP_NT) {
    double v = qb1[i];
    if (tmp) v += tmp[i];
    if (ext) v = fma(ce, ext[i], v);
    qb1[i] = v;
    const double x1 = q1[i];
    d1 = fma(v, x1, d1);
    if (!fin) {
      const double x0 = q0[i], xm = qm ? qm[i] : 0.0;
      d2 = fma(v, x0, d2);
      d3 = fma(v, xm, d3);
      d4 = fma(x1, x0, d4);
      d5 = fma(x1, xm, d5);
    }
  }
  const int nd = fin ? 1 : 5;
  double dv[5] = {d1, d2, d3, d4, d5};
  for (int j = 0; j < nd; ++j) {
    const double s = block_sum<TP_NT>(dv[j], sm);
    if (threadIdx.x == 0) partial[(int64_t)j * G + blockIdx.x] = s;
  }
  if (tp_last_block(ticket)) {
    double t[5];
    for (int j = 0; j < nd; ++j) t[j] = tp_row_sum(partial + (int64_t)j * G, G, sm);
    if (threadIdx.x == 0) {
      if (fin) {
        *res = t[0];
      } else {
        const double bk1 = beta[k + 1];
        const double bb1 = bbar[k + 1] - t[0] / bk1;
        bbar[k + 1] = bb1;
        abar[k] -= t[1] / bk1 + bb1 * t[3];
        if (k > 0) bbar[k] -= t[2] / bk1 + bb1 * t[4];
      }
      *ticket = 0;
    }
  }
}

// Reverse step k, part 2 (elementwise) fused with the parameter term w_bar^T (dH/dtheta) q_k:
//   r_bar = q_bar_{k+1}/beta_{k+1} + beta_bar_{k+1} q_{k+1}   (0 for the last step)
//   w_bar = r_bar + alpha_bar_k q_k
//   q_bar_k += -alpha_k r_bar + alpha_bar_k w_k                (first: q_bar_k starts here)
//   q_bar_{k-1} = -beta_k r_bar                                 (its first contribution)
// Each block adds its parameter sums to its own row of psw (same grid every step).
__global__ void __launch_bounds__(SW_NT) k_tp_rstep(SandwichArgs g, int ns, int P, const double* __restrict__ qb1,
                                                    const double* __restrict__ q1, const double* __restrict__ q0,
                                                    const double* __restrict__ w0, double* __restrict__ qbk,
                                                    double* __restrict__ qbm, double* __restrict__ wbar,
                                                    const double* alpha, const double* beta, const double* abar,
                                                    const double* bbar, int k, int has_next, int first,
                                                    double* __restrict__ pracc, double* __restrict__ psw) {
  extern __shared__ double sacc[];  // [P][SW_NT]
  sandwich_zero(sacc, P);
  const double ak = alpha[k], ab = abar[k];
  const double inv = has_next ? 1.0 / beta[k + 1] : 0.0, bb1 = has_next ? bbar[k + 1] : 0.0;
  const double bk = k > 0 ? beta[k] : 0.0;
  const int64_t D = g.nu * g.nd;
  for (int64_t i = blockIdx.x * (int64_t)SW_NT + threadIdx.x; i < D; i += (int64_t)gridDim.x * SW_NT) {
    const double rb = has_next ? fma(bb1, q1[i], qb1[i] * inv) : 0.0;
    const double x0 = q0[i];
    const double wb = fma(ab, x0, rb);
    qbk[i] = fma(ab, w0[i], fma(-ak, rb, first ? 0.0 : qbk[i]));
    if (qbm) qbm[i] = -bk * rb;
    wbar[i] = wb;
    // w_bar^T (dH/dtheta) q_k, row i: the hop part now, the diagonal part through sum_k w_bar q_k
    pracc[i] = fma(wb, x0, first ? 0.0 : pracc[i]);
    sandwich_hop_terms(g, ns, i, wb, q0, sacc + threadIdx.x);
  }
  sandwich_block_out(sacc, P, psw + (int64_t)blockIdx.x * SW_P, true);
}

// the diagonal (eps, U) part of sum_k w_bar_k^T (dH/dtheta) q_k from pracc = sum_k w_bar_k q_k,
// added to the block rows of psw (same grid as the steps)
__global__ void __launch_bounds__(SW_NT) k_tp_diag_terms(SandwichArgs g, int ns, int P, const double* __restrict__ pracc,
                                                         double* __restrict__ psw) {
  extern __shared__ double sacc[];  // [P][SW_NT]
  sandwich_zero(sacc, P);
  const int64_t D = g.nu * g.nd;
  for (int64_t i = blockIdx.x * (int64_t)SW_NT + threadIdx.x; i < D; i += (int64_t)gridDim.x * SW_NT)
    sandwich_diag_terms(g, ns, i, pracc[i], sacc + threadIdx.x);
  sandwich_block_out(sacc, P, psw + (int64_t)blockIdx.x * SW_P, true);
}

// start_bar = (q_bar_0 - (q_bar_0.q_0) q_0) / beta_0 + beta_bar_0 q_0   (q_0 = s/||s||, beta_0 = ||s||)
__global__ void k_tp_startbar(const double* __restrict__ qb0, const double* __restrict__ q0, int64_t n,
                              const double* beta, const double* bbar, const double* dres, double* __restrict__ out) {
  const double d = *dres, ib = 1.0 / beta[0], b0 = bbar[0];
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = fma(b0, q0[i], (qb0[i] - d * q0[i]) * ib);
}

}  // namespace ed

using namespace ed;

// the parameter accumulators need up to SW_P * SW_NT doubles (64 KB) of dynamic shared memory
// (set on the current device at every call; a host-side attribute write)
static ed_status sandwich_attrs() {
  ED_CUDA(cudaFuncSetAttribute(k_sandwich, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sandwich_smem(SW_P)));
  ED_CUDA(cudaFuncSetAttribute(k_tp_rstep, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sandwich_smem(SW_P)));
  ED_CUDA(cudaFuncSetAttribute(k_tp_diag_terms, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sandwich_smem(SW_P)));
  return ED_OK;
}

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
  const SandwichArgs g = sandwich_args(p);
  const int P = 2 * p->n_sites + (int)p->hop.size();
  ED_TRY(sandwich_attrs());
  k_sandwich<<<nb, SW_NT, sandwich_smem(P), s>>>(g, p->n_sites, P, d_a, d_b, partial);
  k_param_reduce<<<1, SW_P, 0, s>>>(partial, nb, P, d_out, accumulate);
  ED_CHECK_LAUNCH_N("ed_param_sandwich", 2);
  ED_CUDA(cudaFreeAsync(partial, s));
  return ED_OK;
}

}  // extern "C"

// ---- taped Lanczos / reverse sweep: host side -------------------------------------------------
namespace {

struct TapeLayout {
  int nvec, nparts, nsw;
  size_t off_vec, off_part, off_psw, off_scal, off_state, total;
};

size_t tp_align(size_t x) { return (x + 255) & ~(size_t)255; }

TapeLayout tape_layout(const ed_plan_s* p, int K, int c) {
  TapeLayout L;
  const int64_t D = p->dim;
  L.nvec = std::max(4, 2 * c + 6);
  L.nparts = (int)std::max<int64_t>(1, std::min<int64_t>((D + TP_NT - 1) / TP_NT, (int64_t)p->ctx->num_sms * 4));
  L.nsw = (int)std::max<int64_t>(1, std::min<int64_t>((D + SW_NT - 1) / SW_NT, (int64_t)p->ctx->num_sms * 2));
  size_t o = 0;
  L.off_vec = o; o = tp_align(o + (size_t)L.nvec * D * sizeof(double));
  L.off_part = o; o = tp_align(o + (size_t)5 * L.nparts * sizeof(double));
  L.off_psw = o; o = tp_align(o + (size_t)L.nsw * SW_P * sizeof(double));
  // abar[K], bbar[K+1], c[K+2], tridiag work 5(K+2), 16 scalars
  L.off_scal = o; o = tp_align(o + (size_t)(K + (K + 1) + (K + 2) + 5 * (K + 2) + 16) * sizeof(double));
  L.off_state = o; o = tp_align(o + sizeof(TapeState));
  L.total = o;
  return L;
}

ed_status tape_check(const ed_plan_s* p, int K, int c) {
  if (p->kind != 0) return fail(ED_ERR_INVALID_ARG, "the taped Lanczos needs a fermionic plan");
  if (p->dim < 1) return fail(ED_ERR_INVALID_ARG, "empty sector");
  if (K < 1 || K > 4096) return fail(ED_ERR_INVALID_ARG, "max_steps must be in [1, 4096]");
  if (c < 1 || c > 256) return fail(ED_ERR_INVALID_ARG, "checkpoint spacing must be in [1, 256]");
  return ED_OK;
}

}  // namespace

extern "C" {

ED_API ed_status ed_tape_workspace(ed_plan p, int max_steps, int ckpt, size_t* bytes) {
  ED_TRY(check_plan(p));
  if (!bytes) return fail(ED_ERR_INVALID_ARG, "null argument");
  ED_TRY(tape_check(p, max_steps, ckpt));
  *bytes = tape_layout(p, max_steps, ckpt).total;
  return ED_OK;
}

ED_API ed_status ed_lanczos_tape(ed_plan p, const double* d_start, int max_steps, int ckpt, double tol,
                                 int check_every, double breakdown, void* d_work, size_t work_bytes, double* d_alpha,
                                 double* d_beta, double* d_ckpt, int* h_steps, ed_stream_t stream) {
  ED_TRY(check_plan(p));
  if (!d_start || !d_alpha || !d_beta || !d_ckpt || !h_steps) return fail(ED_ERR_INVALID_ARG, "null argument");
  ED_TRY(tape_check(p, max_steps, ckpt));
  const TapeLayout L = tape_layout(p, max_steps, ckpt);
  if (!d_work || work_bytes < L.total) return fail(ED_ERR_INVALID_ARG, "workspace too small (see ed_tape_workspace)");
  const int64_t D = p->dim;
  const int K = max_steps, c = ckpt;
  cudaStream_t s = as_stream(stream);
  char* base = (char*)d_work;
  double* V = (double*)(base + L.off_vec);
  double* part = (double*)(base + L.off_part);
  double* scal = (double*)(base + L.off_scal);
  // scalar region: abar[K], bbar[K+1], c[K+2], tridiagonal work 5(K+2), 16 scalars
  double* cvec = scal + K + (K + 1);
  double* twork = cvec + (K + 2);
  double* n2 = twork + 5 * (K + 2);          // start norm^2
  TriResult* tri = (TriResult*)(n2 + 2);  // 5 of the 16 scalars
  TapeState* st = (TapeState*)(base + L.off_state);
  ED_CUDA(cudaMemsetAsync(st, 0, sizeof(TapeState), s));
  ED_CUDA(cudaMemsetAsync(tri, 0, sizeof(TriResult), s));  // no earlier test to start from
  ED_CUDA(cudaMemsetAsync(d_alpha, 0, K * sizeof(double), s));
  ED_CUDA(cudaMemsetAsync(d_beta, 0, (K + 1) * sizeof(double), s));
  const int gv = L.nparts;
  const int gs = grid_for(D, 256, p->ctx->num_sms * 8);
  double* w = V + 3 * D;
  auto qv = [&](int k) -> double* { return V + (int64_t)(k % 3) * D; };
  const int* stopf = &st->stop;
  k_tp_dot<<<gv, TP_NT, 0, s>>>(d_start, d_start, D, part, &st->ticket[0], n2, d_beta, nullptr);
  k_tp_scale<<<gs, 256, 0, s>>>(d_start, qv(0), D, d_beta, nullptr);
  ED_CHECK_LAUNCH_N("ed_lanczos_tape start", 2);
  double hn2 = 0.0;
  ED_CUDA(cudaMemcpyAsync(&hn2, n2, sizeof(double), cudaMemcpyDeviceToHost, s));
  ED_CUDA(cudaStreamSynchronize(s));
  if (!std::isfinite(hn2)) return fail(ED_ERR_NONFINITE, "start vector is not finite");
  if (hn2 == 0.0) { *h_steps = 0; return ED_OK; }
  const int Km = (int)std::min<int64_t>(K, D);
  // convergence tests on a side stream, on the device (ed_lzcheck.cuh); the host never waits
  const bool checks = check_every > 0 && tol > 0.0;
  SideChecks chk;
  ED_TRY(chk.init(checks ? Km / check_every + 1 : 0));
  int launched = 0;
  for (int k = 0; k < Km; ++k) {
    if (checks && chk.stopped()) break;
    double* q = qv(k);
    double* qp = k > 0 ? qv(k - 1) : nullptr;
    int nl = 4;
    if (k % c == 0) {
      k_tp_ckpt<<<gs, 256, 0, s>>>(q, qp, d_ckpt + (int64_t)(k / c) * 2 * D, D, stopf);
      ++nl;
    }
    ED_TRY(matvec_f64(p, q, w, 1, D, s, stopf));
    k_tp_dot<<<gv, TP_NT, 0, s>>>(q, w, D, part, &st->ticket[0], d_alpha + k, nullptr, stopf);
    k_tp_update<<<gv, TP_NT, 0, s>>>(w, q, qp, D, d_alpha, d_beta, k, breakdown, part, st);
    k_tp_scale<<<gs, 256, 0, s>>>(w, qv(k + 1), D, d_beta + k + 1, stopf);
    ED_CHECK_LAUNCH_N("ed_lanczos_tape step", nl);
    launched = k + 1;
    if (checks && (k + 1) % check_every == 0 && k + 1 < Km)
      ED_TRY(chk.launch(s, d_alpha, d_beta, k + 1, tol, &st->stop, &st->steps, tri, cvec, twork));
  }
  ED_TRY(chk.join(s));
  TapeState hs;
  ED_CUDA(cudaMemcpyAsync(&hs, st, sizeof(TapeState), cudaMemcpyDeviceToHost, s));
  ED_CUDA(cudaStreamSynchronize(s));
  *h_steps = hs.stop ? hs.steps : launched;
  return ED_OK;
}

ED_API ed_status ed_tape_combine(ed_plan p, int m, int ckpt, const double* d_alpha, const double* d_beta,
                                 const double* d_ckpt, const double* d_coef, double* d_out, const double* d_probe,
                                 double* d_dots, void* d_work, size_t work_bytes, ed_stream_t stream) {
  ED_TRY(check_plan(p));
  if (!d_alpha || !d_beta || !d_ckpt) return fail(ED_ERR_INVALID_ARG, "null argument");
  if ((d_out != nullptr) != (d_coef != nullptr) || (d_probe != nullptr) != (d_dots != nullptr))
    return fail(ED_ERR_INVALID_ARG, "d_out needs d_coef and d_probe needs d_dots");
  ED_TRY(tape_check(p, m, ckpt));
  const TapeLayout L = tape_layout(p, m, ckpt);
  if (!d_work || work_bytes < L.total) return fail(ED_ERR_INVALID_ARG, "workspace too small (see ed_tape_workspace)");
  const int64_t D = p->dim;
  const int c = ckpt;
  cudaStream_t s = as_stream(stream);
  char* base = (char*)d_work;
  double* V = (double*)(base + L.off_vec);
  double* part = (double*)(base + L.off_part);
  TapeState* st = (TapeState*)(base + L.off_state);
  double* w = V + 3 * D;
  ED_CUDA(cudaMemsetAsync(st, 0, sizeof(TapeState), s));
  if (d_out) ED_CUDA(cudaMemsetAsync(d_out, 0, D * sizeof(double), s));
  const int gv = L.nparts;
  for (int s0 = 0; s0 < m; s0 += c) {
    const int s1 = std::min(s0 + c, m);
    const double* slot = d_ckpt + (int64_t)(s0 / c) * 2 * D;
    auto q = [&](int k) -> const double* {
      if (k == s0 - 1) return slot;
      if (k == s0) return slot + D;
      return V + (int64_t)((k - s0 - 1) % 3) * D;
    };
    k_tp_acc<<<gv, TP_NT, 0, s>>>(q(s0), D, s0, d_coef, d_out, d_probe, part, &st->ticket[0], d_dots);
    ED_CHECK_LAUNCH("k_tp_acc");
    for (int k = s0; k + 1 < s1; ++k) {
      ED_TRY(matvec_f64(p, q(k), w, 1, D, s, nullptr));
      k_tp_next<<<gv, TP_NT, 0, s>>>(w, q(k), k > 0 ? q(k - 1) : nullptr, D, d_alpha, d_beta, k,
                                     (double*)q(k + 1), d_coef, d_out, d_probe, part, &st->ticket[0], d_dots);
      ED_CHECK_LAUNCH("k_tp_next");
    }
  }
  return ED_OK;
}

ED_API ed_status ed_tape_reverse(ed_plan p, int m, int ckpt, const double* d_alpha, const double* d_beta,
                                 const double* d_ckpt, const double* d_abar, const double* d_bbar,
                                 const double* d_ext_coef, const double* d_ext_vec, void* d_work, size_t work_bytes,
                                 double* d_theta_bar, double* d_start_bar, ed_stream_t stream) {
  ED_TRY(check_plan(p));
  if (!d_alpha || !d_beta || !d_ckpt || !d_abar || !d_bbar || !d_theta_bar || !d_start_bar)
    return fail(ED_ERR_INVALID_ARG, "null argument");
  if ((d_ext_coef != nullptr) != (d_ext_vec != nullptr))
    return fail(ED_ERR_INVALID_ARG, "d_ext_coef and d_ext_vec go together");
  ED_TRY(tape_check(p, m, ckpt));
  if (p->n_sites > SW_SITES || (int)p->hop.size() > SW_BONDS)
    return fail(ED_ERR_TOO_LARGE, "parameter derivatives support up to 16 sites and 32 bonds");
  const TapeLayout L = tape_layout(p, m, ckpt);
  if (!d_work || work_bytes < L.total) return fail(ED_ERR_INVALID_ARG, "workspace too small (see ed_tape_workspace)");
  const int64_t D = p->dim;
  const int c = ckpt;
  cudaStream_t s = as_stream(stream);
  char* base = (char*)d_work;
  double* V = (double*)(base + L.off_vec);
  double* part = (double*)(base + L.off_part);
  double* psw = (double*)(base + L.off_psw);
  double* AB = (double*)(base + L.off_scal);  // alpha_bar [m]
  double* BB = AB + m;                          // beta_bar [m+1]
  double* res = BB + (m + 1);                   // q_bar_0 . q_0
  TapeState* st = (TapeState*)(base + L.off_state);
  // vectors: Qseg [c] (q_{s0+1} .. q_{s1-1}), Wseg [c] (w_{s0} .. w_{s1-1}), q_bar x3, w_bar, tmp,
  // sum_k w_bar_k q_k
  double* Qs = V;
  double* Ws = V + (int64_t)c * D;
  double* QB = V + (int64_t)2 * c * D;
  double* wbar = QB + 3 * D;
  double* tmp = wbar + D;
  double* pracc = tmp + D;
  auto qb = [&](int k) -> double* { return QB + (int64_t)(k % 3) * D; };
  ED_CUDA(cudaMemsetAsync(st, 0, sizeof(TapeState), s));
  ED_CUDA(cudaMemsetAsync(psw, 0, (size_t)L.nsw * SW_P * sizeof(double), s));
  ED_CUDA(cudaMemcpyAsync(AB, d_abar, m * sizeof(double), cudaMemcpyDeviceToDevice, s));
  ED_CUDA(cudaMemcpyAsync(BB, d_bbar, (m + 1) * sizeof(double), cudaMemcpyDeviceToDevice, s));
  const SandwichArgs g = sandwich_args(p);
  const int gv = L.nparts;
  const int P = 2 * p->n_sites + (int)p->hop.size();
  ED_TRY(sandwich_attrs());
  bool have_tmp = false;
  const int last_seg = ((m - 1) / c) * c;
  for (int s0 = last_seg; s0 >= 0; s0 -= c) {
    const int s1 = std::min(s0 + c, m);
    const double* slot = d_ckpt + (int64_t)(s0 / c) * 2 * D;
    auto q = [&](int k) -> const double* {
      if (k == s0 - 1) return k >= 0 ? slot : nullptr;
      if (k == s0) return slot + D;
      if (k == s1) return s1 < m ? d_ckpt + (int64_t)(s1 / c) * 2 * D + D : nullptr;
      return Qs + (int64_t)(k - s0 - 1) * D;
    };
    // recompute the segment: w_k = H q_k and q_{k+1}
    for (int k = s0; k < s1; ++k) {
      ED_TRY(matvec_f64(p, q(k), Ws + (int64_t)(k - s0) * D, 1, D, s, nullptr));
      if (k + 1 < s1) {
        k_tp_next<<<gv, TP_NT, 0, s>>>(Ws + (int64_t)(k - s0) * D, q(k), k > 0 ? q(k - 1) : nullptr, D, d_alpha,
                                       d_beta, k, (double*)q(k + 1), nullptr, nullptr, nullptr, part,
                                       &st->ticket[0], nullptr);
        ED_CHECK_LAUNCH("k_tp_next");
      }
    }
    for (int k = s1 - 1; k >= s0; --k) {
      const bool has_next = k + 1 < m;
      if (has_next) {
        k_tp_radot<<<gv, TP_NT, 0, s>>>(qb(k + 1), have_tmp ? tmp : nullptr, d_ext_vec, d_ext_coef, q(k + 1), q(k),
                                        k > 0 ? q(k - 1) : nullptr, D, d_beta, AB, BB, k, part, &st->ticket[0],
                                        nullptr);
        ED_CHECK_LAUNCH("k_tp_radot");
      }
      k_tp_rstep<<<L.nsw, SW_NT, sandwich_smem(P), s>>>(g, p->n_sites, P, has_next ? qb(k + 1) : nullptr, has_next ? q(k + 1) : nullptr, q(k),
                                         Ws + (int64_t)(k - s0) * D, qb(k), k > 0 ? qb(k - 1) : nullptr, wbar,
                                         d_alpha, d_beta, AB, BB, k, has_next ? 1 : 0, k == m - 1 ? 1 : 0, pracc,
                                         psw);
      ED_CHECK_LAUNCH("k_tp_rstep");
      ED_TRY(matvec_f64(p, wbar, tmp, 1, D, s, nullptr));
      have_tmp = true;
    }
  }
  // q_bar_0 complete, then the start vector's adjoint
  const double* q0 = d_ckpt + D;
  k_tp_radot<<<gv, TP_NT, 0, s>>>(qb(0), tmp, d_ext_vec, d_ext_coef, q0, nullptr,
                                  nullptr, D, d_beta, AB, BB, -1, part, &st->ticket[0], res);
  k_tp_startbar<<<grid_for(D, 256, p->ctx->num_sms * 8), 256, 0, s>>>(qb(0), q0, D, d_beta, BB, res, d_start_bar);
  k_tp_diag_terms<<<L.nsw, SW_NT, sandwich_smem(P), s>>>(g, p->n_sites, P, pracc, psw);
  k_param_reduce<<<1, SW_P, 0, s>>>(psw, L.nsw, P, d_theta_bar, 1);
  ED_CHECK_LAUNCH_N("ed_tape_reverse final", 4);
  return ED_OK;
}

ED_API ed_status ed_cf_adjoint(const double* d_alpha, const double* d_beta, int m, double norm2, double shift,
                               int sign, const double* d_z, int64_t n_z, const double* d_gbar, double* d_abar,
                               double* d_bbar, double* d_scal, ed_stream_t stream) {
  if (m < 1 || m > 4096) return fail(ED_ERR_INVALID_ARG, "m must be in [1, 4096]");
  if (n_z < 1 || n_z > (int64_t)CFA_NT * 65535) return fail(ED_ERR_INVALID_ARG, "n_z out of range");
  if (sign != 1 && sign != -1) return fail(ED_ERR_INVALID_ARG, "sign must be +1 or -1");
  if (!d_alpha || !d_beta || !d_z || !d_gbar || !d_abar || !d_bbar || !d_scal)
    return fail(ED_ERR_INVALID_ARG, "null argument");
  CfaBatch cb{d_alpha, m, d_beta, m + 1, nullptr, nullptr, nullptr, m, norm2, shift, sign, d_gbar, d_abar, d_bbar, d_scal};
  return cf_adjoint_launch(cb, 1, m, (const double2*)d_z, n_z, as_stream(stream));
}

}  // extern "C"
