// Fermionic creation/annihilation between neighbouring sectors: replaces
// _apply_creation_up/dn and _apply_annihilation_up/dn (cmpy/operators.py:652-703) behind
// CreationOperator/AnnihilationOperator (cmpy/operators.py:706-791).
//
// Target-centric: every element of the target sector is written exactly once (zero when
// no source state maps onto it), so the kernel needs no pre-zeroed output and no atomics.
// For target state t the source is s = t ^ (1 << pos) when t has (create) / lacks
// (annihilate) the bit pos; its index in the source list is the colex rank.
#include <algorithm>

#include "ed_plan.cuh"

namespace ed {

// sigma = up: one block per (vector, target up-row); the dn row is copied with a sign.
__global__ void k_fermion_up(const uint64_t* __restrict__ tab, const uint64_t* __restrict__ t_up, int64_t nu_t,
                             int64_t nd, int pos, int create, int jw, const double* __restrict__ x,
                             double* __restrict__ y, int64_t nvec, int64_t ldx, int64_t ldy) {
  const uint64_t op = 1ull << pos;
  const int64_t rows = nu_t * nvec;
  for (int64_t r = blockIdx.x; r < rows; r += gridDim.x) {
    const int64_t v = r / nu_t, ut = r - v * nu_t;
    const uint64_t t = t_up[ut];
    const bool valid = create ? (t & op) != 0 : (t & op) == 0;
    double* yrow = y + v * ldy + ut * nd;
    if (!valid) {
      for (int64_t d = threadIdx.x; d < nd; d += blockDim.x) yrow[d] = 0.0;
      continue;
    }
    const uint64_t s = t ^ op;
    const int64_t us = colex_rank(tab, s);
    double sg = 1.0;
    if (jw && (__popcll(s & (op - 1)) & 1)) sg = -1.0;
    const double* xrow = x + v * ldx + us * nd;
    for (int64_t d = threadIdx.x; d < nd; d += blockDim.x) yrow[d] = sg * xrow[d];
  }
}

// sigma = dn: one block per (vector, up-row), threads over target dn states.
__global__ void k_fermion_dn(const uint64_t* __restrict__ tab, const uint64_t* __restrict__ up,
                             const uint64_t* __restrict__ t_dn, int64_t nu, int64_t nd_s, int64_t nd_t, int pos,
                             int create, int jw, const double* __restrict__ x, double* __restrict__ y,
                             int64_t nvec, int64_t ldx, int64_t ldy) {
  const uint64_t op = 1ull << pos;
  const int64_t rows = nu * nvec;
  for (int64_t r = blockIdx.x; r < rows; r += gridDim.x) {
    const int64_t v = r / nu, u = r - v * nu;
    // with the up-before-dn operator ordering the dn operator passes all up electrons
    const int up_par = jw ? (__popcll(up[u]) & 1) : 0;
    const double* xv = x + v * ldx;
    double* yv = y + v * ldy;
    for (int64_t dt = threadIdx.x; dt < nd_t; dt += blockDim.x) {
      const uint64_t t = t_dn[dt];
      const bool valid = create ? (t & op) != 0 : (t & op) == 0;
      double val = 0.0;
      if (valid) {
        const uint64_t s = t ^ op;
        const int64_t ds = colex_rank(tab, s);
        val = xv[u * nd_s + ds];
        if (jw && ((__popcll(s & (op - 1)) + up_par) & 1)) val = -val;
      }
      yv[u * nd_t + dt] = val;
    }
  }
}

}  // namespace ed

using namespace ed;

extern "C" {

// argument checks shared by the single and the batched entry point
static ed_status check_fermion_pair(const ed_plan_s* p, const ed_plan_s* pt, int pos, int sigma, int create) {
  ED_TRY(check_plan(p));
  ED_TRY(check_plan(pt));
  if (p->kind != 0 || pt->kind != 0) return fail(ED_ERR_INVALID_ARG, "fermion operators need fermionic plans");
  if (pos < 0 || pos >= p->n_sites) return fail(ED_ERR_INVALID_ARG, "pos outside [0, n_sites)");
  if (pt->n_sites != p->n_sites) return fail(ED_ERR_INVALID_ARG, "plans have different n_sites");
  if (sigma != 1 && sigma != 2) return fail(ED_ERR_INVALID_ARG, "sigma must be 1 (up) or 2 (dn)");
  const int dn_ = create ? 1 : -1;
  if (sigma == 1 && (pt->n_up != p->n_up + dn_ || pt->n_dn != p->n_dn))
    return fail(ED_ERR_INVALID_ARG, "target plan is not the neighbouring up sector");
  if (sigma == 2 && (pt->n_dn != p->n_dn + dn_ || pt->n_up != p->n_up))
    return fail(ED_ERR_INVALID_ARG, "target plan is not the neighbouring dn sector");
  return ED_OK;
}

static void launch_fermion(const ed_plan_s* p, const ed_plan_s* pt, int pos, int sigma, int create, int jw_sign,
                           const double* d_x, double* d_y, int64_t nvec, int64_t ldx, int64_t ldy, cudaStream_t s) {
  const int sms = p->ctx->num_sms;
  const int g = (int)std::min<int64_t>(pt->num_up * nvec, (int64_t)sms * 16);
  if (sigma == 1) {
    k_fermion_up<<<g, 256, 0, s>>>(p->ctx->d_binom, pt->up.states, pt->num_up, pt->num_dn, pos, create, jw_sign, d_x,
                                   d_y, nvec, ldx, ldy);
  } else {
    k_fermion_dn<<<g, 256, 0, s>>>(p->ctx->d_binom, pt->up.states, pt->dn.states, pt->num_up, p->num_dn, pt->num_dn,
                                   pos, create, jw_sign, d_x, d_y, nvec, ldx, ldy);
  }
}

ED_API ed_status ed_apply_fermion(ed_plan p, ed_plan pt, int pos, int sigma, int create, int jw_sign,
                                  const double* d_x, double* d_y, int64_t nvec, int64_t ldx, int64_t ldy,
                                  ed_stream_t stream) {
  ED_TRY(check_fermion_pair(p, pt, pos, sigma, create));
  if (nvec < 0 || ldx < p->dim || ldy < pt->dim) return fail(ED_ERR_INVALID_ARG, "bad n_vec / leading dimensions");
  if (pt->dim == 0 || nvec == 0) return ED_OK;
  if (!d_x || !d_y) return fail(ED_ERR_INVALID_ARG, "null vector");
  launch_fermion(p, pt, pos, sigma, create, jw_sign, d_x, d_y, nvec, ldx, ldy, as_stream(stream));
  ED_CHECK_LAUNCH("ed_apply_fermion");
  return ED_OK;
}

ED_API ed_status ed_apply_fermion_batch(const ed_plan* plans, const ed_plan* targets, int n, int pos, int sigma,
                                        int create, int jw_sign, const double* d_x, const int64_t* x_off,
                                        double* d_y, const int64_t* y_off, ed_stream_t stream) {
  if (n < 0) return fail(ED_ERR_INVALID_ARG, "negative problem count");
  if (n == 0) return ED_OK;
  if (!plans || !targets || !x_off || !y_off) return fail(ED_ERR_INVALID_ARG, "null plan or offset array");
  if (!d_x || !d_y) return fail(ED_ERR_INVALID_ARG, "null vector");
  // every problem is checked before the first launch: an error leaves d_y untouched
  for (int i = 0; i < n; ++i) {
    ED_TRY(check_fermion_pair(plans[i], targets[i], pos, sigma, create));
    if (x_off[i] < 0 || y_off[i] < 0) return fail(ED_ERR_INVALID_ARG, "negative vector offset");
  }
  const cudaStream_t s = as_stream(stream);
  int launched = 0;
  for (int i = 0; i < n; ++i) {
    const ed_plan_s* p = plans[i];
    const ed_plan_s* pt = targets[i];
    if (pt->dim == 0) continue;
    launch_fermion(p, pt, pos, sigma, create, jw_sign, d_x + x_off[i], d_y + y_off[i], 1, p->dim, pt->dim, s);
    ++launched;
  }
  ED_CHECK_LAUNCH_N("ed_apply_fermion_batch", launched);
  return ED_OK;
}

}  // extern "C"
