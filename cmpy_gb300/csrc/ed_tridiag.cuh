// Lowest eigenpair of a symmetric tridiagonal matrix on one thread block, FP64 — the
// device replacement of scipy.linalg.eigh_tridiagonal(select="i") used by
// cmpy/exactdiag.py:368-375. Shared by the FP64 and the fixed-point Lanczos drivers.
#pragma once

#include <algorithm>
#include <cmath>
#include <vector>

#include "ed_common.cuh"

namespace ed {

// ---- symmetric tridiagonal eigen-solver (one block) ----------------------------------------
// Number of eigenvalues of T (alpha[0..m), beta[1..m)) below x: sign changes of the sequence
// p_i = (a_i - x) p_{i-1} - b_i^2 p_{i-2} (the leading principal minors of T - x, so
// p_i / p_{i-1} are the LDL^T pivots), without divisions. A zero p_i is replaced by a tiny
// value of the opposite sign of p_{i-1} (a tiny negative pivot, the usual convention for an
// eigenvalue exactly at x); the pair is rescaled by an exact power of two when p_i leaves
// [2^-400, 2^400]. The signs, the zero test and the exponent are read from the bit patterns
// (integer operations), so the FP64 pipe, narrow on this GPU, only runs the recurrence.
// bb = b^2 when precomputed (may be null).
static __device__ int sturm_count(const double* a, const double* b, const double* bb, int m, double x) {
  double p0 = 1.0, p1 = a[0] - x;
  long long s1 = __double_as_longlong(p1);
  if ((s1 << 1) == 0) { p1 = -0x1.0p-900; s1 = __double_as_longlong(p1); }
  int cnt = (int)((unsigned long long)s1 >> 63);
  for (int i = 1; i < m; ++i) {
    const double bbi = bb ? bb[i] : b[i] * b[i];
    double p2 = fma(a[i] - x, p1, -bbi * p0);
    long long s2 = __double_as_longlong(p2);
    if ((s2 << 1) == 0) { p2 = -p1 * 0x1.0p-60; s2 = __double_as_longlong(p2); }
    cnt += (int)((unsigned long long)(s2 ^ s1) >> 63);
    const int ex = (int)((s2 >> 52) & 0x7ff);
    if (ex > 1023 + 400 || ex < 1023 - 400) {
      const double sc = __longlong_as_double((long long)(2046 - ex) << 52);  // 2^-(ex - 1023)
      p2 *= sc;
      p1 *= sc;
    }
    p0 = p1;
    p1 = p2;
    s1 = s2;
  }
  return cnt;
}

// Lowest eigenvalue by 128-way multisection (four warps evaluate the Sturm counts, one per
// SM sub-partition: a warp's FP64 recurrence is bound by its sub-partition's FP64 pipe, so
// more points per warp would not come for free), then optionally the eigenvector by inverse
// iteration (thread 0, FP64, partial pivoting). Needs blockDim.x >= MS_PTS.
constexpr int MS_PTS = 128;
//
// SM_M > 0 (single-block callers): for m <= SM_M the tridiagonal (with b^2), the elimination
// work and the vector live in static shared memory instead of global memory. Batched callers
// keep SM_M = 0.
//
// lo_hint < hi_hint (optional): a bracket of the lowest eigenvalue to start from (e.g. from a
// convergence test of a shorter run of the same Lanczos recurrence); it is used only when the
// Sturm counts confirm it (no eigenvalue below lo_hint, at least one below hi_hint), otherwise
// the Gershgorin interval is.
template <int SM_M = 0>
static __device__ double tridiag_lowest_block(const double* a_g, const double* b_g, int m, double* vec_g,
                                              double* work_g, double lo_hint = 0.0, double hi_hint = 0.0) {
  __shared__ double lo_s, hi_s;
  __shared__ int cnt_s[MS_PTS];
  const double* a = a_g;
  const double* b = b_g;
  const double* bb = nullptr;
  double* vec = vec_g;
  double* work = work_g;
  bool in_smem = false;
  if constexpr (SM_M > 0) {
    __shared__ double s_ab[3 * SM_M];
    __shared__ double s_w[5 * SM_M];
    __shared__ double s_v[SM_M];
    if (m <= SM_M) {
      for (int i = threadIdx.x; i < m; i += blockDim.x) {
        s_ab[i] = a_g[i];
        s_ab[SM_M + i] = b_g[i];
        s_ab[2 * SM_M + i] = b_g[i] * b_g[i];
      }
      __syncthreads();
      a = s_ab;
      b = s_ab + SM_M;
      bb = s_ab + 2 * SM_M;
      work = s_w;
      if (vec_g) vec = s_v;
      in_smem = true;
    }
  }
  const bool hinted = lo_hint < hi_hint;  // block-uniform
  if (hinted && threadIdx.x < 2) cnt_s[threadIdx.x] = sturm_count(a, b, bb, m, threadIdx.x ? hi_hint : lo_hint);
  __syncthreads();
  if (threadIdx.x == 0) {
    double lo = a[0], hi = a[0];
    for (int i = 0; i < m; ++i) {
      const double r = (i > 0 ? fabs(b[i]) : 0.0) + (i + 1 < m ? fabs(b[i + 1]) : 0.0);
      lo = fmin(lo, a[i] - r);
      hi = fmax(hi, a[i] + r);
    }
    const double pad = 1e-12 * fmax(fabs(lo), fabs(hi)) + 1e-300;
    lo_s = lo - pad;
    hi_s = hi + pad;
    if (hinted && cnt_s[0] == 0 && cnt_s[1] >= 1) {
      lo_s = fmax(lo_s, lo_hint);
      hi_s = fmin(hi_s, hi_hint);
    }
  }
  __syncthreads();
  for (int round = 0; round < 16; ++round) {
    const double lo = lo_s, hi = hi_s;
    if (threadIdx.x < MS_PTS) {
      const double x = lo + (hi - lo) * (double)(threadIdx.x + 1) / (double)(MS_PTS + 1);
      cnt_s[threadIdx.x] = sturm_count(a, b, bb, m, x);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      int t = 0;
      while (t < MS_PTS && cnt_s[t] == 0) ++t;  // first point with >=1 eigenvalue below
      const double nlo = (t == 0) ? lo : lo + (hi - lo) * (double)t / (double)(MS_PTS + 1);
      const double nhi = (t == MS_PTS) ? hi : lo + (hi - lo) * (double)(t + 1) / (double)(MS_PTS + 1);
      lo_s = nlo;
      hi_s = nhi;
    }
    __syncthreads();
    if (hi_s - lo_s <= 4e-16 * fmax(fabs(lo_s), fabs(hi_s)) + 1e-300) break;
  }
  const double ev = 0.5 * (lo_s + hi_s);
  if (vec && threadIdx.x == 0) {
    // inverse iteration: (T - ev I) y = v, Gaussian elimination with partial pivoting, factored
    // once; the pivots are kept as reciprocals, so the whole solve takes m FP64 divisions (the
    // FP64 pipe of this GPU is narrow and a division is a long dependent sequence on it).
    // work: 5*m doubles (reciprocal pivots, super, super2, sub multipliers, pivot flags)
    double* dd = work;           // diagonal of U, then its reciprocals
    double* du = work + m;       // first super-diagonal of U
    double* du2 = work + 2 * m;  // second super-diagonal of U
    double* ml = work + 3 * m;   // multipliers
    double* pv = work + 4 * m;   // 1.0 if rows swapped at step i
    const double tiny = 1e-300 + 1e-15 * fmax(fabs(ev), 1.0) * 1e-3;
    for (int i = 0; i < m; ++i) vec[i] = 1.0 / sqrt((double)m) * (1.0 + 0.01 * (double)((i * 7919) % 13) / 13.0);
    for (int i = 0; i < m; ++i) { dd[i] = a[i] - ev; du[i] = (i + 1 < m) ? b[i + 1] : 0.0; du2[i] = 0.0; }
    // magnitude comparisons and zero tests on the bit patterns (integer operations)
    const long long mag = 0x7fffffffffffffffll;
    for (int i = 0; i < m - 1; ++i) {
      const double sub = b[i + 1];
      if ((__double_as_longlong(dd[i]) & mag) >= (__double_as_longlong(sub) & mag)) {
        pv[i] = 0.0;
        if ((__double_as_longlong(dd[i]) & mag) == 0) dd[i] = tiny;
        const double r = 1.0 / dd[i];
        const double l = sub * r;
        ml[i] = l;
        dd[i + 1] -= l * du[i];
        dd[i] = r;
      } else {
        pv[i] = 1.0;
        const double r = 1.0 / sub;
        const double l = dd[i] * r;
        ml[i] = l;
        // swap rows i and i+1
        const double t0 = dd[i + 1], t1 = (i + 2 < m) ? du[i + 1] : 0.0;
        const double odu = du[i];
        du[i] = t0;
        du2[i] = t1;
        dd[i + 1] = odu - l * t0;
        if (i + 2 < m) du[i + 1] = -l * t1;
        dd[i] = r;
      }
    }
    if (dd[m - 1] == 0.0) dd[m - 1] = tiny;
    dd[m - 1] = 1.0 / dd[m - 1];
    for (int it = 0; it < 2; ++it) {
      // forward: apply L^-1 to vec
      for (int i = 0; i < m - 1; ++i) {
        if (pv[i] != 0.0) { const double t = vec[i]; vec[i] = vec[i + 1]; vec[i + 1] = t - ml[i] * vec[i]; }
        else vec[i + 1] -= ml[i] * vec[i];
      }
      // back substitution
      for (int i = m - 1; i >= 0; --i) {
        double s = vec[i];
        if (i + 1 < m) s -= du[i] * vec[i + 1];
        if (i + 2 < m) s -= du2[i] * vec[i + 2];
        vec[i] = s * dd[i];
      }
      double nrm = 0.0;
      for (int i = 0; i < m; ++i) nrm = fma(vec[i], vec[i], nrm);
      nrm = 1.0 / sqrt(nrm);
      for (int i = 0; i < m; ++i) vec[i] *= nrm;
    }
    // sign convention: first nonzero component positive
    double sg = 1.0;
    for (int i = 0; i < m; ++i) if (vec[i] != 0.0) { sg = vec[i] > 0 ? 1.0 : -1.0; break; }
    for (int i = 0; i < m; ++i) vec[i] *= sg;
  }
  __syncthreads();
  if (in_smem && vec_g) {
    for (int i = threadIdx.x; i < m; i += blockDim.x) vec_g[i] = vec[i];
    __syncthreads();
  }
  return ev;
}

// v = -(T - e0)^+ r on the complement of c (c the unit eigenvector of T for its lowest
// eigenvalue e0), the tridiagonal part of the adjoint of that eigenpair. Thread 0: the shifted
// system (T - (e0 - delta)) y = r - (r.c) c by Gaussian elimination with partial pivoting, then
// v = -(y - (y.c) c). delta = 1e-13 max(1, |e0|) keeps the factorisation regular; off c it
// changes the solution by a relative delta / (gap to the next eigenvalue). work: 5*m doubles.
static __device__ void tridiag_pinv_solve(const double* a, const double* b, int m, double e0, const double* c,
                                          const double* r, double* v, double* work) {
  if (threadIdx.x != 0) return;
  double rc = 0.0;
  for (int i = 0; i < m; ++i) rc = fma(r[i], c[i], rc);
  for (int i = 0; i < m; ++i) v[i] = r[i] - rc * c[i];
  const double shift = e0 - 1e-13 * fmax(1.0, fabs(e0));
  double* dd = work;           // diagonal of U
  double* du = work + m;       // first super-diagonal of U
  double* du2 = work + 2 * m;  // second super-diagonal of U
  double* ml = work + 3 * m;   // multipliers
  double* pv = work + 4 * m;   // 1.0 if rows swapped at step i
  for (int i = 0; i < m; ++i) { dd[i] = a[i] - shift; du[i] = (i + 1 < m) ? b[i + 1] : 0.0; du2[i] = 0.0; }
  for (int i = 0; i < m - 1; ++i) {
    const double sub = b[i + 1];
    if (fabs(dd[i]) >= fabs(sub)) {
      pv[i] = 0.0;
      ml[i] = dd[i] != 0.0 ? sub / dd[i] : 0.0;
      dd[i + 1] -= ml[i] * du[i];
    } else {
      pv[i] = 1.0;
      const double l = dd[i] / sub, t0 = dd[i + 1], t1 = (i + 2 < m) ? du[i + 1] : 0.0, odu = du[i];
      ml[i] = l;
      dd[i] = sub;
      du[i] = t0;
      du2[i] = t1;
      dd[i + 1] = odu - l * t0;
      if (i + 2 < m) du[i + 1] = -l * t1;
    }
  }
  for (int i = 0; i < m - 1; ++i) {
    if (pv[i] != 0.0) { const double t = v[i]; v[i] = v[i + 1]; v[i + 1] = t - ml[i] * v[i]; }
    else v[i + 1] -= ml[i] * v[i];
  }
  for (int i = m - 1; i >= 0; --i) {
    double t = v[i];
    if (i + 1 < m) t -= du[i] * v[i + 1];
    if (i + 2 < m) t -= du2[i] * v[i + 2];
    v[i] = dd[i] != 0.0 ? t / dd[i] : 0.0;
  }
  double yc = 0.0;
  for (int i = 0; i < m; ++i) yc = fma(v[i], c[i], yc);
  for (int i = 0; i < m; ++i) v[i] = -(v[i] - yc * c[i]);
}

}  // namespace ed
