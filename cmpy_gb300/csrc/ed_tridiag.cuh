// Lowest eigenpair of a symmetric tridiagonal matrix on one thread block, FP64 — the
// device replacement of scipy.linalg.eigh_tridiagonal(select="i") used by
// cmpy/exactdiag.py:368-375. Shared by the FP64 and the fixed-point Lanczos drivers.
#pragma once

#include "ed_common.cuh"

namespace ed {

// ---- symmetric tridiagonal eigen-solver (one block) ----------------------------------------
// Number of eigenvalues of T (alpha[0..m), beta[1..m)) below x: sign changes of the LDL^T
// pivots, computed without divisions by rescaling a three-term recurrence.
static __device__ int sturm_count(const double* a, const double* b, int m, double x) {
  // p_i = (a_i - x) p_{i-1} - b_i^2 p_{i-2}; count sign changes of p_i / p_{i-1}
  // a zero p_i is replaced by a tiny value of the opposite sign of p_{i-1} (a tiny negative
  // pivot), the usual convention for an eigenvalue exactly at x
  double p0 = 1.0, p1 = a[0] - x;
  if (p1 == 0.0) p1 = -0x1.0p-900;
  int cnt = (p1 < 0.0) ? 1 : 0;
  for (int i = 1; i < m; ++i) {
    const double bb = b[i] * b[i];
    double p2 = (a[i] - x) * p1 - bb * p0;
    if (p2 == 0.0) p2 = -p1 * 0x1.0p-60;
    if ((p2 < 0.0) != (p1 < 0.0)) ++cnt;
    // rescale to avoid overflow/underflow (exact powers of two)
    const double ap = fabs(p2);
    if (ap > 0x1.0p+400 || ap < 0x1.0p-400) {
      const int e = ilogb(ap);
      p2 = scalbn(p2, -e);
      p1 = scalbn(p1, -e);
    }
    p0 = p1;
    p1 = p2;
  }
  return cnt;
}

// Lowest eigenvalue by 32-way multisection (warp 0 evaluates the Sturm counts; FP64 is a
// scarce pipe on this GPU, so fewer points per round cost less in total), then optionally
// the eigenvector by inverse iteration (thread 0, FP64, partial pivoting).
constexpr int MS_PTS = 32;
//
// SM_M > 0 (single-block callers): for m <= SM_M the tridiagonal, the elimination work and the
// vector live in static shared memory (7 * SM_M doubles) instead of global memory, which takes
// the inverse iteration's dependent loads off the L2 round trip. Batched callers keep SM_M = 0.
template <int SM_M = 0>
static __device__ double tridiag_lowest_block(const double* a_g, const double* b_g, int m, double* vec_g,
                                              double* work_g) {
  __shared__ double lo_s, hi_s;
  __shared__ int cnt_s[MS_PTS];
  const double* a = a_g;
  const double* b = b_g;
  double* vec = vec_g;
  double* work = work_g;
  bool in_smem = false;
  if constexpr (SM_M > 0) {
    __shared__ double s_ab[2 * SM_M];
    __shared__ double s_w[5 * SM_M];
    __shared__ double s_v[SM_M];
    if (m <= SM_M) {
      for (int i = threadIdx.x; i < m; i += blockDim.x) {
        s_ab[i] = a_g[i];
        s_ab[SM_M + i] = b_g[i];
      }
      __syncthreads();
      a = s_ab;
      b = s_ab + SM_M;
      work = s_w;
      if (vec_g) vec = s_v;
      in_smem = true;
    }
  }
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
  }
  __syncthreads();
  for (int round = 0; round < 16; ++round) {
    const double lo = lo_s, hi = hi_s;
    if (threadIdx.x < MS_PTS) {
      const double x = lo + (hi - lo) * (double)(threadIdx.x + 1) / (double)(MS_PTS + 1);
      cnt_s[threadIdx.x] = sturm_count(a, b, m, x);
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
    // inverse iteration: (T - ev I) y = v, Gaussian elimination with partial pivoting.
    // work: 5*m doubles (diag, super, super2, sub multipliers, pivot flags)
    double* dd = work;           // diagonal of U
    double* du = work + m;       // first super-diagonal of U
    double* du2 = work + 2 * m;  // second super-diagonal of U
    double* ml = work + 3 * m;   // multipliers
    double* pv = work + 4 * m;   // 1.0 if rows swapped at step i
    const double tiny = 1e-300 + 1e-15 * fmax(fabs(ev), 1.0) * 1e-3;
    for (int i = 0; i < m; ++i) vec[i] = 1.0 / sqrt((double)m) * (1.0 + 0.01 * (double)((i * 7919) % 13) / 13.0);
    for (int it = 0; it < 3; ++it) {
      // factor T - ev I (rebuilt each iteration; m is small)
      for (int i = 0; i < m; ++i) { dd[i] = a[i] - ev; du[i] = (i + 1 < m) ? b[i + 1] : 0.0; du2[i] = 0.0; }
      for (int i = 0; i < m - 1; ++i) {
        const double sub = b[i + 1];
        if (fabs(dd[i]) >= fabs(sub)) {
          pv[i] = 0.0;
          if (dd[i] == 0.0) dd[i] = tiny;
          const double l = sub / dd[i];
          ml[i] = l;
          dd[i + 1] -= l * du[i];
        } else {
          pv[i] = 1.0;
          const double l = dd[i] / sub;
          ml[i] = l;
          // swap rows i and i+1
          const double t0 = dd[i + 1], t1 = (i + 2 < m) ? du[i + 1] : 0.0;
          dd[i] = sub;
          const double odu = du[i];
          du[i] = t0;
          du2[i] = t1;
          dd[i + 1] = odu - l * t0;
          if (i + 2 < m) du[i + 1] = -l * t1;
        }
      }
      if (dd[m - 1] == 0.0) dd[m - 1] = tiny;
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
        vec[i] = s / dd[i];
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

}  // namespace ed
