// Dense symmetric eigensolver for batches of sector matrices, FP64 — the device replacement of
// numpy.linalg.eigh in cmpy/exactdiag.py:46-57 (solve_sector: every eigenpair of a sector's
// dense Hamiltonian) and the dense branch of exactdiag.py:24-43.
//
// For every matrix of the batch (order n_b <= n_max, row-major, overwritten):
// 1. Householder tridiagonalisation A = Q T Q^T. Step k takes the reflector of row k beyond
//    the diagonal, p = tau A22 v, w = p - (tau/2)(p.v) v, A22 -= v w^T + w v^T; the FP64 pipe
//    of this GPU (two FMAs per clock per SM) and the latency of its dependent FP64 chains bound
//    the O(n^3) parts. Three forms: orders <= 128 take every step in one CTA per matrix (block
//    barriers between the phases); orders <= 640, or batches that fill the GPU with clusters,
//    one thread-block cluster of 16 (else 8) CTAs per matrix (cluster barriers, p broadcast
//    through distributed shared memory); larger orders four launches per step over the whole
//    batch (reflector, matrix-vector product with one warp per row, the dot product, rank-2
//    update), so a single large matrix uses every SM. The rank-2 update is formed as
//    v_i w_j + w_i v_j with separately rounded products, so A stays exactly symmetric.
// 2. All eigenvalues of T by multisection on Sturm counts (a group of 1-32 lanes per
//    eigenvalue, sized to fill the GPU), ascending.
// 3. Eigenvectors of T by inverse iteration (Gaussian elimination with partial pivoting of
//    T - lambda I, start vectors that differ per index), one warp per cluster of eigenvalues
//    closer than 1e-7 max(1, |lambda|max) with its work arrays in shared memory: each iterate
//    is re-orthogonalised against the cluster's earlier members, so degenerate sector
//    eigenvalues (symmetries) give an orthonormal basis of the eigenspace.
// 4. Back-transformation y = Q z (one warp per eigenvector, reflectors in reverse order).
// Output: eigenvalues ascending, eigenvector i as row i of Z (Z = V^T).
#include <algorithm>
#include <atomic>
#include <cstdlib>
#include <cmath>
#include <vector>

#include <cooperative_groups.h>

#include "ed_common.cuh"
#include "ed_tridiag.cuh"

namespace ed {

namespace cg = cooperative_groups;

constexpr int DE_NT = 256;

struct DenseBatch {
  double* A;          // [B] matrices, row-major
  int64_t lda, sa;    // leading dimension, matrix stride
  const int* n;       // [B] orders
  double* d;          // [B][nmax] diagonal of T
  double* bet;        // [B][nmax] bet[i] couples i-1 and i (bet[0] = 0)
  double* tau;        // [B][nmax] reflector scales
  double* P;          // [B][nmax] p, then w
  double* glim;       // [B][2] Gershgorin bounds of T
  int nmax;
};

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// step k, one CTA per matrix: the reflector of row k (A[k][k+1..n)), kept in that row with its
// first element replaced by x0 - alpha; tau[k]; d[k] = A[k][k]; bet[k+1] = alpha
__global__ void __launch_bounds__(DE_NT) k_hh_column(DenseBatch m, int k) {
  __shared__ double sm[DE_NT / 32];
  const int b = blockIdx.x, n = m.n[b];
  if (k > n - 3) return;
  double* row = m.A + (size_t)b * m.sa + (size_t)k * m.lda;
  double s = 0.0;
  for (int i = k + 2 + threadIdx.x; i < n; i += DE_NT) s = fma(row[i], row[i], s);
  s = block_sum<DE_NT>(s, sm);
  if (threadIdx.x == 0) {
    const double x0 = row[k + 1];
    double t = 0.0, alpha = x0;
    if (s > 0.0) {
      const double nrm = sqrt(fma(x0, x0, s));
      alpha = x0 >= 0.0 ? -nrm : nrm;
      const double v0 = x0 - alpha;
      t = 2.0 / fma(v0, v0, s);
      row[k + 1] = v0;
    }
    m.tau[(size_t)b * m.nmax + k] = t;
    m.d[(size_t)b * m.nmax + k] = row[k];
    m.bet[(size_t)b * m.nmax + k + 1] = alpha;
  }
}

// step k: p_i = tau sum_{j>k} A[i][j] v_j for i > k (one warp per row)
__global__ void __launch_bounds__(DE_NT) k_hh_matvec(DenseBatch m, int k) {
  const int b = blockIdx.y, n = m.n[b];
  if (k > n - 3) return;
  const int i = k + 1 + blockIdx.x * (DE_NT / 32) + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (i >= n) return;
  const double t = m.tau[(size_t)b * m.nmax + k];
  const double* Ab = m.A + (size_t)b * m.sa;
  const double* v = Ab + (size_t)k * m.lda;
  const double* ai = Ab + (size_t)i * m.lda;
  double s = 0.0;
  for (int j = k + 1 + lane; j < n; j += 32) s = fma(ai[j], v[j], s);
  s = warp_sum_d(s);
  if (lane == 0) m.P[(size_t)b * m.nmax + i] = t * s;
}

// step k, one CTA per matrix: w = p - (tau/2)(p.v) v in place of p
__global__ void __launch_bounds__(DE_NT) k_hh_dot(DenseBatch m, int k) {
  __shared__ double sm[DE_NT / 32];
  __shared__ double kk;
  const int b = blockIdx.x, n = m.n[b];
  if (k > n - 3) return;
  const double* v = m.A + (size_t)b * m.sa + (size_t)k * m.lda;
  double* p = m.P + (size_t)b * m.nmax;
  double s = 0.0;
  for (int i = k + 1 + threadIdx.x; i < n; i += DE_NT) s = fma(p[i], v[i], s);
  s = block_sum<DE_NT>(s, sm);
  if (threadIdx.x == 0) kk = 0.5 * m.tau[(size_t)b * m.nmax + k] * s;
  __syncthreads();
  for (int i = k + 1 + threadIdx.x; i < n; i += DE_NT) p[i] = fma(-kk, v[i], p[i]);
}

// step k: A[i][j] -= v_i w_j + w_i v_j for i, j > k (products rounded separately: symmetric)
__global__ void __launch_bounds__(DE_NT) k_hh_update(DenseBatch m, int k) {
  const int b = blockIdx.y, n = m.n[b];
  if (k > n - 3) return;
  const int i = k + 1 + blockIdx.x;
  if (i >= n) return;
  if (m.tau[(size_t)b * m.nmax + k] == 0.0) return;
  double* Ab = m.A + (size_t)b * m.sa;
  const double* v = Ab + (size_t)k * m.lda;
  const double* w = m.P + (size_t)b * m.nmax;
  const double vi = v[i], wi = w[i];
  double* ai = Ab + (size_t)i * m.lda;
  for (int j = k + 1 + threadIdx.x; j < n; j += DE_NT)
    ai[j] = __dsub_rn(ai[j], __dadd_rn(__dmul_rn(vi, w[j]), __dmul_rn(wi, v[j])));
}

// All Householder steps of one matrix per thread-block cluster of CS CTAs (one per SM), for
// orders where per-step launches cost more than the FP64 work they spread: the matrix stays in
// global memory (L2-resident at these orders) and the phases of a step are separated by
// cluster barriers instead of launches. Row i > k of step k belongs to warp (i - k - 1) mod NW
// of the cluster (NW = 8 CS warps) for both the product p = tau A22 v and the rank-2 update.
// Each p_i is written into the shared memory of every CTA of the cluster (distributed shared
// memory), so after the barrier every CTA forms w = p - (tau/2)(p.v) v from local copies. The
// warp that owns row k + 1 (warp 0 of rank 0) forms reflector k + 1 as soon as it has updated
// that row, while the other rows are still being updated. A step takes two cluster barriers.
// Shared memory: p and w, 2 n_max doubles. Same arithmetic as the per-step kernels, except
// that the norm of the reflector row and the dot p.v are summed in another order.
template <int CS>
__global__ void __launch_bounds__(DE_NT) k_hh_cluster(DenseBatch m) {
  extern __shared__ double hsm[];
  __shared__ double red[DE_NT / 32];
  __shared__ double kk_s;
  cg::cluster_group cl = cg::this_cluster();
  const int b = blockIdx.y, n = m.n[b];
  double* ps = hsm;           // p, written by every CTA of the cluster
  double* ws = hsm + m.nmax;  // w
  const int rank = (int)cl.block_rank();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int gw = rank * (DE_NT / 32) + warp, NW = CS * (DE_NT / 32);
  double* Ab = m.A + (size_t)b * m.sa;
  double* tau = m.tau + (size_t)b * m.nmax;
  // reflector of row k (warp 0 of rank 0), as k_hh_column
  auto reflector = [&](int k) {
    double* row = Ab + (size_t)k * m.lda;
    double sq = 0.0;
    for (int i = k + 2 + lane; i < n; i += 32) sq = fma(row[i], row[i], sq);
    sq = warp_sum_d(sq);
    if (lane == 0) {
      const double x0 = row[k + 1];
      double t = 0.0, alpha = x0;
      if (sq > 0.0) {
        const double nrm = sqrt(fma(x0, x0, sq));
        alpha = x0 >= 0.0 ? -nrm : nrm;
        const double v0 = x0 - alpha;
        t = 2.0 / fma(v0, v0, sq);
        row[k + 1] = v0;
      }
      tau[k] = t;
      m.d[(size_t)b * m.nmax + k] = row[k];
      m.bet[(size_t)b * m.nmax + k + 1] = alpha;
    }
    __syncwarp();
  };
  if (n >= 3 && rank == 0 && warp == 0) reflector(0);
  cl.sync();
  for (int k = 0; k + 3 <= n; ++k) {
    const double t = tau[k];
    const double* v = Ab + (size_t)k * m.lda;
    // p_i = t sum_{j>k} A[i][j] v_j, one warp per row, into every CTA's copy of p
    for (int i = k + 1 + gw; i < n; i += NW) {
      const double* ai = Ab + (size_t)i * m.lda;
      double sp = 0.0;
      for (int j = k + 1 + lane; j < n; j += 32) sp = fma(ai[j], v[j], sp);
      sp = warp_sum_d(sp);
      if (lane < CS) *cl.map_shared_rank(ps + i, lane) = t * sp;
    }
    cl.sync();
    // w = p - (t/2)(p.v) v from the local copy of p
    double sd = 0.0;
    for (int i = k + 1 + threadIdx.x; i < n; i += DE_NT) sd = fma(ps[i], v[i], sd);
    sd = block_sum<DE_NT>(sd, red);
    if (threadIdx.x == 0) kk_s = 0.5 * t * sd;
    __syncthreads();
    const double kk = kk_s;
    for (int i = k + 1 + threadIdx.x; i < n; i += DE_NT) ws[i] = fma(-kk, v[i], ps[i]);
    __syncthreads();
    // A[i][j] -= v_i w_j + w_i v_j for i, j > k (products rounded separately: symmetric)
    for (int i = k + 1 + gw; i < n; i += NW) {
      if (t != 0.0) {
        double* ai = Ab + (size_t)i * m.lda;
        const double vi = v[i], wi = ws[i];
        for (int j = k + 1 + lane; j < n; j += 32)
          ai[j] = __dsub_rn(ai[j], __dadd_rn(__dmul_rn(vi, ws[j]), __dmul_rn(wi, v[j])));
      }
      if (i == k + 1 && k + 4 <= n) {  // warp 0 of rank 0: row k + 1 is final for this step
        __syncwarp();
        reflector(k + 1);
      }
    }
    cl.sync();
  }
}

// All Householder steps of one matrix per CTA (matrices of order <= DE_SMALL): the four phases
// of a step separated by block barriers instead of launches. One SM's FP64 pipe does the
// O(n^3) work, so this pays only for small orders: at n = 128 about 0.2 ms against ~1.5 ms of
// per-step launches; at n = 300 the per-step launches over every SM are faster.
constexpr int DE_SMALL = 128;
constexpr int DE_CLUSTER_MAX = 640;  // largest order reduced by one cluster per matrix when the batch is small
constexpr int DE_NTS = 1024;
__global__ void __launch_bounds__(DE_NTS) k_hh_small(DenseBatch m) {
  __shared__ double sm[DE_NTS / 32];
  __shared__ double sh_t, sh_k;
  const int b = blockIdx.x, n = m.n[b];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  double* Ab = m.A + (size_t)b * m.sa;
  double* p = m.P + (size_t)b * m.nmax;
  for (int k = 0; k + 3 <= n; ++k) {
    double* v = Ab + (size_t)k * m.lda;
    // reflector of row k
    double s = 0.0;
    for (int i = k + 2 + tid; i < n; i += DE_NTS) s = fma(v[i], v[i], s);
    s = block_sum<DE_NTS>(s, sm);
    if (tid == 0) {
      const double x0 = v[k + 1];
      double t = 0.0, alpha = x0;
      if (s > 0.0) {
        const double nrm = sqrt(fma(x0, x0, s));
        alpha = x0 >= 0.0 ? -nrm : nrm;
        const double v0 = x0 - alpha;
        t = 2.0 / fma(v0, v0, s);
        v[k + 1] = v0;
      }
      m.tau[(size_t)b * m.nmax + k] = t;
      m.d[(size_t)b * m.nmax + k] = v[k];
      m.bet[(size_t)b * m.nmax + k + 1] = alpha;
      sh_t = t;
    }
    __syncthreads();
    const double t = sh_t;
    if (t == 0.0) continue;  // uniform: nothing to transform at this step
    // p = tau A22 v, one warp per row
    for (int i = k + 1 + warp; i < n; i += DE_NTS / 32) {
      const double* ai = Ab + (size_t)i * m.lda;
      double acc = 0.0;
      for (int j = k + 1 + lane; j < n; j += 32) acc = fma(ai[j], v[j], acc);
      acc = warp_sum_d(acc);
      if (lane == 0) p[i] = t * acc;
    }
    __syncthreads();
    // w = p - (tau/2)(p.v) v
    double d = 0.0;
    for (int i = k + 1 + tid; i < n; i += DE_NTS) d = fma(p[i], v[i], d);
    d = block_sum<DE_NTS>(d, sm);
    if (tid == 0) sh_k = 0.5 * t * d;
    __syncthreads();
    const double kk = sh_k;
    for (int i = k + 1 + tid; i < n; i += DE_NTS) p[i] = fma(-kk, v[i], p[i]);
    __syncthreads();
    // A22 -= v w^T + w v^T (products rounded separately: A stays symmetric)
    const int r = n - k - 1;
    for (int e = tid; e < r * r; e += DE_NTS) {
      const int i = k + 1 + e / r, j = k + 1 + e % r;
      double* aij = Ab + (size_t)i * m.lda + j;
      *aij = __dsub_rn(*aij, __dadd_rn(__dmul_rn(v[i], p[j]), __dmul_rn(p[i], v[j])));
    }
    __syncthreads();
  }
}

// the last diagonal entries and the Gershgorin bounds of T (one thread per matrix)
// the last two entries of T, its Gershgorin bounds and the squared couplings (P is free after
// the reduction), one 128-thread block per matrix
__global__ void __launch_bounds__(128) k_hh_finish(DenseBatch m, int B) {
  __shared__ double slo[4], shi[4];
  const int b = blockIdx.x;
  if (b >= B) return;
  const int n = m.n[b];
  const double* Ab = m.A + (size_t)b * m.sa;
  double* d = m.d + (size_t)b * m.nmax;
  double* bt = m.bet + (size_t)b * m.nmax;
  if (threadIdx.x == 0) {
    bt[0] = 0.0;
    if (n >= 2) {
      d[n - 2] = Ab[(size_t)(n - 2) * m.lda + n - 2];
      bt[n - 1] = Ab[(size_t)(n - 2) * m.lda + n - 1];
    }
    d[n - 1] = Ab[(size_t)(n - 1) * m.lda + n - 1];
  }
  __syncthreads();
  double lo = d[0], hi = d[0];
  double* bb = m.P + (size_t)b * m.nmax;
  for (int i = threadIdx.x; i < n; i += 128) {
    const double r = (i > 0 ? fabs(bt[i]) : 0.0) + (i + 1 < n ? fabs(bt[i + 1]) : 0.0);
    lo = fmin(lo, d[i] - r);
    hi = fmax(hi, d[i] + r);
    bb[i] = bt[i] * bt[i];
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    lo = fmin(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    hi = fmax(hi, __shfl_xor_sync(0xffffffffu, hi, o));
  }
  if ((threadIdx.x & 31) == 0) {
    slo[threadIdx.x >> 5] = lo;
    shi[threadIdx.x >> 5] = hi;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    lo = fmin(fmin(slo[0], slo[1]), fmin(slo[2], slo[3]));
    hi = fmax(fmax(shi[0], shi[1]), fmax(shi[2], shi[3]));
    const double pad = 1e-12 * fmax(fabs(lo), fabs(hi)) + 1e-300;
    m.glim[2 * b] = lo - pad;
    m.glim[2 * b + 1] = hi + pad;
  }
}

// a given tridiagonal (alpha[0..m), beta[1..m)) as T of a one-matrix batch, and its Gershgorin
// bounds (one thread)
__global__ void k_tri_setup(DenseBatch m, const double* alpha, const double* beta, int n) {
  for (int i = 0; i < n; ++i) {
    m.d[i] = alpha[i];
    m.bet[i] = i > 0 ? beta[i] : 0.0;
  }
  double lo = m.d[0], hi = m.d[0];
  for (int i = 0; i < n; ++i) {
    const double r = (i > 0 ? fabs(m.bet[i]) : 0.0) + (i + 1 < n ? fabs(m.bet[i + 1]) : 0.0);
    lo = fmin(lo, m.d[i] - r);
    hi = fmax(hi, m.d[i] + r);
  }
  const double pad = 1e-12 * fmax(fabs(lo), fabs(hi)) + 1e-300;
  m.glim[0] = lo - pad;
  m.glim[1] = hi + pad;
  for (int i = 0; i < n; ++i) m.P[i] = m.bet[i] * m.bet[i];
}

// All eigenvalues of T by multisection: a group of P lanes (P a power of two <= 32) per
// eigenvalue. Each round the group counts the eigenvalues below P equidistant interior points
// of its bracket and keeps the gap where the count first reaches i + 1, so a bracket shrinks by
// P + 1 per round (P = 1 is bisection). The launch picks P so that the batch fills the GPU: a
// few eigenvalues take whole warps (fewer rounds of the latency-bound FP64 recurrence), many
// take single lanes (the FP64 pipe's throughput is then the bound). A bracket stops when a
// round makes no progress (its points round onto its ends); W = its midpoint, ascending in i.
// bb: the squared couplings (m.P after k_hh_finish / k_tri_setup).
__global__ void k_tri_eigvals_ms(DenseBatch m, int B, double* W, int P) {
  const int lane = threadIdx.x & 31;
  const int64_t gw = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int gpw = 32 / P, grp = lane / P, j = lane - grp * P;
  const int64_t e = gw * gpw + grp;  // eigenvalue slot over the batch (b, i)
  const int b = (int)(e / m.nmax), i = (int)(e % m.nmax);
  const int n = b < B ? m.n[b] : 0;
  bool done = !(b < B && i < n);  // uniform within a group
  const double* d = m.d + (size_t)(done ? 0 : b) * m.nmax;
  const double* bt = m.bet + (size_t)(done ? 0 : b) * m.nmax;
  const double* bb = m.P + (size_t)(done ? 0 : b) * m.nmax;
  double lo = done ? 0.0 : m.glim[2 * b], hi = done ? 0.0 : m.glim[2 * b + 1];
  const unsigned gmask = (P == 32) ? 0xffffffffu : (((1u << P) - 1u) << (grp * P));
  const double den = 1.0 / (double)(P + 1);
  for (int round = 0; round < 256; ++round) {
    if (__all_sync(0xffffffffu, done)) break;
    int cnt = 0;
    if (!done) cnt = sturm_count(d, bt, bb, n, lo + (hi - lo) * ((double)(j + 1) * den));
    const unsigned hit = __ballot_sync(0xffffffffu, !done && cnt >= i + 1) & gmask;
    if (!done) {
      const int t = hit ? (__ffs(hit) - 1 - grp * P) : P;  // first point with >= i + 1 below
      const double nlo = (t == 0) ? lo : lo + (hi - lo) * ((double)t * den);
      const double nhi = (t == P) ? hi : lo + (hi - lo) * ((double)(t + 1) * den);
      if (!(nlo > lo) && !(nhi < hi)) done = true;  // the points rounded onto the ends
      lo = nlo;
      hi = nhi;
    }
  }
  if (b < B && i < n && j == 0) W[(size_t)b * m.nmax + i] = 0.5 * (lo + hi);
}

// bytes of shared memory k_tri_eigvecs_warp takes for order n
__host__ __device__ inline size_t eigvec_smem(int n) { return (size_t)5 * n * sizeof(double) + (((size_t)n + 15) & ~(size_t)15); }

// The eigenvectors of T by inverse iteration as in k_tri_eigvecs, one warp (one block) per
// cluster of eigenvalues, with the elimination's work arrays and the iterate in shared memory
// (eigvec_smem(n) bytes): lane 0 runs the sequential elimination and the two triangular
// solves, the whole warp the start vector, the scaling, the re-orthogonalisation against the
// cluster's earlier members and the normalisation. Same clusters, same steps.
__global__ void __launch_bounds__(32) k_tri_eigvecs_warp(DenseBatch m, int B, const double* W, double* Z,
                                                         int64_t ldz, int64_t sz) {
  extern __shared__ __align__(16) double ws[];
  const int lane = threadIdx.x;
  const int64_t e = blockIdx.x;
  const int b = (int)(e / m.nmax), i0 = (int)(e % m.nmax);
  if (b >= B) return;
  const int n = m.n[b];
  if (i0 >= n) return;
  const double* w = W + (size_t)b * m.nmax;
  const double ctol = 1e-7 * fmax(1.0, fmax(fabs(w[0]), fabs(w[n - 1])));
  if (i0 > 0 && w[i0] - w[i0 - 1] <= ctol) return;  // not the first member of its cluster
  int i1 = i0 + 1;
  while (i1 < n && w[i1] - w[i1 - 1] <= ctol) ++i1;
  const double* a = m.d + (size_t)b * m.nmax;
  const double* bt = m.bet + (size_t)b * m.nmax;
  double* Zb = Z + (size_t)b * sz;
  double* dd = ws;
  double* du = ws + n;
  double* du2 = ws + 2 * n;
  double* ml = ws + 3 * n;
  double* vec = ws + 4 * n;
  unsigned char* pv = (unsigned char*)(ws + 5 * n);  // 1 if rows r and r + 1 were swapped
  for (int q = i0; q < i1; ++q) {
    const double ev = w[q];
    const double tiny = 1e-300 + 1e-18 * fmax(fabs(ev), 1.0);
    // start vector in [0.5, 1.5), a hash of (q, r): differs with the index
    for (int r = lane; r < n; r += 32) {
      uint32_t h = 2654435761u * (uint32_t)(q + 1) ^ (2246822519u * (uint32_t)(r + 1));
      h ^= h >> 15;
      h *= 2246822519u;
      h ^= h >> 13;
      vec[r] = 0.5 + (double)(h & 0xffffu) / 65536.0;
      dd[r] = a[r] - ev;
      du[r] = (r + 1 < n) ? bt[r + 1] : 0.0;
      du2[r] = 0.0;
    }
    __syncwarp();
    if (lane == 0) {
      for (int r = 0; r < n - 1; ++r) {
        const double sub = bt[r + 1];
        if (fabs(dd[r]) >= fabs(sub)) {
          pv[r] = 0;
          if (dd[r] == 0.0) dd[r] = tiny;
          const double rc = 1.0 / dd[r];
          const double l = sub * rc;
          ml[r] = l;
          dd[r + 1] -= l * du[r];
          dd[r] = rc;
        } else {
          pv[r] = 1;
          const double rc = 1.0 / sub;
          const double l = dd[r] * rc;
          ml[r] = l;
          const double t0 = dd[r + 1], t1 = (r + 2 < n) ? du[r + 1] : 0.0, odu = du[r];
          du[r] = t0;
          du2[r] = t1;
          dd[r + 1] = odu - l * t0;
          if (r + 2 < n) du[r + 1] = -l * t1;
          dd[r] = rc;
        }
      }
      if (dd[n - 1] == 0.0) dd[n - 1] = tiny;
      dd[n - 1] = 1.0 / dd[n - 1];
    }
    __syncwarp();
    for (int it = 0; it < 3; ++it) {
      if (lane == 0) {
        for (int r = 0; r < n - 1; ++r) {
          if (pv[r]) {
            const double t = vec[r];
            vec[r] = vec[r + 1];
            vec[r + 1] = t - ml[r] * vec[r];
          } else {
            vec[r + 1] -= ml[r] * vec[r];
          }
        }
        for (int r = n - 1; r >= 0; --r) {
          double sacc = vec[r];
          if (r + 1 < n) sacc -= du[r] * vec[r + 1];
          if (r + 2 < n) sacc -= du2[r] * vec[r + 2];
          vec[r] = sacc * dd[r];
        }
      }
      __syncwarp();
      double mx = 0.0;
      for (int r = lane; r < n; r += 32) mx = fmax(mx, fabs(vec[r]));
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
      const double sc = mx > 0.0 ? 1.0 / mx : 1.0;  // keep the iterate in range
      for (int r = lane; r < n; r += 32) vec[r] *= sc;
      __syncwarp();
      for (int pass = 0; pass < 2; ++pass)
        for (int l = i0; l < q; ++l) {
          const double* zl = Zb + (size_t)l * ldz;
          double sp = 0.0;
          for (int r = lane; r < n; r += 32) sp = fma(zl[r], vec[r], sp);
          sp = warp_sum_d(sp);
          for (int r = lane; r < n; r += 32) vec[r] = fma(-sp, zl[r], vec[r]);
          __syncwarp();
        }
      double nrm = 0.0;
      for (int r = lane; r < n; r += 32) nrm = fma(vec[r], vec[r], nrm);
      nrm = 1.0 / sqrt(warp_sum_d(nrm));
      for (int r = lane; r < n; r += 32) vec[r] *= nrm;
      __syncwarp();
    }
    double* zq = Zb + (size_t)q * ldz;
    for (int r = lane; r < n; r += 32) zq[r] = vec[r];
    __syncwarp();
  }
}

// The eigenvectors of T by inverse iteration, one thread per cluster of eigenvalues (values
// closer than ctol = 1e-7 max(1, |lambda|max) to their neighbour; most clusters are single
// values). Each member: Gaussian elimination with partial pivoting of T - lambda I (pivots
// kept as reciprocals), three solves from a start vector that differs with the index, each
// followed by modified Gram-Schmidt against the cluster's earlier members, so that the
// members of a degenerate eigenvalue converge to an orthonormal basis of its eigenspace.
// work: 5 n doubles of the thread.
__global__ void k_tri_eigvecs(DenseBatch m, int B, const double* W, double* Z, int64_t ldz, int64_t sz,
                              double* work) {
  const int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int b = (int)(g / m.nmax), i0 = (int)(g % m.nmax);
  if (b >= B) return;
  const int n = m.n[b];
  if (i0 >= n) return;
  const double* w = W + (size_t)b * m.nmax;
  const double ctol = 1e-7 * fmax(1.0, fmax(fabs(w[0]), fabs(w[n - 1])));
  if (i0 > 0 && w[i0] - w[i0 - 1] <= ctol) return;  // not the first member of its cluster
  int i1 = i0 + 1;
  while (i1 < n && w[i1] - w[i1 - 1] <= ctol) ++i1;
  const double* a = m.d + (size_t)b * m.nmax;
  const double* bt = m.bet + (size_t)b * m.nmax;
  double* Zb = Z + (size_t)b * sz;
  double* wk = work + ((size_t)b * m.nmax + i0) * 5 * (size_t)m.nmax;
  double* dd = wk;
  double* du = wk + n;
  double* du2 = wk + 2 * n;
  double* ml = wk + 3 * n;
  double* pv = wk + 4 * n;
  for (int q = i0; q < i1; ++q) {
    const double ev = w[q];
    double* vec = Zb + (size_t)q * ldz;
    const double tiny = 1e-300 + 1e-18 * fmax(fabs(ev), 1.0);
    uint32_t h = 2654435761u * (uint32_t)(q + 1);
    for (int r = 0; r < n; ++r) {
      h ^= h << 13;
      h ^= h >> 17;
      h ^= h << 5;
      vec[r] = 0.5 + (double)(h & 0xffffu) / 65536.0;
    }
    for (int r = 0; r < n; ++r) {
      dd[r] = a[r] - ev;
      du[r] = (r + 1 < n) ? bt[r + 1] : 0.0;
      du2[r] = 0.0;
    }
    for (int r = 0; r < n - 1; ++r) {
      const double sub = bt[r + 1];
      if (fabs(dd[r]) >= fabs(sub)) {
        pv[r] = 0.0;
        if (dd[r] == 0.0) dd[r] = tiny;
        const double rc = 1.0 / dd[r];
        const double l = sub * rc;
        ml[r] = l;
        dd[r + 1] -= l * du[r];
        dd[r] = rc;
      } else {
        pv[r] = 1.0;
        const double rc = 1.0 / sub;
        const double l = dd[r] * rc;
        ml[r] = l;
        const double t0 = dd[r + 1], t1 = (r + 2 < n) ? du[r + 1] : 0.0, odu = du[r];
        du[r] = t0;
        du2[r] = t1;
        dd[r + 1] = odu - l * t0;
        if (r + 2 < n) du[r + 1] = -l * t1;
        dd[r] = rc;
      }
    }
    if (dd[n - 1] == 0.0) dd[n - 1] = tiny;
    dd[n - 1] = 1.0 / dd[n - 1];
    for (int it = 0; it < 3; ++it) {
      for (int r = 0; r < n - 1; ++r) {
        if (pv[r] != 0.0) {
          const double t = vec[r];
          vec[r] = vec[r + 1];
          vec[r + 1] = t - ml[r] * vec[r];
        } else {
          vec[r + 1] -= ml[r] * vec[r];
        }
      }
      for (int r = n - 1; r >= 0; --r) {
        double sacc = vec[r];
        if (r + 1 < n) sacc -= du[r] * vec[r + 1];
        if (r + 2 < n) sacc -= du2[r] * vec[r + 2];
        vec[r] = sacc * dd[r];
      }
      double mx = 0.0;
      for (int r = 0; r < n; ++r) mx = fmax(mx, fabs(vec[r]));
      const double sc = mx > 0.0 ? 1.0 / mx : 1.0;  // keep the iterate in range
      for (int r = 0; r < n; ++r) vec[r] *= sc;
      for (int pass = 0; pass < 2; ++pass)
        for (int l = i0; l < q; ++l) {
          const double* zl = Zb + (size_t)l * ldz;
          double sp = 0.0;
          for (int r = 0; r < n; ++r) sp = fma(zl[r], vec[r], sp);
          for (int r = 0; r < n; ++r) vec[r] = fma(-sp, zl[r], vec[r]);
        }
      double nrm = 0.0;
      for (int r = 0; r < n; ++r) nrm = fma(vec[r], vec[r], nrm);
      nrm = 1.0 / sqrt(nrm);
      for (int r = 0; r < n; ++r) vec[r] *= nrm;
    }
  }
}

// y = Q z for every eigenvector (one warp per vector): reflectors n-3 .. 0
__global__ void __launch_bounds__(DE_NT) k_hh_back(DenseBatch m, int B, double* Z, int64_t ldz, int64_t sz) {
  const int64_t gw = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  const int b = (int)(gw / m.nmax), i = (int)(gw % m.nmax);
  if (b >= B) return;
  const int n = m.n[b];
  if (i >= n) return;
  const double* Ab = m.A + (size_t)b * m.sa;
  double* y = Z + (size_t)b * sz + (size_t)i * ldz;
  for (int k = n - 3; k >= 0; --k) {
    const double t = m.tau[(size_t)b * m.nmax + k];
    if (t == 0.0) continue;
    const double* v = Ab + (size_t)k * m.lda;
    double s = 0.0;
    for (int j = k + 1 + lane; j < n; j += 32) s = fma(v[j], y[j], s);
    s = t * warp_sum_d(s);
    for (int j = k + 1 + lane; j < n; j += 32) y[j] = fma(-s, v[j], y[j]);
    __syncwarp();
  }
}

// Householder reduction of the batch by one cluster of CS CTAs per matrix; false when the
// device cannot co-schedule such a cluster (the caller then launches per step)
template <int CS>
static bool hh_cluster_launch(const DeviceContext* ctx, DenseBatch m, int B, cudaStream_t s, ed_status* st) {
  static std::atomic<uint64_t> done{0}, usable{0};
  const uint64_t bit = 1ull << (ctx->device & 63);
  const size_t smem = (size_t)2 * m.nmax * sizeof(double);
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(CS, B);
  cfg.blockDim = dim3(DE_NT);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = CS;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  if (!(done.load() & bit)) {
    bool ok = true;
    if (CS > 8)
      ok = cudaFuncSetAttribute(k_hh_cluster<CS>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) == cudaSuccess;
    if (ok)
      ok = cudaFuncSetAttribute(k_hh_cluster<CS>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                ctx->smem_optin - 1024) == cudaSuccess;
    int nc = 0;
    if (ok) {
      cudaLaunchConfig_t probe = cfg;
      probe.gridDim = dim3(CS, 1);
      probe.dynamicSmemBytes = 48 * 1024;
      ok = cudaOccupancyMaxActiveClusters(&nc, k_hh_cluster<CS>, &probe) == cudaSuccess && nc >= 1;
    }
    (void)cudaGetLastError();
    if (ok) usable.fetch_or(bit);
    done.fetch_or(bit);
  }
  if (!(usable.load() & bit) || smem > 48 * 1024) return false;
  const cudaError_t e = cudaLaunchKernelEx(&cfg, k_hh_cluster<CS>, m);
  count_launches(1);
  *st = e == cudaSuccess ? ED_OK : cuda_fail(e, "k_hh_cluster");
  return true;
}

// lanes per eigenvalue of k_tri_eigvals_ms for E eigenvalues on a GPU with `sms` SMs: the
// largest power of two <= 32 that keeps the launch near four warps per SM
static int eigvals_lanes(int64_t E, int sms) {
  int P = 1;
  while (P < 32 && E * (int64_t)(2 * P) <= (int64_t)sms * 4 * 32) P *= 2;
  return P;
}

// eigenvalues (ascending) and eigenvectors of the B tridiagonals of m (d, bet, glim and the
// squared couplings in P set) into W [B][nmax] and Z (row i = eigenvector i). The eigenvectors
// take the shared-memory kernel when its arrays fit in one CTA's shared memory, else the
// kernel with global work arrays (5 nmax^2 doubles per matrix, allocated here).
static ed_status tridiag_eigenpairs(const DeviceContext* ctx, DenseBatch m, int B, double* W, double* Z, int64_t ldz,
                                    int64_t sz, cudaStream_t s) {
  const int64_t E = (int64_t)B * m.nmax;
  const int P = eigvals_lanes(E, ctx->num_sms);
  const int64_t warps = (E + (32 / P) - 1) / (32 / P);
  k_tri_eigvals_ms<<<(int)((warps + 3) / 4), 128, 0, s>>>(m, B, W, P);
  ED_CHECK_LAUNCH("k_tri_eigvals_ms");
  const size_t sm = eigvec_smem(m.nmax);
  if (sm + 1024 <= (size_t)ctx->smem_optin) {
    static std::atomic<uint64_t> done{0};
    const uint64_t bit = 1ull << (ctx->device & 63);
    if (sm > 48 * 1024 && !(done.load() & bit)) {
      ED_CUDA(cudaFuncSetAttribute(k_tri_eigvecs_warp, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   ctx->smem_optin - 1024));
      done.fetch_or(bit);
    }
    k_tri_eigvecs_warp<<<(unsigned)E, 32, sm, s>>>(m, B, W, Z, ldz, sz);
    ED_CHECK_LAUNCH("k_tri_eigvecs_warp");
    return ED_OK;
  }
  double* work = nullptr;
  ED_CUDA(cudaMallocAsync((void**)&work, (size_t)5 * E * m.nmax * sizeof(double), s));
  k_tri_eigvecs<<<(int)((E + 31) / 32), 32, 0, s>>>(m, B, W, Z, ldz, sz, work);
  const cudaError_t e = cudaGetLastError();
  count_launches(1);
  ED_CUDA(cudaFreeAsync(work, s));
  if (e != cudaSuccess) return cuda_fail(e, "k_tri_eigvecs");
  return ED_OK;
}

}  // namespace ed

using namespace ed;

extern "C" {

ED_API ed_status ed_dense_eigh_batch(double* d_a, int64_t lda, int64_t stride_a, const int* h_n, int B, int n_max,
                                     double* d_w, double* d_z, int64_t ldz, int64_t stride_z, ed_stream_t stream) {
  if (B < 1 || n_max < 1) return fail(ED_ERR_INVALID_ARG, "B and n_max must be >= 1");
  if (!d_a || !h_n || !d_w || !d_z) return fail(ED_ERR_INVALID_ARG, "null pointer");
  if (lda < n_max || stride_a < (int64_t)n_max * lda || ldz < n_max || stride_z < (int64_t)n_max * ldz)
    return fail(ED_ERR_INVALID_ARG, "leading dimensions or strides smaller than n_max");
  for (int b = 0; b < B; ++b)
    if (h_n[b] < 1 || h_n[b] > n_max) return fail(ED_ERR_INVALID_ARG, "matrix order outside [1, n_max]");
  DeviceContext* ctx;
  ED_TRY(device_context(&ctx));
  cudaStream_t s = as_stream(stream);
  const size_t nm = (size_t)B * n_max;
  double* buf = nullptr;
  int* dn = nullptr;
  // d, bet, tau, P (4 nm), Gershgorin (2 B)
  ED_CUDA(cudaMallocAsync((void**)&buf, (4 * nm + 2 * (size_t)B) * sizeof(double), s));
  ED_CUDA(cudaMallocAsync((void**)&dn, (size_t)B * sizeof(int), s));
  ED_CUDA(cudaMemcpyAsync(dn, h_n, (size_t)B * sizeof(int), cudaMemcpyHostToDevice, s));
  DenseBatch m;
  m.A = d_a;
  m.lda = lda;
  m.sa = stride_a;
  m.n = dn;
  m.d = buf;
  m.bet = buf + nm;
  m.tau = buf + 2 * nm;
  m.P = buf + 3 * nm;
  m.glim = buf + 4 * nm;
  m.nmax = n_max;
  ed_status st = ED_OK;
  const int rows_per = DE_NT / 32;
  if (n_max <= DE_SMALL) {
    // every step of each matrix in one CTA
    k_hh_small<<<B, DE_NTS, 0, s>>>(m);
    const cudaError_t e = cudaGetLastError();
    count_launches(1);
    if (e != cudaSuccess) st = cuda_fail(e, "Householder (one CTA per matrix)");
  }
  // orders above DE_SMALL: one cluster of 16 (else 8) CTAs per matrix while the clusters'
  // SMs do the FP64 work faster than per-step launches over every SM would (order <= 640, or a
  // batch that occupies the GPU with clusters); else four launches per step
  // CMPY_ED_HH_CLUSTER=16, 8 or 0 forces that cluster size or the per-step launches (for tests
  // and comparisons; read once per process)
  static int env_cluster = -2;
  if (env_cluster == -2) {
    const char* e = getenv("CMPY_ED_HH_CLUSTER");
    env_cluster = e ? atoi(e) : -1;
  }
  bool stepped = n_max <= DE_SMALL;
  const bool want = env_cluster >= 0 ? env_cluster > 0
                                     : (n_max <= DE_CLUSTER_MAX || (int64_t)B * 16 >= ctx->num_sms);
  if (!stepped && want) {
    if (env_cluster != 8) stepped = hh_cluster_launch<16>(ctx, m, B, s, &st);
    if (!stepped) stepped = hh_cluster_launch<8>(ctx, m, B, s, &st);
  }
  for (int k = 0; !stepped && k + 3 <= n_max && st == ED_OK; ++k) {
    const int rem = n_max - k - 1;
    k_hh_column<<<B, DE_NT, 0, s>>>(m, k);
    k_hh_matvec<<<dim3((rem + rows_per - 1) / rows_per, B), DE_NT, 0, s>>>(m, k);
    k_hh_dot<<<B, DE_NT, 0, s>>>(m, k);
    k_hh_update<<<dim3(rem, B), DE_NT, 0, s>>>(m, k);
    const cudaError_t e = cudaGetLastError();
    count_launches(4);
    if (e != cudaSuccess) st = cuda_fail(e, "Householder step");
  }
  if (st == ED_OK) {
    k_hh_finish<<<B, 128, 0, s>>>(m, B);
    const cudaError_t e = cudaGetLastError();
    count_launches(1);
    if (e != cudaSuccess) st = cuda_fail(e, "k_hh_finish");
  }
  if (st == ED_OK) st = tridiag_eigenpairs(ctx, m, B, d_w, d_z, ldz, stride_z, s);
  if (st == ED_OK) {
    const int64_t nt = (int64_t)B * n_max;
    k_hh_back<<<(int)((nt * 32 + DE_NT - 1) / DE_NT), DE_NT, 0, s>>>(m, B, d_z, ldz, stride_z);
    const cudaError_t e = cudaGetLastError();
    count_launches(1);
    if (e != cudaSuccess) st = cuda_fail(e, "k_hh_back");
  }
  cudaFreeAsync(buf, s);
  cudaFreeAsync(dn, s);
  return st;
}

ED_API ed_status ed_tridiag_eigh(const double* d_alpha, const double* d_beta, int m, double* d_w, double* d_z,
                                 int64_t ldz, ed_stream_t stream) {
  if (m < 1) return fail(ED_ERR_INVALID_ARG, "m must be >= 1");
  if (!d_alpha || !d_beta || !d_w || !d_z) return fail(ED_ERR_INVALID_ARG, "null pointer");
  if (ldz < m) return fail(ED_ERR_INVALID_ARG, "ldz smaller than m");
  DeviceContext* ctx;
  ED_TRY(device_context(&ctx));
  cudaStream_t s = as_stream(stream);
  double* buf = nullptr;
  int* dn = nullptr;
  ED_CUDA(cudaMallocAsync((void**)&buf, (4 * (size_t)m + 2) * sizeof(double), s));
  ED_CUDA(cudaMallocAsync((void**)&dn, sizeof(int), s));
  ED_CUDA(cudaMemcpyAsync(dn, &m, sizeof(int), cudaMemcpyHostToDevice, s));
  DenseBatch b{};
  b.n = dn;
  b.d = buf;
  b.bet = buf + m;
  b.tau = buf + 2 * (size_t)m;
  b.P = buf + 3 * (size_t)m;
  b.glim = buf + 4 * (size_t)m;
  b.nmax = m;
  k_tri_setup<<<1, 1, 0, s>>>(b, d_alpha, d_beta, m);
  const cudaError_t e = cudaGetLastError();
  count_launches(1);
  ed_status st = e != cudaSuccess ? cuda_fail(e, "k_tri_setup") : ED_OK;
  if (st == ED_OK) st = tridiag_eigenpairs(ctx, b, 1, d_w, d_z, ldz, (int64_t)m * ldz, s);
  cudaFreeAsync(buf, s);
  cudaFreeAsync(dn, s);
  return st;
}

}  // extern "C"
