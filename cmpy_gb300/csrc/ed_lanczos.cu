// Device Lanczos: the ground state that cmpy obtains from ARPACK eigsh(k=1, which="SA")
// (cmpy/exactdiag.py:24-43) and the Lanczos coefficients of cmpy/exactdiag.py:324-375,
// run on the GPU. The recurrence's scalars (alpha, beta, norms, flags) stay in device memory
// and the host enqueues the steps without waiting; the convergence tests and the final
// tridiagonal eigenpair also run on the device (ed_lzcheck.cuh), so the host waits once, at
// the end.
//
// Reductions are deterministic: each block writes a partial, the last block to arrive
// (atomic ticket, no waiting) sums the partials in block order.
#include <algorithm>
#include <cmath>
#include <vector>

#include "ed_lzcheck.cuh"
#include "ed_plan.cuh"
#include "ed_tridiag.cuh"

namespace ed {

constexpr int LZ_NT = 256;

struct LzState {
  int stop;          // 0 running, 1 converged, 2 invariant subspace
  int steps;         // size m of the tridiagonal matrix once stopped
  int status;
  int pad;
  double e_prev;     // last convergence-check energy
  double energy;
  double residual;
  double nrm2;       // scratch: last norm^2
  unsigned int ticket[8];
};

__device__ __forceinline__ bool lz_stopped(const LzState* st) { return *(volatile const int*)&st->stop != 0; }

// Last-block detection; every thread of the block gets the answer.
__device__ __forceinline__ bool last_block(unsigned int* ticket) {
  __shared__ bool am_last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) am_last = (atomicAdd(ticket, 1u) == gridDim.x - 1);
  __syncthreads();
  if (am_last) __threadfence();
  return am_last;
}

// sum partials[0..n) with the whole block (NT threads), in a fixed order
template <int NT = LZ_NT>
__device__ double block_sum_array(const double* p, int n, double* smem) {
  double v = 0.0;
  for (int i = threadIdx.x; i < n; i += NT) v += ((volatile const double*)p)[i];
  return block_sum<NT>(v, smem);
}

// ---- start vector ------------------------------------------------------------------------
__device__ __forceinline__ uint64_t splitmix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

// uniform(0,1) like the reference's np.random.uniform(0, 1) start (exactdiag.py:326), seeded
__global__ void k_random_start(double* v, int64_t n, uint64_t seed) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    v[i] = (double)(splitmix64(seed * 0x100000001B3ull + (uint64_t)i) >> 11) * 0x1.0p-53 + 0x1.0p-54;
}

// out = <a, b> (or ||a||^2 with b == a); result -> *res (and optionally its sqrt -> *res_sqrt)
__global__ void k_dot(const double* __restrict__ a, const double* __restrict__ b, int64_t n, double* partial,
                      LzState* st, int tk, double* res, double* res_sqrt, const int* stop) {
  if (stop && *(volatile const int*)stop) return;
  __shared__ double sm[LZ_NT / 32];
  double v = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)LZ_NT + threadIdx.x; i < n; i += (int64_t)gridDim.x * LZ_NT)
    v = fma(a[i], b[i], v);
  v = block_sum<LZ_NT>(v, sm);
  if (threadIdx.x == 0) partial[blockIdx.x] = v;
  if (last_block(&st->ticket[tk])) {
    const double s = block_sum_array(partial, gridDim.x, sm);
    if (threadIdx.x == 0) {
      *res = s;
      if (res_sqrt) *res_sqrt = sqrt(s);
      st->ticket[tk] = 0;
    }
  }
}

// v *= 1/ *scale (scale read from device memory); out may equal v
__global__ void k_scale(const double* __restrict__ v, double* __restrict__ out, int64_t n, const double* scale,
                        const int* stop) {
  if (stop && *(volatile const int*)stop) return;
  const double s = 1.0 / *scale;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = v[i] * s;
}

// w -= alpha*q + beta*qprev; norm^2 -> st->nrm2; when final (no reorth) also beta_{k+1}
// and the breakdown test.
__global__ void k_lz_update(double* __restrict__ w, const double* __restrict__ q, const double* __restrict__ qp,
                            int64_t n, const double* alpha_k, const double* beta_k, double* partial, LzState* st,
                            double* beta_next, int k, int final_norm) {
  if (lz_stopped(st)) return;
  __shared__ double sm[LZ_NT / 32];
  const double a = *alpha_k, b = *beta_k;
  double v = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)LZ_NT + threadIdx.x; i < n; i += (int64_t)gridDim.x * LZ_NT) {
    double x = w[i] - a * q[i];
    if (qp) x -= b * qp[i];
    w[i] = x;
    v = fma(x, x, v);
  }
  v = block_sum<LZ_NT>(v, sm);
  if (threadIdx.x == 0) partial[blockIdx.x] = v;
  if (last_block(&st->ticket[1])) {
    const double s = block_sum_array(partial, gridDim.x, sm);
    if (threadIdx.x == 0) {
      st->nrm2 = s;
      if (final_norm) {
        const double bn = sqrt(s);
        *beta_next = bn;
        const double scale = fmax(fabs(a), fmax(b, 1e-300));
        if (!(bn > 1e-13 * scale)) { st->steps = k + 1; st->stop = 2; }
      }
      st->ticket[1] = 0;
    }
  }
}

// ---- full reorthogonalisation: classical Gram-Schmidt against Q[0..m) -----------------------
// h = Q^T w, pass 1: block b owns the element chunk [b*ch, (b+1)*ch) (ch = ceil(n / gridDim)) and
// writes partial[j*gridDim + b] for every vector j. FP64 is the narrow pipe on this part, so the
// kernel keeps its FP64 work close to one FMA per element and vector:
//  * one-tile chunks (ch <= RD_TILE, the usual case): w stays in registers; a warp takes four
//    vectors at a time, issues each vector's RD_EPL loads before its FMAs (two chains per lane),
//    and folds the four per-lane sums with one transposing butterfly (6 adds per lane for four
//    dot products instead of 4 x 5);
//  * longer chunks: one vector per warp, tiles of RD_TILE, q and w loads in flight together.
// The partials are summed in block order by k_multidot_reduce (one block per vector).
constexpr int RD_EPL = 20;  // even (two FMA chains); 640-element tiles, two CTAs per SM
constexpr int RD_TILE = 32 * RD_EPL;
__device__ __forceinline__ double rd_tile_dot(const double* __restrict__ q, const double (&wr)[RD_EPL], int64_t i0,
                                              int64_t i1, int lane) {
  double qv[RD_EPL];
#pragma unroll
  for (int e = 0; e < RD_EPL; ++e) {
    const int64_t i = i0 + lane + 32 * e;
    qv[e] = i < i1 ? __ldg(q + i) : 0.0;
  }
  double a0 = 0.0, a1 = 0.0;
#pragma unroll
  for (int e = 0; e < RD_EPL; e += 2) {
    a0 = fma(qv[e], wr[e], a0);
    a1 = fma(qv[e + 1], wr[e + 1], a1);
  }
  return a0 + a1;
}
__global__ void __launch_bounds__(LZ_NT, 2) k_multidot(const double* __restrict__ Q, int64_t ldq, int m,
                                                    const double* __restrict__ w, int64_t n, double* partial,
                                                    LzState* st) {
  if (lz_stopped(st)) return;
  const int64_t ch = (n + gridDim.x - 1) / gridDim.x;
  const int64_t i0 = (int64_t)blockIdx.x * ch;
  const int64_t i1 = min(n, i0 + ch);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  if (i1 - i0 <= RD_TILE) {
    double wr[RD_EPL];
#pragma unroll
    for (int e = 0; e < RD_EPL; ++e) {
      const int64_t i = i0 + lane + 32 * e;
      wr[e] = i < i1 ? __ldg(w + i) : 0.0;
    }
    for (int j0 = 4 * warp; j0 < m; j0 += 4 * nw) {
      double p[4];
#pragma unroll
      for (int v = 0; v < 4; ++v)  // j0 + v < m is uniform across the warp
        p[v] = (j0 + v < m) ? rd_tile_dot(Q + (int64_t)(j0 + v) * ldq, wr, i0, i1, lane) : 0.0;
      // butterfly over the four sums: after the xor-16 and xor-8 exchanges each lane holds one
      // vector's partial (vector 2*bit4 + bit3 of the lane id), then three more halvings
      const bool hi = lane & 16, b8 = lane & 8;
      const double k0 = (hi ? p[2] : p[0]) + __shfl_xor_sync(0xffffffffu, hi ? p[0] : p[2], 16);
      const double k1 = (hi ? p[3] : p[1]) + __shfl_xor_sync(0xffffffffu, hi ? p[1] : p[3], 16);
      double t = (b8 ? k1 : k0) + __shfl_xor_sync(0xffffffffu, b8 ? k0 : k1, 8);
      t += __shfl_xor_sync(0xffffffffu, t, 4);
      t += __shfl_xor_sync(0xffffffffu, t, 2);
      t += __shfl_xor_sync(0xffffffffu, t, 1);
      const int v = (hi ? 2 : 0) + (b8 ? 1 : 0);
      if ((lane & 7) == 0 && j0 + v < m) partial[(int64_t)(j0 + v) * gridDim.x + blockIdx.x] = t;
    }
  } else {
    for (int j = warp; j < m; j += nw) {
      const double* q = Q + (int64_t)j * ldq;
      double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
      for (int64_t t0 = i0; t0 < i1; t0 += RD_TILE) {
        double qv[RD_EPL], wv[RD_EPL];
#pragma unroll
        for (int e = 0; e < RD_EPL; ++e) {
          const int64_t i = t0 + lane + 32 * e;
          const bool ok = i < i1;
          qv[e] = ok ? __ldg(q + i) : 0.0;
          wv[e] = ok ? __ldg(w + i) : 0.0;
        }
#pragma unroll
        for (int e = 0; e < RD_EPL; e += 4) {
          a0 = fma(qv[e], wv[e], a0);
          a1 = fma(qv[e + 1], wv[e + 1], a1);
          a2 = fma(qv[e + 2], wv[e + 2], a2);
          a3 = fma(qv[e + 3], wv[e + 3], a3);
        }
      }
      double acc = (a0 + a1) + (a2 + a3);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
      if (lane == 0) partial[(int64_t)j * gridDim.x + blockIdx.x] = acc;
    }
  }
}

// h = Q^T w, pass 2: block j sums partial[j*nb + b] over b in a fixed order (deterministic)
__global__ void k_multidot_reduce(const double* __restrict__ partial, int nb, double* h, const LzState* st) {
  if (lz_stopped(st)) return;
  const int j = blockIdx.x, lane = threadIdx.x;
  double acc = 0.0;
  for (int b = lane; b < nb; b += 32) acc += partial[(int64_t)j * nb + b];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if (lane == 0) h[j] = acc;
}

// w -= sum_j h[j] Q[j]; optionally accumulates ||w||^2 and finalises beta_{k+1}. Each thread owns
// two elements per grid-stride step (i and i + RA_NT, each coalesced across the warp), so one
// shared-memory read of h_j serves two FMAs, and walks j in groups of RA_J: the 2*RA_J loads of a
// group are issued before their FMAs (four chains per element). Small CTAs (2*RA_NT elements)
// spread the last partial wave evenly over the SMs. m <= RO_MAX (checked by the host).
constexpr int RO_MAX = 1024;
constexpr int RA_J = 8;
constexpr int RA_NT = 128;
__global__ void __launch_bounds__(RA_NT, 6) k_multiaxpy(const double* __restrict__ Q, int64_t ldq, int m,
                                                     const double* __restrict__ h, double* __restrict__ w, int64_t n,
                                                     double* partial, LzState* st, double* beta_next, int k,
                                                     int final_norm, const double* alpha_k) {
  if (lz_stopped(st)) return;
  __shared__ double sm[RA_NT / 32];
  __shared__ double hs[RO_MAX + RA_J];
  for (int j = threadIdx.x; j < m + RA_J; j += RA_NT) hs[j] = j < m ? h[j] : 0.0;
  __syncthreads();
  double v = 0.0;
  const int mf = m - m % RA_J;  // vectors in full groups
  const int64_t step = (int64_t)gridDim.x * 2 * RA_NT;
  for (int64_t ia = blockIdx.x * (int64_t)(2 * RA_NT) + threadIdx.x; ia < n; ia += step) {
    const int64_t ib = ia + RA_NT;
    const bool hb = ib < n;
    const int64_t ibc = hb ? ib : ia;  // a valid address for the second element's loads
    double xa0 = w[ia], xa1 = 0.0, xa2 = 0.0, xa3 = 0.0;
    double xb0 = hb ? w[ib] : 0.0, xb1 = 0.0, xb2 = 0.0, xb3 = 0.0;
    for (int j = 0; j < mf; j += RA_J) {
      double qa[RA_J], qb[RA_J];
#pragma unroll
      for (int e = 0; e < RA_J; ++e) {
        qa[e] = __ldg(Q + (int64_t)(j + e) * ldq + ia);
        qb[e] = __ldg(Q + (int64_t)(j + e) * ldq + ibc);
      }
#pragma unroll
      for (int e = 0; e < RA_J; e += 4) {
        const double h0 = -hs[j + e], h1 = -hs[j + e + 1], h2 = -hs[j + e + 2], h3 = -hs[j + e + 3];
        xa0 = fma(h0, qa[e], xa0);
        xa1 = fma(h1, qa[e + 1], xa1);
        xa2 = fma(h2, qa[e + 2], xa2);
        xa3 = fma(h3, qa[e + 3], xa3);
        xb0 = fma(h0, qb[e], xb0);
        xb1 = fma(h1, qb[e + 1], xb1);
        xb2 = fma(h2, qb[e + 2], xb2);
        xb3 = fma(h3, qb[e + 3], xb3);
      }
    }
    for (int j = mf; j < m; ++j) {
      xa0 = fma(-hs[j], __ldg(Q + (int64_t)j * ldq + ia), xa0);
      xb0 = fma(-hs[j], __ldg(Q + (int64_t)j * ldq + ibc), xb0);
    }
    const double xa = (xa0 + xa1) + (xa2 + xa3);
    w[ia] = xa;
    v = fma(xa, xa, v);
    if (hb) {
      const double xb = (xb0 + xb1) + (xb2 + xb3);
      w[ib] = xb;
      v = fma(xb, xb, v);
    }
  }
  v = block_sum<RA_NT>(v, sm);
  if (threadIdx.x == 0) partial[blockIdx.x] = v;
  if (last_block(&st->ticket[3])) {
    const double s = block_sum_array<RA_NT>(partial, gridDim.x, sm);
    if (threadIdx.x == 0) {
      st->nrm2 = s;
      if (final_norm) {
        const double bn = sqrt(s);
        *beta_next = bn;
        const double scale = fmax(fabs(*alpha_k), 1e-300);
        if (!(bn > 1e-13 * scale)) { st->steps = k + 1; st->stop = 2; }
      }
      st->ticket[3] = 0;
    }
  }
}

// B tridiagonals, one block each: problem b has alpha[b*lda ..], beta[b*ldb ..], size m[b]
__global__ void k_tridiag_batch(const double* alpha, int lda, const double* beta, int ldb, const int* m, double* value,
                                double* vec, int ldv, double* work) {
  const int b = blockIdx.x;
  if (m[b] < 1) {  // an empty run (zero start vector)
    if (threadIdx.x == 0) value[b] = 0.0;
    return;
  }
  const double e = tridiag_lowest_block<512>(alpha + (size_t)b * lda, beta + (size_t)b * ldb, m[b],
                                             vec ? vec + (size_t)b * ldv : nullptr, work + (size_t)b * 5 * ldv);
  if (threadIdx.x == 0) value[b] = e;
}

__global__ void k_tridiag_pinv_batch(const double* alpha, int lda, const double* beta, int ldb, const int* m,
                                     const double* e0, const double* c, int ldc, const double* rhs, double* out,
                                     int ldr, double* work) {
  const int b = blockIdx.x;
  if (m[b] < 1) return;
  tridiag_pinv_solve(alpha + (size_t)b * lda, beta + (size_t)b * ldb, m[b], e0[b], c + (size_t)b * ldc,
                     rhs + (size_t)b * ldr, out + (size_t)b * ldr, work + (size_t)b * 5 * ldr);
}

__global__ void k_tridiag(const double* alpha, const double* beta, int m, double* value, double* vec, double* work) {
  const double e = tridiag_lowest_block<512>(alpha, beta, m, vec, work);
  if (threadIdx.x == 0) *value = e;
}

// psi = sum_{k<m} c_k Q[k]
__global__ void k_ritz(const double* __restrict__ Q, int64_t ldq, const double* __restrict__ c, const LzState* st,
                       double* __restrict__ out, int64_t n) {
  const int m = st->steps;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    double x = 0.0;
    for (int k = 0; k < m; ++k) x = fma(c[k], Q[(int64_t)k * ldq + i], x);
    out[i] = x;
  }
}

// ---- workspace layout ----------------------------------------------------------------------
struct LzLayout {
  int64_t nvec;      // vectors in the basis store
  size_t off_basis, off_w, off_partial, off_h, off_c, off_work, off_state, off_scalars, off_tri, total;
  int nparts;
};

static size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

static LzLayout lz_layout(int64_t D, int K, bool store, int nparts) {
  LzLayout L;
  L.nparts = nparts;
  L.nvec = store ? (int64_t)K + 1 : 3;
  size_t o = 0;
  L.off_basis = o; o = align256(o + (size_t)L.nvec * D * sizeof(double));
  L.off_w = o; o = align256(o + (size_t)D * sizeof(double));
  L.off_partial = o; o = align256(o + (size_t)nparts * (K + 2) * sizeof(double));
  L.off_h = o; o = align256(o + (size_t)(K + 2) * sizeof(double));
  L.off_c = o; o = align256(o + (size_t)(K + 2) * sizeof(double));
  L.off_work = o; o = align256(o + (size_t)5 * (K + 2) * sizeof(double));
  L.off_scalars = o; o = align256(o + 8 * sizeof(double));
  L.off_state = o; o = align256(o + sizeof(LzState));
  L.off_tri = o; o = align256(o + sizeof(TriResult));
  L.total = o;
  return L;
}

static int lz_parts(const ed_plan_s* p, int64_t D) {
  return (int)std::max<int64_t>(1, std::min<int64_t>((D + LZ_NT - 1) / LZ_NT, (int64_t)p->ctx->num_sms * 4));
}

}  // namespace ed

using namespace ed;

extern "C" {

// fixed-point vectors: automatic when the sector allows them and no reorthogonalisation
static ed_status use_fixed(const ed_plan_s* p, const ed_lanczos_params* prm, bool* out) {
  const bool ok = p->bfp.eligible && !prm->reorth;
  if (prm->arithmetic == 2 && !ok)
    return fail(ED_ERR_INVALID_ARG, "fixed-point Lanczos needs a fixed-point sector and reorth = 0");
  *out = ok && prm->arithmetic != 1;
  return ED_OK;
}

ED_API ed_status ed_lanczos_workspace(ed_plan p, const ed_lanczos_params* prm, size_t* bytes) {
  ED_TRY(check_plan(p));
  if (!prm || !bytes) return fail(ED_ERR_INVALID_ARG, "null argument");
  if (prm->max_steps < 1 || prm->max_steps > 4096) return fail(ED_ERR_INVALID_ARG, "max_steps must be in [1, 4096]");
  bool fixed = false;
  ED_TRY(use_fixed(p, prm, &fixed));
  const bool store = prm->want_vector || prm->reorth;
  *bytes = fixed ? bfp_workspace_bytes(p, prm->max_steps, store)
                 : lz_layout(p->dim, prm->max_steps, store, lz_parts(p, p->dim)).total;
  return ED_OK;
}

// normalises d_evec in place (FP64)
static ed_status normalise(const ed_plan_s* p, double* v, int64_t D, double* part, double* scal, LzState* st,
                           cudaStream_t s) {
  k_dot<<<lz_parts(p, D), LZ_NT, 0, s>>>(v, v, D, part, st, 0, scal, scal + 1, nullptr);
  k_scale<<<grid_for(D, 256, p->ctx->num_sms * 8), 256, 0, s>>>(v, v, D, scal + 1, nullptr);
  ED_CHECK_LAUNCH_N("normalise", 2);
  return ED_OK;
}

ED_API ed_status ed_lanczos(ed_plan p, const ed_lanczos_params* prm, const double* d_v0, void* d_work, size_t work_bytes,
                            double* d_alpha, double* d_beta, double* d_evec, ed_lanczos_result* res,
                            ed_stream_t stream) {
  ED_TRY(check_plan(p));
  if (!prm || !res || !d_alpha || !d_beta) return fail(ED_ERR_INVALID_ARG, "null argument");
  const int K = prm->max_steps;
  if (K < 1 || K > 4096) return fail(ED_ERR_INVALID_ARG, "max_steps must be in [1, 4096]");
  const int64_t D = p->dim;
  if (D < 1) return fail(ED_ERR_INVALID_ARG, "empty sector");
  if (prm->want_vector && !d_evec) return fail(ED_ERR_INVALID_ARG, "want_vector needs d_evec");
  bool fixed = false;
  ED_TRY(use_fixed(p, prm, &fixed));
  if (fixed) {
    const size_t need = bfp_workspace_bytes(p, K, prm->want_vector != 0);
    if (!d_work || work_bytes < need) return fail(ED_ERR_INVALID_ARG, "workspace too small (see ed_lanczos_workspace)");
    cudaStream_t s = as_stream(stream);
    // FP64 start vector: the caller's, else a seeded uniform(0,1) one generated into d_evec
    // (overwritten by the Ritz vector at the end) or into a temporary buffer
    const double* v0 = d_v0;
    double* tmp_alloc = nullptr;
    if (!v0) {
      double* tmp = d_evec;
      if (!tmp) {
        ED_CUDA(cudaMallocAsync(&tmp_alloc, D * sizeof(double), s));
        tmp = tmp_alloc;
      }
      k_random_start<<<grid_for(D, 256, p->ctx->num_sms * 8), 256, 0, s>>>(tmp, D, prm->seed);
      ED_CHECK_LAUNCH("k_random_start");
      v0 = tmp;
    }
    const ed_status rs = bfp_lanczos(p, prm, v0, d_work, d_alpha, d_beta, d_evec, res, s, nullptr);
    if (tmp_alloc) cudaFreeAsync(tmp_alloc, s);
    ED_TRY(rs);
    if (d_evec) {
      double* scratch = nullptr;
      ED_CUDA(cudaMallocAsync(&scratch, (lz_parts(p, D) + 8) * sizeof(double) + sizeof(LzState) + 256, s));
      LzState* st = (LzState*)((char*)scratch + ((lz_parts(p, D) + 8) * sizeof(double) + 255) / 256 * 256);
      ED_CUDA(cudaMemsetAsync(st, 0, sizeof(LzState), s));
      ed_status r = normalise(p, d_evec, D, scratch, scratch + lz_parts(p, D), st, s);
      ED_CUDA(cudaStreamSynchronize(s));
      cudaFreeAsync(scratch, s);
      ED_TRY(r);
    }
    return ED_OK;
  }
  const bool store = prm->want_vector || prm->reorth;
  const int nparts = lz_parts(p, D);
  const LzLayout L = lz_layout(D, K, store, nparts);
  if (!d_work || work_bytes < L.total) return fail(ED_ERR_INVALID_ARG, "workspace too small (see ed_lanczos_workspace)");
  if (prm->reorth && K + 1 > 1024) return fail(ED_ERR_INVALID_ARG, "reorth supports max_steps <= 1023");
  cudaStream_t s = as_stream(stream);
  char* base = (char*)d_work;
  double* Q = (double*)(base + L.off_basis);
  double* w = (double*)(base + L.off_w);
  double* part = (double*)(base + L.off_partial);
  double* h = (double*)(base + L.off_h);
  double* c = (double*)(base + L.off_c);
  double* scal = (double*)(base + L.off_scalars);
  LzState* st = (LzState*)(base + L.off_state);
  double* twork = (double*)(base + L.off_work);
  TriResult* tri = (TriResult*)(base + L.off_tri);
  ED_CUDA(cudaMemsetAsync(st, 0, sizeof(LzState), s));
  ED_CUDA(cudaMemsetAsync(tri, 0, sizeof(TriResult), s));
  ED_CUDA(cudaMemsetAsync(d_alpha, 0, K * sizeof(double), s));
  ED_CUDA(cudaMemsetAsync(d_beta, 0, (K + 1) * sizeof(double), s));
  const int gv = nparts;
  const int gs = grid_for(D, 256, p->ctx->num_sms * 8);
  // reorthogonalisation dots: element chunks of one tile (RD_TILE) per block where the
  // partial store (nparts blocks) allows it
  const int gmd = (int)std::max<int64_t>(1, std::min<int64_t>((D + RD_TILE - 1) / RD_TILE, nparts));
  // reorthogonalisation axpy: one CTA per 2*RA_NT elements, at most 2*nparts CTAs (their norm
  // partials fit the partial store, which holds nparts * (K + 2) values)
  const int gax = (int)std::max<int64_t>(1, std::min<int64_t>((D + 2 * RA_NT - 1) / (2 * RA_NT), 2 * (int64_t)nparts));
  auto qv = [&](int k) -> double* { return Q + (int64_t)(store ? k : (k % 3)) * D; };
  // q_0
  if (d_v0) {
    ED_CUDA(cudaMemcpyAsync(qv(0), d_v0, D * sizeof(double), cudaMemcpyDeviceToDevice, s));
  } else {
    k_random_start<<<gs, 256, 0, s>>>(qv(0), D, prm->seed);
    ED_CHECK_LAUNCH("k_random_start");
  }
  k_dot<<<gv, LZ_NT, 0, s>>>(qv(0), qv(0), D, part, st, 0, scal, scal + 1, nullptr);
  k_scale<<<gs, 256, 0, s>>>(qv(0), qv(0), D, scal + 1, nullptr);
  ED_CHECK_LAUNCH_N("lanczos start", 2);
  {
    double n2 = 0.0;
    ED_CUDA(cudaMemcpyAsync(&n2, scal, sizeof(double), cudaMemcpyDeviceToHost, s));
    ED_CUDA(cudaStreamSynchronize(s));
    if (!std::isfinite(n2)) return fail(ED_ERR_NONFINITE, "start vector is not finite");
    if (n2 == 0.0) return fail(ED_ERR_ZERO_VECTOR, "start vector has zero norm");
  }
  // optional per-matvec CUDA events on the launching stream
  std::vector<cudaEvent_t> ev;
  if (prm->profile) {
    ev.resize(2 * (size_t)K);
    for (auto& e : ev) ED_CUDA(cudaEventCreate(&e));
  }
  const int* stopf = &st->stop;
  // the Krylov dimension cannot exceed D; without reorthogonalisation rounding would
  // otherwise keep beta alive past it
  const int Km = (int)std::min<int64_t>(K, D);
  // convergence tests on a side stream and the final eigenpair, on the device (ed_lzcheck.cuh)
  const bool checks = prm->check_every > 0 && prm->tol > 0.0;
  SideChecks chk;
  ED_TRY(chk.init(checks ? Km / prm->check_every + 1 : 0));
  int launched = 0;
  for (int k = 0; k < Km; ++k) {
    if (checks && chk.stopped()) break;
    double* q = qv(k);
    double* qp = k > 0 ? qv(k - 1) : nullptr;
    if (prm->profile) ED_CUDA(cudaEventRecord(ev[2 * k], s));
    ED_TRY(matvec_f64(p, q, w, 1, D, s, stopf));
    if (prm->profile) ED_CUDA(cudaEventRecord(ev[2 * k + 1], s));
    k_dot<<<gv, LZ_NT, 0, s>>>(q, w, D, part, st, 0, d_alpha + k, nullptr, stopf);
    const bool last_norm = !prm->reorth;
    k_lz_update<<<gv, LZ_NT, 0, s>>>(w, q, qp, D, d_alpha + k, d_beta + k, part, st, d_beta + k + 1, k, last_norm);
    uint64_t nl = 3;
    if (prm->reorth) {
      for (int pass = 0; pass < 2; ++pass) {
        k_multidot<<<gmd, LZ_NT, 0, s>>>(Q, D, k + 1, w, D, part, st);
        k_multidot_reduce<<<k + 1, 32, 0, s>>>(part, gmd, h, st);
        k_multiaxpy<<<gax, RA_NT, 0, s>>>(Q, D, k + 1, h, w, D, part, st, d_beta + k + 1, k, pass == 1, d_alpha + k);
        nl += 3;
      }
    }
    k_scale<<<gs, 256, 0, s>>>(w, qv(k + 1), D, d_beta + k + 1, stopf);
    ED_CHECK_LAUNCH_N("lanczos step", nl);
    launched = k + 1;
    if (checks && ((k + 1) % prm->check_every == 0) && k + 1 < Km)
      ED_TRY(chk.launch(s, d_alpha, d_beta, k + 1, prm->tol, &st->stop, &st->steps, tri, c, twork));
  }
  ED_TRY(chk.join(s));
  k_tri_final<<<1, TRI_NT, 0, s>>>(d_alpha, d_beta, launched, &st->stop, &st->steps, tri, c, twork);
  ED_CHECK_LAUNCH("k_tri_final");
  if (prm->want_vector) {
    k_ritz<<<gs, 256, 0, s>>>(Q, D, c, st, d_evec, D);
    k_dot<<<gv, LZ_NT, 0, s>>>(d_evec, d_evec, D, part, st, 0, scal, scal + 1, nullptr);
    k_scale<<<gs, 256, 0, s>>>(d_evec, d_evec, D, scal + 1, nullptr);
    ED_CHECK_LAUNCH_N("lanczos ritz", 3);
  }
  LzState hs;
  TriResult ht;
  ED_CUDA(cudaMemcpyAsync(&hs, st, sizeof(LzState), cudaMemcpyDeviceToHost, s));
  ED_CUDA(cudaMemcpyAsync(&ht, tri, sizeof(TriResult), cudaMemcpyDeviceToHost, s));
  ED_CUDA(cudaStreamSynchronize(s));
  const int m = ht.m_final;
  res->energy = ht.energy;
  res->residual = ht.residual;
  res->steps = m;
  res->converged = hs.stop;
  res->status = hs.status;
  res->matvec_ms = 0.0;
  res->matvecs = 0;
  if (prm->profile) {
    // matvecs after a stop return immediately; count only the steps that ran
    for (int k = 0; k < m; ++k) {
      float ms = 0.f;
      ED_CUDA(cudaEventElapsedTime(&ms, ev[2 * k], ev[2 * k + 1]));
      res->matvec_ms += ms;
      res->matvecs += 1;
    }
    for (auto& e : ev) cudaEventDestroy(e);
  }
  return ED_OK;
}

ED_API ed_status ed_lanczos_coeffs_multi(int n, const ed_plan* plans, int K, const double* const* d_starts,
                                         void* const* d_work, const size_t* work_bytes, double* const* d_alpha,
                                         double* const* d_beta, int* h_steps, double* h_norm, ed_stream_t stream) {
  if (n < 1 || !plans || !d_starts || !d_work || !work_bytes || !d_alpha || !d_beta || !h_steps || !h_norm)
    return fail(ED_ERR_INVALID_ARG, "null argument or n < 1");
  if (K < 1 || K > 4096) return fail(ED_ERR_INVALID_ARG, "max_steps must be in [1, 4096]");
  bool all_fixed = true;
  for (int i = 0; i < n; ++i) {
    ED_TRY(check_plan(plans[i]));
    if (!d_starts[i] || !d_alpha[i] || !d_beta[i]) return fail(ED_ERR_INVALID_ARG, "null argument");
    if (plans[i]->dim < 1) return fail(ED_ERR_INVALID_ARG, "empty sector");
    if (plans[i]->bfp.eligible) {
      if (!d_work[i] || work_bytes[i] < bfp_workspace_bytes(plans[i], K, false))
        return fail(ED_ERR_INVALID_ARG, "workspace too small (see ed_lanczos_workspace)");
    } else {
      all_fixed = false;
    }
    for (int j = 0; j < i; ++j)
      if (d_work[j] == d_work[i] || d_alpha[j] == d_alpha[i] || d_beta[j] == d_beta[i])
        return fail(ED_ERR_INVALID_ARG, "the runs must not share workspaces or outputs");
  }
  if (!all_fixed) {
    // FP64 runs: one after another on the caller's stream
    for (int i = 0; i < n; ++i)
      ED_TRY(ed_lanczos_coeffs(plans[i], K, d_starts[i], d_work[i], work_bytes[i], d_alpha[i], d_beta[i],
                               &h_steps[i], &h_norm[i], stream));
    return ED_OK;
  }
  std::vector<const ed_plan_s*> ps(plans, plans + n);
  return bfp_lanczos_coeffs_multi(n, ps.data(), K, d_starts, d_work, d_alpha, d_beta, h_steps, h_norm,
                                  as_stream(stream));
}

ED_API ed_status ed_lanczos_coeffs(ed_plan p, int K, const double* d_start, void* d_work, size_t work_bytes,
                                   double* d_alpha, double* d_beta, int* h_steps, double* h_norm, ed_stream_t stream) {
  ED_TRY(check_plan(p));
  if (!d_start || !d_alpha || !d_beta || !h_steps || !h_norm) return fail(ED_ERR_INVALID_ARG, "null argument");
  if (K < 1 || K > 4096) return fail(ED_ERR_INVALID_ARG, "max_steps must be in [1, 4096]");
  const int64_t D = p->dim;
  if (D < 1) return fail(ED_ERR_INVALID_ARG, "empty sector");
  if (p->bfp.eligible) {
    if (!d_work || work_bytes < bfp_workspace_bytes(p, K, false))
      return fail(ED_ERR_INVALID_ARG, "workspace too small (see ed_lanczos_workspace)");
    return bfp_lanczos_coeffs(p, K, d_start, d_work, d_alpha, d_beta, h_steps, h_norm, as_stream(stream));
  }
  const int nparts = lz_parts(p, D);
  const LzLayout L = lz_layout(D, K, false, nparts);
  if (!d_work || work_bytes < L.total) return fail(ED_ERR_INVALID_ARG, "workspace too small (see ed_lanczos_workspace)");
  cudaStream_t s = as_stream(stream);
  char* base = (char*)d_work;
  double* Q = (double*)(base + L.off_basis);
  double* w = (double*)(base + L.off_w);
  double* part = (double*)(base + L.off_partial);
  double* scal = (double*)(base + L.off_scalars);
  LzState* st = (LzState*)(base + L.off_state);
  ED_CUDA(cudaMemsetAsync(st, 0, sizeof(LzState), s));
  ED_CUDA(cudaMemsetAsync(d_alpha, 0, K * sizeof(double), s));
  ED_CUDA(cudaMemsetAsync(d_beta, 0, (K + 1) * sizeof(double), s));
  const int gv = nparts;
  const int gs = grid_for(D, 256, p->ctx->num_sms * 8);
  auto qv = [&](int k) -> double* { return Q + (int64_t)(k % 3) * D; };
  k_dot<<<gv, LZ_NT, 0, s>>>(d_start, d_start, D, part, st, 0, scal, scal + 1, nullptr);
  k_scale<<<gs, 256, 0, s>>>(d_start, qv(0), D, scal + 1, nullptr);
  ED_CHECK_LAUNCH_N("lanczos_coeffs start", 2);
  double n2 = 0.0;
  ED_CUDA(cudaMemcpyAsync(&n2, scal, sizeof(double), cudaMemcpyDeviceToHost, s));
  ED_CUDA(cudaStreamSynchronize(s));
  if (!std::isfinite(n2)) return fail(ED_ERR_NONFINITE, "start vector is not finite");
  if (n2 == 0.0) { *h_steps = 0; *h_norm = 0.0; return ED_OK; }
  const int* stopf = &st->stop;
  const int Km = (int)std::min<int64_t>(K, D);
  for (int k = 0; k < Km; ++k) {
    double* q = qv(k);
    double* qp = k > 0 ? qv(k - 1) : nullptr;
    ED_TRY(matvec_f64(p, q, w, 1, D, s, stopf));
    k_dot<<<gv, LZ_NT, 0, s>>>(q, w, D, part, st, 0, d_alpha + k, nullptr, stopf);
    k_lz_update<<<gv, LZ_NT, 0, s>>>(w, q, qp, D, d_alpha + k, d_beta + k, part, st, d_beta + k + 1, k, 1);
    k_scale<<<gs, 256, 0, s>>>(w, qv(k + 1), D, d_beta + k + 1, stopf);
    ED_CHECK_LAUNCH_N("lanczos_coeffs step", 3);
  }
  LzState hs;
  ED_CUDA(cudaMemcpyAsync(&hs, st, sizeof(LzState), cudaMemcpyDeviceToHost, s));
  ED_CUDA(cudaStreamSynchronize(s));
  *h_steps = hs.stop ? hs.steps : Km;
  *h_norm = std::sqrt(n2);
  return ED_OK;
}

ED_API ed_status ed_tridiag_lowest_batch(const double* d_alpha, int lda, const double* d_beta, int ldb,
                                         const int* d_m, int B, int max_m, double* d_values, double* d_vecs, int ldv,
                                         ed_stream_t stream) {
  if (B < 0 || max_m < 1 || max_m > 4096 || lda < max_m || ldb < max_m + 1 || ldv < max_m)
    return fail(ED_ERR_INVALID_ARG, "bad batch shape (1 <= m <= 4096, lda >= m, ldb >= m + 1, ldv >= m)");
  if (B == 0) return ED_OK;
  if (!d_alpha || !d_beta || !d_m || !d_values || !d_vecs) return fail(ED_ERR_INVALID_ARG, "null argument");
  cudaStream_t s = as_stream(stream);
  double* work = nullptr;
  ED_CUDA(cudaMallocAsync(&work, 5 * (size_t)B * ldv * sizeof(double), s));
  k_tridiag_batch<<<B, LZ_NT, 0, s>>>(d_alpha, lda, d_beta, ldb, d_m, d_values, d_vecs, ldv, work);
  ED_CHECK_LAUNCH("k_tridiag_batch");
  ED_CUDA(cudaFreeAsync(work, s));
  return ED_OK;
}

ED_API ed_status ed_tridiag_pinv_solve_batch(const double* d_alpha, int lda, const double* d_beta, int ldb,
                                             const int* d_m, int B, int max_m, const double* d_e0, const double* d_c,
                                             int ldc, const double* d_rhs, double* d_out, int ldr,
                                             ed_stream_t stream) {
  if (B < 0 || max_m < 1 || max_m > 4096 || lda < max_m || ldb < max_m + 1 || ldc < max_m || ldr < max_m)
    return fail(ED_ERR_INVALID_ARG, "bad batch shape (1 <= m <= 4096, leading dimensions >= m)");
  if (B == 0) return ED_OK;
  if (!d_alpha || !d_beta || !d_m || !d_e0 || !d_c || !d_rhs || !d_out) return fail(ED_ERR_INVALID_ARG, "null argument");
  if (d_rhs == d_out) return fail(ED_ERR_INVALID_ARG, "d_rhs and d_out must not alias");
  cudaStream_t s = as_stream(stream);
  double* work = nullptr;
  ED_CUDA(cudaMallocAsync(&work, 5 * (size_t)B * ldr * sizeof(double), s));
  k_tridiag_pinv_batch<<<B, 32, 0, s>>>(d_alpha, lda, d_beta, ldb, d_m, d_e0, d_c, ldc, d_rhs, d_out, ldr, work);
  ED_CHECK_LAUNCH("k_tridiag_pinv_batch");
  ED_CUDA(cudaFreeAsync(work, s));
  return ED_OK;
}

ED_API ed_status ed_tridiag_lowest(const double* d_alpha, const double* d_beta, int m, double* d_value, double* d_vec,
                                   ed_stream_t stream) {
  if (m < 1 || m > 4096) return fail(ED_ERR_INVALID_ARG, "m must be in [1, 4096]");
  if (!d_alpha || !d_beta || !d_value) return fail(ED_ERR_INVALID_ARG, "null argument");
  cudaStream_t s = as_stream(stream);
  double* work = nullptr;
  if (d_vec) ED_CUDA(cudaMallocAsync(&work, 5 * (size_t)m * sizeof(double), s));
  k_tridiag<<<1, LZ_NT, 0, s>>>(d_alpha, d_beta, m, d_value, d_vec, work);
  ED_CHECK_LAUNCH("k_tridiag");
  if (work) ED_CUDA(cudaFreeAsync(work, s));
  return ED_OK;
}

}  // extern "C"
