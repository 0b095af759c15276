// COO triplet generators, bit-exact and in the emission order of the reference projectors:
//   project_onsite_energy  cmpy/operators.py:359-422
//   project_hubbard_inter  cmpy/operators.py:305-356
//   project_hopping        cmpy/operators.py:463-527 (via _compute_hopping_term :436-460)
//   HubbardModel/_ham_data cmpy/models/hubbard.py:13-22, SIAM anderson.py:147-158,
//   HeisenbergModel        cmpy/models/heisenberg.py:19-40.
// Every segment is generated by (count -> exclusive scan -> fill) so the output positions
// are exactly the reference's generator order, including its skipping of exact zeros.
#include <algorithm>
#include <cmath>
#include <vector>

#include "ed_plan.cuh"

namespace ed {

// ---- exclusive scan of int64 counts ----------------------------------------------------
constexpr int SCAN_NT = 256;
constexpr int SCAN_IPT = 8;
constexpr int SCAN_TILE = SCAN_NT * SCAN_IPT;

__global__ void k_tile_sum(const int64_t* __restrict__ cnt, int64_t n, int64_t* __restrict__ bsum) {
  __shared__ int64_t sm[SCAN_NT];
  const int64_t base = (int64_t)blockIdx.x * SCAN_TILE;
  int64_t s = 0;
  for (int k = 0; k < SCAN_IPT; ++k) {
    const int64_t i = base + (int64_t)k * SCAN_NT + threadIdx.x;
    if (i < n) s += cnt[i];
  }
  sm[threadIdx.x] = s;
  __syncthreads();
  for (int o = SCAN_NT / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) sm[threadIdx.x] += sm[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) bsum[blockIdx.x] = sm[0];
}

// single block: exclusive scan of bsum[0..nb), total into bsum[nb]
__global__ void k_scan_bsum(int64_t* __restrict__ bsum, int64_t nb) {
  __shared__ int64_t sm[SCAN_NT];
  __shared__ int64_t carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int64_t c0 = 0; c0 < nb; c0 += SCAN_NT) {
    const int64_t i = c0 + threadIdx.x;
    const int64_t v = i < nb ? bsum[i] : 0;
    sm[threadIdx.x] = v;
    __syncthreads();
    for (int o = 1; o < SCAN_NT; o <<= 1) {
      const int64_t t = threadIdx.x >= o ? sm[threadIdx.x - o] : 0;
      __syncthreads();
      sm[threadIdx.x] += t;
      __syncthreads();
    }
    if (i < nb) bsum[i] = carry + sm[threadIdx.x] - v;
    __syncthreads();
    if (threadIdx.x == 0) carry += sm[SCAN_NT - 1];
    __syncthreads();
  }
  if (threadIdx.x == 0) bsum[nb] = carry;
}

__global__ void k_tile_scan(const int64_t* __restrict__ cnt, int64_t n, const int64_t* __restrict__ bsum,
                            int64_t* __restrict__ off) {
  __shared__ int64_t sm[SCAN_NT];
  __shared__ int64_t carry;
  const int64_t base = (int64_t)blockIdx.x * SCAN_TILE;
  if (threadIdx.x == 0) carry = bsum[blockIdx.x];
  __syncthreads();
  for (int k = 0; k < SCAN_IPT; ++k) {
    const int64_t i = base + (int64_t)k * SCAN_NT + threadIdx.x;
    const int64_t v = i < n ? cnt[i] : 0;
    sm[threadIdx.x] = v;
    __syncthreads();
    for (int o = 1; o < SCAN_NT; o <<= 1) {
      const int64_t t = threadIdx.x >= o ? sm[threadIdx.x - o] : 0;
      __syncthreads();
      sm[threadIdx.x] += t;
      __syncthreads();
    }
    if (i < n) off[i] = carry + sm[threadIdx.x] - v;
    __syncthreads();
    if (threadIdx.x == 0) carry += sm[SCAN_NT - 1];
    __syncthreads();
  }
}

// off[i] = sum_{k<i} cnt[k]; returns the total (synchronous).
static ed_status exclusive_scan(const int64_t* d_cnt, int64_t n, int64_t* d_off, int64_t* total, cudaStream_t s) {
  *total = 0;
  if (n == 0) return ED_OK;
  const int64_t nb = (n + SCAN_TILE - 1) / SCAN_TILE;
  int64_t* d_b = nullptr;
  ED_CUDA(cudaMallocAsync(&d_b, (nb + 1) * sizeof(int64_t), s));
  k_tile_sum<<<(unsigned)nb, SCAN_NT, 0, s>>>(d_cnt, n, d_b);
  k_scan_bsum<<<1, SCAN_NT, 0, s>>>(d_b, nb);
  k_tile_scan<<<(unsigned)nb, SCAN_NT, 0, s>>>(d_cnt, n, d_b, d_off);
  ED_CHECK_LAUNCH_N("exclusive_scan", 3);
  ED_CUDA(cudaMemcpyAsync(total, d_b + nb, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
  ED_CUDA(cudaStreamSynchronize(s));
  ED_CUDA(cudaFreeAsync(d_b, s));
  return ED_OK;
}

// ---- kernels -------------------------------------------------------------------------------
struct Values {
  int n;
  double v[ED_MAX_SITES + 2];
};

__device__ __forceinline__ bool truthy(double e) { return e != 0.0 || isnan(e); }  // python `if energy:`

// flag/count per spin state for the onsite segment: cnt = mult if weighted_element != 0
__global__ void k_onsite_count(const uint64_t* __restrict__ st, int64_t n, Values vals, int64_t mult,
                               int64_t* __restrict__ cnt, double* __restrict__ energy) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double e = weighted_element(st[i], vals.v, vals.n);
    energy[i] = e;
    cnt[i] = truthy(e) ? mult : 0;
  }
}

// up block: origin = i*nd + d for all d; dn block (dn_mode): origin = u*nd + j for all u
__global__ void k_onsite_fill(const double* __restrict__ energy, const int64_t* __restrict__ cnt,
                              const int64_t* __restrict__ off, int64_t n, int64_t nu, int64_t nd, int dn_mode,
                              int64_t base, int64_t* __restrict__ rows, int64_t* __restrict__ cols,
                              double* __restrict__ out) {
  // one block per spin state, threads over the other species
  for (int64_t i = blockIdx.x; i < n; i += gridDim.x) {
    if (cnt[i] == 0) continue;
    const int64_t o = base + off[i];
    const double e = energy[i];
    const int64_t m = dn_mode ? nu : nd;
    for (int64_t k = threadIdx.x; k < m; k += blockDim.x) {
      const int64_t origin = dn_mode ? k * nd + i : i * nd + k;
      rows[o + k] = origin;
      cols[o + k] = origin;
      out[o + k] = e;
    }
  }
}

__global__ void k_inter_count(const uint64_t* __restrict__ up, const uint64_t* __restrict__ dn, int64_t nu,
                              int64_t nd, Values vals, int64_t* __restrict__ cnt) {
  const int64_t D = nu * nd;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < D; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t u = i / nd, d = i - u * nd;
    cnt[i] = truthy(weighted_element(up[u] & dn[d], vals.v, vals.n)) ? 1 : 0;
  }
}

__global__ void k_inter_fill(const uint64_t* __restrict__ up, const uint64_t* __restrict__ dn, int64_t nu,
                             int64_t nd, Values vals, const int64_t* __restrict__ cnt,
                             const int64_t* __restrict__ off, int64_t base, int64_t* __restrict__ rows,
                             int64_t* __restrict__ cols, double* __restrict__ out) {
  const int64_t D = nu * nd;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < D; i += (int64_t)gridDim.x * blockDim.x) {
    if (!cnt[i]) continue;
    const int64_t u = i / nd, d = i - u * nd;
    const int64_t o = base + off[i];
    rows[o] = i;
    cols[o] = i;
    out[o] = weighted_element(up[u] & dn[d], vals.v, vals.n);
  }
}

__global__ void k_hop_flag(const uint64_t* __restrict__ st, int64_t n, int s1, int s2, int64_t mult,
                           int64_t* __restrict__ cnt) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t s = st[i];
    cnt[i] = (((s >> s1) ^ (s >> s2)) & 1ull) ? mult : 0;
  }
}

__global__ void k_hop_emit(const uint64_t* __restrict__ st, int64_t n, int width, int s1, int s2, double hop,
                           const int64_t* __restrict__ cnt, const int64_t* __restrict__ off, int64_t nu,
                           int64_t nd, int dn_mode, int64_t base, int64_t* __restrict__ rows,
                           int64_t* __restrict__ cols, double* __restrict__ out) {
  for (int64_t i = blockIdx.x; i < n; i += gridDim.x) {
    if (!cnt[i]) continue;
    const uint64_t s = st[i];
    const uint64_t t = s ^ (1ull << s1) ^ (1ull << s2);
    const int64_t j = bisect_left(st, n, t);
    const double val = hop_sign(s, width, s1, s2) < 0 ? -hop : hop;
    const int64_t o = base + off[i];
    const int64_t m = dn_mode ? nu : nd;
    for (int64_t k = threadIdx.x; k < m; k += blockDim.x) {
      rows[o + k] = dn_mode ? k * nd + i : i * nd + k;
      cols[o + k] = dn_mode ? k * nd + j : j * nd + k;
      out[o + k] = val;
    }
  }
}

// Heisenberg: per state, n_pairs diagonals + one triplet per pair with differing bits
struct PairArgs {
  int n;
  int p1[256];
  int p2[256];
  double j[256];
  double jz[256];
};

__global__ void k_spin_coo_count(const uint64_t* __restrict__ st, int64_t n, const PairArgs* __restrict__ pa,
                                 int64_t* __restrict__ cnt) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t s = st[i];
    int64_t c = pa->n;
    for (int p = 0; p < pa->n; ++p) c += (((s >> pa->p1[p]) ^ (s >> pa->p2[p])) & 1ull) ? 1 : 0;
    cnt[i] = c;
  }
}

__global__ void k_spin_coo_fill(const uint64_t* __restrict__ st, int64_t n, const PairArgs* __restrict__ pa,
                                const int64_t* __restrict__ off, int64_t* __restrict__ rows,
                                int64_t* __restrict__ cols, double* __restrict__ out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t s = st[i];
    int64_t o = off[i];
    for (int p = 0; p < pa->n; ++p) {
      const int b1 = (int)((s >> pa->p1[p]) & 1ull), b2 = (int)((s >> pa->p2[p]) & 1ull);
      // sign * factor * jz with sign = (-1)**b1 * (-1)**b2 (heisenberg.py:27-29)
      const double sign = (b1 == b2) ? 1.0 : -1.0;
      rows[o] = i; cols[o] = i; out[o] = __dmul_rn(__dmul_rn(sign, 0.25), pa->jz[p]); ++o;
      if (b1 != b2) {
        const uint64_t t = s ^ (1ull << pa->p1[p]) ^ (1ull << pa->p2[p]);
        rows[o] = i; cols[o] = bisect_left(st, n, t); out[o] = __dmul_rn(0.25, pa->j[p]) / 2.0; ++o;
      }
    }
  }
}

// ---- host drivers ------------------------------------------------------------------------
struct CooOut {
  int64_t* rows; int64_t* cols; double* vals; int64_t capacity;
  bool count_only() const { return rows == nullptr; }
};

static int grid1(int64_t n, int sms) { return grid_for(n, 256, sms * 8); }

// onsite segment starting at `base`; adds its size to *seg.
static ed_status seg_onsite(const uint64_t* up, int64_t nu, const uint64_t* dn, int64_t nd, const Values& v,
                            const CooOut& o, int64_t base, int64_t* seg, int sms, cudaStream_t s) {
  *seg = 0;
  const int64_t nmax = std::max<int64_t>(std::max(nu, nd), 1);
  int64_t *cnt = nullptr, *off = nullptr;
  double* en = nullptr;
  ED_CUDA(cudaMallocAsync(&cnt, nmax * sizeof(int64_t), s));
  ED_CUDA(cudaMallocAsync(&off, nmax * sizeof(int64_t), s));
  ED_CUDA(cudaMallocAsync(&en, nmax * sizeof(double), s));
  for (int dn_mode = 0; dn_mode < 2; ++dn_mode) {
    const uint64_t* st = dn_mode ? dn : up;
    const int64_t n = dn_mode ? nd : nu;
    const int64_t mult = dn_mode ? nu : nd;
    if (n == 0) continue;
    k_onsite_count<<<grid1(n, sms), 256, 0, s>>>(st, n, v, mult, cnt, en);
    ED_CHECK_LAUNCH("k_onsite_count");
    int64_t tot = 0;
    ED_TRY(exclusive_scan(cnt, n, off, &tot, s));
    if (!o.count_only()) {
      if (base + *seg + tot > o.capacity) return fail(ED_ERR_INVALID_ARG, "COO capacity too small");
      k_onsite_fill<<<(unsigned)std::min<int64_t>(n, 65535), 128, 0, s>>>(en, cnt, off, n, nu, nd, dn_mode,
                                                                          base + *seg, o.rows, o.cols, o.vals);
      ED_CHECK_LAUNCH("k_onsite_fill");
    }
    *seg += tot;
  }
  ED_CUDA(cudaFreeAsync(cnt, s));
  ED_CUDA(cudaFreeAsync(off, s));
  ED_CUDA(cudaFreeAsync(en, s));
  return ED_OK;
}

static ed_status seg_inter(const uint64_t* up, int64_t nu, const uint64_t* dn, int64_t nd, const Values& v,
                           const CooOut& o, int64_t base, int64_t* seg, int sms, cudaStream_t s) {
  *seg = 0;
  const int64_t D = nu * nd;
  if (D == 0) return ED_OK;
  int64_t *cnt = nullptr, *off = nullptr;
  ED_CUDA(cudaMallocAsync(&cnt, D * sizeof(int64_t), s));
  ED_CUDA(cudaMallocAsync(&off, D * sizeof(int64_t), s));
  k_inter_count<<<grid1(D, sms), 256, 0, s>>>(up, dn, nu, nd, v, cnt);
  ED_CHECK_LAUNCH("k_inter_count");
  int64_t tot = 0;
  ED_TRY(exclusive_scan(cnt, D, off, &tot, s));
  if (!o.count_only()) {
    if (base + tot > o.capacity) return fail(ED_ERR_INVALID_ARG, "COO capacity too small");
    k_inter_fill<<<grid1(D, sms), 256, 0, s>>>(up, dn, nu, nd, v, cnt, off, base, o.rows, o.cols, o.vals);
    ED_CHECK_LAUNCH("k_inter_fill");
  }
  *seg = tot;
  ED_CUDA(cudaFreeAsync(cnt, s));
  ED_CUDA(cudaFreeAsync(off, s));
  return ED_OK;
}

static ed_status seg_hopping(const uint64_t* up, int64_t nu, const uint64_t* dn, int64_t nd, int width, int s1,
                             int s2, double hop, const CooOut& o, int64_t base, int64_t* seg, int sms,
                             cudaStream_t s) {
  *seg = 0;
  const int64_t nmax = std::max<int64_t>(std::max(nu, nd), 1);
  int64_t *cnt = nullptr, *off = nullptr;
  ED_CUDA(cudaMallocAsync(&cnt, nmax * sizeof(int64_t), s));
  ED_CUDA(cudaMallocAsync(&off, nmax * sizeof(int64_t), s));
  for (int dn_mode = 0; dn_mode < 2; ++dn_mode) {
    const uint64_t* st = dn_mode ? dn : up;
    const int64_t n = dn_mode ? nd : nu;
    const int64_t mult = dn_mode ? nu : nd;
    if (n == 0) continue;
    k_hop_flag<<<grid1(n, sms), 256, 0, s>>>(st, n, s1, s2, mult, cnt);
    ED_CHECK_LAUNCH("k_hop_flag");
    int64_t tot = 0;
    ED_TRY(exclusive_scan(cnt, n, off, &tot, s));
    if (!o.count_only()) {
      if (base + *seg + tot > o.capacity) return fail(ED_ERR_INVALID_ARG, "COO capacity too small");
      k_hop_emit<<<(unsigned)std::min<int64_t>(n, 65535), 128, 0, s>>>(st, n, width, s1, s2, hop, cnt, off, nu, nd,
                                                                      dn_mode, base + *seg, o.rows, o.cols, o.vals);
      ED_CHECK_LAUNCH("k_hop_emit");
    }
    *seg += tot;
  }
  ED_CUDA(cudaFreeAsync(cnt, s));
  ED_CUDA(cudaFreeAsync(off, s));
  return ED_OK;
}

static ed_status values_from(const double* h, int n, Values* v) {
  if (n < 0 || n > ED_MAX_SITES) return fail(ED_ERR_INVALID_ARG, "value array length must be in [0, 62]");
  if (n > 0 && !h) return fail(ED_ERR_INVALID_ARG, "null value array");
  v->n = n;
  for (int i = 0; i < ED_MAX_SITES + 2; ++i) v->v[i] = i < n ? h[i] : 0.0;
  return ED_OK;
}

static ed_status check_out(const CooOut& o, int64_t* h_nnz) {
  if (!h_nnz) return fail(ED_ERR_INVALID_ARG, "null nnz output");
  if (!o.count_only() && (!o.cols || !o.vals)) return fail(ED_ERR_INVALID_ARG, "null COO output arrays");
  return ED_OK;
}

static ed_status finish(const CooOut& o, cudaStream_t s) {
  if (!o.count_only()) ED_CUDA(cudaStreamSynchronize(s));
  return ED_OK;
}

}  // namespace ed

using namespace ed;

extern "C" {

ED_API ed_status ed_coo_onsite(const uint64_t* up, int64_t nu, const uint64_t* dn, int64_t nd, const double* h_eps,
                               int n_values, int64_t* rows, int64_t* cols, double* vals, int64_t capacity,
                               int64_t* h_nnz, ed_stream_t stream) {
  CooOut o{rows, cols, vals, capacity};
  ED_TRY(check_out(o, h_nnz));
  Values v;
  ED_TRY(values_from(h_eps, n_values, &v));
  DeviceContext* ctx;
  ED_TRY(device_context(&ctx));
  ED_TRY(seg_onsite(up, nu, dn, nd, v, o, 0, h_nnz, ctx->num_sms, as_stream(stream)));
  return finish(o, as_stream(stream));
}

ED_API ed_status ed_coo_inter(const uint64_t* up, int64_t nu, const uint64_t* dn, int64_t nd, const double* h_u,
                              int n_values, int64_t* rows, int64_t* cols, double* vals, int64_t capacity,
                              int64_t* h_nnz, ed_stream_t stream) {
  CooOut o{rows, cols, vals, capacity};
  ED_TRY(check_out(o, h_nnz));
  Values v;
  ED_TRY(values_from(h_u, n_values, &v));
  DeviceContext* ctx;
  ED_TRY(device_context(&ctx));
  ED_TRY(seg_inter(up, nu, dn, nd, v, o, 0, h_nnz, ctx->num_sms, as_stream(stream)));
  return finish(o, as_stream(stream));
}

ED_API ed_status ed_coo_hopping(const uint64_t* up, int64_t nu, const uint64_t* dn, int64_t nd, int width, int site1,
                                int site2, double hop, int64_t* rows, int64_t* cols, double* vals, int64_t capacity,
                                int64_t* h_nnz, ed_stream_t stream) {
  CooOut o{rows, cols, vals, capacity};
  ED_TRY(check_out(o, h_nnz));
  if (!(0 <= site1 && site1 < site2 && site2 <= ED_MAX_SITES)) return fail(ED_ERR_INVALID_ARG, "requires 0 <= site1 < site2 <= 62 (operators.py:438 asserts site1 < site2)");
  DeviceContext* ctx;
  ED_TRY(device_context(&ctx));
  ED_TRY(seg_hopping(up, nu, dn, nd, width, site1, site2, hop, o, 0, h_nnz, ctx->num_sms, as_stream(stream)));
  return finish(o, as_stream(stream));
}

ED_API ed_status ed_coo_plan(ed_plan p, int64_t* rows, int64_t* cols, double* vals, int64_t capacity, int64_t* h_nnz,
                             ed_stream_t stream) {
  ED_TRY(check_plan(p));
  CooOut o{rows, cols, vals, capacity};
  ED_TRY(check_out(o, h_nnz));
  cudaStream_t s = as_stream(stream);
  const int sms = p->ctx->num_sms;
  int64_t total = 0, seg = 0;
  if (p->kind == 0) {
    Values ve, vu;
    ED_TRY(values_from(p->eps.data(), p->n_sites, &ve));
    ED_TRY(values_from(p->u.data(), p->n_sites, &vu));
    const uint64_t *up = p->up.states, *dn = p->dn.states;
    ED_TRY(seg_onsite(up, p->num_up, dn, p->num_dn, ve, o, total, &seg, sms, s));
    total += seg;
    ED_TRY(seg_inter(up, p->num_up, dn, p->num_dn, vu, o, total, &seg, sms, s));
    total += seg;
    for (size_t b = 0; b < p->hop.size(); ++b) {
      ED_TRY(seg_hopping(up, p->num_up, dn, p->num_dn, p->sign_width, p->b1[b], p->b2[b], p->hop[b], o, total, &seg,
                         sms, s));
      total += seg;
    }
  } else {
    PairArgs* h_pa = new PairArgs();
    h_pa->n = (int)p->p1.size();
    for (int q = 0; q < h_pa->n; ++q) {
      h_pa->p1[q] = p->p1[q]; h_pa->p2[q] = p->p2[q]; h_pa->j[q] = p->pj[q]; h_pa->jz[q] = p->pjz[q];
    }
    PairArgs* d_pa = nullptr;
    int64_t *cnt = nullptr, *off = nullptr;
    const int64_t D = std::max<int64_t>(p->dim, 1);
    auto run = [&]() -> ed_status {
      ED_CUDA(cudaMallocAsync(&d_pa, sizeof(PairArgs), s));
      ED_CUDA(cudaMemcpyAsync(d_pa, h_pa, sizeof(PairArgs), cudaMemcpyHostToDevice, s));
      ED_CUDA(cudaMallocAsync(&cnt, D * sizeof(int64_t), s));
      ED_CUDA(cudaMallocAsync(&off, D * sizeof(int64_t), s));
      k_spin_coo_count<<<grid1(p->dim, sms), 256, 0, s>>>(p->up.states, p->dim, d_pa, cnt);
      ED_CHECK_LAUNCH("k_spin_coo_count");
      ED_TRY(exclusive_scan(cnt, p->dim, off, &total, s));
      if (!o.count_only()) {
        if (total > o.capacity) return fail(ED_ERR_INVALID_ARG, "COO capacity too small");
        k_spin_coo_fill<<<grid1(p->dim, sms), 256, 0, s>>>(p->up.states, p->dim, d_pa, off, o.rows, o.cols, o.vals);
        ED_CHECK_LAUNCH("k_spin_coo_fill");
      }
      ED_CUDA(cudaStreamSynchronize(s));
      return ED_OK;
    };
    ed_status st = run();
    cudaFreeAsync(d_pa, s);
    cudaFreeAsync(cnt, s);
    cudaFreeAsync(off, s);
    delete h_pa;
    ED_TRY(st);
  }
  *h_nnz = total;
  p->nnz = total;
  return finish(o, s);
}

}  // extern "C"
