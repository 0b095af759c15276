// Green's-function kernels: the continued fraction of the Lanczos coefficients (new; the
// reference only has dense Lanczos helpers, cmpy/exactdiag.py:324-375) and the thermal
// Lehmann pole sum of _accumulate_sum (cmpy/exactdiag.py:110-129).
// Complex numbers are interleaved (re, im) FP64 pairs.
#include <cmath>

#include "ed_plan.cuh"

namespace ed {

// G(z) = sign * norm2 / (z' - a0 - b1^2 / (z' - a1 - ...)),  z' = sign * z + shift
__global__ void k_cf(const double* __restrict__ a, const double* __restrict__ b, int n, double norm2, double shift,
                     int sign, const double2* __restrict__ z, int64_t nz, double2* __restrict__ g, int accumulate) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nz; i += (int64_t)gridDim.x * blockDim.x) {
    const double2 zi = z[i];
    const double zr = sign * zi.x + shift, zm = sign * zi.y;
    double tr = zr - a[n - 1], tm = zm;
    for (int l = n - 2; l >= 0; --l) {
      const double bb = b[l + 1] * b[l + 1];
      const double inv = bb / (tr * tr + tm * tm);
      tr = zr - a[l] - tr * inv;
      tm = zm + tm * inv;
    }
    const double inv = sign * norm2 / (tr * tr + tm * tm);
    double2 r = make_double2(tr * inv, -tm * inv);
    if (accumulate) { r.x += g[i].x; r.y += g[i].y; }
    g[i] = r;
  }
}

// coef[m*nd + n] = ov[m, n] * (w_n + w'_m),  pole = E'_m - E_n;  w = exp(-beta (E - emin))
// (all ones when beta is not finite, cmpy/exactdiag.py:114-119)
__global__ void k_lehmann_poles(const double* __restrict__ e, int64_t nd, const double* __restrict__ ep, int64_t ndp,
                                const double* __restrict__ ov, double beta, double emin, double* __restrict__ coef,
                                double* __restrict__ pole) {
  const int64_t tot = nd * ndp;
  const bool fin = isfinite(beta);
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < tot; k += (int64_t)gridDim.x * blockDim.x) {
    const int64_t m = k / nd, n = k - m * nd;
    const double wn = fin ? exp(-beta * (e[n] - emin)) : 1.0;
    const double wm = fin ? exp(-beta * (ep[m] - emin)) : 1.0;
    coef[k] = ov[k] * (wn + wm);
    pole[k] = ep[m] - e[n];
  }
}

// g[z] += sum_k coef_k / (z - pole_k); one block per frequency chunk, terms staged in smem
constexpr int LEH_T = 1024;
__global__ void k_lehmann_sum(const double* __restrict__ coef, const double* __restrict__ pole, int64_t nt,
                              const double2* __restrict__ z, int64_t nz, double2* __restrict__ g) {
  __shared__ double sc[LEH_T], sp[LEH_T];
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const double2 zi = i < nz ? z[i] : make_double2(0.0, 1.0);
  const double zm2 = zi.y * zi.y;
  double gr = 0.0, gm = 0.0;
  for (int64_t t0 = 0; t0 < nt; t0 += LEH_T) {
    __syncthreads();
    for (int t = threadIdx.x; t < LEH_T; t += blockDim.x) {
      const int64_t k = t0 + t;
      sc[t] = k < nt ? coef[k] : 0.0;
      sp[t] = k < nt ? pole[k] : 0.0;
    }
    __syncthreads();
    const int tn = (int)((nt - t0) < LEH_T ? (nt - t0) : LEH_T);
    for (int t = 0; t < tn; ++t) {
      const double c = sc[t];
      if (c == 0.0) continue;
      const double ar = zi.x - sp[t];
      const double inv = c / (ar * ar + zm2);
      gr = fma(ar, inv, gr);
      gm = fma(-zi.y, inv, gm);
    }
  }
  if (i < nz) {
    double2 r = g[i];
    r.x += gr;
    r.y += gm;
    g[i] = r;
  }
}

}  // namespace ed

using namespace ed;

extern "C" {

ED_API ed_status ed_gf_continued_fraction(const double* d_alpha, const double* d_beta, int n_lev, double norm2,
                                          double shift, int sign, const double* d_z, int64_t n_z, double* d_g,
                                          int accumulate, ed_stream_t stream) {
  if (n_lev < 1) return fail(ED_ERR_INVALID_ARG, "n_lev must be >= 1");
  if (sign != 1 && sign != -1) return fail(ED_ERR_INVALID_ARG, "sign must be +1 or -1");
  if (n_z < 0) return fail(ED_ERR_INVALID_ARG, "negative n_z");
  if (n_z == 0) return ED_OK;
  if (!d_alpha || !d_beta || !d_z || !d_g) return fail(ED_ERR_INVALID_ARG, "null argument");
  DeviceContext* ctx;
  ED_TRY(device_context(&ctx));
  k_cf<<<grid_for(n_z, 128, ctx->num_sms * 8), 128, 0, as_stream(stream)>>>(
      d_alpha, d_beta, n_lev, norm2, shift, sign, (const double2*)d_z, n_z, (double2*)d_g, accumulate);
  ED_CHECK_LAUNCH("k_cf");
  return ED_OK;
}

ED_API ed_status ed_lehmann_accumulate(const double* d_e, int64_t nd, const double* d_ep, int64_t ndp,
                                       const double* d_ov, double beta, double emin, const double* d_z, int64_t nz,
                                       double* d_g, ed_stream_t stream) {
  if (nd < 0 || ndp < 0 || nz < 0) return fail(ED_ERR_INVALID_ARG, "negative size");
  if (nd == 0 || ndp == 0 || nz == 0) return ED_OK;
  if (!d_e || !d_ep || !d_ov || !d_z || !d_g) return fail(ED_ERR_INVALID_ARG, "null argument");
  if (std::isnan(beta)) return fail(ED_ERR_NONFINITE, "beta is NaN");
  DeviceContext* ctx;
  ED_TRY(device_context(&ctx));
  cudaStream_t s = as_stream(stream);
  const int64_t nt = nd * ndp;
  double *coef = nullptr, *pole = nullptr;
  ED_CUDA(cudaMallocAsync(&coef, nt * sizeof(double), s));
  ED_CUDA(cudaMallocAsync(&pole, nt * sizeof(double), s));
  k_lehmann_poles<<<grid_for(nt, 256, ctx->num_sms * 8), 256, 0, s>>>(d_e, nd, d_ep, ndp, d_ov, beta, emin, coef, pole);
  k_lehmann_sum<<<(unsigned)((nz + 127) / 128), 128, 0, s>>>(coef, pole, nt, (const double2*)d_z, nz, (double2*)d_g);
  ED_CHECK_LAUNCH_N("ed_lehmann_accumulate", 2);
  ED_CUDA(cudaFreeAsync(coef, s));
  ED_CUDA(cudaFreeAsync(pole, s));
  return ED_OK;
}

}  // extern "C"
