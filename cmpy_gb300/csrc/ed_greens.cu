// Green's-function kernels: the continued fraction of the Lanczos coefficients (new; the
// reference only has dense Lanczos helpers, cmpy/exactdiag.py:324-375), the thermal
// Lehmann pole sum of _accumulate_sum (cmpy/exactdiag.py:110-129), the real-time Green's
// function from Krylov spectral weights (gf_greater / gf_lesser, cmpy/exactdiag.py:248-302)
// and its Laplace transform to complex frequencies (fourier_t2z, cmpy/exactdiag.py:311-316).
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


// out[n] (+)= -i*sign * sum_k w_k exp(-i sign (lam_k - e0) t_n)
// (sign = +1: greater function of c^dag|gs>; sign = -1: lesser function of c|gs>)
constexpr int TEVO_T = 1024;
__global__ void k_tevo_sum(const double* __restrict__ lam, const double* __restrict__ w, int64_t m, double e0, int sign,
                           const double* __restrict__ t, int64_t nt, double2* __restrict__ out, int accumulate) {
  __shared__ double sl[TEVO_T], sw[TEVO_T];
  const int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const double tn = n < nt ? t[n] : 0.0;
  double sr = 0.0, si = 0.0;
  for (int64_t k0 = 0; k0 < m; k0 += TEVO_T) {
    __syncthreads();
    for (int k = threadIdx.x; k < TEVO_T; k += blockDim.x) {
      sl[k] = k0 + k < m ? lam[k0 + k] - e0 : 0.0;
      sw[k] = k0 + k < m ? w[k0 + k] : 0.0;
    }
    __syncthreads();
    const int kn = (int)((m - k0) < TEVO_T ? (m - k0) : TEVO_T);
    for (int k = 0; k < kn; ++k) {
      double sn, cs;
      sincos(sign * sl[k] * tn, &sn, &cs);
      sr = fma(sw[k], cs, sr);
      si = fma(-sw[k], sn, si);
    }
  }
  if (n < nt) {
    // -i*sign * (sr + i si) = sign*si - i sign*sr
    double2 r = make_double2(sign * si, -sign * sr);
    if (accumulate) { r.x += out[n].x; r.y += out[n].y; }
    out[n] = r;
  }
}

__device__ __forceinline__ double2 cmul(double2 a, double2 b) { return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
__device__ __forceinline__ double2 cexp_(double2 x) {
  double sn, cs;
  sincos(x.y, &sn, &cs);
  const double r = exp(x.x);
  return make_double2(r * cs, r * sn);
}
__device__ __forceinline__ double2 cdiv(double2 a, double2 b) {
  const double d = b.x * b.x + b.y * b.y;
  return make_double2((a.x * b.x + a.y * b.y) / d, (a.y * b.x - a.x * b.y) / d);
}
// phi1(x) = (e^x - 1)/x and phi2(x) = (e^x - 1 - x)/x^2 of a complex x; Taylor series for |x| < 1/4
__device__ __forceinline__ void phi12(double2 x, double2* p1, double2* p2) {
  const double ax = sqrt(x.x * x.x + x.y * x.y);
  if (ax < 0.25) {
    // phi1 = sum x^k/(k+1)!, phi2 = sum x^k/(k+2)!  (16 terms: |x|^16/16! << 1e-16)
    double2 a = make_double2(0.0, 0.0), b = make_double2(0.0, 0.0);
    for (int k = 16; k >= 0; --k) {
      a = cmul(a, x);
      b = cmul(b, x);
      double fa = 1.0, fb = 1.0;
      for (int j = 2; j <= k + 1; ++j) fa *= j;
      for (int j = 2; j <= k + 2; ++j) fb *= j;
      a.x += 1.0 / fa;
      b.x += 1.0 / fb;
    }
    *p1 = a;
    *p2 = b;
  } else {
    const double2 ex = cexp_(x);
    const double2 em1 = make_double2(ex.x - 1.0, ex.y);
    *p1 = cdiv(em1, x);
    *p2 = cdiv(make_double2(em1.x - x.x, em1.y - x.y), cmul(x, x));
  }
}

// Laplace transform G(z) = int_{t_0}^{t_{N-1}} e^{i z t} g(t) dt of samples g(t_j):
//   method 0: exact integral of the piecewise-linear interpolant, segment by segment
//     int_{t_j}^{t_j+h} e^{u t} g dt = h e^{u t_j} [g_j phi2(u h) + g_{j+1} (phi1 - phi2)(u h)],  u = i z;
//   method 1: trapezoidal rule.
__global__ void k_laplace_t2z(const double* __restrict__ t, const double2* __restrict__ g, int64_t nt,
                              const double2* __restrict__ z, int64_t nz, int method, double2* __restrict__ out) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= nz) return;
  const double2 u = make_double2(-z[i].y, z[i].x);  // i z
  double2 acc = make_double2(0.0, 0.0);
  for (int64_t j = 0; j + 1 < nt; ++j) {
    const double h = t[j + 1] - t[j];
    const double2 ej = cexp_(make_double2(u.x * t[j], u.y * t[j]));
    if (method == 0) {
      double2 p1, p2;
      phi12(make_double2(u.x * h, u.y * h), &p1, &p2);
      const double2 c0 = cmul(g[j], p2);
      const double2 c1 = cmul(g[j + 1], make_double2(p1.x - p2.x, p1.y - p2.y));
      const double2 seg = cmul(ej, make_double2(h * (c0.x + c1.x), h * (c0.y + c1.y)));
      acc.x += seg.x;
      acc.y += seg.y;
    } else {
      const double2 ej1 = cexp_(make_double2(u.x * t[j + 1], u.y * t[j + 1]));
      const double2 a = cmul(ej, g[j]), b = cmul(ej1, g[j + 1]);
      acc.x += 0.5 * h * (a.x + b.x);
      acc.y += 0.5 * h * (a.y + b.y);
    }
  }
  out[i] = acc;
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

ED_API ed_status ed_tevo_sum(const double* d_lam, const double* d_w, int64_t m, double e0, int sign, const double* d_t,
                             int64_t n_t, double* d_out, int accumulate, ed_stream_t stream) {
  if (m < 0 || n_t < 0) return fail(ED_ERR_INVALID_ARG, "negative size");
  if (sign != 1 && sign != -1) return fail(ED_ERR_INVALID_ARG, "sign must be +1 or -1");
  if (n_t == 0) return ED_OK;
  if ((m > 0 && (!d_lam || !d_w)) || !d_t || !d_out) return fail(ED_ERR_INVALID_ARG, "null argument");
  if (!std::isfinite(e0)) return fail(ED_ERR_NONFINITE, "e0 is not finite");
  k_tevo_sum<<<(unsigned)((n_t + 127) / 128), 128, 0, as_stream(stream)>>>(d_lam, d_w, m, e0, sign, d_t, n_t,
                                                                           (double2*)d_out, accumulate);
  ED_CHECK_LAUNCH("k_tevo_sum");
  return ED_OK;
}

ED_API ed_status ed_laplace_t2z(const double* d_t, const double* d_gt, int64_t n_t, const double* d_z, int64_t n_z,
                                int method, double* d_out, ed_stream_t stream) {
  if (n_t < 0 || n_z < 0) return fail(ED_ERR_INVALID_ARG, "negative size");
  if (method != 0 && method != 1) return fail(ED_ERR_INVALID_ARG, "method must be 0 (linear) or 1 (trapezoid)");
  if (n_z == 0) return ED_OK;
  if (!d_t || !d_gt || !d_z || !d_out) return fail(ED_ERR_INVALID_ARG, "null argument");
  k_laplace_t2z<<<(unsigned)((n_z + 127) / 128), 128, 0, as_stream(stream)>>>(d_t, (const double2*)d_gt, n_t,
                                                                              (const double2*)d_z, n_z, method,
                                                                              (double2*)d_out);
  ED_CHECK_LAUNCH("k_laplace_t2z");
  return ED_OK;
}

}  // extern "C"
