// Generic CSR operator for user-supplied triplets (HamiltonOperator(size, data, indices),
// cmpy/operators.py:617-630). Bit-for-bit agreement with the reference's sequential
// `y[col] += val * x[row]` needs strictly sequential accumulation, so each row is summed
// by one thread in storage order with separately rounded multiply and add. This path is
// for user-defined models only; the built-in models use the matrix-free kernels.
#include "ed_plan.cuh"

namespace ed {

__global__ void k_csr_matvec(int64_t n, const int64_t* __restrict__ rowptr, const int64_t* __restrict__ cols,
                             const double* __restrict__ vals, const double* __restrict__ x, double* __restrict__ y) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
    double acc = 0.0;
    const int64_t k1 = rowptr[r + 1];
    for (int64_t k = rowptr[r]; k < k1; ++k) acc = __dadd_rn(acc, __dmul_rn(vals[k], x[cols[k]]));
    y[r] = acc;
  }
}

}  // namespace ed

using namespace ed;

extern "C" {

ED_API ed_status ed_csr_matvec(int64_t n, const int64_t* rowptr, const int64_t* cols, const double* vals,
                               const double* x, double* y, ed_stream_t stream) {
  if (n < 0) return fail(ED_ERR_INVALID_ARG, "negative n_rows");
  if (n == 0) return ED_OK;
  if (!rowptr || !x || !y) return fail(ED_ERR_INVALID_ARG, "null argument");
  DeviceContext* ctx;
  ED_TRY(device_context(&ctx));
  k_csr_matvec<<<grid_for(n, 128, ctx->num_sms * 16), 128, 0, as_stream(stream)>>>(n, rowptr, cols, vals, x, y);
  ED_CHECK_LAUNCH("k_csr_matvec");
  return ED_OK;
}

}  // extern "C"
