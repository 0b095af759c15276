// Internal layout of an ed_plan: one Hamiltonian sector resident on one device.
//
// Fermionic sectors keep, per spin species, the sorted states, the on-site energy of each
// state and a target-centric hopping table (CSR): row i lists (j, c) with H_ij = c for the
// single-spin hops out of state i. Because a hop only flips the two bond bits, the
// reference's sign (cmpy/operators.py:425-433) is the same in both directions, so the table
// also gives y_i += c * x_j for the matvec (the reference's y[col] += val * x[row]).
// Spin sectors keep one table over the states plus the precomputed diagonal.
#pragma once

#include <vector>

#include "ed_common.cuh"

namespace ed {

struct SpinTable {
  int64_t n = 0;              // number of states of this spin species
  int64_t nnz = 0;            // table entries
  uint64_t* states = nullptr; // [n] ascending
  double* energy = nullptr;   // [n] weighted_element(state, eps)
  int32_t* off = nullptr;     // [n+1]
  int32_t* idx = nullptr;     // [nnz] target state index j
  double* coef = nullptr;     // [nnz] hop value with sign
  int32_t max_row = 0;        // longest row
};

struct FermionParams {
  int n_sites;
  int u_uniform;   // 1 if all u[i] equal (then U-term = u0 * popcount)
  double u0;
  double u[ED_MAX_SITES + 2];
};

}  // namespace ed

struct ed_plan_s {
  int kind = 0;  // 0 fermion, 1 spin
  int device = -1;
  int n_sites = 0, n_up = 0, n_dn = 0;
  int64_t num_up = 0, num_dn = 0, dim = 0;
  int64_t nnz = 0;
  double hnorm_bound = 0.0;
  // model copy (host)
  std::vector<double> eps, u;
  std::vector<int32_t> b1, b2;
  std::vector<double> hop;
  int sign_width = 0;
  // spin model copy (host)
  std::vector<int32_t> p1, p2;
  std::vector<double> pj, pjz;
  // device tables
  ed::SpinTable up, dn;       // fermion: up/dn species; spin: `up` holds the states
  ed::FermionParams fp;
  double* spin_diag = nullptr;  // spin: [D]
  ed::DeviceContext* ctx = nullptr;
};

namespace ed {
ed_status enumerate_into(int n_sites, int n, uint64_t* d_out, cudaStream_t s);
ed_status check_plan(const ed_plan_s* p);
// y = H x for nvec vectors (leading dimension ld); skipped when *stop != 0 (stop may be null).
ed_status matvec_f64(const ed_plan_s* p, const double* x, double* y, int64_t nvec, int64_t ld, cudaStream_t s,
                     const int* stop = nullptr);
}  // namespace ed
