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
  int16_t* bond = nullptr;    // [nnz] bond of the entry (fermion tables)
  int32_t max_row = 0;        // longest row
};

struct FermionParams {
  int n_sites;
  int u_uniform;   // 1 if all u[i] equal (then U-term = u0 * popcount)
  double u0;
  double u[ED_MAX_SITES + 2];
};

// Tables of the banded two-pass ("sweep") fixed-point matvec (ed_sweep.cuh). The up and the
// dn states are renumbered (reverse Cuthill-McKee order of each spin's hop graph) so that the
// single-spin hop matrices are banded; a Lanczos run that uses this matvec keeps its vectors
// in the renumbered basis (index u' * num_dn + d').
// tables of the stripe matvec (variant 6, ed_stripe.cuh): states renumbered by hop count, hop
// lists in list-major pairs of 16-bit record slots
struct StripeTables {
  int on = 0;
  int per_sm_up = 0, per_sm_dn = 0;  // CTAs per SM of pass 1 / pass 2 (shared memory)
  int pmax_up = 0, pmax_dn = 0;      // list pairs per target, largest
  int32_t* perm_up = nullptr;        // [nu] renumbered -> original up index
  int32_t* perm_dn = nullptr;        // [nd]
  // per renumbered target: pairs of partner record slots (+ pairs first, then - pairs, each
  // segment padded to whole pairs with the zero record), list-major [pair][n] uint32
  uint32_t* lst_up = nullptr;
  uint32_t* lst_dn = nullptr;
  uint16_t* meta_up = nullptr;       // [nu]: + pairs | - pairs << 8
  uint16_t* meta_dn = nullptr;       // [nd]
  uint64_t* s_up = nullptr;          // states, renumbered
  uint64_t* s_dn = nullptr;
  int32_t* e_up = nullptr;           // diagonal mode 0 energies, renumbered
  int32_t* e_dn = nullptr;
  int64_t* f_up = nullptr;           // diagonal mode 1 energies, renumbered
  int64_t* f_dn = nullptr;
  int pol = 0;                       // L2 policy selection (see ed_stripe.cuh)
};

// tables of variant 7: the single-pass matvec with the dn states renumbered by their numbers
// of + and - hops (the up states keep their order), so that each 64-column chunk of a warp
// loops over its own list lengths instead of every bond slot
struct DnCompactTables {
  int on = 0;
  int rows = 0;                  // table words per column (largest + and - pair counts of a chunk)
  uint32_t* tab = nullptr;       // [rows][nd]: two partner byte offsets (16 * column) per word
  uint16_t* chunk = nullptr;     // [nd / 64]: + pairs | - pairs << 8 of each 64-column chunk
  int32_t* perm_up = nullptr;    // [nu] identity
  int32_t* perm_dn = nullptr;    // [nd] renumbered -> original dn index
  uint64_t* s_dn = nullptr;      // dn states, renumbered
  int32_t* e_dn = nullptr;       // diagonal mode 0 dn energies, renumbered
  int64_t* f_dn = nullptr;       // diagonal mode 1 dn energies, renumbered
};

struct SweepTables {
  int on = 0;
  int ring_up = 0, ring_dn = 0;  // ring capacity in chunks of 32 rows (pass 1) / 32 columns (pass 2)
  int nblk_up = 0, nblk_dn = 0;  // target blocks of 32 rows / 32 columns
  int32_t* perm_up = nullptr;    // [nu] renumbered -> original up index
  int32_t* perm_dn = nullptr;    // [nd]
  // hop lists per renumbered target, 16 uint16 each: entries (ring offset | 0x8000 for a
  // negative sign), entry 15 = count
  uint16_t* lst_up = nullptr;    // [nu][16]
  uint16_t* lst_dn = nullptr;    // [nd][16]
  int2* win_up = nullptr;        // [nblk_up] (first chunk still needed, last chunk needed)
  int2* win_dn = nullptr;        // [nblk_dn]
  uint64_t* s_up = nullptr;      // states, renumbered
  uint64_t* s_dn = nullptr;
  int32_t* e_up = nullptr;       // diagonal mode 0 energies, renumbered
  int32_t* e_dn = nullptr;
  int64_t* f_up = nullptr;       // diagonal mode 1 energies, renumbered
  int64_t* f_dn = nullptr;
  int pol = 0;                   // L2 policy selection of the two passes (see ed_sweep.cuh)
};

// Tables of the block-fixed-point (BFP) matvec. Eligible sectors have one hopping magnitude
// |t| = t_int * 2^-F (t_int a small integer). Output exponent e_w = e_x - F and
//   W = t_int * sum(+-X_nbr) + D(X)
// for input mantissas |X| <= 2^m_in, where the diagonal term D is
//   diag64 = 0: diag_int * X, exact (eps, U exact integers times 2^-F);
//   diag64 = 1: round(diag_fx * X / 2^(Fd - F)) with diag_fx = diag * 2^Fd in int64
//               (arbitrary FP64 on-site energies; one rounding per element).
struct BfpTables {
  int eligible = 0;
  int F = 0;              // hopping scale: |t| = t_int * 2^-F
  int m_in = 56;          // input mantissa bound 2^m_in
  int32_t t_int = 0;      // hop magnitude as integer
  int diag64 = 0;         // diagonal mode (see above)
  int Fd = 0;             // diag64: fractional bits of diag_fx
  int u_uniform = 1;
  int32_t u0_int = 0;
  int32_t u_int[ED_MAX_SITES + 2] = {};
  int64_t u0_fx = 0;
  int64_t u_fx[ED_MAX_SITES + 2] = {};
  int64_t* e_up_fx = nullptr;  // diag64: [nu]
  int64_t* e_dn_fx = nullptr;  // diag64: [nd]
  int max_dn = 0;         // dn table entries per column (padded)
  int vec2 = 0;           // num_dn even: 128-bit row loads
  // up: per target row, neighbours with + sign first, then - sign
  int32_t* up_off = nullptr;   // [nu+1]
  int32_t* up_npos = nullptr;  // [nu]
  int32_t* up_idx = nullptr;   // [nnz]
  // dn: column-major [max_dn][nd] shared-memory slots: j (+), nd + j (-), 2*nd (zero)
  uint16_t* dn_tab = nullptr;
  // dn, bond-major: one row of partner columns per (bond, sign) that occurs, nd marking "no
  // hop" (a zero slot); + rows first, each sign class padded to an even count with zero rows;
  // rows packed in pairs as byte offsets into the interleaved row pair (16 bytes per column):
  // [n_b2][nd] uint32 = 16*slot(2p) | 16*slot(2p+1) << 16
  uint32_t* dn_btab2 = nullptr;
  int n_b2 = 0, n_b2pos = 0;
  int max_up = 0;               // most up-neighbours of one row
  // up lists as the v3 matvec stages them, one bulk copy per row group: [nu + 1][up_lstride]
  // element offsets idx * nd (+ segment, then - segment, each padded to a multiple of 4 with
  // the row's own offset), and [nu + 1][4] = (+ length, - length, padding correction, 0);
  // row nu is an empty list (read by the second row slot of a final one-row group)
  int32_t* up_lst = nullptr;
  int32_t* up_cnt = nullptr;
  int up_lstride = 0;
  int32_t* e_up_int = nullptr;  // [nu]
  int32_t* e_dn_int = nullptr;  // [nd]
  SweepTables sw;
  StripeTables sp;
  DnCompactTables dc;
  long wait_limit = 0;          // polls of a first bulk-copy wait before giving up (0: default)
  int force_var = 0;            // matvec variant chosen for this plan (0: automatic)
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
  ed::BfpTables bfp;
};

namespace ed {
ed_status enumerate_into(int n_sites, int n, uint64_t* d_out, cudaStream_t s);
ed_status check_plan(const ed_plan_s* p);
// y = H x for nvec vectors (leading dimension ld); skipped when *stop != 0 (stop may be null).
ed_status matvec_f64(const ed_plan_s* p, const double* x, double* y, int64_t nvec, int64_t ld, cudaStream_t s,
                     const int* stop = nullptr);
// Builds p->bfp when the sector qualifies (called at plan creation; synchronous).
ed_status build_bfp(ed_plan_s* p, cudaStream_t s);
void free_bfp(ed_plan_s* p);
// fixed-point Lanczos (ed_bfp.cu)
size_t bfp_workspace_bytes(const ed_plan_s* p, int K, bool store);
ed_status bfp_lanczos(const ed_plan_s* p, const ed_lanczos_params* prm, const double* v0_dev, void* work,
                      double* alpha, double* beta, double* evec, ed_lanczos_result* res, cudaStream_t s,
                      double* v0_tmp);
ed_status bfp_lanczos_coeffs_multi(int n, const ed_plan_s* const* plans, int K, const double* const* starts,
                                   void* const* works, double* const* alphas, double* const* betas, int* steps,
                                   double* norms, cudaStream_t s);
ed_status bfp_lanczos_coeffs(const ed_plan_s* p, int K, const double* start, void* work, double* alpha,
                             double* beta, int* steps, double* norm, cudaStream_t s);
}  // namespace ed
