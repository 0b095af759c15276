/*
 * cmpy_ed.h — C ABI of the GB300 exact-diagonalisation engine (libcmpy_ed.so).
 *
 * The engine replaces the hot path of cmpy: Fock-sector enumeration (cmpy/basis.py),
 * the COO Hamiltonian projectors (cmpy/operators.py), the HamiltonOperator matvec
 * (cmpy/operators.py:614-646), the fermionic creation/annihilation operators
 * (cmpy/operators.py:652-791), the ground-state driver (cmpy/exactdiag.py:24-57) and the
 * Green's functions (cmpy/exactdiag.py:110-245).
 *
 * Conventions (identical to the reference):
 *   - site i <-> bit i of a uint64 bitstring (LSB = site 0);
 *   - a spin sector lists the ascending integers with popcount n (colex order), so the
 *     index of a state is rank(s) = sum_k C(p_k, k) over its set-bit positions p_1<p_2<...;
 *   - many-body index is up-major: idx = up_idx * num_dn + dn_idx;
 *   - values are IEEE FP64, indices int64.
 *
 * Memory: every vector/array argument prefixed d_ is caller-owned DEVICE memory; h_ is
 * host memory. Plans (opaque) own only their small per-spin tables. Every call is
 * asynchronous on the given stream unless its comment says "synchronous", and returns an
 * ed_status; nothing throws. A plan is not thread-safe; separate plans are.
 */
#ifndef CMPY_ED_H
#define CMPY_ED_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define ED_API __attribute__((visibility("default")))
#else
#define ED_API
#endif

typedef void* ed_stream_t; /* a cudaStream_t; NULL = legacy default stream */

typedef enum ed_status {
  ED_OK = 0,
  ED_ERR_INVALID_ARG = 1,  /* bad size/pointer/site index (reference: assert / ValueError) */
  ED_ERR_CUDA = 2,         /* a CUDA runtime call failed; see ed_last_error() */
  ED_ERR_TIMEOUT = 3,      /* a bounded device-side wait ran out */
  ED_ERR_NONFINITE = 4,    /* NaN/Inf in model parameters or start vector */
  ED_ERR_TOO_LARGE = 5,    /* dimension beyond the engine's index range / capacity */
  ED_ERR_ZERO_VECTOR = 6,  /* start vector has zero norm */
  ED_ERR_DEVICE = 7,       /* a kernel's own bounds check fired (device status word) */
  ED_ERR_NOT_FOUND = 8     /* target sector does not exist (e.g. c^dag on a full sector) */
} ed_status;

/* ---- library ------------------------------------------------------------------------ */

ED_API const char* ed_status_string(int status);
/* Last error message of the calling thread (CUDA error string or argument diagnostic). */
ED_API const char* ed_last_error(void);
ED_API int ed_version(void); /* major*10000 + minor*100 + patch */
/* Number of kernels this library has launched in the process (all devices, all threads). */
ED_API uint64_t ed_launch_count(void);

/* ---- basis: cmpy/basis.py ----------------------------------------------------------- */

/* Binomial coefficient C(n, k) for 0 <= k <= n <= 63 (else 0). Host function. */
ED_API int64_t ed_binomial(int n, int k);

/* Number of states of a spin sector: C(n_sites, n), or 2^n_sites when n < 0 ("n=None"). */
ED_API int64_t ed_sector_size(int n_sites, int n);

/* Replaces Basis.generate_states / get_states (cmpy/basis.py:655-676) and the
 * init_sectors scan (cmpy/basis.py:644-653): writes the ascending states with popcount
 * n into d_out[0 .. ed_sector_size(n_sites, n)). n < 0 writes 0 .. 2^n_sites - 1.
 * n_sites <= 62. capacity is the length of d_out in elements. */
ED_API ed_status ed_enumerate(int n_sites, int n, uint64_t* d_out, int64_t capacity,
                              ed_stream_t stream);

/* Index of each state inside its own popcount sector (the combinatorial number system);
 * equals bisect_left(get_states(popcount(s)), s) (cmpy/operators.py:276-299). */
ED_API ed_status ed_rank(const uint64_t* d_states, int64_t count, int64_t* d_ranks,
                         ed_stream_t stream);

/* ---- models: cmpy/models/hubbard.py, anderson.py, heisenberg.py --------------------- */

/* Fermionic model descriptor (host memory, copied at plan creation).
 *   eps[i]  on-site energy of site i, chemical potential already subtracted
 *           (HubbardModel: eps - mu, cmpy/models/hubbard.py:77;
 *            SIAM: [eps_imp - mu, eps_bath...], cmpy/models/anderson.py:151);
 *   u[i]    Hubbard U of site i (SIAM: [U, 0, ...], cmpy/models/anderson.py:150);
 *   bonds   (site1 < site2, hop) in emission order (hubbard.py:19-21 keeps i<j pairs of
 *           the neighbour list; anderson.py:156-158 has (0, j+1, v_j));
 *   sign_width  the `width` of the reference's fermionic sign bit_count
 *           (cmpy/operators.py:253-273,425-433): n_sites for HubbardModel, 0 for the SIAM
 *           (cmpy/models/anderson.py:149 passes nsites = 0, i.e. no sign). */
typedef struct ed_fermion_model {
  int32_t n_sites;
  int32_t n_bonds;
  int32_t sign_width;
  int32_t reserved;
  const double* h_eps;
  const double* h_u;
  const int32_t* h_bond_site1;
  const int32_t* h_bond_site2;
  const double* h_bond_hop;
} ed_fermion_model;

/* Spin-1/2 XXZ model on directed site pairs, in the emission order of
 * HeisenbergModel._hamiltonian_data (cmpy/models/heisenberg.py:19-40): for every state,
 * for pos1 in 0..n_sites-1, for pos2 in neighbours(pos1). Each pair carries its own
 * coupling (the reference has one uniform j, jz; per-pair values generalise it). Per
 * directed pair the diagonal gets sign*0.25*jz and a flip gets (0.25*j)/2. */
typedef struct ed_spin_model {
  int32_t n_sites;
  int32_t n_pairs;
  const int32_t* h_pos1;
  const int32_t* h_pos2;
  const double* h_j;
  const double* h_jz;
} ed_spin_model;

/* ---- plans: one Hamiltonian sector on one device ------------------------------------- */

typedef struct ed_plan_s* ed_plan;

typedef struct ed_plan_info {
  int64_t dim;        /* sector dimension D */
  int64_t num_up;     /* number of up states (spin model: D) */
  int64_t num_dn;     /* number of dn states (spin model: 1) */
  int64_t hop_up;     /* single-spin hopping table entries, up */
  int64_t hop_dn;     /* single-spin hopping table entries, dn */
  int64_t nnz;        /* triplets the reference generator would emit for this sector */
  int32_t n_sites;
  int32_t kind;       /* 0 fermion, 1 spin */
  int32_t n_up;
  int32_t n_dn;
  double hnorm_bound; /* upper bound of ||H||_inf (max row abs sum) */
} ed_plan_info;

/* Build the sector basis and hopping tables on the device (replaces
 * AbstractManyBodyModel.hamilton_operator's setup, cmpy/models/abc.py:250-256).
 * n_up/n_dn in 0..n_sites. Synchronous on `stream` (it reads back table sizes). */
ED_API ed_status ed_plan_create_fermion(const ed_fermion_model* model, int n_up, int n_dn,
                                        ed_plan* out, ed_stream_t stream);
/* Spin model: sector with n_up up-spins (AbstractSpinModel.hamilton_operator,
 * cmpy/models/abc.py:194-199; SpinBasis.get_states(s) with n_up = N/2 + s). */
ED_API ed_status ed_plan_create_spin(const ed_spin_model* model, int n_up, ed_plan* out,
                                     ed_stream_t stream);
ED_API ed_status ed_plan_destroy(ed_plan plan);
ED_API ed_status ed_plan_get_info(ed_plan plan, ed_plan_info* out);
/* Device pointers to the plan's sorted spin-sector states (valid until destroy). */
ED_API ed_status ed_plan_states(ed_plan plan, const uint64_t** d_up, const uint64_t** d_dn);

/* ---- Hamiltonian application: HamiltonOperator._matvec (cmpy/operators.py:626-630) --- */

/* y = H x for the plan's sector (H is real symmetric, so this equals the reference's
 * y[col] += val * x[row] loop over its triplets). d_x, d_y: FP64[D], must not alias. */
ED_API ed_status ed_matvec(ed_plan plan, const double* d_x, double* d_y, ed_stream_t stream);
/* Y = H X for n_vec column-major vectors with leading dimension ld >= D
 * (LinearOperator._matmat). */
ED_API ed_status ed_matmat(ed_plan plan, const double* d_x, double* d_y, int64_t n_vec,
                           int64_t ld, ed_stream_t stream);
/* Dense H (row-major D x D) for small sectors, summed in triplet order like
 * HamiltonOperator.toarray (cmpy/operators.py:632-635). D <= 32768. */
ED_API ed_status ed_dense(ed_plan plan, double* d_out, ed_stream_t stream);
/* Diagonal of H (HamiltonOperator._trace sums it, cmpy/operators.py:641-646). */
ED_API ed_status ed_diagonal(ed_plan plan, double* d_out, ed_stream_t stream);

/* Generic sparse operator for user-supplied triplets (HamiltonOperator(size, data, indices),
 * cmpy/operators.py:617-630): y[r] = sum_k vals[k] * x[cols[k]] over k in
 * [rowptr[r], rowptr[r+1]), accumulated in storage order from 0.0 with separately rounded
 * multiply and add. Storing the triplets transposed and stably sorted by their column
 * reproduces the reference loop `y[col] += val * x[row]` bit for bit. */
ED_API ed_status ed_csr_matvec(int64_t n_rows, const int64_t* d_rowptr, const int64_t* d_cols,
                               const double* d_vals, const double* d_x, double* d_y,
                               ed_stream_t stream);

/* ---- COO projectors: cmpy/operators.py:305-527, hubbard.py:13-22, heisenberg.py:19-40 */

/* Triplet segments in the reference's emission order. Each function works in two calls:
 * with d_rows == NULL it only counts (synchronous; *h_nnz receives the count), otherwise it
 * writes exactly that many triplets into d_rows/d_cols/d_vals (capacity elements). The
 * state arrays may be any ascending list (bisect_left semantics are kept exactly). */

/* project_onsite_energy(up_states, dn_states, eps) — cmpy/operators.py:359-422 */
ED_API ed_status ed_coo_onsite(const uint64_t* d_up, int64_t num_up, const uint64_t* d_dn,
                               int64_t num_dn, const double* h_eps, int n_values,
                               int64_t* d_rows, int64_t* d_cols, double* d_vals,
                               int64_t capacity, int64_t* h_nnz, ed_stream_t stream);
/* project_hubbard_inter(up_states, dn_states, u) — cmpy/operators.py:305-356 */
ED_API ed_status ed_coo_inter(const uint64_t* d_up, int64_t num_up, const uint64_t* d_dn,
                              int64_t num_dn, const double* h_u, int n_values,
                              int64_t* d_rows, int64_t* d_cols, double* d_vals,
                              int64_t capacity, int64_t* h_nnz, ed_stream_t stream);
/* project_hopping(up_states, dn_states, num_sites, site1, site2, hop) —
 * cmpy/operators.py:463-527 (width = num_sites for the sign). site1 < site2. */
ED_API ed_status ed_coo_hopping(const uint64_t* d_up, int64_t num_up, const uint64_t* d_dn,
                                int64_t num_dn, int width, int site1, int site2, double hop,
                                int64_t* d_rows, int64_t* d_cols, double* d_vals,
                                int64_t capacity, int64_t* h_nnz, ed_stream_t stream);
/* Whole model, the concatenation _ham_data emits (hubbard.py:13-22 / anderson.py:147-158
 * / heisenberg.py:19-40) for the plan's sector. */
ED_API ed_status ed_coo_plan(ed_plan plan, int64_t* d_rows, int64_t* d_cols, double* d_vals,
                             int64_t capacity, int64_t* h_nnz, ed_stream_t stream);

/* ---- fermion operators: cmpy/operators.py:652-791 ------------------------------------ */

/* y = c^dag_{pos,sigma} x (create=1) or c_{pos,sigma} x (create=0), from the plan's sector
 * to the plan_target sector (n_sigma +/- 1). jw_sign=0 reproduces the reference (no
 * Jordan-Wigner sign, cmpy/operators.py:652-703); jw_sign=1 applies the fermionic sign
 * (-1)^(number of same-spin electrons below pos, plus all up electrons for sigma=dn).
 * sigma: 1 = up, 2 = dn (cmpy/basis.py:39). d_y is fully written (zeros where no source).
 * Applies to n_vec column vectors (leading dimensions ld_x >= D, ld_y >= D_target), the
 * matmat of CreationOperator.matmat(evecs) in cmpy/exactdiag.py:132-134. */
ED_API ed_status ed_apply_fermion(ed_plan plan, ed_plan plan_target, int pos, int sigma,
                                  int create, int jw_sign, const double* d_x, double* d_y,
                                  int64_t n_vec, int64_t ld_x, int64_t ld_y,
                                  ed_stream_t stream);

/* The same operator on n independent problems in one call (no reference counterpart; the
 * batched Green's-function driver applies c^dag / c to every realisation's ground state):
 * problem i maps d_x + x_off[i] (plans[i]->dim values) to d_y + y_off[i] (targets[i]->dim
 * values). x_off / y_off are HOST arrays of element offsets. Every problem is checked (as in
 * ed_apply_fermion) before the first launch, so an error leaves d_y untouched. */
ED_API ed_status ed_apply_fermion_batch(const ed_plan* plans, const ed_plan* targets, int n,
                                        int pos, int sigma, int create, int jw_sign,
                                        const double* d_x, const int64_t* x_off, double* d_y,
                                        const int64_t* y_off, ed_stream_t stream);

/* ---- Lanczos ground state (replaces eigsh in cmpy/exactdiag.py:24-43) ----------------- */

typedef struct ed_lanczos_params {
  int32_t max_steps;     /* Krylov dimension limit K */
  int32_t reorth;        /* 0 = none (plain three-term), 1 = full (classical Gram-Schmidt twice) */
  int32_t check_every;   /* device-side convergence test period (0 = never, run K steps) */
  int32_t want_vector;   /* 1 = form the Ritz ground-state vector (needs the stored basis) */
  double tol;            /* stop when the Ritz residual |beta_m s_m| <= tol * max(1, |E|) */
  uint64_t seed;         /* start vector seed when d_v0 == NULL */
  int32_t profile;       /* 1 = time every matvec launch with CUDA events on `stream` */
  int32_t arithmetic;    /* 0 auto: block-fixed-point vectors when the sector allows it
                            (ed_plan_fixed_point > 0, no reorth), else FP64;
                            1 FP64 vectors; 2 fixed-point (error if the sector does not allow it) */
} ed_lanczos_params;

typedef struct ed_lanczos_result {
  double energy;         /* lowest Ritz value */
  double residual;       /* |beta_m * s_m| Ritz residual estimate */
  double matvec_ms;      /* total matvec kernel time (profile = 1), else 0 */
  int32_t steps;         /* Lanczos steps taken (size m of T) */
  int32_t converged;     /* 1 if tol met, 2 if invariant subspace (breakdown) */
  int32_t status;        /* device status word */
  int32_t matvecs;       /* matvec launches timed */
} ed_lanczos_result;

/* Bytes of caller-provided device workspace for ed_lanczos (Krylov basis included). */
ED_API ed_status ed_lanczos_workspace(ed_plan plan, const ed_lanczos_params* params,
                                      size_t* h_bytes);
/* Runs the Lanczos iteration on the device. d_v0: optional start vector FP64[D].
 * Writes alpha[0..steps) and beta[0..steps] (beta[0] = 0, beta[k] couples k-1 and k,
 * beta[steps] is the residual coupling) into d_alpha (FP64[max_steps]) and d_beta
 * (FP64[max_steps+1]), the normalised ground state to d_evec (FP64[D], if want_vector).
 * The steps are enqueued without waiting; with tol > 0 the host reads the scalars every
 * check_every steps and tests convergence, and at the end it solves the m x m tridiagonal
 * eigenproblem (a serial FP64 chain, faster on a host core than in one GPU block).
 * Synchronous at the end (fills *h_result). */
ED_API ed_status ed_lanczos(ed_plan plan, const ed_lanczos_params* params,
                            const double* d_v0, void* d_work, size_t work_bytes,
                            double* d_alpha, double* d_beta, double* d_evec,
                            ed_lanczos_result* h_result, ed_stream_t stream);

/* Lanczos coefficients of the Krylov space of d_start (not normalised; its norm is
 * returned in *h_norm): the continued-fraction input of the Green's function. No basis is
 * stored (three vectors of workspace; size from ed_lanczos_workspace with want_vector = 0,
 * reorth = 0, arithmetic = 0). Uses the fixed-point vectors when the sector allows it.
 * Returns the number of steps in *h_steps. */
ED_API ed_status ed_lanczos_coeffs(ed_plan plan, int max_steps, const double* d_start,
                                   void* d_work, size_t work_bytes, double* d_alpha,
                                   double* d_beta, int* h_steps, double* h_norm,
                                   ed_stream_t stream);
/* n independent ed_lanczos_coeffs runs in one call (e.g. the particle and the hole part of a
 * Green's function, cmpy/exactdiag.py:215-245 takes both from one ground state): with
 * fixed-point plans their steps interleave on n internal streams forked from `stream`, so one
 * run's kernels fill the SMs that the other's leave idle; results equal the runs done one after
 * another. Run i: plans[i], d_starts[i], d_work[i] (work_bytes[i]), d_alpha[i], d_beta[i] ->
 * h_steps[i], h_norm[i]; workspaces and outputs must be distinct. Synchronous. */
ED_API ed_status ed_lanczos_coeffs_multi(int n, const ed_plan* plans, int max_steps,
                                         const double* const* d_starts, void* const* d_work,
                                         const size_t* work_bytes, double* const* d_alpha,
                                         double* const* d_beta, int* h_steps, double* h_norm,
                                         ed_stream_t stream);

/* Lowest eigenpair of the symmetric tridiagonal matrix (alpha[0..m), beta[1..m)) on the
 * device, FP64 (replaces scipy.linalg.eigh_tridiagonal in cmpy/exactdiag.py:368-375).
 * d_vec (FP64[m]) may be NULL. */
ED_API ed_status ed_tridiag_lowest(const double* d_alpha, const double* d_beta, int m,
                                   double* d_value, double* d_vec, ed_stream_t stream);
/* The same for B tridiagonals in one launch (one block each): problem b is alpha[b*lda ..],
 * beta[b*ldb ..] of size d_m[b] <= max_m (device int array); eigenvalue -> d_values[b],
 * eigenvector -> d_vecs[b*ldv ..]. Used by the adjoint Green's function for the ground state
 * of each taped Lanczos run (the reference's eigh_tridiagonal, cmpy/exactdiag.py:368-375). */
ED_API ed_status ed_tridiag_lowest_batch(const double* d_alpha, int lda, const double* d_beta, int ldb,
                                         const int* d_m, int B, int max_m, double* d_values, double* d_vecs,
                                         int ldv, ed_stream_t stream);
/* v_b = -(T_b - e0_b)^+ r_b on the complement of c_b, for B tridiagonals (c_b the unit
 * eigenvector of T_b's lowest eigenvalue e0_b, d_e0 on the device): the tridiagonal part of the
 * reverse pass through a Lanczos ground state. No reference counterpart (cmpy has no
 * derivatives). d_rhs and d_out must not alias. */
ED_API ed_status ed_tridiag_pinv_solve_batch(const double* d_alpha, int lda, const double* d_beta, int ldb,
                                             const int* d_m, int B, int max_m, const double* d_e0,
                                             const double* d_c, int ldc, const double* d_rhs, double* d_out,
                                             int ldr, ed_stream_t stream);
/* Every eigenpair of B real symmetric matrices, FP64 (replaces numpy.linalg.eigh in
 * solve_sector, cmpy/exactdiag.py:46-57, and the dense branch of exactdiag.py:24-43).
 * Matrix b has order h_n[b] (host array, 1 <= h_n[b] <= n_max), row-major at
 * d_a + b*stride_a with leading dimension lda, and is overwritten (Householder reflectors).
 * Eigenvalues ascending -> d_w[b*n_max + i]; eigenvector i -> row i of
 * d_z + b*stride_z (leading dimension ldz), i.e. Z = V^T. Degenerate eigenvalues get an
 * orthonormal basis of their eigenspace. Asynchronous on `stream` (work memory from
 * cudaMallocAsync: (4 + 5 n_max) B n_max doubles). */
ED_API ed_status ed_dense_eigh_batch(double* d_a, int64_t lda, int64_t stride_a, const int* h_n, int B, int n_max,
                                     double* d_w, double* d_z, int64_t ldz, int64_t stride_z,
                                     ed_stream_t stream);
/* Every eigenpair of the symmetric tridiagonal (d_alpha[0..m), d_beta[1..m)): eigenvalues
 * ascending -> d_w, eigenvector i -> row i of d_z (leading dimension ldz). The same bisection
 * and inverse iteration as ed_dense_eigh_batch; used for the real-time Green's function of a
 * Lanczos tridiagonal (no reference counterpart: the reference's gf_greater/gf_lesser evolve
 * states with expm_multiply, cmpy/exactdiag.py:280-330). Asynchronous on `stream`. */
ED_API ed_status ed_tridiag_eigh(const double* d_alpha, const double* d_beta, int m, double* d_w, double* d_z,
                                 int64_t ldz, ed_stream_t stream);

/* ---- batched form: many sectors / realisations in one persistent launch -----------------
 * No reference counterpart: the reference solves sectors one after another on the host
 * (cmpy/exactdiag.py:24-43). A batch holds n fixed-point sector plans (ed_plan_fixed_point
 * > 0; the plans must outlive the batch). One launch runs every problem's Lanczos in its own
 * CTA (largest first from a device work queue); nothing in it allocates or synchronises with
 * the host, so sequences of batched launches can be captured in a CUDA graph. */
typedef struct ed_batch_s* ed_batch;
ED_API ed_status ed_batch_create(const ed_plan* plans, int n, ed_batch* out);
ED_API ed_status ed_batch_destroy(ed_batch batch);
/* Workspace bytes for max_steps and a launch configuration (threads per CTA in
 * {128,256,512,1024}, CTAs per SM); threads <= 0 uses the tuned (or default) configuration. */
ED_API ed_status ed_batch_workspace(ed_batch batch, int max_steps, int threads, int ctas_per_sm,
                                    int cluster_size, size_t* h_bytes);
/* Ground states of every problem. Outputs (device, problem p): alpha[p*K + k], beta[p*(K+1) + k]
 * (beta[p*(K+1)] = start-vector norm), energy[p], residual[p], steps[p]. d_starts: optional
 * DEVICE array of n device pointers to FP64 start vectors (NULL: seeded uniform(0,1)). With
 * want_vector the normalised ground state of problem p is written to d_vecs + d_vec_offsets[p]
 * (d_vec_offsets is a device array). tol/check_every as in ed_lanczos_params. Asynchronous. */
ED_API ed_status ed_batch_lanczos(ed_batch batch, int max_steps, double tol, int check_every,
                                  uint64_t seed, const double* const* d_starts, int want_vector,
                                  void* d_work, size_t work_bytes, double* d_alpha, double* d_beta,
                                  double* d_energy, double* d_residual, int32_t* d_steps,
                                  double* d_vecs, const int64_t* d_vec_offsets, int threads,
                                  int ctas_per_sm, int cluster_size, ed_stream_t stream);
/* Launch configuration: threads per CTA (128, 256, 512, 1024), CTAs per SM, and the
 * thread-block cluster size per problem (1, or 2/4/8 with 512 or 1024 threads: the cluster's
 * CTAs share each problem's vectors and exchange their partial sums through distributed
 * shared memory). threads <= 0 selects the tuned (or default) configuration.
 * Autotuner: times the candidate configurations on a tune_steps run and keeps the fastest for
 * this batch (used when ed_batch_lanczos gets threads <= 0). Synchronous. */
ED_API ed_status ed_batch_tune(ed_batch batch, int tune_steps, void* d_work, size_t work_bytes,
                               double* d_alpha, double* d_beta, double* d_energy,
                               double* d_residual, int32_t* d_steps, int* h_threads,
                               int* h_ctas_per_sm, int* h_cluster_size, float* h_ms,
                               ed_stream_t stream);
/* Adds the continued fraction of every problem (layout of ed_batch_lanczos, norm^2 =
 * beta[p*(K+1)]^2, shift d_e0[p]) at n_z frequencies into d_g[p*n_z + j] (complex FP64). */
ED_API ed_status ed_batch_gf_continued_fraction(int n, int max_steps, const double* d_alpha,
                                                const double* d_beta, const int32_t* d_steps,
                                                const double* d_e0, int sign, const double* d_z,
                                                int64_t n_z, double* d_g, ed_stream_t stream);

/* ---- parameter derivatives (adjoint form; no reference counterpart) ---------------------
 * Number of model parameters of a fermionic plan: 2*n_sites + n_bonds, in the order
 * [eps_0..eps_{N-1}, U_0..U_{N-1}, t_0..t_{nb-1}] (cmpy/models/hubbard.py:13-22 and
 * cmpy/models/anderson.py:147-158 give their meaning). */
ED_API int ed_plan_num_params(ed_plan plan);
/* d_out[theta] (+)= a^T (dH/dtheta) b for every parameter at once (a, b: FP64[D]);
 * dH/deps_j = n_j_up + n_j_dn, dH/dU_j = n_j_up n_j_dn, dH/dt_b = the hopping of bond b with
 * its fermionic sign. Supports n_sites <= 16, n_bonds <= 32. */
ED_API ed_status ed_param_sandwich(ed_plan plan, const double* d_a, const double* d_b, double* d_out,
                                   int accumulate, ed_stream_t stream);

/* Taped FP64 Lanczos for reverse mode. The plain three-term recurrence of cmpy's Lanczos
 * coefficients (cmpy/exactdiag.py:324-365), normalised, from d_start: alpha[0..m),
 * beta[0..m] (beta[0] = ||start||, beta[m] the last residual norm). Every ckpt-th step k
 * stores [q_{k-1}, q_k] in d_ckpt + (k/ckpt)*2*D (q_{-1} = 0): ceil(min(max_steps, D)/ckpt)
 * slots of 2*D doubles. Stops on breakdown (beta_{k+1} <= breakdown*(|alpha_k| + beta_k))
 * and, with tol > 0, when the lowest Ritz pair has |beta_{k+1} c_k| <= tol*max(1, |E|)
 * (tested every check_every steps; the host reads the stop flag then). Synchronous; h_steps
 * = m (0 for a zero start vector). Fermionic plans; workspace from ed_tape_workspace
 * (shared by the three tape calls). */
ED_API ed_status ed_tape_workspace(ed_plan plan, int max_steps, int ckpt, size_t* bytes);
ED_API ed_status ed_lanczos_tape(ed_plan plan, const double* d_start, int max_steps, int ckpt,
                                 double tol, int check_every, double breakdown, void* d_work,
                                 size_t work_bytes, double* d_alpha, double* d_beta,
                                 double* d_ckpt, int* h_steps, ed_stream_t stream);
/* Replays a tape segment by segment from its checkpoints (bit-identical Krylov vectors):
 * d_out = sum_{k<m} d_coef[k] q_k (the Ritz vector) and/or d_dots[k] = q_k . d_probe. */
ED_API ed_status ed_tape_combine(ed_plan plan, int m, int ckpt, const double* d_alpha,
                                 const double* d_beta, const double* d_ckpt, const double* d_coef,
                                 double* d_out, const double* d_probe, double* d_dots,
                                 void* d_work, size_t work_bytes, ed_stream_t stream);
/* Reverse sweep of a tape: given the adjoints of the scalars (d_abar[m], d_bbar[m+1], d_bbar[0]
 * for ||start||) and optional external adjoints of the Krylov vectors q_bar_k +=
 * d_ext_coef[k] * d_ext_vec, accumulates d_theta_bar[p] += dL/dtheta_p (parameter layout of
 * ed_plan_num_params) and writes the adjoint of the start vector to d_start_bar. Each
 * segment is recomputed from its checkpoint; two matvecs per step. */
ED_API ed_status ed_tape_reverse(ed_plan plan, int m, int ckpt, const double* d_alpha,
                                 const double* d_beta, const double* d_ckpt, const double* d_abar,
                                 const double* d_bbar, const double* d_ext_coef,
                                 const double* d_ext_vec, void* d_work, size_t work_bytes,
                                 double* d_theta_bar, double* d_start_bar, ed_stream_t stream);
/* Batched tape: B problems sharing one structure plan (the sector and bonds of `plan`, which
 * is built with t = 1 on every bond, so its coefficients are the fermionic signs; its eps and
 * U are unused) with per-problem parameters d_theta[B][P] (layout of ed_plan_num_params).
 * Vectors are problem-major [B][D]; alpha is [B][max_steps], beta [B][max_steps+1], the
 * checkpoints [slot][2][B][D]. Problem b's arithmetic is that of the single-problem tape;
 * h_steps / h_m hold the B tape lengths. ed_batch_diag writes the per-problem diagonal
 * d_diag[B][D] that the others take; ed_batch_matvec_params applies H_b to x[b]. */
ED_API ed_status ed_batch_diag(ed_plan plan, int B, const double* d_theta, double* d_diag,
                               ed_stream_t stream);
ED_API ed_status ed_batch_matvec_params(ed_plan plan, int B, const double* d_theta,
                                        const double* d_diag, const double* d_x, double* d_y,
                                        ed_stream_t stream);
ED_API ed_status ed_batch_tape_workspace(ed_plan plan, int B, int max_steps, int ckpt,
                                         size_t* bytes);
ED_API ed_status ed_batch_lanczos_tape(ed_plan plan, int B, const double* d_theta,
                                       const double* d_diag, const double* d_start, int max_steps,
                                       int ckpt, double tol, int check_every, double breakdown,
                                       void* d_work, size_t work_bytes, double* d_alpha,
                                       double* d_beta, double* d_ckpt, int* h_steps,
                                       ed_stream_t stream);
ED_API ed_status ed_batch_tape_combine(ed_plan plan, int B, const double* d_theta,
                                       const double* d_diag, const int* h_m, int max_steps,
                                       int ckpt, const double* d_alpha, const double* d_beta,
                                       const double* d_ckpt, const double* d_coef, double* d_out,
                                       const double* d_probe, double* d_dots, void* d_work,
                                       size_t work_bytes, ed_stream_t stream);
ED_API ed_status ed_batch_tape_reverse(ed_plan plan, int B, const double* d_theta,
                                       const double* d_diag, const int* h_m, int max_steps,
                                       int ckpt, const double* d_alpha, const double* d_beta,
                                       const double* d_ckpt, const double* d_abar,
                                       const double* d_bbar, const double* d_ext_coef,
                                       const double* d_ext_vec, void* d_work, size_t work_bytes,
                                       double* d_theta_bar, double* d_start_bar,
                                       ed_stream_t stream);
/* Continued fractions of B tapes at once (the arithmetic of ed_gf_continued_fraction):
 * d_g[b][j] += sign n2[b] / (z'_j - alpha[b][0] - beta[b][1]^2 / ...), z' = sign z + shift[b],
 * m[b] levels (problems with m[b] = 0 are skipped); alpha[b][l] = d_alpha[b*ka + l],
 * beta[b][l] = d_beta[b*kb + l]. ed_batch_cf_adjoint is ed_cf_adjoint per problem
 * (d_abar[b*ka + l], d_bbar[b*kb + l], d_scal[2b], d_scal[2b+1]); m_max = max m[b]. */
ED_API ed_status ed_batch_cf(int B, const double* d_alpha, int64_t ka, const double* d_beta,
                             int64_t kb, const int* d_m, const double* d_n2, const double* d_shift,
                             int sign, const double* d_z, int64_t n_z, double* d_g,
                             ed_stream_t stream);
ED_API ed_status ed_batch_cf_adjoint(int B, const double* d_alpha, int64_t ka,
                                     const double* d_beta, int64_t kb, const int* d_m, int m_max,
                                     const double* d_n2, const double* d_shift, int sign,
                                     const double* d_z, int64_t n_z, const double* d_gbar,
                                     double* d_abar, double* d_bbar, double* d_scal,
                                     ed_stream_t stream);
/* Adjoint of the continued fraction of ed_gf_continued_fraction: for
 * L = Re sum_j conj(gbar_j) G(z_j) (d_z, d_gbar interleaved complex), d_abar[l] = dL/dalpha_l,
 * d_bbar[l] = dL/dbeta_l (l = 1..m-1; d_bbar[0] = dL/d sqrt(norm2), d_bbar[m] = 0),
 * d_scal[0] = dL/dshift, d_scal[1] = dL/dnorm2. */
ED_API ed_status ed_cf_adjoint(const double* d_alpha, const double* d_beta, int m, double norm2,
                               double shift, int sign, const double* d_z, int64_t n_z,
                               const double* d_gbar, double* d_abar, double* d_bbar,
                               double* d_scal, ed_stream_t stream);

/* ---- block-fixed-point vectors (no reference counterpart: GB300 arithmetic) ------------
 * A vector is stored as int64 mantissas m[i] with one exponent e: x[i] = m[i] * 2^e. On
 * GB300 the FP64 pipe is ~60x narrower than the integer pipe, so the engine's fast matvec
 * and Lanczos run on these integer vectors (exact adds, 128-bit dot products).
 *
 * ed_plan_fixed_point: m_in > 0 (the input mantissa bound 2^m_in) when the sector has a
 * fixed-point matvec (one hopping magnitude, eps/U/t exact integers times 2^-F), else 0. */
ED_API int ed_plan_fixed_point(ed_plan plan);
/* d_xm = round(d_x * 2^-e) with max |d_xm| < 2^m_bits; *h_exp = e. Synchronous. */
ED_API ed_status ed_fixed_from_f64(const double* d_x, int64_t n, int m_bits, int64_t* d_xm,
                                   int32_t* h_exp, ed_stream_t stream);
/* d_x = d_xm * 2^exp. Synchronous. */
ED_API ed_status ed_fixed_to_f64(const int64_t* d_xm, int64_t n, int32_t exp, double* d_x,
                                 ed_stream_t stream);
/* W = H X exactly in integers: input mantissas |d_xm| <= 2^m_in (m_in from
 * ed_plan_fixed_point, also returned in *h_m_in), output exponent *h_ew = ex - F. */
ED_API ed_status ed_matvec_fixed(ed_plan plan, const int64_t* d_xm, int32_t ex, int64_t* d_wm,
                                 int32_t* h_ew, int* h_m_in, ed_stream_t stream);
/* Which fixed-point matvec the plan uses (0: none). 7: the single-pass kernel with the dn
 * states renumbered by their numbers of + and - hops (the default where its tables fit); 3, 2,
 * 1: single-pass kernels in the sector's own order; 5: the banded two-pass sweep (up and dn
 * states in reverse Cuthill-McKee order) and 6: two-pass stripes (states sorted by hop count),
 * chosen when forced (5 also where 3 does not fit). Variants 5, 6 and 7 keep the vectors of
 * their Lanczos runs in their renumbered basis; ed_matvec_fixed still takes and returns vectors
 * in the sector's ascending-state order. All variants give bit-identical results. The
 * environment variable CMPY_ED_MATVEC=1..7 forces a variant where the sector allows it. */
ED_API int ed_plan_matvec_variant(ed_plan plan);
/* Chooses the fixed-point matvec variant of this plan (0: automatic, 1..7 as above when the
 * sector allows it, else the automatic choice); for comparisons and benchmarks. Takes effect
 * for the next call; not while a Lanczos run of the plan is in flight. */
ED_API ed_status ed_plan_set_matvec_variant(ed_plan plan, int variant);
/* Polls of a first wait for a bulk copy in the fixed-point matvec before the kernel gives up
 * (records ED_ERR_TIMEOUT in the solve, lets its copies land and returns); 0 restores the
 * default (2^22 polls); -1 makes the first wait give up without polling, which lets tests
 * exercise the give-up path. */
ED_API ed_status ed_plan_set_wait_limit(ed_plan plan, int64_t polls);

/* Allocation-free ed_tridiag_lowest (no counterpart in the reference). For callers that
 * cannot allocate device memory where they need the result: hosts whose device memory
 * belongs to their own allocator (a framework's caching allocator or a fixed pool), plugin
 * hosts that forbid libraries from allocating, and latency-critical loops where an
 * allocation's bookkeeping or implicit synchronisation is not acceptable. The
 * inverse-iteration scratch is a static array of the library's device image holding
 * 5 * 4096 doubles (160 KB on every GPU that loads the library, until the process exits), so
 * m <= 4096; larger m returns ED_ERR_INVALID_ARG, like ed_tridiag_lowest. The first call on a
 * device (and the first after its context was replaced, e.g. by cudaDeviceReset) looks up the
 * array's device address (cudaGetSymbolAddress); that call should come before any stream
 * capture on the device, and later calls can be captured into a CUDA graph. All calls share
 * the array: calls that overlap on the GPU race on it. Calls no cudaMalloc and no allocating
 * library routine; cudaFree(NULL), which frees nothing, only on a thread without a current
 * context, to make the device's primary context current. */
ED_API ed_status ed_tridiag_lowest_noalloc(const double* d_alpha, const double* d_beta, int m,
                                           double* d_value, double* d_vec, ed_stream_t stream);

/* ---- Green's functions -------------------------------------------------------------- */

/* Continued fraction G(z) = sign * norm2 / (z' - a0 - b1^2 / (z' - a1 - ...)) with
 * z' = sign * z + shift over n_z complex frequencies (interleaved re,im FP64), adding into
 * d_g when accumulate=1. With E0 the ground-state energy and (a, b, norm2) the Lanczos
 * coefficients of c^dag|gs> (resp. c|gs>): electron part sign=+1, shift=E0; hole part
 * sign=-1, shift=E0. */
ED_API ed_status ed_gf_continued_fraction(const double* d_alpha, const double* d_beta,
                                          int n_lev, double norm2, double shift, int sign,
                                          const double* d_z, int64_t n_z, double* d_g,
                                          int accumulate, ed_stream_t stream);

/* Lehmann pole sum of cmpy/exactdiag.py:110-129 (_accumulate_sum): with the overlap
 * matrix ov[m, n] = |<m|c^dag|n>|^2 (FP64, d_p1 x d, row-major), adds
 *   sum_{m,n} ov[m,n] (w_n + w'_m) / (z - E'_m + E_n),  w = exp(-beta (E - emin))
 * to g[z] (interleaved complex FP64). beta = +inf gives unit weights like the reference. */
ED_API ed_status ed_lehmann_accumulate(const double* d_evals, int64_t n_d,
                                       const double* d_evals_p1, int64_t n_dp1,
                                       const double* d_overlap, double beta, double emin,
                                       const double* d_z, int64_t n_z, double* d_g,
                                       ed_stream_t stream);

/* Real-time Green's function from Krylov spectral data: with (lam_k, w_k) the eigenvalues of
 * the Lanczos tridiagonal of c^dag|gs> (resp. c|gs>) and w_k = norm^2 * U_0k^2 their weights,
 *   out[n] (+)= -i*sign * sum_k w_k exp(-i sign (lam_k - e0) t_n)
 * over n_t times (interleaved complex FP64 out). sign = +1 gives the greater function
 * -i e^{i E0 t} <gs|c e^{-iHt} c^dag|gs> of gf_greater (cmpy/exactdiag.py:248-273), sign = -1
 * the lesser function +i e^{-i E0 t} <gs|c^dag e^{iHt} c|gs> of gf_lesser (exactdiag.py:276-301),
 * which the reference evaluates with scipy expm_multiply. */
ED_API ed_status ed_tevo_sum(const double* d_lam, const double* d_w, int64_t m, double e0, int sign,
                             const double* d_t, int64_t n_t, double* d_out, int accumulate,
                             ed_stream_t stream);

/* Laplace transform G(z) = int_{t_0}^{t_last} e^{i z t} g(t) dt of complex samples g(t_j) to n_z
 * complex frequencies — fourier_t2z (cmpy/exactdiag.py:311-316), which calls
 * gftool.fourier.tt2z. method 0: exact integral of the piecewise-linear interpolant of g
 * (gftool's default rule, tt2z_lin); method 1: trapezoidal rule (tt2z_trapz). */
ED_API ed_status ed_laplace_t2z(const double* d_t, const double* d_gt, int64_t n_t,
                                const double* d_z, int64_t n_z, int method, double* d_out,
                                ed_stream_t stream);

#ifdef __cplusplus
}
#endif

#endif /* CMPY_ED_H */
