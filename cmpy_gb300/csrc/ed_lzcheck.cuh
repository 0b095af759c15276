// Convergence tests and the final eigenpair of a Lanczos run's tridiagonal matrix, on the
// device (cmpy/exactdiag.py:368-375 solves the same eigenproblem with LAPACK on the host).
//
// The drivers enqueue their Lanczos steps on the caller's stream without waiting. Every
// `check_every` steps a one-block kernel on a side stream (ordered after that step by an
// event) computes the lowest eigenpair of T_m and the residual estimate |beta_m c_{m-1}|; when
// it is below tol * max(1, |E|) it stops the run at m steps (the step kernels read the stop
// flag and return at once). The side stream also copies the stop flag into pinned host
// memory, and the host polls those copies with non-blocking event queries to stop enqueueing;
// it never waits for a check. At the end the caller's stream waits for the side stream and a
// final kernel forms the eigenpair of the run's T_m (reusing the last check when it had the
// same m). The state words are the driver's own (stop, steps).
#pragma once

#include <vector>

#include "ed_tridiag.cuh"

namespace ed {

// result of the device tridiagonal solves of one run (device memory)
struct TriResult {
  int m_checked;    // size of the eigenpair held in cvec from the last check (0: none)
  int m_final;      // size of the final eigenproblem (0: the run stopped on an error)
  double e_checked;
  double r_checked; // residual estimate of that check
  double energy;    // lowest eigenvalue of T_m_final
  double residual;  // |beta[m] c[m-1]|
};

constexpr int TRI_NT = 512;
constexpr int TRI_SM = 512;  // tridiagonals up to this size are solved in shared memory

// the bracket a test after a shorter run gives for the lowest eigenvalue of T_m: by
// interlacing it is at most the earlier value; the earlier residual estimate sets how far below
// it is looked for (the Sturm counts in tridiag_lowest_block confirm the bracket before use)
__device__ __forceinline__ void tri_hint(const TriResult* tr, double* lo, double* hi) {
  *lo = *hi = 0.0;
  if (tr->m_checked <= 0) return;
  const double e = tr->e_checked, s = fmax(1.0, fabs(e));
  *hi = e + 1e-13 * s;
  *lo = e - fmax(16.0 * tr->r_checked, 1e-9 * s);
}

// one convergence test after m steps (side stream)
static __global__ void __launch_bounds__(TRI_NT) k_tri_check(const double* alpha, const double* beta, int m, double tol,
                                                            int* stop, int* steps, TriResult* tr, double* cvec,
                                                            double* work) {
  if (*(volatile int*)stop) return;  // converged, invariant subspace or failed wait already
  double lo, hi;
  tri_hint(tr, &lo, &hi);
  const double e = tridiag_lowest_block<TRI_SM>(alpha, beta, m, cvec, work, lo, hi);
  if (threadIdx.x == 0) {
    const double res = fabs(beta[m] * cvec[m - 1]);
    tr->m_checked = m;
    tr->e_checked = e;
    tr->r_checked = res;
    if (res <= tol * fmax(1.0, fabs(e)) && atomicCAS(stop, 0, 1) == 0) *steps = m;
  }
}

// convergence tests of B problems after m steps, one block per problem (alpha [B][lda],
// beta [B][lda + 1]; per-problem vectors cvec [B][ldw] and work [B][5 ldw])
static __global__ void __launch_bounds__(TRI_NT) k_tri_check_batch(const double* alpha, const double* beta, int lda,
                                                                  int m, double tol, int* stop, int* steps,
                                                                  double* cvec, double* work, int ldw) {
  const int b = blockIdx.x;
  if (*(volatile int*)&stop[b]) return;
  const double* a = alpha + (size_t)b * lda;
  const double* bb = beta + (size_t)b * (lda + 1);
  double* c = cvec + (size_t)b * ldw;
  const double e = tridiag_lowest_block<TRI_SM>(a, bb, m, c, work + (size_t)b * 5 * ldw);
  if (threadIdx.x == 0) {
    const double res = fabs(bb[m] * c[m - 1]);
    if (res <= tol * fmax(1.0, fabs(e)) && atomicCAS(&stop[b], 0, 1) == 0) steps[b] = m;
  }
}

// the final eigenpair (caller's stream, after the side stream): m = steps once stopped, else
// `launched`; stop code 3 (a failed wait) leaves m_final = 0
static __global__ void __launch_bounds__(TRI_NT) k_tri_final(const double* alpha, const double* beta, int launched,
                                                            const int* stop, int* steps, TriResult* tr,
                                                            double* cvec, double* work) {
  const int sc = *(volatile const int*)stop;
  if (sc == 3) {
    if (threadIdx.x == 0) tr->m_final = 0;
    return;
  }
  const int m = sc ? *(volatile int*)steps : launched;
  double e;
  if (tr->m_checked == m) {
    e = tr->e_checked;  // the vector of that check is still in cvec
  } else {
    double lo, hi;
    tri_hint(tr, &lo, &hi);
    e = tridiag_lowest_block<TRI_SM>(alpha, beta, m, cvec, work, lo, hi);
  }
  if (threadIdx.x == 0) {
    tr->m_final = m;
    tr->energy = e;
    tr->residual = fabs(beta[m] * cvec[m - 1]);
    *steps = m;
  }
}

// host side: the side stream, its events and the pinned copies of the stop flags (one flag
// per problem: nflags > 1 for batched runs, where the run ends when every problem stopped)
class SideChecks {
 public:
  ~SideChecks() { release(); }

  // enabled only when the run has convergence tests
  ed_status init(int max_checks, int nflags = 1) {
    if (max_checks <= 0) return ED_OK;
    ED_CUDA(cudaStreamCreateWithFlags(&s2_, cudaStreamNonBlocking));
    ED_CUDA(cudaEventCreateWithFlags(&fence_, cudaEventDisableTiming));
    done_.resize(max_checks, nullptr);
    for (auto& e : done_) ED_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    nflags_ = nflags;
    ED_TRY(pinned_flags(max_checks * nflags));
    n_ = 0;
    polled_ = 0;
    return ED_OK;
  }

  // a test after the work enqueued so far on s: launch(s2) enqueues the check kernel(s) on the
  // side stream, then the stop flags are copied out
  template <class Launch>
  ed_status launch(cudaStream_t s, Launch&& launch_on, const int* d_flags) {
    if (!s2_ || n_ >= (int)done_.size()) return ED_OK;
    ED_CUDA(cudaEventRecord(fence_, s));
    ED_CUDA(cudaStreamWaitEvent(s2_, fence_, 0));
    launch_on(s2_);
    ED_CHECK_LAUNCH("side-stream convergence test");
    ED_CUDA(cudaMemcpyAsync(flags() + (size_t)n_ * nflags_, d_flags, sizeof(int) * nflags_, cudaMemcpyDeviceToHost,
                            s2_));
    ED_CUDA(cudaEventRecord(done_[n_], s2_));
    ++n_;
    return ED_OK;
  }

  // a single-run test of T_m (k_tri_check)
  ed_status launch(cudaStream_t s, const double* alpha, const double* beta, int m, double tol, int* stop, int* steps,
                   TriResult* tr, double* cvec, double* work) {
    return launch(
        s, [&](cudaStream_t s2) { k_tri_check<<<1, TRI_NT, 0, s2>>>(alpha, beta, m, tol, stop, steps, tr, cvec, work); },
        stop);
  }

  // true when a finished test shows every flag set (the run has stopped); never waits
  bool stopped() {
    while (polled_ < n_) {
      const cudaError_t q = cudaEventQuery(done_[polled_]);
      if (q == cudaErrorNotReady) return false;
      if (q != cudaSuccess) {
        (void)cudaGetLastError();
        return false;
      }
      const int* f = flags() + (size_t)polled_ * nflags_;
      bool all = true;
      for (int i = 0; i < nflags_ && all; ++i) all = f[i] != 0;
      if (all) return true;
      ++polled_;
    }
    return false;
  }

  // the caller's stream waits for every test
  ed_status join(cudaStream_t s) {
    if (!s2_) return ED_OK;
    ED_CUDA(cudaEventRecord(fence_, s2_));
    ED_CUDA(cudaStreamWaitEvent(s, fence_, 0));
    return ED_OK;
  }

 private:
  void release() {
    for (auto& e : done_)
      if (e) cudaEventDestroy(e);
    done_.clear();
    if (fence_) cudaEventDestroy(fence_);
    if (s2_) cudaStreamDestroy(s2_);
    fence_ = nullptr;
    s2_ = nullptr;
  }
  // per-thread pinned buffer for the flag copies (grown on demand, kept for the thread's life)
  static ed_status pinned_flags(int n) {
    Pinned& p = pinned();
    if (p.cap >= n) return ED_OK;
    if (p.ptr) cudaFreeHost(p.ptr);
    p.ptr = nullptr;
    p.cap = 0;
    ED_CUDA(cudaHostAlloc((void**)&p.ptr, sizeof(int) * (size_t)n, cudaHostAllocDefault));
    p.cap = n;
    return ED_OK;
  }
  struct Pinned {
    int* ptr = nullptr;
    int cap = 0;
  };
  static Pinned& pinned() {
    static thread_local Pinned p;
    return p;
  }
  int* flags() { return pinned().ptr; }

  cudaStream_t s2_ = nullptr;
  cudaEvent_t fence_ = nullptr;
  std::vector<cudaEvent_t> done_;
  int n_ = 0, polled_ = 0, nflags_ = 1;
};

}  // namespace ed
