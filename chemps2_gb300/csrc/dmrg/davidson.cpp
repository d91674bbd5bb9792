#include "davidson.hpp"

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <vector>

namespace c2g {

namespace {
// Offsets in the small device scratch sm_.
constexpr int kMxM = 0;         // 32 x 32 Rayleigh-Ritz matrix (ld 32)
constexpr int kEvecs = 1024;    // its eigenvectors (ld 32)
constexpr int kEvals = 2048;    // eigenvalues, ascending
constexpr int kDots = 2112;     // up to 64 dot products
constexpr int kDots2 = 2176;    // w.t, w.u
constexpr int kOverlap = 2184;  // keep x keep overlap
constexpr int kLowdin = 2200;   // keep x keep Loewdin matrix
constexpr int kSumSq = 2216;    // one sum of squares
constexpr int kSmall = 2304;
constexpr int kLd = 32;
// Mixed-precision refinement: cycles, FP32 expansions per cycle, and the residual
// reduction (relative to the cycle's exact first residual) that ends a cycle.
constexpr int kRefineCycles = 8;
constexpr int kRefineExpand = 12;
constexpr double kRefineRel = 1e-3;
// A stall of the reduced-precision phase (no 0.7x residual reduction in 6 iterations)
// with a residual of at most kStallCeiling |theta| is its arithmetic's floor: the
// refinement cycles take over. A stall above it marks a hard step: a residual plateau from
// a poor guess (the first sweep from a random start), on which the FP64 solver may still
// turn to a lower eigenpair after many more products while the reduced-precision one
// settles on an excited state. Such a step, and one that needs more than kLoMaxMatvec
// reduced-precision products, is solved by the FP64 solver from the guess.
constexpr double kStallCeiling = 1e-3;
constexpr int kLoMaxMatvec = 1000;
}  // namespace

DeviceDavidson::DeviceDavidson(Runtime& rt, int64_t n, int max_vec, int keep, double rtol, double cutoff)
    : rt_(rt), n_(n), max_vec_(max_vec), keep_(keep), rtol_(rtol), cutoff_(cutoff) {
  if (max_vec > kLd || keep < 1 || keep > 4 || keep >= max_vec)
    throw std::invalid_argument("Davidson: unsupported number of vectors");
  V_ = rt_.alloc(n_ * max_vec_);
  HV_ = rt_.alloc(n_ * max_vec_);
  W_ = rt_.alloc(n_ * (3 + keep_));
  sm_ = rt_.alloc(kSmall);
  rt_.zero(sm_, kSmall);
  host_ = rt_.pinned_scalars();
}

DeviceDavidson::~DeviceDavidson() {
  rt_.release_quiet(V_);
  rt_.release_quiet(HV_);
  rt_.release_quiet(W_);
  rt_.release_quiet(sm_);
}

void DeviceDavidson::multi_dot(const double* A, int ncol, const double* x, double* out) {
  C2G_CUDA(launch_multi_dot(A, n_, ncol, x, n_, rt_.partial(), out, rt_.stream()));
  count_launches(2);
}

double DeviceDavidson::norm2(const double* x, double* theta) {
  multi_dot(x, 1, x, sm_ + kSumSq);
  C2G_CUDA(cudaMemcpyAsync(host_, sm_ + kSumSq, sizeof(double), cudaMemcpyDeviceToHost, rt_.stream()));
  if (theta) C2G_CUDA(cudaMemcpyAsync(host_ + 1, sm_ + kEvals, sizeof(double), cudaMemcpyDeviceToHost, rt_.stream()));
  rt_.sync();
  if (theta) *theta = host_[1];
  return host_[0];
}

// CheMPS2/Davidson.cpp:216-236 (AddNewVec): t <- t - V V^T t (twice), t <- t / |t|, V[nv] <- t.
void DeviceDavidson::add_new_vec(double* t, int nv) {
  cudaStream_t s = rt_.stream();
  for (int pass = 0; pass < 2 && nv > 0; pass++) {
    multi_dot(V_, nv, t, sm_ + kDots);
    C2G_CUDA(launch_neg(sm_ + kDots, nv, s));
    C2G_CUDA(launch_combine(t, 1.0, V_, n_, sm_ + kDots, nv, n_, s));
    count_launches(2);
  }
  multi_dot(t, 1, t, sm_ + kSumSq);
  C2G_CUDA(launch_inv_sqrt_scale(t, sm_ + kSumSq, n_, s));
  count_launches(1);
  C2G_CUDA(cudaMemcpyAsync(V(nv), t, sizeof(double) * n_, cudaMemcpyDeviceToDevice, s));
}

bool DeviceDavidson::run(const double* diag, const MatVec& matvec, Precision prec, double tol, bool stop_on_stall,
                         DavidsonStats& st) {
  cudaStream_t s = rt_.stream();
  double* t = W(0);
  double* u = W(1);
  double* w = W(2);
  auto mv = [&](const double* x, double* y) {
    matvec(x, y, prec);
    st.n_matvec++;
    if (prec != Precision::kFP64) st.n_matvec_fp32++;
  };
  int nv = 0;
  eig_n_ = -1;
  add_new_vec(t, nv);
  mv(V(nv), HV(nv));
  double best = 1e300;
  int since_best = 0;
  const int matvec0 = st.n_matvec;
  for (;;) {
    // DiagonalizeSmallMatrixAndCalcResidual (CheMPS2/Davidson.cpp:238-289)
    multi_dot(HV_, nv + 1, V(nv), sm_ + kDots);
    C2G_CUDA(launch_mxm_row(sm_ + kMxM, kLd, nv, sm_ + kDots, nv + 1, s));
    nv++;
    // warm start when the previous solve was of this matrix's leading block
    C2G_CUDA(launch_small_eig(sm_ + kMxM, nv, kLd, sm_ + kEvals, sm_ + kEvecs, s, eig_n_ == nv - 1));
    eig_n_ = nv;
    C2G_CUDA(launch_combine(t, 0.0, HV_, n_, sm_ + kEvecs, nv, n_, s));
    C2G_CUDA(launch_combine(u, 0.0, V_, n_, sm_ + kEvecs, nv, n_, s));
    C2G_CUDA(launch_residual(t, u, sm_ + kEvals, n_, s));
    count_launches(5);
    double theta = 0.0;
    const double rnorm = std::sqrt(norm2(t, stop_on_stall ? &theta : nullptr));
    st.n_iter++;
    st.rnorm = rnorm;
    if (!(rnorm > tol)) break;
    if (stop_on_stall) {  // reduced-precision phase: stop when the residual no longer improves
      if (rnorm < 0.7 * best) {
        best = rnorm;
        since_best = 0;
      } else if (++since_best >= 6) {
        st.lo_stalled = true;
        if (rnorm > kStallCeiling * std::fabs(theta)) return false;
        break;
      }
      if (st.n_matvec - matvec0 >= kLoMaxMatvec) return false;
    }
    // CalculateNewVec (CheMPS2/Davidson.cpp:291-317)
    C2G_CUDA(launch_precond_w(w, u, diag, sm_ + kEvals, cutoff_, n_, s));
    multi_dot(W(0), 2, w, sm_ + kDots2);  // w.t, w.u
    C2G_CUDA(launch_precond_t(t, u, diag, sm_ + kEvals, sm_ + kDots2, cutoff_, n_, s));
    count_launches(2);
    if (nv == max_vec_) {
      // Deflation (CheMPS2/Davidson.cpp:319-384): keep the lowest keep_ Ritz vectors
      C2G_CUDA(cudaMemcpyAsync(W(3), u, sizeof(double) * n_, cudaMemcpyDeviceToDevice, s));
      for (int c = 1; c < keep_; c++) {
        C2G_CUDA(launch_combine(W(3 + c), 0.0, V_, n_, sm_ + kEvecs + kLd * c, nv, n_, s));
        count_launches(1);
      }
      for (int c = 0; c < keep_; c++) multi_dot(W(3), keep_, W(3 + c), sm_ + kOverlap + keep_ * c);
      C2G_CUDA(launch_lowdin(sm_ + kOverlap, keep_, sm_ + kLowdin, s));
      count_launches(1);
      for (int c = 0; c < keep_; c++) {
        C2G_CUDA(launch_combine(V(c), 0.0, W(3), n_, sm_ + kLowdin + keep_ * c, keep_, n_, s));
        count_launches(1);
      }
      for (int c = 0; c < keep_; c++) mv(V(c), HV(c));
      // MxMafterDeflation (CheMPS2/Davidson.cpp:510-536)
      eig_n_ = -1;  // the projected matrix is rebuilt
      for (int j = 0; j < keep_; j++) {
        multi_dot(V_, j + 1, HV(j), sm_ + kDots);
        C2G_CUDA(launch_mxm_row(sm_ + kMxM, kLd, j, sm_ + kDots, j + 1, s));
        count_launches(1);
      }
      nv = keep_;
    }
    add_new_vec(t, nv);
    mv(V(nv), HV(nv));
  }
  return true;
}

bool DeviceDavidson::refine_cycle(const double* diag, const MatVec& matvec, double tol, int max_expand, double rel,
                                  DavidsonStats& st, double* r_exact) {
  cudaStream_t s = rt_.stream();
  double* t = W(0);
  double* u = W(1);
  double* w = W(2);
  int nv = 0;
  eig_n_ = -1;
  add_new_vec(t, nv);
  matvec(V(0), HV(0), Precision::kFP64);
  st.n_matvec++;
  double r0 = 0.0;
  for (int it = 0;; it++) {
    multi_dot(HV_, nv + 1, V(nv), sm_ + kDots);
    C2G_CUDA(launch_mxm_row(sm_ + kMxM, kLd, nv, sm_ + kDots, nv + 1, s));
    nv++;
    C2G_CUDA(launch_small_eig(sm_ + kMxM, nv, kLd, sm_ + kEvals, sm_ + kEvecs, s, eig_n_ == nv - 1));
    eig_n_ = nv;
    C2G_CUDA(launch_combine(t, 0.0, HV_, n_, sm_ + kEvecs, nv, n_, s));
    C2G_CUDA(launch_combine(u, 0.0, V_, n_, sm_ + kEvecs, nv, n_, s));
    C2G_CUDA(launch_residual(t, u, sm_ + kEvals, n_, s));
    count_launches(5);
    const double rnorm = std::sqrt(norm2(t));
    st.n_iter++;
    st.rnorm = rnorm;
    if (it == 0) {
      // V = {u} with its FP64 product: the exact residual
      r0 = rnorm;
      *r_exact = rnorm;
      if (!(rnorm > tol)) return true;
    } else if (rnorm <= rel * r0 || it >= max_expand || nv >= max_vec_) {
      return false;
    }
    C2G_CUDA(launch_precond_w(w, u, diag, sm_ + kEvals, cutoff_, n_, s));
    multi_dot(W(0), 2, w, sm_ + kDots2);
    C2G_CUDA(launch_precond_t(t, u, diag, sm_ + kEvals, sm_ + kDots2, cutoff_, n_, s));
    count_launches(2);
    add_new_vec(t, nv);
    matvec(V(nv), HV(nv), lo_);
    st.n_matvec++;
    st.n_matvec_fp32++;
  }
}

DavidsonStats DeviceDavidson::solve(double* guess, const double* diag, const MatVec& matvec, bool mixed,
                                    double lo_tol, Precision lo) {
  lo_ = lo;
  cudaStream_t s = rt_.stream();
  DavidsonStats st;
  double* t = W(0);
  double* u = W(1);
  C2G_CUDA(cudaMemcpyAsync(t, guess, sizeof(double) * n_, cudaMemcpyDeviceToDevice, s));
  // SafetyCheckGuess (CheMPS2/Davidson.cpp:204-214)
  if (norm2(t) == 0.0) {
    std::vector<double> r(n_);
    HostRand libc;
    HostRand& g = rand_ ? *rand_ : libc;
    for (int64_t i = 0; i < n_; i++) r[i] = g.unit();
    C2G_CUDA(cudaMemcpyAsync(t, r.data(), sizeof(double) * n_, cudaMemcpyHostToDevice, s));
    // the start vector also stays in guess (overwritten by the result at the end), for a
    // restart of the mixed solve
    C2G_CUDA(cudaMemcpyAsync(guess, t, sizeof(double) * n_, cudaMemcpyDeviceToDevice, s));
    rt_.sync();
  }
  bool done = false;
  if (mixed) {
    const bool lo_done = run(diag, matvec, lo_, std::max(lo_tol, rtol_), true, st);
    st.n_lo = st.n_matvec;
    st.lo_rnorm = st.rnorm;
    if (!lo_done) {  // a hard step: the FP64 solver from the guess
      st.fp64_fallback = true;
      C2G_CUDA(cudaMemcpyAsync(t, guess, sizeof(double) * n_, cudaMemcpyDeviceToDevice, s));
      run(diag, matvec, Precision::kFP64, rtol_, false, st);
      C2G_CUDA(cudaMemcpyAsync(guess, u, sizeof(double) * n_, cudaMemcpyDeviceToDevice, s));
      C2G_CUDA(cudaMemcpyAsync(host_, sm_ + kEvals, sizeof(double), cudaMemcpyDeviceToHost, s));
      rt_.sync();
      st.energy = host_[0];
      return st;
    }
    // refinement cycles from the FP32 Ritz vector; a cycle that cannot improve (for
    // example an FP32 floor above the target) leaves it to the FP64 Davidson below
    double last = 1e300;
    for (int cycle = 0; cycle < kRefineCycles && !done; cycle++) {
      C2G_CUDA(cudaMemcpyAsync(t, u, sizeof(double) * n_, cudaMemcpyDeviceToDevice, s));
      double r = 0.0;
      st.n_cycles++;
      done = refine_cycle(diag, matvec, rtol_, kRefineExpand, kRefineRel, st, &r);
      if (cycle == 0) st.r_exact0 = r;
      if (!done && r > 0.5 * last) break;  // the exact residual no longer drops
      last = r;
    }
    if (!done) C2G_CUDA(cudaMemcpyAsync(t, u, sizeof(double) * n_, cudaMemcpyDeviceToDevice, s));
  }
  if (!done) run(diag, matvec, Precision::kFP64, rtol_, false, st);
  C2G_CUDA(cudaMemcpyAsync(guess, u, sizeof(double) * n_, cudaMemcpyDeviceToDevice, s));
  C2G_CUDA(cudaMemcpyAsync(host_, sm_ + kEvals, sizeof(double), cudaMemcpyDeviceToHost, s));
  rt_.sync();
  st.energy = host_[0];
  return st;
}

}  // namespace c2g
