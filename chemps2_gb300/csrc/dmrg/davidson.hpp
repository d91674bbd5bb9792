// Davidson eigensolver for the lowest eigenpair of the effective Hamiltonian, on the GPU.
//
// Same algorithm and state sequence as CheMPS2::Davidson with problem type 'E'
// (CheMPS2/Davidson.cpp:31-536): at most MAX_NUM_VEC basis vectors, deflation to
// NUM_VEC_KEEP Ritz vectors with Loewdin re-orthonormalisation, the diagonal
// preconditioner with cutoff, and convergence when the residual 2-norm <= rtol. All
// vectors, the Rayleigh-Ritz matrix and its eigendecomposition stay on the device in
// FP64; only the residual norm travels to the host, once per iteration, to drive the
// state machine. Orthogonalisation is classical Gram-Schmidt applied twice (the reference
// applies one modified Gram-Schmidt pass; both are exact in exact arithmetic).
//
// Mixed precision: the matvec is requested in FP32 until the residual reaches a looser
// tolerance (or stops improving). Refinement cycles follow: each restarts the subspace from
// the current Ritz vector u with its FP64 product H u, so the first Rayleigh-Ritz step of a
// cycle gives the exact residual of u (the convergence test), and expands it with FP32
// products; the cross terms with u use the exact H u, so only the small correction
// coefficients carry FP32 error and every cycle reduces the residual by orders of
// magnitude at the cost of one FP64 matvec. The returned eigenpair is an FP64 one.
#pragma once

#include <functional>

#include "rng.hpp"
#include "runtime.hpp"

namespace c2g {

struct DavidsonStats {
  double energy = 0.0;
  int n_matvec = 0;       // all matvecs
  int n_matvec_fp32 = 0;  // of which in FP32
  int n_iter = 0;
  double rnorm = 0.0;
  // mixed solves: matvecs of the reduced-precision phase, its last residual and whether it
  // ended on a stall; refinement cycles run
  int n_lo = 0;
  double lo_rnorm = 0.0;
  bool lo_stalled = false;
  bool fp64_fallback = false;  // a hard step: solved by the FP64 solver from the guess
  int n_cycles = 0;
  double r_exact0 = 0.0;  // exact (FP64) residual at the start of the first cycle
};

class DeviceDavidson {
 public:
  using MatVec = std::function<void(const double* x, double* y, Precision prec)>;

  DeviceDavidson(Runtime& rt, int64_t n, int max_vec, int keep, double rtol, double cutoff);
  ~DeviceDavidson();
  DeviceDavidson(const DeviceDavidson&) = delete;
  DeviceDavidson& operator=(const DeviceDavidson&) = delete;

  // guess: device vector of length n (in: start vector; out: converged eigenvector).
  // diag: device vector, the diagonal of the operator. mixed: run the FP32 phase first,
  // down to residual lo_tol (never below rtol).
  // `lo`: the arithmetic of the reduced-precision matvecs of the mixed mode (kFP32, or kTC
  // for the tensor-core products of the large groups).
  DavidsonStats solve(double* guess, const double* diag, const MatVec& matvec, bool mixed = false,
                      double lo_tol = 1e-5, Precision lo = Precision::kFP32);
  // source of the random start that replaces a zero guess (the C library's rand() unless set)
  void set_rand(HostRand* r) { rand_ = r; }

 private:
  Precision lo_ = Precision::kFP32;
  // order of the projected matrix whose eigenvectors are in the evecs scratch (-1: none
  // valid for the matrix now being built)
  int eig_n_ = -1;
  double* V(int i) { return V_ + n_ * i; }
  double* HV(int i) { return HV_ + n_ * i; }
  double* W(int i) { return W_ + n_ * i; }
  void add_new_vec(double* t, int nv);  // orthonormalise t against V[0..nv) into V[nv]
  // synchronising host read of x.x (and, with theta, of the lowest Ritz value)
  double norm2(const double* x, double* theta = nullptr);
  void multi_dot(const double* A, int ncol, const double* x, double* out);
  // One Davidson run from the vector in W(0); the Ritz vector ends in W(1). False when a
  // reduced-precision run (stop_on_stall) met a hard step (a stall far above its
  // arithmetic's floor, or its product limit).
  bool run(const double* diag, const MatVec& matvec, Precision prec, double tol, bool stop_on_stall,
           DavidsonStats& st);
  // One refinement cycle from the vector in W(0) (first product FP64, then FP32, at most
  // max_expand expansions, until the residual estimate falls below rel * the exact first
  // residual); true when that exact first residual is <= tol. The Ritz vector ends in W(1).
  bool refine_cycle(const double* diag, const MatVec& matvec, double tol, int max_expand, double rel,
                    DavidsonStats& st, double* r_exact);

  Runtime& rt_;
  int64_t n_;
  int max_vec_, keep_;
  double rtol_, cutoff_;
  double* V_ = nullptr;
  double* HV_ = nullptr;
  double* W_ = nullptr;   // columns: 0 t, 1 u, 2 w, 3.. deflation vectors
  double* sm_ = nullptr;  // small device scalars (layout in davidson.cpp)
  double* host_ = nullptr;  // pinned host scalars of the runtime
  HostRand* rand_ = nullptr;
};

}  // namespace c2g
