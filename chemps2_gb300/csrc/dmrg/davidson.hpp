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
#pragma once

#include <functional>

#include "runtime.hpp"

namespace c2g {

struct DavidsonStats {
  double energy = 0.0;
  int n_matvec = 0;
  int n_iter = 0;
  double rnorm = 0.0;
};

class DeviceDavidson {
 public:
  using MatVec = std::function<void(const double* x, double* y)>;

  DeviceDavidson(Runtime& rt, int64_t n, int max_vec, int keep, double rtol, double cutoff);
  ~DeviceDavidson();
  DeviceDavidson(const DeviceDavidson&) = delete;
  DeviceDavidson& operator=(const DeviceDavidson&) = delete;

  // guess: device vector of length n (in: start vector; out: converged eigenvector).
  // diag: device vector, the diagonal of the operator.
  DavidsonStats solve(double* guess, const double* diag, const MatVec& matvec);

 private:
  double* V(int i) { return V_ + n_ * i; }
  double* HV(int i) { return HV_ + n_ * i; }
  double* W(int i) { return W_ + n_ * i; }
  void add_new_vec(double* t, int nv);  // orthonormalise t against V[0..nv) into V[nv]
  double norm2(const double* x);         // synchronising host read of x.x
  void multi_dot(const double* A, int ncol, const double* x, double* out);

  Runtime& rt_;
  int64_t n_;
  int max_vec_, keep_;
  double rtol_, cutoff_;
  double* V_ = nullptr;
  double* HV_ = nullptr;
  double* W_ = nullptr;   // columns: 0 t, 1 u, 2 w, 3.. deflation vectors
  double* sm_ = nullptr;  // small device scalars (layout in davidson.cpp)
  double* host_ = nullptr;  // pinned host scalars
};

}  // namespace c2g
