// Extension without a counterpart in the reference: many independent DMRG problems solved
// on one GPU. The reference solves one problem per DMRG object, one object at a time; its
// callers loop over problems. SolveBatch is that loop run concurrently: each problem gets
// its own DMRG object, whose operators and MPS stay in GPU memory and whose kernels run on
// its own CUDA stream.
#pragma once

#include <string>
#include <vector>

#include "ConvergenceScheme.h"
#include "DMRG.h"
#include "Problem.h"

namespace CheMPS2 {

struct BatchResult {
  double energy = 0.0;         // DMRG::Solve() of this problem
  long long n_matvec = 0;      // its Heff applications
  double seconds = 0.0;        // wall clock of its construction and Solve()
  double matvec_seconds = 0.0; // device time of its Heff applications
  // 0 solved; 1 invalid input (what the reference asserts); 2 a CUDA call failed; 3 no
  // CUDA device; 4 another failure. `error` says why.
  int status = 0;
  std::string error;
  DMRGStats stats;             // the DMRG's statistics after Solve()
};

// Solves problems[i] with schemes[i] for every i. Problem i's random start is the one that
// srand(seeds[i]) gives a DMRG constructed right after it, drawn from a generator of its
// own, so results do not depend on the order or concurrency of the solves. At most
// `workers` problems are in flight (workers <= 1: one after another, in input order); each
// worker is a host thread that takes the largest remaining problem, so the device overlaps
// the streams of several problems and one problem's host work (task compiler, truncation)
// with another's kernels. Every problem is attempted; failures are reported in its result.
// The Problems are modified as by DMRG construction (matrix elements are built).
std::vector<BatchResult> SolveBatch(const std::vector<Problem*>& problems,
                                    const std::vector<ConvergenceScheme*>& schemes,
                                    const std::vector<unsigned>& seeds, int workers);

}  // namespace CheMPS2
