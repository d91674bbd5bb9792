// Compiler of the effective-Hamiltonian matvec and of its diagonal.
//
// compile_heff() records, for every block kappa of the two-site object, the
// contractions that CheMPS2::Heff::makeHeff issues (CheMPS2/Heff.cpp:43-248): diagram
// groups 1 to 5 of CheMPS2/HeffDiagrams1-5.cpp. The input vector is bound to slot X and
// the output to slot Y, in the reference's "symmetric" normalisation (the Davidson
// vectors are the two-site blocks scaled by sqrt(2S_R + 1), CheMPS2/Sobject.cpp:624-650).
//
// compile_heff_diag() records the diagonal used by the Davidson preconditioner
// (CheMPS2/Heff.cpp:250-315, CheMPS2/HeffDiagonal.cpp) as rank-1 contractions of
// operator diagonals against a vector of ones (slot kSlotOnes).
#pragma once

#include "chemps2/Problem.h"
#include "chemps2/SyBookkeeper.h"
#include "layout.hpp"
#include "operators.hpp"
#include "tasks.hpp"

namespace c2g {

struct HeffContext {
  const CheMPS2::SyBookkeeper* bk = nullptr;
  const CheMPS2::Problem* prob = nullptr;
  const TwoSiteLayout* S = nullptr;
  const BoundaryOps* left = nullptr;   // operators at boundary index (built moving right)
  const BoundaryOps* right = nullptr;  // operators at boundary index + 2 (built moving left)
};

// Both compilers visit the blocks in the reference's size-sorted order; with nshards > 1
// only every nshards-th block of that order (starting at shard) is emitted.
void compile_heff(TaskBuilder& tb, const HeffContext& ctx, int shard = 0, int nshards = 1);
void compile_heff_diag(TaskBuilder& tb, const HeffContext& ctx, int shard = 0, int nshards = 1);

}  // namespace c2g
