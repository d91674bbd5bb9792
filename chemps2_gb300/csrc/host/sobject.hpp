// Two-site object tasks: Join (CheMPS2/Sobject.cpp:212-258) and the sector planning and
// block copies of Split (CheMPS2/Sobject.cpp:260-621).
//
// The two-site vector is kept in the reference's "symmetric" convention throughout (block
// kappa scaled by sqrt(2S_R + 1), CheMPS2/Sobject.cpp:624-650): Join writes it directly and
// Split reads it, folding prog2symm / symm2prog into their prefactors.
#pragma once

#include <vector>

#include "chemps2/SyBookkeeper.h"
#include "layout.hpp"
#include "operators.hpp"
#include "tasks.hpp"

namespace c2g {

// Y (slot Y, TwoSiteLayout S) = Join(left MPS tensor of site S.index, right of site + 1)
void compile_join(TaskBuilder& tb, const CheMPS2::SyBookkeeper& bk, const TwoSiteLayout& S, const MpsT& left,
                  const MpsT& right);

// One center symmetry sector (N_M, 2S_M, I_M) at boundary index + 1, with the left and
// right sectors that couple to it through the two local sites, in the reference's order.
struct SplitPart {
  int n = 0, two_s = 0, irrep = 0, dim = 0, off = 0;
};
struct SplitCenter {
  int NM = 0, TwoSM = 0, IM = 0;
  int dimL = 0, dimR = 0, cd = 0;  // DimLtotal, DimRtotal, min of both
  std::vector<SplitPart> lparts, rparts;
  int64_t offA = 0;  // assembled DimL x DimR matrix in the work slot
  int64_t offG = 0;  // Gram matrix g x g (g = DimL moving right, DimR moving left)
  int64_t offU = 0;  // its eigenvectors, largest eigenvalue first
  int64_t offE = 0;  // eigenvalues (ascending, as the eigensolver writes them)
  int g = 0;
};
struct SplitPlan {
  int index = 0;
  bool moving_right = true;
  std::vector<SplitCenter> centers;
  int64_t work_size = 0;  // doubles
};

SplitPlan plan_split(const CheMPS2::SyBookkeeper& bk, int index, bool moving_right);

// Stage 1: assemble every center-sector matrix from the two-site blocks (slot X); stage 2:
// its Gram matrix. Outputs go to slot kSlotWork, which must be zero-filled before.
void compile_split_assemble(TaskBuilder& tb, const CheMPS2::SyBookkeeper& bk, const TwoSiteLayout& S,
                            const SplitPlan& plan);

// Copies the kept singular vectors into the new MPS tensors (already zero-filled), with the
// singular values and spin factors of CheMPS2/Sobject.cpp:521-590. dims_m[c] is the new
// dimension of center sector c.
void compile_split_copy(TaskBuilder& tb, const SplitPlan& plan, const std::vector<int>& dims_m, const MpsT& left,
                        const MpsT& right);

}  // namespace c2g
