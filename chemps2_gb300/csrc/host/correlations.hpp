// Task compiler of the correlation pass of DMRG::calc2DMandCorrelations
// (CheMPS2/DMRGtechnics.cpp:157-176): the tensors G, Y, Z (TensorGYZ.cpp) and K, M
// (TensorKM.cpp) of every orbital p left of the current site, carried from boundary to
// boundary with the generic operator update (CheMPS2/DMRGoperators3RDM.cpp:415-466), and
// the diagrams of Correlations::FillSite (CheMPS2/Correlations.cpp:353-560) that turn them
// into the two-orbital density matrices of (p, site).
#pragma once

#include <memory>
#include <vector>

#include "chemps2/Problem.h"
#include "chemps2/SyBookkeeper.h"
#include "operators.hpp"
#include "tasks.hpp"

namespace c2g {

// G, Y, Z (2j = 0, n = 0, trivial irrep) and K, M (2j = 1, n = 1, irrep of p) of the
// orbitals p = 0 .. boundary - 1 at one boundary, all moving right, packed into one slot.
struct CorrTensors {
  int boundary = 0;
  int slot = -1;
  int64_t size = 0;  // doubles
  std::unique_ptr<OpLayoutCache> layouts;
  std::vector<OpT> G, Y, Z, K, M;  // [p]
};

void allocate_corr(CorrTensors& c, const CheMPS2::SyBookkeeper& bk, int boundary, int slot);

// Tensors of boundary `site` (next) from those of boundary site - 1 (prev, null when
// site == 1) through T = MPS[site - 1]: the generic update for p < site - 1 and the
// construction of p = site - 1 (TensorGYZ::construct, TensorKM::construct).
void compile_corr_update(TaskBuilder& tb, const CheMPS2::SyBookkeeper& bk, const CheMPS2::Problem& prob, int L,
                         int site, const CorrTensors* prev, const CorrTensors& next, const MpsT& T);

// Values per orbital p < site, in this order (the diagrams of Correlations::FillSite):
// diagram3(G), diagram1(Y), diagram2(Z), diagram1(G), diagram3(Y), diagram4(K),
// diagram2(G), diagram3(Z), diagram5(M), diagram1(Z), diagram5(K), diagram4(M),
// diagram2(Y); diagrams 4 and 5 only when p and site share their irrep (zero otherwise).
constexpr int kCorrValues = 13;
// Two stages like the 2-RDM programs: products into the work slot (offsets from 0), then
// Frobenius products into slot Y (value p * kCorrValues + n). Returns the work size.
int64_t compile_corr_fill(TaskBuilder& tb, const CheMPS2::SyBookkeeper& bk, int site, const MpsT& T,
                          const CorrTensors& c);

}  // namespace c2g
