// Task compiler of the two-particle density matrix (CheMPS2/TwoDM.cpp:445-1592,
// TwoDM::FillSite and its diagrams D1-D24).
//
// With the MPS in mixed-canonical form around `site`, every diagram value is a sum over
// symmetry blocks of factor * < T_up, P > with P = op(L_left) T_down op(O_right), a product
// of the site tensor with renormalized operators of the left boundary (site - 1, moving
// right) and of the right boundary (site, moving left). A compiled program has two stages:
// the first writes every product P (scaled by its factor) into the work slot, the second
// accumulates the Frobenius products < T_up, P > into scalar diagram values in slot Y.
// twodm_assemble then sets the density-matrix elements from the values exactly as
// FillSite does.
#pragma once

#include <vector>

#include "chemps2/SyBookkeeper.h"
#include "chemps2/TwoDM.h"
#include "operators.hpp"
#include "tasks.hpp"

namespace c2g {

struct TwoDMContext {
  const CheMPS2::SyBookkeeper* bk = nullptr;
  int L = 0;
  int site = 0;
  MpsT T;                            // the site tensor (orthogonality centre)
  const BoundaryOps* left = nullptr;   // boundary site - 1, moving right (null at site 0)
  const BoundaryOps* right = nullptr;  // boundary site, moving left (null at site L - 1)
};

// The groups of diagrams FillSite evaluates per orbital combination, with their number of
// scalar values: D1 (1), D2 (1), D3-D6 (4), D7 (1), D8-D12 (5: d8 d9 d10 d11 d12) and
// D13-D24 (12: d13 ... d24).
enum TwoDMKind : int { kTdmD1, kTdmD2, kTdmD3to6, kTdmD7, kTdmD8to12, kTdmD13to24 };
int twodm_num_values(int kind);

struct TwoDMInstance {
  int kind;
  int g, j, k;   // orbitals (unused ones -1)
  int value0;    // first scalar of the instance in slot Y
  int64_t work;  // doubles of products it writes to the work slot
};

// The diagram instances of FillSite(site), in FillSite's order, with their value offsets
// and work sizes.
std::vector<TwoDMInstance> twodm_instances(const TwoDMContext& ctx);

// Records instances [first, last): stage 1 the products (work offsets from 0, in instance
// order), stage 2 the Frobenius products into slot Y at the instances' value0 minus the
// value0 of `first`.
void compile_twodm(TaskBuilder& tb, const TwoDMContext& ctx, const std::vector<TwoDMInstance>& inst, size_t first,
                   size_t last);

// Sets the density-matrix elements of FillSite(site) from the diagram values (values[v]
// for instance value v, indexed as value0 + offset).
void twodm_assemble(CheMPS2::TwoDM& dm, int site, const std::vector<TwoDMInstance>& inst,
                    const std::vector<double>& values);

}  // namespace c2g
