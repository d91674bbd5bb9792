// Task compilers of the excited-state machinery (CheMPS2/DMRG.cpp:464-505,
// CheMPS2/DMRGtechnics.cpp:509-620, CheMPS2/TensorO.cpp, CheMPS2/HeffDiagrams1.cpp:65-86):
// overlap tensors between the current MPS and a stored (lower) state, carried from
// boundary to boundary with the sweeps, and the projection vector
//   V = sqrt(E_shift) / (2S + 1) * O_left S_stored O_right^T
// of the stored state onto the current two-site basis, which adds E_shift-weighted
// projectors (x . V) V to the effective Hamiltonian.
#pragma once

#include <memory>
#include <vector>

#include "chemps2/SyBookkeeper.h"
#include "layout.hpp"
#include "operators.hpp"
#include "tasks.hpp"

namespace c2g {

// Blocks (N, 2S, I) of one boundary that both bookkeepers populate, each
// dim_up (current) x dim_down (stored), column-major.
struct OverlapLayout {
  int boundary = 0;
  int nkappa = 0;
  std::vector<int> N, S, I, rows, cols;
  std::vector<int64_t> k2i;
  void build(const CheMPS2::SyBookkeeper& up, const CheMPS2::SyBookkeeper& down, int boundary);
  int kappa(int n, int s, int i) const;
  int64_t size() const { return k2i[nkappa]; }

 private:
  const CheMPS2::SyBookkeeper* up_ = nullptr;
  std::vector<int> by_sector_;  // [sector id of up] -> kappa or -1
};

struct OverlapT {
  const OverlapLayout* lay = nullptr;
  Ref base = 0;
  Blk blk(int n, int s, int i) const {
    const int k = lay->kappa(n, s, i);
    if (k < 0) return Blk();
    return Blk::make(base + lay->k2i[k], lay->rows[k], lay->cols[k]);
  }
};

// The overlap tensor `out` of boundary index + 1 from `prev` (boundary index when moving
// right, index + 2 when moving left; null at the edge, where it is the 1 x 1 identity)
// through the site tensors of site index (moving right) or index + 1 (moving left) of the
// current (up) and the stored (down) MPS (TensorO::create / update_ownmem).
void compile_overlap_update(TaskBuilder& tb, const CheMPS2::SyBookkeeper& up, const CheMPS2::SyBookkeeper& down,
                            bool moving_right, int index, const OverlapT* prev, const OverlapT& out, const MpsT& Tup,
                            const MpsT& Tdown);

// V (slot / offsets of the current two-site layout S) from the stored state's joined
// two-site vector (layout Sk at base sup), the overlaps left (boundary index, null at
// index 0) and right (boundary index + 2, null at the right edge) and the prefactor
// sqrt(E_shift) / (2S + 1) (CheMPS2/DMRGtechnics.cpp:540-620).
void compile_veff(TaskBuilder& tb, const TwoSiteLayout& S, const TwoSiteLayout& Sk, Ref sup, const OverlapT* left,
                  const OverlapT* right, double prefactor, Ref out);

}  // namespace c2g
