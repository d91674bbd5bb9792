// Drop-in replacement for CheMPS2::SyBookkeeper (CheMPS2/include/chemps2/SyBookkeeper.h,
// CheMPS2/SyBookkeeper.cpp:29-323).
//
// For every boundary b = 0..L it knows the allowed particle numbers N, spins 2S and irreps
// I, the FCI virtual dimension of each (b, N, 2S, I) sector (capped at 262144,
// CheMPS2/include/chemps2/Options.h:76) and the current dimension. The FCI dimensions are
// filled by the same left-to-right and right-to-left recurrences, and the initial current
// dimensions are scaled with ceil(D / total * dim) exactly as ScaleCURdim, so every
// sector dimension is bit-identical to the reference.
//
// Sectors of a boundary are numbered densely (sector_id): N outermost, then 2S, then the
// irrep, which is the loop order every reference layout uses. The id gives O(1) lookups
// for the block tables of the MPS, two-site and operator tensors.
#pragma once

#include <vector>

#include "Problem.h"

namespace CheMPS2 {

class SyBookkeeper {
 public:
  SyBookkeeper(const Problem* Prob, const int D);
  SyBookkeeper(const SyBookkeeper& other) = default;

  const Problem* gProb() const { return Prob; }
  int gL() const { return L; }
  int gIrrep(const int orbital) const { return orb_irrep[orbital]; }
  int gTwoS() const { return TwoS; }
  int gN() const { return N; }
  int gIrrep() const { return Irrep; }
  int getNumberOfIrreps() const { return nirrep; }

  int gNmin(const int b) const { return Nmin[b]; }
  int gNmax(const int b) const { return Nmax[b]; }
  int gTwoSmin(const int b, const int n) const { return TwoSmin[b][n - Nmin[b]]; }
  int gTwoSmax(const int b, const int n) const { return TwoSmax[b][n - Nmin[b]]; }

  // Dense sector index at boundary b, or -1 when (N, 2S, I) is outside the ranges.
  int sector_id(const int b, const int n, const int two_s, const int irrep) const {
    if (b < 0 || b > L) return -1;
    if (n < Nmin[b] || n > Nmax[b]) return -1;
    const int smin = TwoSmin[b][n - Nmin[b]];
    const int smax = TwoSmax[b][n - Nmin[b]];
    if ((two_s % 2) != (smin % 2)) return -1;
    if (two_s < smin || two_s > smax) return -1;
    if (irrep < 0 || irrep >= nirrep) return -1;
    return sec_base[b][n - Nmin[b]] + ((two_s - smin) / 2) * nirrep + irrep;
  }
  int num_sectors(const int b) const { return nsec[b]; }
  void sector_labels(const int b, const int id, int* n, int* two_s, int* irrep) const;

  int gFCIdim(const int b, const int n, const int two_s, const int irrep) const {
    const int id = sector_id(b, n, two_s, irrep);
    return id < 0 ? 0 : fci[b][id];
  }
  int gCurrentDim(const int b, const int n, const int two_s, const int irrep) const {
    const int id = sector_id(b, n, two_s, irrep);
    return id < 0 ? 0 : cur[b][id];
  }
  int cur_dim_by_id(const int b, const int id) const { return id < 0 ? 0 : cur[b][id]; }
  int fci_dim_by_id(const int b, const int id) const { return id < 0 ? 0 : fci[b][id]; }
  void SetDim(const int b, const int n, const int two_s, const int irrep, const int value);

  int gMaxDimAtBound(const int b) const;
  int gTotDimAtBound(const int b) const;
  bool IsPossible() const;

 private:
  const Problem* Prob;
  int L, N, TwoS, Irrep, nirrep;
  std::vector<int> orb_irrep;
  std::vector<int> Nmin, Nmax, nsec;
  std::vector<std::vector<int>> TwoSmin, TwoSmax, sec_base;
  std::vector<std::vector<int>> fci, cur;

  void fill_fci_dim_right(std::vector<std::vector<int>>& st, int start, int stop);
  void fill_fci_dim_left(std::vector<std::vector<int>>& st, int start, int stop);
  int dim_private(const std::vector<std::vector<int>>& st, int b, int n, int two_s, int irrep) const {
    const int id = sector_id(b, n, two_s, irrep);
    return id < 0 ? 0 : st[b][id];
  }
  void scale_cur_dim(int virtual_dim, int start, int stop);
};

}  // namespace CheMPS2
