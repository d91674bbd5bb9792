// Block layouts of the three tensor kinds on the DMRG hot path. Every layout enumerates
// its symmetry blocks in exactly the reference's loop order, so block numbers (kappa) and
// storage offsets (kappa2index) are bit-identical to the reference; the lookup tables
// replace the reference's linear scans (gKappa) with O(1) probes.
//
//   MpsLayout     CheMPS2/TensorT.cpp:38-110    blocks (NL,2SL,IL) -> (NR,2SR,IR)
//   TwoSiteLayout CheMPS2/Sobject.cpp:36-145    blocks (NL,2SL,IL,N1,N2,2J,NR,2SR,IR),
//                                               plus the size-sorted visiting order
//   OpLayout      CheMPS2/TensorOperator.cpp:29-105  blocks keyed by the upper sector and
//                                               the lower spin, dim_up x dim_down
//
// All blocks are column-major, dim_left (or dim_up) rows.
#pragma once

#include <cstdint>
#include <map>
#include <memory>
#include <tuple>
#include <vector>

#include "chemps2/SyBookkeeper.h"

namespace c2g {

using CheMPS2::SyBookkeeper;

struct MpsLayout {
  int index = 0;  // site; left boundary = index, right boundary = index + 1
  int nkappa = 0;
  std::vector<int> NL, TwoSL, IL, NR, TwoSR, IR, rows, cols;
  std::vector<int64_t> k2i;
  std::vector<int> lookup;  // [left sector id * 4 + variant] -> kappa or -1

  void build(const SyBookkeeper& bk, int site);
  int kappa(int nl, int sl, int il, int nr, int sr, int ir) const;
  int64_t size() const { return k2i[nkappa]; }

 private:
  const SyBookkeeper* bk_ = nullptr;
};

struct TwoSiteLayout {
  int index = 0;  // sites index, index + 1; boundaries index and index + 2
  int nkappa = 0;
  std::vector<int> NL, TwoSL, IL, N1, N2, TwoJ, NR, TwoSR, IR, rows, cols;
  std::vector<int64_t> k2i;
  std::vector<int> reorder;  // visiting order: block size non-increasing (stable)
  std::vector<int> lookup;   // [((sidL*9 + N1*3 + N2)*3 + 2J)*5 + (2SR-2SL+2)] -> kappa

  void build(const SyBookkeeper& bk, int site);
  int kappa(int nl, int sl, int il, int n1, int n2, int tj, int nr, int sr, int ir) const;
  int64_t size() const { return k2i[nkappa]; }

 private:
  const SyBookkeeper* bk_ = nullptr;
};

struct OpLayout {
  int index = 0;  // boundary
  int two_j = 0, n_elec = 0, n_irrep = 0;
  int nkappa = 0;
  std::vector<int> n_up, irrep_up, spin_up, spin_down, rows, cols;
  std::vector<int64_t> k2i;
  std::vector<int> lookup;  // [sector id up * 5 + (2S_down - 2S_up + 2)] -> kappa

  void build(const SyBookkeeper& bk, int boundary, int two_j, int n_elec, int n_irrep);
  // Block index for (upper sector) -> (lower sector), -1 if the block does not exist.
  int kappa(int n1, int s1, int i1, int n2, int s2, int i2) const;
  int64_t size() const { return k2i[nkappa]; }

 private:
  const SyBookkeeper* bk_ = nullptr;
};

// Shares one OpLayout between all operator tensors of equal (boundary, 2j, n, irrep).
class OpLayoutCache {
 public:
  explicit OpLayoutCache(const SyBookkeeper* bk) : bk_(bk) {}
  const OpLayout* get(int boundary, int two_j, int n_elec, int n_irrep);
  void invalidate_boundary(int boundary);
  void clear() { cache_.clear(); }

 private:
  const SyBookkeeper* bk_;
  std::map<std::tuple<int, int, int, int>, std::unique_ptr<OpLayout>> cache_;
};

}  // namespace c2g
