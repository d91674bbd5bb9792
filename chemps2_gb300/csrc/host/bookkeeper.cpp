// SyBookkeeper: FCI and current virtual dimensions per symmetry sector.
// Same recurrences, bounds and scaling as CheMPS2/SyBookkeeper.cpp:29-323.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <stdexcept>

#include "chemps2/SyBookkeeper.h"
#include "symm.hpp"

namespace CheMPS2 {

namespace {
constexpr int kDimensionCutoff = 262144;  // CheMPS2/include/chemps2/Options.h:76
}

SyBookkeeper::SyBookkeeper(const Problem* P, const int D)
    : Prob(P), L(P->gL()), N(P->gN()), TwoS(P->gTwoS()), Irrep(P->gIrrep()),
      nirrep(c2g::num_irreps(P->gSy())) {
  orb_irrep.resize(L);
  for (int o = 0; o < L; o++) orb_irrep[o] = P->gIrrep(o);
  Nmin.resize(L + 1);
  Nmax.resize(L + 1);
  nsec.resize(L + 1);
  TwoSmin.resize(L + 1);
  TwoSmax.resize(L + 1);
  sec_base.resize(L + 1);
  fci.resize(L + 1);
  cur.resize(L + 1);
  // Allowed ranges: CheMPS2/SyBookkeeper.cpp:76-111
  for (int b = 0; b <= L; b++) {
    Nmin[b] = std::max(std::max(0, N + 2 * (b - L)), b - L + (N + TwoS) / 2);
    Nmax[b] = std::min(std::min(2 * b, N), b + (N - TwoS) / 2);
    const int nn = std::max(0, Nmax[b] - Nmin[b] + 1);
    TwoSmin[b].resize(nn);
    TwoSmax[b].resize(nn);
    sec_base[b].resize(nn);
    int count = 0;
    for (int n = Nmin[b]; n <= Nmax[b]; n++) {
      const int temporary = L - b - std::abs(N - n - L + b);
      TwoSmin[b][n - Nmin[b]] = std::max(n % 2, TwoS - temporary);
      TwoSmax[b][n - Nmin[b]] = std::min(b - std::abs(b - n), TwoS + temporary);
      sec_base[b][n - Nmin[b]] = count;
      const int ns = (TwoSmax[b][n - Nmin[b]] - TwoSmin[b][n - Nmin[b]]) / 2 + 1;
      count += std::max(0, ns) * nirrep;
    }
    nsec[b] = count;
    fci[b].assign(count, 0);
    cur[b].assign(count, 0);
  }
  // fillFCIdim: CheMPS2/SyBookkeeper.cpp:175-194
  fci[0][sector_id(0, 0, 0, 0)] = 1;
  fill_fci_dim_right(fci, 1, L);
  const int rhs = gFCIdim(L, N, TwoS, Irrep);
  for (int i = 0; i < (int)fci[L].size(); i++) fci[L][i] = 0;
  {
    const int id = sector_id(L, N, TwoS, Irrep);
    if (id >= 0) fci[L][id] = std::min(1, rhs);
  }
  fill_fci_dim_left(fci, 0, L - 1);
  cur = fci;
  scale_cur_dim(D, 1, L - 1);
  if (!IsPossible()) throw std::invalid_argument("SyBookkeeper: the targeted symmetry sector is empty");
}

void SyBookkeeper::sector_labels(const int b, const int id, int* n, int* two_s, int* irrep) const {
  for (int nn = Nmax[b]; nn >= Nmin[b]; nn--) {
    if (sec_base[b][nn - Nmin[b]] <= id) {
      const int rel = id - sec_base[b][nn - Nmin[b]];
      *n = nn;
      *two_s = TwoSmin[b][nn - Nmin[b]] + 2 * (rel / nirrep);
      *irrep = rel % nirrep;
      return;
    }
  }
  *n = *two_s = *irrep = -1;
}

void SyBookkeeper::SetDim(const int b, const int n, const int s, const int i, const int value) {
  // CheMPS2/SyBookkeeper.cpp:167-173: only sectors that exist at FCI level are set.
  if (gFCIdim(b, n, s, i) != 0) cur[b][sector_id(b, n, s, i)] = value;
}

void SyBookkeeper::fill_fci_dim_right(std::vector<std::vector<int>>& st, int start, int stop) {
  // CheMPS2/SyBookkeeper.cpp:196-215
  for (int b = start; b <= stop; b++) {
    for (int n = Nmin[b]; n <= Nmax[b]; n++) {
      for (int s = gTwoSmin(b, n); s <= gTwoSmax(b, n); s += 2) {
        for (int i = 0; i < nirrep; i++) {
          const int ip = c2g::irrep_prod(i, orb_irrep[b - 1]);
          const int value = std::min(
              kDimensionCutoff, dim_private(st, b - 1, n, s, i) + dim_private(st, b - 1, n - 2, s, i) +
                                    dim_private(st, b - 1, n - 1, s + 1, ip) +
                                    dim_private(st, b - 1, n - 1, s - 1, ip));
          st[b][sector_id(b, n, s, i)] = value;
        }
      }
    }
  }
}

void SyBookkeeper::fill_fci_dim_left(std::vector<std::vector<int>>& st, int start, int stop) {
  // CheMPS2/SyBookkeeper.cpp:217-236
  for (int b = stop; b >= start; b--) {
    for (int n = Nmin[b]; n <= Nmax[b]; n++) {
      for (int s = gTwoSmin(b, n); s <= gTwoSmax(b, n); s += 2) {
        for (int i = 0; i < nirrep; i++) {
          const int ip = c2g::irrep_prod(i, orb_irrep[b]);
          const int value = std::min(
              dim_private(st, b, n, s, i),
              std::min(kDimensionCutoff,
                       dim_private(st, b + 1, n, s, i) + dim_private(st, b + 1, n + 2, s, i) +
                           dim_private(st, b + 1, n + 1, s + 1, ip) +
                           dim_private(st, b + 1, n + 1, s - 1, ip)));
          st[b][sector_id(b, n, s, i)] = value;
        }
      }
    }
  }
}

void SyBookkeeper::scale_cur_dim(int virtual_dim, int start, int stop) {
  // CheMPS2/SyBookkeeper.cpp:250-269
  for (int b = start; b <= stop; b++) {
    const int total = gTotDimAtBound(b);
    if (total > virtual_dim) {
      const double factor = (1.0 * virtual_dim) / total;
      for (int n = Nmin[b]; n <= Nmax[b]; n++)
        for (int s = gTwoSmin(b, n); s <= gTwoSmax(b, n); s += 2)
          for (int i = 0; i < nirrep; i++) {
            const int value = static_cast<int>(std::ceil(factor * gCurrentDim(b, n, s, i)) + 0.1);
            SetDim(b, n, s, i, value);
          }
    }
  }
}

int SyBookkeeper::gMaxDimAtBound(const int b) const {
  int m = 0;
  for (int v : cur[b]) m = std::max(m, v);
  return m;
}

int SyBookkeeper::gTotDimAtBound(const int b) const {
  int t = 0;
  for (int v : cur[b]) t += v;
  return t;
}

bool SyBookkeeper::IsPossible() const { return gCurrentDim(L, N, TwoS, Irrep) == 1; }

}  // namespace CheMPS2
