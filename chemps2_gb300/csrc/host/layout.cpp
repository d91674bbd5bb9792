#include "layout.hpp"

#include <algorithm>
#include <cstdlib>
#include <numeric>

#include "symm.hpp"

namespace c2g {

// ------------------------------------------------------------------ MpsLayout ----
// Loop order of CheMPS2/TensorT.cpp:38-110.
void MpsLayout::build(const SyBookkeeper& bk, int site) {
  index = site;
  nkappa = 0;
  NL.clear(); TwoSL.clear(); IL.clear(); NR.clear(); TwoSR.clear(); IR.clear();
  rows.clear(); cols.clear();
  k2i.assign(1, 0);
  lookup.assign(static_cast<size_t>(bk.num_sectors(index)) * 4, -1);
  const int nirr = bk.getNumberOfIrreps();
  for (int nl = bk.gNmin(index); nl <= bk.gNmax(index); nl++) {
    for (int sl = bk.gTwoSmin(index, nl); sl <= bk.gTwoSmax(index, nl); sl += 2) {
      for (int il = 0; il < nirr; il++) {
        const int dimL = bk.gCurrentDim(index, nl, sl, il);
        if (dimL <= 0) continue;
        const int sid = bk.sector_id(index, nl, sl, il);
        for (int nr = nl; nr <= nl + 2; nr++) {
          const int tj = (nr == nl + 1) ? 1 : 0;
          for (int sr = sl - tj; sr <= sl + tj; sr += 2) {
            if (sr < 0) continue;
            const int ir = (nr == nl + 1) ? irrep_prod(il, bk.gIrrep(index)) : il;
            const int dimR = bk.gCurrentDim(index + 1, nr, sr, ir);
            if (dimR <= 0) continue;
            const int variant = (nr == nl) ? 0 : (nr == nl + 2 ? 3 : (sr < sl ? 1 : 2));
            lookup[sid * 4 + variant] = nkappa;
            NL.push_back(nl); TwoSL.push_back(sl); IL.push_back(il);
            NR.push_back(nr); TwoSR.push_back(sr); IR.push_back(ir);
            rows.push_back(dimL); cols.push_back(dimR);
            k2i.push_back(k2i.back() + static_cast<int64_t>(dimL) * dimR);
            nkappa++;
          }
        }
      }
    }
  }
  bk_ = &bk;
}

int MpsLayout::kappa(int nl, int sl, int il, int nr, int sr, int ir) const {
  const int sid = bk_->sector_id(index, nl, sl, il);
  if (sid < 0) return -1;
  int variant;
  if (nr == nl) variant = 0;
  else if (nr == nl + 2) variant = 3;
  else if (nr == nl + 1 && sr == sl - 1) variant = 1;
  else if (nr == nl + 1 && sr == sl + 1) variant = 2;
  else return -1;
  const int k = lookup[sid * 4 + variant];
  if (k < 0) return -1;
  if (NR[k] != nr || TwoSR[k] != sr || IR[k] != ir) return -1;
  return k;
}

// -------------------------------------------------------------- TwoSiteLayout ----
// Loop order of CheMPS2/Sobject.cpp:36-128; size-sorted order of :130-145.
void TwoSiteLayout::build(const SyBookkeeper& bk, int site) {
  index = site;
  bk_ = &bk;
  nkappa = 0;
  for (auto* v : {&NL, &TwoSL, &IL, &N1, &N2, &TwoJ, &NR, &TwoSR, &IR, &rows, &cols}) v->clear();
  k2i.assign(1, 0);
  lookup.assign(static_cast<size_t>(bk.num_sectors(index)) * 135, -1);
  const int nirr = bk.getNumberOfIrreps();
  const int I1 = bk.gIrrep(index), I2 = bk.gIrrep(index + 1);
  for (int nl = bk.gNmin(index); nl <= bk.gNmax(index); nl++) {
    for (int sl = bk.gTwoSmin(index, nl); sl <= bk.gTwoSmax(index, nl); sl += 2) {
      for (int il = 0; il < nirr; il++) {
        const int dimL = bk.gCurrentDim(index, nl, sl, il);
        if (dimL <= 0) continue;
        const int sid = bk.sector_id(index, nl, sl, il);
        for (int n1 = 0; n1 <= 2; n1++) {
          for (int n2 = 0; n2 <= 2; n2++) {
            const int nr = nl + n1 + n2;
            const int im = (n1 == 1) ? irrep_prod(il, I1) : il;
            const int ir = (n2 == 1) ? irrep_prod(im, I2) : im;
            const int tjmin = (n1 + n2) % 2;
            const int tjmax = (n1 == 1 && n2 == 1) ? 2 : tjmin;
            for (int tj = tjmin; tj <= tjmax; tj += 2) {
              for (int sr = sl - tj; sr <= sl + tj; sr += 2) {
                if (sr < 0) continue;
                const int dimR = bk.gCurrentDim(index + 2, nr, sr, ir);
                if (dimR <= 0) continue;
                lookup[((sid * 9 + n1 * 3 + n2) * 3 + tj) * 5 + (sr - sl + 2)] = nkappa;
                NL.push_back(nl); TwoSL.push_back(sl); IL.push_back(il);
                N1.push_back(n1); N2.push_back(n2); TwoJ.push_back(tj);
                NR.push_back(nr); TwoSR.push_back(sr); IR.push_back(ir);
                rows.push_back(dimL); cols.push_back(dimR);
                k2i.push_back(k2i.back() + static_cast<int64_t>(dimL) * dimR);
                nkappa++;
              }
            }
          }
        }
      }
    }
  }
  // The reference bubble-sorts with a strict "<" swap, which is a stable sort by
  // non-increasing block size; std::stable_sort gives the identical permutation.
  reorder.resize(nkappa);
  std::iota(reorder.begin(), reorder.end(), 0);
  std::stable_sort(reorder.begin(), reorder.end(), [&](int a, int b) {
    return (k2i[a + 1] - k2i[a]) > (k2i[b + 1] - k2i[b]);
  });
}

int TwoSiteLayout::kappa(int nl, int sl, int il, int n1, int n2, int tj, int nr, int sr,
                         int ir) const {
  if (n1 < 0 || n1 > 2 || n2 < 0 || n2 > 2 || tj < 0 || tj > 2) return -1;
  const int ds = sr - sl;
  if (ds < -2 || ds > 2) return -1;
  const int sid = bk_->sector_id(index, nl, sl, il);
  if (sid < 0) return -1;
  const int k = lookup[((sid * 9 + n1 * 3 + n2) * 3 + tj) * 5 + (ds + 2)];
  if (k < 0) return -1;
  if (NR[k] != nr || IR[k] != ir) return -1;
  return k;
}

// ------------------------------------------------------------------- OpLayout ----
// Loop order of CheMPS2/TensorOperator.cpp:29-105; lookup semantics of :121-141.
void OpLayout::build(const SyBookkeeper& bk, int boundary, int tj, int ne, int nirrep) {
  index = boundary;
  two_j = tj;
  n_elec = ne;
  n_irrep = nirrep;
  bk_ = &bk;
  nkappa = 0;
  for (auto* v : {&n_up, &irrep_up, &spin_up, &spin_down, &rows, &cols}) v->clear();
  k2i.assign(1, 0);
  lookup.assign(static_cast<size_t>(bk.num_sectors(index)) * 5, -1);
  const int nirr = bk.getNumberOfIrreps();
  for (int nu = bk.gNmin(index); nu <= bk.gNmax(index); nu++) {
    for (int su = bk.gTwoSmin(index, nu); su <= bk.gTwoSmax(index, nu); su += 2) {
      for (int iu = 0; iu < nirr; iu++) {
        const int dim_up = bk.gCurrentDim(index, nu, su, iu);
        if (dim_up <= 0) continue;
        const int sid = bk.sector_id(index, nu, su, iu);
        const int id = irrep_prod(n_irrep, iu);
        const int nd = nu + n_elec;
        for (int sd = su - two_j; sd <= su + two_j; sd += 2) {
          if (sd < 0) continue;
          const int dim_down = bk.gCurrentDim(index, nd, sd, id);
          if (dim_down <= 0) continue;
          lookup[sid * 5 + (sd - su + 2)] = nkappa;
          n_up.push_back(nu); irrep_up.push_back(iu); spin_up.push_back(su); spin_down.push_back(sd);
          rows.push_back(dim_up); cols.push_back(dim_down);
          k2i.push_back(k2i.back() + static_cast<int64_t>(dim_up) * dim_down);
          nkappa++;
        }
      }
    }
  }
}

int OpLayout::kappa(int n1, int s1, int i1, int n2, int s2, int i2) const {
  if (irrep_prod(i1, n_irrep) != i2) return -1;
  if (n2 != n1 + n_elec) return -1;
  if (std::abs(s1 - s2) > two_j) return -1;
  const int sid = bk_->sector_id(index, n1, s1, i1);
  if (sid < 0) return -1;
  return lookup[sid * 5 + (s2 - s1 + 2)];
}

const OpLayout* OpLayoutCache::get(int boundary, int two_j, int n_elec, int n_irrep) {
  auto key = std::make_tuple(boundary, two_j, n_elec, n_irrep);
  auto it = cache_.find(key);
  if (it != cache_.end()) return it->second.get();
  auto lay = std::make_unique<OpLayout>();
  lay->build(*bk_, boundary, two_j, n_elec, n_irrep);
  const OpLayout* p = lay.get();
  cache_[key] = std::move(lay);
  return p;
}

void OpLayoutCache::invalidate_boundary(int boundary) {
  for (auto it = cache_.begin(); it != cache_.end();) {
    if (std::get<0>(it->first) == boundary) it = cache_.erase(it);
    else ++it;
  }
}

}  // namespace c2g
