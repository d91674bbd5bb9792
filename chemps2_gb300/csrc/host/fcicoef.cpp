#include "fcicoef.hpp"

#include <cmath>
#include <stdexcept>

#include "symm.hpp"

namespace c2g {

double fci_coefficient(const CheMPS2::SyBookkeeper& bk, const CheMPS2::Problem& prob,
                       const std::vector<const MpsLayout*>& lay, const std::vector<const double*>& T,
                       const int* alpha, const int* beta) {
  const int L = prob.gL();
  auto ham = [&](int k) { return prob.gReorder() ? prob.gf2(k) : k; };
  // CheMPS2/DMRGtechnics.cpp:346-371: the determinant must lie in the targeted sector
  int n_tot = 0, two_sz = 0, irrep = 0;
  for (int k = 0; k < L; k++) {
    const int h = ham(k);
    if ((alpha[h] != 0 && alpha[h] != 1) || (beta[h] != 0 && beta[h] != 1))
      throw std::invalid_argument("getFCIcoefficient: occupations must be 0 or 1");
    n_tot += alpha[h] + beta[h];
    two_sz += alpha[h] - beta[h];
    if (alpha[h] + beta[h] == 1) irrep = irrep_prod(irrep, bk.gIrrep(k));
  }
  if (n_tot != prob.gN() || two_sz > prob.gTwoS() || two_sz < -prob.gTwoS() || (prob.gTwoS() - two_sz) % 2 != 0 ||
      irrep != prob.gIrrep())
    return 0.0;
  // :373-491: a row vector over the states of boundary k, one segment per spin 2S_L (the
  // particle number, irrep and 2S_z of the boundary are fixed by the determinant), times
  // the site tensor's blocks, with the Clebsch-Gordan coefficient that couples the local
  // spin projection written as a 3j symbol
  struct Sector {
    int two_s;
    std::vector<double> v;
  };
  std::vector<Sector> left{{0, {1.0}}};
  int NL = 0, IL = 0, two_szl = 0;
  for (int k = 0; k < L; k++) {
    const int h = ham(k);
    const int n_loc = alpha[h] + beta[h];
    const int two_sz_loc = alpha[h] - beta[h];
    const int NR = NL + n_loc;
    const int two_szr = two_szl + two_sz_loc;
    const int IR = (n_loc == 1) ? irrep_prod(IL, bk.gIrrep(k)) : IL;
    const int spread = (n_loc == 1) ? 1 : 0;
    std::vector<Sector> right;
    for (const Sector& sl : left)
      for (int two_sr = sl.two_s - spread; two_sr <= sl.two_s + spread; two_sr += 2) {
        bool seen = false;
        for (const Sector& sr : right) seen = seen || sr.two_s == two_sr;
        if (seen || two_sr < 0) continue;
        const int dim_r = bk.gCurrentDim(k + 1, NR, two_sr, IR);
        if (dim_r > 0) right.push_back({two_sr, std::vector<double>(dim_r, 0.0)});
      }
    for (Sector& sr : right) {
      const int dim_r = static_cast<int>(sr.v.size());
      for (int two_sl = sr.two_s - spread; two_sl <= sr.two_s + spread; two_sl += 2) {
        const Sector* sl = nullptr;
        for (const Sector& s : left)
          if (s.two_s == two_sl) sl = &s;
        if (!sl) continue;
        const int kap = lay[k]->kappa(NL, two_sl, IL, NR, sr.two_s, IR);
        if (kap < 0) continue;
        const int dim_l = static_cast<int>(sl->v.size());
        if (lay[k]->rows[kap] != dim_l || lay[k]->cols[kap] != dim_r)
          throw std::logic_error("getFCIcoefficient: block dimensions differ from the bookkeeper");
        const double* blk = T[k] + lay[k]->k2i[kap];
        const double pref = std::sqrt(sr.two_s + 1.0) * wigner3j(two_sl, spread, sr.two_s, two_szl, two_sz_loc, -two_szr) *
                            phase(-two_sl + spread - two_szr);
        if (pref == 0.0) continue;
        for (int c = 0; c < dim_r; c++) {
          double acc = 0.0;
          for (int r = 0; r < dim_l; r++) acc += sl->v[r] * blk[r + static_cast<size_t>(dim_l) * c];
          sr.v[c] += pref * acc;
        }
      }
    }
    left.swap(right);
    NL = NR;
    IL = IR;
    two_szl = two_szr;
  }
  if (left.size() != 1 || left[0].v.size() != 1 || left[0].two_s != prob.gTwoS())
    throw std::logic_error("getFCIcoefficient: the chain does not end in the targeted sector");
  return left[0].v[0];
}

}  // namespace c2g
