#include "excite.hpp"

#include <stdexcept>

#include "symm.hpp"

namespace c2g {

void OverlapLayout::build(const CheMPS2::SyBookkeeper& up, const CheMPS2::SyBookkeeper& down, int b) {
  boundary = b;
  up_ = &up;
  N.clear();
  S.clear();
  I.clear();
  rows.clear();
  cols.clear();
  k2i.assign(1, 0);
  by_sector_.clear();
  for (int n = up.gNmin(b); n <= up.gNmax(b); n++)
    for (int s = up.gTwoSmin(b, n); s <= up.gTwoSmax(b, n); s += 2)
      for (int i = 0; i < up.getNumberOfIrreps(); i++) {
        const int du = up.gCurrentDim(b, n, s, i), dd = down.gCurrentDim(b, n, s, i);
        if (du <= 0 || dd <= 0) continue;
        const int sid = up.sector_id(b, n, s, i);
        if (sid >= static_cast<int>(by_sector_.size())) by_sector_.resize(sid + 1, -1);
        by_sector_[sid] = static_cast<int>(N.size());
        N.push_back(n);
        S.push_back(s);
        I.push_back(i);
        rows.push_back(du);
        cols.push_back(dd);
        k2i.push_back(k2i.back() + static_cast<int64_t>(du) * dd);
      }
  nkappa = static_cast<int>(N.size());
}

int OverlapLayout::kappa(int n, int s, int i) const {
  const int sid = up_->sector_id(boundary, n, s, i);
  if (sid < 0 || sid >= static_cast<int>(by_sector_.size())) return -1;
  return by_sector_[sid];
}

namespace {
Blk need(const Blk& b) {
  if (!b.valid) throw std::logic_error("excited states: a block of nonzero dimensions is missing");
  return b;
}
}  // namespace

// CheMPS2/TensorO.cpp:64-192 and the spin-0 case of CheMPS2/TensorOperator.cpp:163-405
void compile_overlap_update(TaskBuilder& tb, const CheMPS2::SyBookkeeper& up, const CheMPS2::SyBookkeeper& down,
                            bool moving_right, int index, const OverlapT* prev, const OverlapT& out, const MpsT& Tup,
                            const MpsT& Tdown) {
  const OverlapLayout& lay = *out.lay;
  const int b = index + 1;  // boundary of `out`
  for (int k = 0; k < lay.nkappa; k++) {
    const Blk ob = Blk::make(out.base + lay.k2i[k], lay.rows[k], lay.cols[k]);
    tb.declare_output(ob);
    const int n = lay.N[k], s = lay.S[k], ir = lay.I[k];
    if (moving_right) {
      // previous boundary index, site index: left sectors of (n, s, ir)
      const int isite = up.gIrrep(index);
      const int nl[4] = {n, n - 2, n - 1, n - 1};
      const int sl[4] = {s, s, s - 1, s + 1};
      const int il[4] = {ir, ir, irrep_prod(ir, isite), irrep_prod(ir, isite)};
      for (int g = 0; g < 4; g++) {
        if (nl[g] < 0 || sl[g] < 0) continue;
        const int du = up.gCurrentDim(b - 1, nl[g], sl[g], il[g]), dd = down.gCurrentDim(b - 1, nl[g], sl[g], il[g]);
        if (du <= 0 || dd <= 0) continue;
        const Blk tu = need(Tup.blk(nl[g], sl[g], il[g], n, s, ir));
        const Blk td = need(Tdown.blk(nl[g], sl[g], il[g], n, s, ir));
        if (prev) tb.contract(ob, 1.0, tu, true, need(prev->blk(nl[g], sl[g], il[g])), false, td, false);
        else if (du == 1 && dd == 1) tb.contract(ob, 1.0, tu, true, td, false, Blk(), false);
      }
    } else {
      // previous boundary index + 2, site index + 1: right sectors of (n, s, ir)
      const int isite = up.gIrrep(index + 1);
      const int nr[4] = {n, n + 2, n + 1, n + 1};
      const int sr[4] = {s, s, s - 1, s + 1};
      const int irr[4] = {ir, ir, irrep_prod(ir, isite), irrep_prod(ir, isite)};
      for (int g = 0; g < 4; g++) {
        if (sr[g] < 0) continue;
        const int du = up.gCurrentDim(b + 1, nr[g], sr[g], irr[g]), dd = down.gCurrentDim(b + 1, nr[g], sr[g], irr[g]);
        if (du <= 0 || dd <= 0) continue;
        const double alpha = (g > 1) ? (sr[g] + 1.0) / (s + 1) : 1.0;
        const Blk tu = need(Tup.blk(n, s, ir, nr[g], sr[g], irr[g]));
        const Blk td = need(Tdown.blk(n, s, ir, nr[g], sr[g], irr[g]));
        if (prev) tb.contract(ob, alpha, tu, false, need(prev->blk(nr[g], sr[g], irr[g])), false, td, true);
        else if (du == 1 && dd == 1) tb.contract(ob, alpha, Blk(), false, tu, false, td, true);
      }
    }
  }
}

// CheMPS2/DMRGtechnics.cpp:540-620 (calcVeffTilde), in the symmetric convention of the
// joined vectors
void compile_veff(TaskBuilder& tb, const TwoSiteLayout& S, const TwoSiteLayout& Sk, Ref sup, const OverlapT* left,
                  const OverlapT* right, double prefactor, Ref out) {
  for (int k = 0; k < S.nkappa; k++) {
    const Blk ob = Blk::make(out + S.k2i[k], S.rows[k], S.cols[k]);
    tb.declare_output(ob);
    const int ks = Sk.kappa(S.NL[k], S.TwoSL[k], S.IL[k], S.N1[k], S.N2[k], S.TwoJ[k], S.NR[k], S.TwoSR[k], S.IR[k]);
    if (ks < 0) continue;
    const Blk sb = Blk::make(sup + Sk.k2i[ks], Sk.rows[ks], Sk.cols[ks]);
    Blk ol, orr;
    if (left) ol = need(left->blk(S.NL[k], S.TwoSL[k], S.IL[k]));
    else if (sb.rows != ob.rows) throw std::logic_error("excited states: left edge dimensions differ");
    if (right) orr = need(right->blk(S.NR[k], S.TwoSR[k], S.IR[k]));
    else if (sb.cols != ob.cols) throw std::logic_error("excited states: right edge dimensions differ");
    tb.contract(ob, prefactor, ol, false, sb, false, orr, true);
  }
}

}  // namespace c2g
