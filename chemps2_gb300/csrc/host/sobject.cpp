#include "sobject.hpp"

#include <algorithm>
#include <cmath>
#include <cstdlib>

#include "symm.hpp"

namespace c2g {

using std::abs;
using std::max;
using std::min;
using std::sqrt;

// CheMPS2/Sobject.cpp:212-258, times sqrt(2S_R + 1) (prog2symm).
void compile_join(TaskBuilder& tb, const CheMPS2::SyBookkeeper& bk, const TwoSiteLayout& S, const MpsT& left,
                  const MpsT& right) {
  const int index = S.index;
  const int Ilocal1 = bk.gIrrep(index);
  for (int k = 0; k < S.nkappa; k++) {
    const int NL = S.NL[k], TwoSL = S.TwoSL[k], IL = S.IL[k];
    const int NR = S.NR[k], TwoSR = S.TwoSR[k], IR = S.IR[k];
    const int TwoJ = S.TwoJ[k], N1 = S.N1[k], N2 = S.N2[k];
    const Blk Y = Blk::make(make_ref(kSlotY, S.k2i[k]), S.rows[k], S.cols[k]);
    tb.declare_output(Y);
    const int TwoS1 = (N1 == 1) ? 1 : 0, TwoS2 = (N2 == 1) ? 1 : 0;
    const int fase = phase(TwoSL + TwoSR + TwoS1 + TwoS2);
    const int NM = NL + N1;
    const int IM = (TwoS1 == 1) ? irrep_prod(IL, Ilocal1) : IL;
    const int lo = max(abs(TwoSL - TwoS1), abs(TwoSR - TwoS2));
    const int hi = min(TwoSL + TwoS1, TwoSR + TwoS2);
    for (int TwoJM = lo; TwoJM <= hi; TwoJM += 2) {
      if (bk.gCurrentDim(index + 1, NM, TwoJM, IM) <= 0) continue;
      const Blk bl = left.blk(NL, TwoSL, IL, NM, TwoJM, IM);
      const Blk br = right.blk(NM, TwoJM, IM, NR, TwoSR, IR);
      if (!bl.valid || !br.valid) continue;
      const double pref = fase * sqrt(1.0 * (TwoJ + 1) * (TwoJM + 1)) * wigner6j(TwoSL, TwoSR, TwoJ, TwoS2, TwoS1, TwoJM) *
                          sqrt(TwoSR + 1.0);
      tb.contract(Y, pref, Blk(), false, bl, false, br, false);
    }
  }
}

// CheMPS2/Sobject.cpp:260-340 (center sectors and their left / right partners).
SplitPlan plan_split(const CheMPS2::SyBookkeeper& bk, int index, bool moving_right) {
  SplitPlan plan;
  plan.index = index;
  plan.moving_right = moving_right;
  const int nirr = bk.getNumberOfIrreps();
  const int Ilocal1 = bk.gIrrep(index), Ilocal2 = bk.gIrrep(index + 1);
  int64_t off = 0;
  auto align = [](int64_t x) { return (x + 31) & ~int64_t(31); };
  for (int NM = bk.gNmin(index + 1); NM <= bk.gNmax(index + 1); NM++) {
    for (int TwoSM = bk.gTwoSmin(index + 1, NM); TwoSM <= bk.gTwoSmax(index + 1, NM); TwoSM += 2) {
      for (int IM = 0; IM < nirr; IM++) {
        if (bk.gFCIdim(index + 1, NM, TwoSM, IM) <= 0) continue;
        SplitCenter c;
        c.NM = NM;
        c.TwoSM = TwoSM;
        c.IM = IM;
        for (int NL = NM - 2; NL <= NM; NL++) {
          const int TwoS1 = (NL + 1 == NM) ? 1 : 0;
          for (int TwoSL = TwoSM - TwoS1; TwoSL <= TwoSM + TwoS1; TwoSL += 2) {
            if (TwoSL < 0) continue;
            const int IL = (TwoS1 == 1) ? irrep_prod(Ilocal1, IM) : IM;
            const int dimL = bk.gCurrentDim(index, NL, TwoSL, IL);
            if (dimL > 0) {
              c.lparts.push_back({NL, TwoSL, IL, dimL, c.dimL});
              c.dimL += dimL;
            }
          }
        }
        for (int NR = NM; NR <= NM + 2; NR++) {
          const int TwoS2 = (NR == NM + 1) ? 1 : 0;
          for (int TwoSR = TwoSM - TwoS2; TwoSR <= TwoSM + TwoS2; TwoSR += 2) {
            if (TwoSR < 0) continue;
            const int IR = (TwoS2 == 1) ? irrep_prod(Ilocal2, IM) : IM;
            const int dimR = bk.gCurrentDim(index + 2, NR, TwoSR, IR);
            if (dimR > 0) {
              c.rparts.push_back({NR, TwoSR, IR, dimR, c.dimR});
              c.dimR += dimR;
            }
          }
        }
        c.cd = min(c.dimL, c.dimR);
        if (c.cd > 0) {
          c.g = moving_right ? c.dimL : c.dimR;
          c.offA = off;
          off = align(off + int64_t(c.dimL) * c.dimR);
          c.offG = off;
          off = align(off + int64_t(c.g) * c.g);
          c.offU = off;
          off = align(off + int64_t(c.g) * c.g);
          c.offE = off;
          off = align(off + c.g);
        }
        plan.centers.push_back(std::move(c));
      }
    }
  }
  plan.work_size = off;
  return plan;
}

// CheMPS2/Sobject.cpp:341-416: mem += prefactor * block, with the symm2prog factor
// 1 / sqrt(2S_R + 1) folded into the prefactor.
void compile_split_assemble(TaskBuilder& tb, const CheMPS2::SyBookkeeper& bk, const TwoSiteLayout& S,
                            const SplitPlan& plan) {
  (void)bk;
  for (const SplitCenter& c : plan.centers) {
    if (c.cd <= 0) continue;
    for (const SplitPart& lp : c.lparts) {
      for (const SplitPart& rp : c.rparts) {
        const int TwoS1 = (lp.n + 1 == c.NM) ? 1 : 0;
        const int TwoS2 = (rp.n == c.NM + 1) ? 1 : 0;
        const int fase = phase(lp.two_s + rp.two_s + TwoS1 + TwoS2);
        const int jmin = max(abs(rp.two_s - lp.two_s), abs(TwoS2 - TwoS1));
        const int jmax = min(TwoS1 + TwoS2, lp.two_s + rp.two_s);
        const Blk out = Blk::make(make_ref(kSlotWork, c.offA + lp.off + int64_t(c.dimL) * rp.off), lp.dim, rp.dim, c.dimL);
        for (int TwoJ = jmin; TwoJ <= jmax; TwoJ += 2) {
          const int k = S.kappa(lp.n, lp.two_s, lp.irrep, c.NM - lp.n, rp.n - c.NM, TwoJ, rp.n, rp.two_s, rp.irrep);
          if (k < 0) continue;
          const double pref = fase * sqrt(TwoJ + 1.0) * wigner6j(lp.two_s, rp.two_s, TwoJ, TwoS2, TwoS1, c.TwoSM);
          const Blk blk = Blk::make(make_ref(kSlotX, S.k2i[k]), S.rows[k], S.cols[k]);
          tb.axpy(out, pref, blk, false);
        }
      }
    }
  }
  tb.next_stage("split.gram");
  for (const SplitCenter& c : plan.centers) {
    if (c.cd <= 0) continue;
    const Blk A = Blk::make(make_ref(kSlotWork, c.offA), c.dimL, c.dimR);
    const Blk G = Blk::make(make_ref(kSlotWork, c.offG), c.g, c.g);
    if (plan.moving_right)
      tb.contract(G, 1.0, Blk(), false, A, false, A, true);  // A A^T
    else
      tb.contract(G, 1.0, Blk(), false, A, true, A, false);  // A^T A
  }
}

void compile_split_copy(TaskBuilder& tb, const SplitPlan& plan, const std::vector<int>& dims_m, const MpsT& left,
                        const MpsT& right) {
  for (size_t ic = 0; ic < plan.centers.size(); ic++) {
    const SplitCenter& c = plan.centers[ic];
    const int dimM = dims_m[ic];
    const int nr = min(dimM, c.cd);
    if (dimM <= 0 || nr <= 0) continue;
    const Blk Ucols = Blk::make(make_ref(kSlotWork, c.offU), c.g, nr, c.g);
    for (const SplitPart& lp : c.lparts) {
      const Blk T = left.blk(lp.n, lp.two_s, lp.irrep, c.NM, c.TwoSM, c.IM);
      if (!T.valid) continue;
      const Blk out = Blk::make(T.ref, lp.dim, nr, lp.dim);
      if (plan.moving_right) {
        // U part, CheMPS2/Sobject.cpp:527-555
        tb.axpy(out, 1.0, Blk::make(make_ref(kSlotWork, c.offU + lp.off), lp.dim, nr, c.g), false);
      } else {
        // U * lambda = A V
        const Blk Asub = Blk::make(make_ref(kSlotWork, c.offA + lp.off), lp.dim, c.dimR, c.dimL);
        tb.contract(out, 1.0, Blk(), false, Asub, false, Ucols, false);
      }
    }
    for (const SplitPart& rp : c.rparts) {
      const Blk T = right.blk(c.NM, c.TwoSM, c.IM, rp.n, rp.two_s, rp.irrep);
      if (!T.valid) continue;
      const Blk out = Blk::make(T.ref, nr, rp.dim, dimM);
      const double fb = sqrt((c.TwoSM + 1.0) / (rp.two_s + 1));
      if (plan.moving_right) {
        // lambda * V^T = U^T A, CheMPS2/Sobject.cpp:557-590
        const Blk Asub = Blk::make(make_ref(kSlotWork, c.offA + int64_t(c.dimL) * rp.off), c.dimL, rp.dim, c.dimL);
        tb.contract(out, fb, Blk(), false, Ucols, true, Asub, false);
      } else {
        tb.axpy(out, fb, Blk::make(make_ref(kSlotWork, c.offU + rp.off), rp.dim, nr, c.g), true);
      }
    }
  }
}

}  // namespace c2g
