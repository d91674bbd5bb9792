// compile_heff / compile_heff_diag: the per-block diagram schedule of
// CheMPS2::Heff::makeHeff and CheMPS2::Heff::fillHeffDiag.
#include "heff_impl.hpp"

namespace c2g {

using std::sqrt;

// CheMPS2/Heff.cpp:43-248. Every block of Y is an output of the single accumulation
// stage; its terms keep the reference's diagram order.
void compile_heff(TaskBuilder& tb, const HeffContext& ctx, int shard, int nshards) {
  HeffEmitter h(tb, ctx);
  const int L = ctx.bk->gL();
  const bool atLeft = (h.theindex == 0);
  const bool atRight = (h.theindex == L - 2);
  const TwoSiteLayout& S = *ctx.S;
  for (int r = shard; r < S.nkappa; r += nshards) {
    const int k = S.reorder[r];
    h.set_block(k, kSlotY);
    tb.declare_output(h.Y);
    h.d1C();
    h.d1D();
    h.d2dall();
    h.d3Eand3H();
    if (!atLeft) {
      h.d1A();
      h.d2b1and2b2();
      h.d2c1and2c2();
      h.d2b3spin0();
      h.d2b3spin1();
      h.d2c3spin0();
      h.d2c3spin1();
      h.d3Aand3D();
      h.d3Band3I();
      h.d4A1and4A2spin0();
      h.d4A1and4A2spin1();
      h.d4A3and4A4spin0();
      h.d4A3and4A4spin1();
      h.d4D();
      h.d4I();
    }
    if (!atRight) {
      h.d1B();
      h.d2e1and2e2();
      h.d2f1and2f2();
      h.d2e3spin0();
      h.d2e3spin1();
      h.d2f3spin0();
      h.d2f3spin1();
      h.d3Kand3F();
      h.d3Land3G();
      h.d4J1and4J2spin0();
      h.d4J1and4J2spin1();
      h.d4J3and4J4spin0();
      h.d4J3and4J4spin1();
      h.d4F();
      h.d4G();
    }
    if (!atLeft && !atRight) {
      h.d2a1spin0();
      h.d2a2spin0();
      h.d2a1spin1();
      h.d2a2spin1();
      h.d2a3spin0();
      h.d2a3spin1();
      h.d3C();
      h.d3J();
      h.d4B1and4B2spin0();
      h.d4B1and4B2spin1();
      h.d4B3and4B4spin0();
      h.d4B3and4B4spin1();
      h.d4C1and4C2spin0();
      h.d4C1and4C2spin1();
      h.d4C3and4C4spin0();
      h.d4C3and4C4spin1();
      h.d4E();
      h.d4H();
      h.d4K1and4K2spin0();
      h.d4L1and4L2spin0();
      h.d4K1and4K2spin1();
      h.d4L1and4L2spin1();
      h.d4K3and4K4spin0();
      h.d4L3and4L4spin0();
      h.d4K3and4K4spin1();
      h.d4L3and4L4spin1();
      h.d5A();
      h.d5B();
      h.d5C();
      h.d5D();
      h.d5E();
      h.d5F();
    }
  }
}

namespace {

// The diagonal of a square operator block as a 1 x d row with stride d + 1.
Blk diag_row(const Blk& b) {
  Blk r = Blk::make(b.ref, 1, b.rows, b.ld + 1);
  return r;
}
Blk ones_col(int n) { return Blk::make(make_ref(kSlotOnes, 0), n, 1); }
Blk ones_row(int n) { return Blk::make(make_ref(kSlotOnes, 0), 1, n, 1); }

}  // namespace

// CheMPS2/Heff.cpp:250-315 with CheMPS2/HeffDiagonal.cpp:27-642. Each contribution is
// a rank-1 update of the block: (left diagonal or ones) x (right diagonal or ones).
void compile_heff_diag(TaskBuilder& tb, const HeffContext& ctx, int shard, int nshards) {
  HeffEmitter h(tb, ctx);
  const int L = ctx.bk->gL();
  const int i = h.theindex;
  const bool atLeft = (i == 0);
  const bool atRight = (i == L - 2);
  const TwoSiteLayout& S = *ctx.S;
  const BoundaryOps* Lt = ctx.left;
  const BoundaryOps* Rt = ctx.right;
  for (int r = shard; r < S.nkappa; r += nshards) {
    const int k = S.reorder[r];
    h.set_block(k, kSlotY);
    tb.declare_output(h.Y);
    const int NL = h.NL, TwoSL = h.TwoSL, IL = h.IL, NR = h.NR, TwoSR = h.TwoSR, IR = h.IR;
    const int N1 = h.N1, N2 = h.N2, TwoJ = h.TwoJ;
    const int dimL = h.dimL, dimR = h.dimR;
    if (dimL == 0 || dimR == 0) continue;
    const Blk oL = ones_col(dimL), oR = ones_row(dimR);
    auto add_const = [&](double a) { tb.contract(h.Y, a, Blk(), false, oL, false, oR, false); };
    auto add_left = [&](double a, const Blk& b) { tb.contract(h.Y, a, Blk(), false, diag_row(b), true, oR, false); };
    auto add_right = [&](double a, const Blk& b) { tb.contract(h.Y, a, Blk(), false, oL, false, diag_row(b), false); };
    auto add_both = [&](double a, const Blk& bl, const Blk& br) {
      tb.contract(h.Y, a, Blk(), false, diag_row(bl), true, diag_row(br), false);
    };
    // 1C, 1D and 2d3 (HeffDiagonal.cpp:50-110)
    double c = 0.0;
    if (N1 == 2) c += h.V(i, i, i, i);
    if (N2 == 2) c += h.V(i + 1, i + 1, i + 1, i + 1);
    const double v1 = h.V(i, i + 1, i, i + 1), v2 = h.V(i, i + 1, i + 1, i);
    if (N1 == 2 && N2 == 2) c += 4 * v1 - 2 * v2;
    if (N1 == 1 && N2 == 1) c += v1 + ((TwoJ == 2) ? -1 : 1) * v2;
    if ((N1 == 2 && N2 == 1) || (N1 == 1 && N2 == 2)) c += 2 * v1 - v2;
    if (c != 0.0) add_const(c);
    if (!atLeft) {
      add_left(1.0, HeffEmitter::need(Lt->X.blk(NL, TwoSL, IL, NL, TwoSL, IL)));  // 1A
      if (N1 != 0) add_left(N1 * sqrt(0.5), HeffEmitter::need(Lt->C[0][0].blk(NL, TwoSL, IL, NL, TwoSL, IL)));
      if (N1 == 1) {
        const int fase = phase(TwoSL + TwoSR + 2 * TwoJ + ((N2 == 1) ? 1 : 0) - 1);
        const double a = fase * (TwoJ + 1) * sqrt(3.0 * (TwoSL + 1)) * wigner6j(TwoJ, TwoJ, 2, 1, 1, (N2 == 1) ? 1 : 0) *
                         wigner6j(TwoJ, TwoJ, 2, TwoSL, TwoSL, TwoSR);
        add_left(a, HeffEmitter::need(Lt->D[0][0].blk(NL, TwoSL, IL, NL, TwoSL, IL)));
      }
      if (N2 != 0) add_left(N2 * sqrt(0.5), HeffEmitter::need(Lt->C[0][1].blk(NL, TwoSL, IL, NL, TwoSL, IL)));
      if (N2 == 1) {
        const int fase = phase(TwoSL + TwoSR + 2 * TwoJ + ((N1 == 1) ? 1 : 0) - 1);
        const double a = fase * (TwoJ + 1) * sqrt(3.0 * (TwoSL + 1)) * wigner6j(TwoJ, TwoJ, 2, 1, 1, (N1 == 1) ? 1 : 0) *
                         wigner6j(TwoJ, TwoJ, 2, TwoSL, TwoSL, TwoSR);
        add_left(a, HeffEmitter::need(Lt->D[0][1].blk(NL, TwoSL, IL, NL, TwoSL, IL)));
      }
    }
    if (!atRight) {
      add_right(1.0, HeffEmitter::need(Rt->X.blk(NR, TwoSR, IR, NR, TwoSR, IR)));  // 1B
      if (N1 != 0) add_right(N1 * sqrt(0.5), HeffEmitter::need(Rt->C[0][1].blk(NR, TwoSR, IR, NR, TwoSR, IR)));
      if (N1 == 1) {
        const int fase = phase(TwoSR + TwoSL + 2 * TwoJ + ((N2 == 1) ? 1 : 0) + 1);
        const double a = fase * (TwoJ + 1) * sqrt(3.0 * (TwoSR + 1)) * wigner6j(TwoJ, TwoJ, 2, 1, 1, (N2 == 1) ? 1 : 0) *
                         wigner6j(TwoJ, TwoJ, 2, TwoSR, TwoSR, TwoSL);
        add_right(a, HeffEmitter::need(Rt->D[0][1].blk(NR, TwoSR, IR, NR, TwoSR, IR)));
      }
      if (N2 != 0) add_right(N2 * sqrt(0.5), HeffEmitter::need(Rt->C[0][0].blk(NR, TwoSR, IR, NR, TwoSR, IR)));
      if (N2 == 1) {
        const int fase = phase(TwoSR + TwoSL + 2 * TwoJ + ((N1 == 1) ? 1 : 0) + 1);
        const double a = fase * (TwoJ + 1) * sqrt(3.0 * (TwoSR + 1)) * wigner6j(TwoJ, TwoJ, 2, 1, 1, (N1 == 1) ? 1 : 0) *
                         wigner6j(TwoJ, TwoJ, 2, TwoSR, TwoSR, TwoSL);
        add_right(a, HeffEmitter::need(Rt->D[0][0].blk(NR, TwoSR, IR, NR, TwoSR, IR)));
      }
    }
    if (!atLeft && !atRight) {
      // 2a3spin0 / 2a3spin1 (HeffDiagonal.cpp:428-642): every unordered pair of orbitals of
      // the shorter side with equal irreps; distinct pairs occur twice in the reference's
      // two loops, coinciding orbitals once.
      const double a1 = phase(TwoSL + TwoSR + TwoJ + 2) * sqrt((TwoSR + 1) * (TwoSL + 1.0)) *
                        wigner6j(TwoSL, TwoSR, TwoJ, TwoSR, TwoSL, 2);
      const bool leftSum = (i < L * 0.5);
      if (leftSum) {
        for (int lo = 0; lo < i; lo++)
          for (int hi = lo; hi < i; hi++) {
            if (h.irr(lo) != h.irr(hi)) continue;
            const double mult = (lo == hi) ? 1.0 : 2.0;
            const Blk f0 = Lt->F0[hi - lo][i - 1 - hi].blk(NL, TwoSL, IL, NL, TwoSL, IL);
            const Blk cc = Rt->C[hi - lo][i + 1 - hi].blk(NR, TwoSR, IR, NR, TwoSR, IR);
            add_both(mult, HeffEmitter::need(f0), HeffEmitter::need(cc));
            const Blk f1 = Lt->F1[hi - lo][i - 1 - hi].blk(NL, TwoSL, IL, NL, TwoSL, IL);
            const Blk dd = Rt->D[hi - lo][i + 1 - hi].blk(NR, TwoSR, IR, NR, TwoSR, IR);
            add_both(mult * a1, HeffEmitter::need(f1), HeffEmitter::need(dd));
          }
      } else {
        for (int lo = i + 2; lo < L; lo++)
          for (int hi = lo; hi < L; hi++) {
            if (h.irr(lo) != h.irr(hi)) continue;
            const double mult = (lo == hi) ? 1.0 : 2.0;
            const Blk cc = Lt->C[hi - lo][lo - i].blk(NL, TwoSL, IL, NL, TwoSL, IL);
            const Blk f0 = Rt->F0[hi - lo][lo - i - 2].blk(NR, TwoSR, IR, NR, TwoSR, IR);
            add_both(mult, HeffEmitter::need(cc), HeffEmitter::need(f0));
            const Blk dd = Lt->D[hi - lo][lo - i].blk(NL, TwoSL, IL, NL, TwoSL, IL);
            const Blk f1 = Rt->F1[hi - lo][lo - i - 2].blk(NR, TwoSR, IR, NR, TwoSR, IR);
            add_both(mult * a1, HeffEmitter::need(dd), HeffEmitter::need(f1));
          }
      }
    }
  }
}

}  // namespace c2g
