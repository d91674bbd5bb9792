// Internal state of the Heff compiler: the labels of the current output block kappa and
// helpers that turn the reference's (sector, operator, block) lookups into Blk operands.
#pragma once

#include <cmath>
#include <cstdlib>
#include <stdexcept>
#include <vector>

#include "heff.hpp"
#include "symm.hpp"

namespace c2g {

struct HeffEmitter {
  TaskBuilder& tb;
  const CheMPS2::SyBookkeeper& bk;
  const CheMPS2::Problem& prob;
  const TwoSiteLayout& S;
  const BoundaryOps* Lt;  // left operators (boundary theindex)
  const BoundaryOps* Rt;  // right operators (boundary theindex + 2)
  int L = 0;
  int theindex = 0;

  // labels of the current output block
  int ik = 0, NL = 0, TwoSL = 0, IL = 0, N1 = 0, N2 = 0, TwoJ = 0, NR = 0, TwoSR = 0, IR = 0;
  int dimL = 0, dimR = 0;
  Blk Y;

  HeffEmitter(TaskBuilder& t, const HeffContext& c)
      : tb(t), bk(*c.bk), prob(*c.prob), S(*c.S), Lt(c.left), Rt(c.right), L(c.bk->gL()),
        theindex(c.S->index) {}

  void set_block(int k, int out_slot) {
    ik = k;
    NL = S.NL[k]; TwoSL = S.TwoSL[k]; IL = S.IL[k];
    N1 = S.N1[k]; N2 = S.N2[k]; TwoJ = S.TwoJ[k];
    NR = S.NR[k]; TwoSR = S.TwoSR[k]; IR = S.IR[k];
    dimL = S.rows[k];
    dimR = S.cols[k];
    Y = Blk::make(make_ref(out_slot, S.k2i[k]), dimL, dimR);
  }

  Blk X(int kp) const { return Blk::make(make_ref(kSlotX, S.k2i[kp]), S.rows[kp], S.cols[kp]); }
  int kap(int nl, int sl, int il, int n1, int n2, int tj, int nr, int sr, int ir) const {
    return S.kappa(nl, sl, il, n1, n2, tj, nr, sr, ir);
  }
  int dL(int n, int s, int i) const { return bk.gCurrentDim(theindex, n, s, i); }
  int dR(int n, int s, int i) const { return bk.gCurrentDim(theindex + 2, n, s, i); }
  double V(int a, int b, int c, int d) const { return prob.gMxElement(a, b, c, d); }
  int irr(int site) const { return bk.gIrrep(site); }

  static Blk need(const Blk& b) {
    if (!b.valid) throw std::logic_error("Heff compiler: a block the reference dereferences is absent");
    return b;
  }
  // Y += alpha * op(A) * X[kp] * op(C); A / C may be invalid (absent)
  void emit(double alpha, const Blk& A, bool ta, int kp, const Blk& C, bool tc) {
    tb.contract(Y, alpha, A, ta, X(kp), false, C, tc);
  }
  // Y += alpha * X[kp]
  void emit_scalar(double alpha, int kp) { tb.axpy(Y, alpha, X(kp), false); }

  // combination of operator blocks (the reference's daxpy into a temporary)
  Blk combine(const std::vector<std::pair<double, Blk>>& parts, int rows, int cols) {
    return tb.combine(parts, rows, cols);
  }

  // diagram groups (CheMPS2/HeffDiagrams1-5.cpp)
  void d1A(); void d1B(); void d1C(); void d1D();
  void d2a1spin0(); void d2a2spin0(); void d2a1spin1(); void d2a2spin1(); void d2a3spin0(); void d2a3spin1();
  void d2b1and2b2(); void d2c1and2c2(); void d2dall(); void d2e1and2e2(); void d2f1and2f2();
  void d2b3spin0(); void d2c3spin0(); void d2e3spin0(); void d2f3spin0();
  void d2b3spin1(); void d2c3spin1(); void d2e3spin1(); void d2f3spin1();
  void d3Aand3D(); void d3Band3I(); void d3C(); void d3Eand3H(); void d3Kand3F(); void d3Land3G(); void d3J();
  void d4A1and4A2spin0(); void d4A1and4A2spin1(); void d4A3and4A4spin0(); void d4A3and4A4spin1();
  void d4B1and4B2spin0(); void d4B1and4B2spin1(); void d4B3and4B4spin0(); void d4B3and4B4spin1();
  void d4C1and4C2spin0(); void d4C1and4C2spin1(); void d4C3and4C4spin0(); void d4C3and4C4spin1();
  void d4D(); void d4E(); void d4F(); void d4G(); void d4H(); void d4I();
  void d4J1and4J2spin0(); void d4J1and4J2spin1(); void d4J3and4J4spin0(); void d4J3and4J4spin1();
  void d4K1and4K2spin0(); void d4L1and4L2spin0(); void d4K1and4K2spin1(); void d4L1and4L2spin1();
  void d4K3and4K4spin0(); void d4L3and4L4spin0(); void d4K3and4K4spin1(); void d4L3and4L4spin1();
  void d5A(); void d5B(); void d5C(); void d5D(); void d5E(); void d5F();
};

inline int heff_phase(int x) { return phase(x); }

}  // namespace c2g
