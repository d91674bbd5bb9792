// Heff diagrams 5A-5F (CheMPS2/HeffDiagrams5.cpp:28-1960): one creator of the left block
// and one of the right block, weighted by two-body integrals with two indices on the two
// local sites. For each left orbital l_a the reference sums the right creators into a
// temporary (sum over l_b of prefac(l_a, l_b) * L_right(l_b)) and applies
// L_left(l_a) * X * temporary; the temporary becomes a combined block here.
#include "heff_impl.hpp"

namespace c2g {

using std::abs;
using std::sqrt;

namespace {

inline int ph(int x) { return heff_phase(x); }
inline int parity(int x) { return ((x % 2) != 0) ? -1 : 1; }

bool any_irrep(const HeffEmitter& h, int lo, int hi, int ir) {
  for (int l = lo; l < hi; l++)
    if (h.irr(l) == ir) return true;
  return false;
}

}  // namespace

namespace {

// Shared body of every 5X case. nld / nrd: particle number of the left / right "down"
// sector; ldn: the left creator block maps (nld -> NL) and is used transposed, otherwise
// (NL -> nld); rdn: the right creator block maps (nrd -> NR) and is used as is, otherwise
// (NR -> nrd) used transposed. Reference loop: CheMPS2/HeffDiagrams5.cpp:66-128.
template <class Coef>
void five_body(HeffEmitter& h, int nld, int SLd, int nrd, int SRd, int kn1, int kn2, int ktj, bool ldn, bool rdn,
               Coef coef) {
  const int i = h.theindex;
  const int mid = irrep_prod(h.irr(i), h.irr(i + 1));
  const int nirr = h.bk.getNumberOfIrreps();
  for (int Irrep = 0; Irrep < nirr; Irrep++) {
    const int IrrepTimesMid = irrep_prod(Irrep, mid);
    if (!any_irrep(h, 0, i, Irrep) || !any_irrep(h, i + 2, h.L, IrrepTimesMid)) continue;
    const int ILd = irrep_prod(h.IL, Irrep), IRd = irrep_prod(h.IR, IrrepTimesMid);
    const int dLd = h.dL(nld, SLd, ILd), dRd = h.dR(nrd, SRd, IRd);
    if (dLd <= 0 || dRd <= 0) continue;
    const int kp = h.kap(nld, SLd, ILd, kn1, kn2, ktj, nrd, SRd, IRd);
    if (kp == -1) continue;
    for (int la = 0; la < i; la++) {
      if (h.irr(la) != Irrep) continue;
      thread_local std::vector<std::pair<double, Blk>> parts;  // reused: no allocation per block
      parts.clear();
      for (int lb = i + 2; lb < h.L; lb++) {
        if (h.irr(lb) != IrrepTimesMid) continue;
        const Blk rb = rdn ? h.Rt->Lop(lb).blk(nrd, SRd, IRd, h.NR, h.TwoSR, h.IR)
                           : h.Rt->Lop(lb).blk(h.NR, h.TwoSR, h.IR, nrd, SRd, IRd);
        parts.push_back({coef(la, lb), HeffEmitter::need(rb)});
      }
      const Blk W = rdn ? h.combine(parts, dRd, h.dimR) : h.combine(parts, h.dimR, dRd);
      const Blk lbk = ldn ? h.Lt->Lop(la).blk(nld, SLd, ILd, h.NL, h.TwoSL, h.IL)
                          : h.Lt->Lop(la).blk(h.NL, h.TwoSL, h.IL, nld, SLd, ILd);
      h.emit(1.0, HeffEmitter::need(lbk), ldn, kp, W, !rdn);
    }
  }
}

}  // namespace

// CheMPS2/HeffDiagrams5.cpp:28-358
void HeffEmitter::d5A() {
  const int i = theindex;
  if (N1 == 0 && N2 == 0)  // 5A1
    for (int SLd = TwoSL - 1; SLd <= TwoSL + 1; SLd += 2)
      for (int SRd = TwoSR - 1; SRd <= TwoSR + 1; SRd += 2)
        for (int TJd = 0; TJd <= 2; TJd += 2) {
          if (abs(SLd - SRd) > TJd || SLd < 0 || SRd < 0) continue;
          const double f = ph(SLd + SRd + 2) * sqrt((TJd + 1) * (SRd + 1.0)) * wigner6j(1, 1, TJd, SLd, SRd, TwoSR);
          five_body(*this, NL - 1, SLd, NR + 1, SRd, 1, 1, TJd, true, false, [&](int la, int lb) {
            return f * (V(la, lb, i, i + 1) + ((TJd == 0) ? 1 : -1) * V(la, lb, i + 1, i));
          });
        }
  if ((N1 == 1 && N2 == 0) || (N1 == 0 && N2 == 1))  // 5A2 and 5A3
    for (int SLd = TwoSL - 1; SLd <= TwoSL + 1; SLd += 2)
      for (int SRd = TwoSR - 1; SRd <= TwoSR + 1; SRd += 2) {
        if (!((TwoSL == SRd) || (SLd == TwoSR)) || abs(SLd - SRd) > 1 || SLd < 0 || SRd < 0) continue;
        double fa = 0.0, fb = 0.0;  // fa multiplies the spin-flip-free term in 5A2
        if (TwoSL == SRd) fb = ph(SRd + 1 - TwoSR);
        if (SLd == TwoSR) fa = ph(SLd + 1 - TwoSL) * sqrt(((SRd + 1) * (TwoSL + 1.0)) / ((TwoSR + 1) * (SLd + 1.0)));
        const double f1 = (N1 == 1) ? fa : fb, f2 = (N1 == 1) ? fb : fa;
        const int kn1 = (N1 == 1) ? 2 : 1, kn2 = (N1 == 1) ? 1 : 2;
        five_body(*this, NL - 1, SLd, NR + 1, SRd, kn1, kn2, 1, true, false,
                  [&](int la, int lb) { return f1 * V(la, lb, i, i + 1) + f2 * V(la, lb, i + 1, i); });
      }
  if (N1 == 1 && N2 == 1)  // 5A4
    for (int SLd = TwoSL - 1; SLd <= TwoSL + 1; SLd += 2) {
      if (SLd < 0 || abs(TwoSR - SLd) > 1) continue;
      const int SRd = SLd;
      const double f = parity(TwoSL + 1) * sqrt((TwoJ + 1) * (TwoSL + 1.0)) * wigner6j(1, 1, TwoJ, TwoSL, TwoSR, SRd);
      five_body(*this, NL - 1, SLd, NR + 1, SRd, 2, 2, 0, true, false, [&](int la, int lb) {
        return f * (V(la, lb, i, i + 1) + ((TwoJ == 0) ? 1 : -1) * V(la, lb, i + 1, i));
      });
    }
}

// CheMPS2/HeffDiagrams5.cpp:360-687
void HeffEmitter::d5B() {
  const int i = theindex;
  if (N1 == 1 && N2 == 1)  // 5B1
    for (int SLd = TwoSL - 1; SLd <= TwoSL + 1; SLd += 2) {
      if (SLd < 0 || abs(TwoSR - SLd) > 1) continue;
      const int SRd = SLd;
      const double f = ph(TwoSL + TwoSR + 2) * sqrt((TwoJ + 1) * (TwoSR + 1.0)) * wigner6j(1, 1, TwoJ, TwoSL, TwoSR, SRd);
      five_body(*this, NL + 1, SLd, NR - 1, SRd, 0, 0, 0, false, true, [&](int la, int lb) {
        return f * (V(la, lb, i, i + 1) + ((TwoJ == 0) ? 1 : -1) * V(la, lb, i + 1, i));
      });
    }
  if ((N1 == 2 && N2 == 1) || (N1 == 1 && N2 == 2))  // 5B2 and 5B3
    for (int SLd = TwoSL - 1; SLd <= TwoSL + 1; SLd += 2)
      for (int SRd = TwoSR - 1; SRd <= TwoSR + 1; SRd += 2) {
        if (!((TwoSL == SRd) || (SLd == TwoSR)) || abs(SLd - SRd) > 1 || SLd < 0 || SRd < 0) continue;
        double fa = 0.0, fb = 0.0;
        if (SLd == TwoSR) fb = ph(TwoSR + 1 - SRd);
        if (TwoSL == SRd) fa = ph(TwoSL + 1 - SLd) * sqrt(((TwoSR + 1) * (SLd + 1.0)) / ((SRd + 1) * (TwoSL + 1.0)));
        const double f1 = (N1 == 2) ? fa : fb, f2 = (N1 == 2) ? fb : fa;
        const int kn1 = (N1 == 2) ? 1 : 0, kn2 = (N1 == 2) ? 0 : 1;
        five_body(*this, NL + 1, SLd, NR - 1, SRd, kn1, kn2, 1, false, true,
                  [&](int la, int lb) { return f1 * V(la, lb, i, i + 1) + f2 * V(la, lb, i + 1, i); });
      }
  if (N1 == 2 && N2 == 2)  // 5B4
    for (int SLd = TwoSL - 1; SLd <= TwoSL + 1; SLd += 2)
      for (int SRd = TwoSR - 1; SRd <= TwoSR + 1; SRd += 2)
        for (int TJd = 0; TJd <= 2; TJd += 2) {
          if (abs(SLd - SRd) > TJd || SLd < 0 || SRd < 0) continue;
          const double f = parity(SLd + 1) * sqrt((TJd + 1) * (SLd + 1.0)) * wigner6j(1, 1, TJd, SLd, SRd, TwoSR);
          five_body(*this, NL + 1, SLd, NR - 1, SRd, 1, 1, TJd, false, true, [&](int la, int lb) {
            return f * (V(la, lb, i, i + 1) + ((TJd == 0) ? 1 : -1) * V(la, lb, i + 1, i));
          });
        }
}

// CheMPS2/HeffDiagrams5.cpp:689-1005 (5C: left annihilated, right annihilated) and
// 1326-1641 (5E, the same with the two local sites swapped in the integrals).
namespace {
void five_ce(HeffEmitter& h, int a, int b) {
  // a, b: the local sites in the order of the reference's integrals (i, i+1 for 5C;
  // i+1, i for 5E). The spin coupling factors below are identical for 5C and 5E once
  // the occupations of the two sites are exchanged accordingly.
  const int NL = h.NL, TwoSL = h.TwoSL, NR = h.NR, TwoSR = h.TwoSR, TwoJ = h.TwoJ;
  const bool is_c = (a == h.theindex);
  const int Nna = is_c ? h.N1 : h.N2;  // occupation of site a
  const int Nnb = is_c ? h.N2 : h.N1;  // occupation of site b
  auto kn = [&](int na, int nb, int& k1, int& k2) {
    k1 = is_c ? na : nb;
    k2 = is_c ? nb : na;
  };
  auto body = [&](int SLd, int SRd, int na, int nb, int tj, double f1, double f2) {
    int k1, k2;
    kn(na, nb, k1, k2);
    five_body(h, NL - 1, SLd, NR - 1, SRd, k1, k2, tj, true, true,
              [&](int la, int lb) { return f1 * h.V(la, a, b, lb) + f2 * h.V(la, a, lb, b); });
  };
  if (Nna == 1 && Nnb == 0)  // 5C1 / 5E1
    for (int SLd = TwoSL - 1; SLd <= TwoSL + 1; SLd += 2)
      for (int SRd = TwoSR - 1; SRd <= TwoSR + 1; SRd += 2) {
        if (abs(SLd - SRd) > 1 || SLd < 0 || SRd < 0) continue;
        const double f2 = ph(TwoSL + SRd) * sqrt((TwoSL + 1) * (TwoSR + 1.0)) * wigner6j(SLd, SRd, 1, TwoSR, TwoSL, 1);
        const double f1 = (TwoSL == SRd) ? sqrt((TwoSR + 1.0) / (SRd + 1.0)) : 0.0;
        body(SLd, SRd, 0, 1, 1, f1, f2);
      }
  if (Nna == 2 && Nnb == 0)  // 5C2 / 5E2
    for (int SLd = TwoSL - 1; SLd <= TwoSL + 1; SLd += 2)
      for (int SRd = TwoSR - 1; SRd <= TwoSR + 1; SRd += 2)
        for (int TJd = 0; TJd <= 2; TJd += 2) {
          if (abs(SLd - SRd) > TJd || SLd < 0 || SRd < 0) continue;
          const int fase = is_c ? ph(TwoSR + SLd + 3 + TJd) : ph(TwoSR + SLd + 3);
          const double f1 = fase * sqrt((TwoSR + 1) * (TJd + 1.0)) * wigner6j(1, 1, TJd, SLd, SRd, TwoSR);
          const double f2 = (TJd == 0) ? sqrt(2.0 * (TwoSR + 1.0) / (SRd + 1.0)) : 0.0;
          body(SLd, SRd, 1, 1, TJd, f1, f2);
        }
  if (Nna == 1 && Nnb == 1)  // 5C3 / 5E3
    for (int SLd = TwoSL - 1; SLd <= TwoSL + 1; SLd += 2) {
      if (SLd < 0 || abs(TwoSR - SLd) > 1) continue;
      const int SRd = SLd;
      const int fase = is_c ? ph(TwoSR + SRd + 3 + TwoJ) : ph(TwoSR + SRd + 3);
      const double f1 = fase * sqrt((TwoSL + 1.0) * (TwoJ + 1.0) * (TwoSR + 1.0) / (SRd + 1.0)) *
                        wigner6j(1, 1, TwoJ, TwoSL, TwoSR, SRd);
      const double f2 = (TwoJ == 0) ? sqrt(2.0 * (TwoSR + 1.0) / (SRd + 1.0)) : 0.0;
      body(SLd, SRd, 0, 2, 0, f1, f2);
    }
  if (Nna == 2 && Nnb == 1)  // 5C4 / 5E4
    for (int SLd = TwoSL - 1; SLd <= TwoSL + 1; SLd += 2)
      for (int SRd = TwoSR - 1; SRd <= TwoSR + 1; SRd += 2) {
        if (abs(SLd - SRd) > 1 || SLd < 0 || SRd < 0) continue;
        const double f1 = (SLd == TwoSR) ? ph(TwoSL - SRd) * sqrt((TwoSL + 1.0) / (SLd + 1.0)) : 0.0;
        const double f2 = ph(TwoSL + SRd + 2) * sqrt((TwoSL + 1) * (TwoSR + 1.0)) * wigner6j(SLd, SRd, 1, TwoSR, TwoSL, 1);
        body(SLd, SRd, 1, 2, 1, f1, f2);
      }
}

// CheMPS2/HeffDiagrams5.cpp:1007-1324 (5D: left created, right created) and 1643-1960
// (5F, the same with the two local sites swapped in the integrals).
void five_df(HeffEmitter& h, int a, int b) {
  const int NL = h.NL, TwoSL = h.TwoSL, NR = h.NR, TwoSR = h.TwoSR, TwoJ = h.TwoJ;
  const bool is_d = (a == h.theindex);
  const int Nna = is_d ? h.N1 : h.N2;
  const int Nnb = is_d ? h.N2 : h.N1;
  auto body = [&](int SLd, int SRd, int na, int nb, int tj, double f1, double f2) {
    const int k1 = is_d ? na : nb, k2 = is_d ? nb : na;
    five_body(h, NL + 1, SLd, NR + 1, SRd, k1, k2, tj, false, false,
              [&](int la, int lb) { return f1 * h.V(la, a, b, lb) + f2 * h.V(la, a, lb, b); });
  };
  if (Nna == 0 && Nnb == 1)  // 5D1 / 5F1
    for (int SLd = TwoSL - 1; SLd <= TwoSL + 1; SLd += 2)
      for (int SRd = TwoSR - 1; SRd <= TwoSR + 1; SRd += 2) {
        if (abs(SLd - SRd) > 1 || SLd < 0 || SRd < 0) continue;
        const double f2 = ph(SLd + TwoSR) * sqrt((SLd + 1) * (SRd + 1.0)) * wigner6j(TwoSL, TwoSR, 1, SRd, SLd, 1);
        const double f1 = (SLd == TwoSR) ? sqrt((SRd + 1.0) / (TwoSR + 1.0)) : 0.0;
        body(SLd, SRd, 1, 0, 1, f1, f2);
      }
  if (Nna == 1 && Nnb == 1)  // 5D2 / 5F2
    for (int SLd = TwoSL - 1; SLd <= TwoSL + 1; SLd += 2) {
      if (SLd < 0 || abs(TwoSR - SLd) > 1) continue;
      const int SRd = SLd;
      const int fase = is_d ? ph(SRd + TwoSL + 3 + TwoJ) : ph(SRd + TwoSL + 3);
      const double f1 = fase * sqrt((SRd + 1) * (TwoJ + 1.0)) * wigner6j(1, 1, TwoJ, TwoSL, TwoSR, SRd);
      const double f2 = (TwoJ == 0) ? sqrt(2.0 * (SRd + 1.0) / (TwoSR + 1.0)) : 0.0;
      body(SLd, SRd, 2, 0, 0, f1, f2);
    }
  if (Nna == 0 && Nnb == 2)  // 5D3 / 5F3
    for (int SLd = TwoSL - 1; SLd <= TwoSL + 1; SLd += 2)
      for (int SRd = TwoSR - 1; SRd <= TwoSR + 1; SRd += 2)
        for (int TJd = 0; TJd <= 2; TJd += 2) {
          if (abs(SLd - SRd) > TJd || SLd < 0 || SRd < 0) continue;
          const int fase = is_d ? ph(TwoSR + SRd + 3 + TJd) : ph(TwoSR + SRd + 3);
          const double f1 = fase * sqrt((SLd + 1.0) * (TJd + 1.0) * (SRd + 1.0) / (TwoSR + 1.0)) *
                            wigner6j(1, 1, TJd, SLd, SRd, TwoSR);
          const double f2 = (TJd == 0) ? sqrt(2.0 * (SRd + 1.0) / (TwoSR + 1.0)) : 0.0;
          body(SLd, SRd, 1, 1, TJd, f1, f2);
        }
  if (Nna == 1 && Nnb == 2)  // 5D4 / 5F4
    for (int SLd = TwoSL - 1; SLd <= TwoSL + 1; SLd += 2)
      for (int SRd = TwoSR - 1; SRd <= TwoSR + 1; SRd += 2) {
        if (abs(SLd - SRd) > 1 || SLd < 0 || SRd < 0) continue;
        const double f1 = (TwoSL == SRd) ? ph(SLd - TwoSR) * sqrt((SLd + 1.0) / (TwoSL + 1.0)) : 0.0;
        const double f2 = ph(SLd + TwoSR + 2) * sqrt((SLd + 1) * (SRd + 1.0)) * wigner6j(TwoSL, TwoSR, 1, SRd, SLd, 1);
        body(SLd, SRd, 2, 1, 1, f1, f2);
      }
}
}  // namespace

void HeffEmitter::d5C() { five_ce(*this, theindex, theindex + 1); }
void HeffEmitter::d5E() { five_ce(*this, theindex + 1, theindex); }
void HeffEmitter::d5D() { five_df(*this, theindex, theindex + 1); }
void HeffEmitter::d5F() { five_df(*this, theindex + 1, theindex); }

}  // namespace c2g
