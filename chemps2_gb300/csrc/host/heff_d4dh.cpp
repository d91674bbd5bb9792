// Heff diagrams 4D, 4E, 4F, 4G, 4H and 4I (CheMPS2/HeffDiagrams4.cpp:2334-4276): a
// creator of the left (4D, 4I) or right (4F, 4G) block weighted by two-body integrals with
// three indices on the two local sites, and products of a left and a right creator
// (4E, 4H). The reference's integral-weighted temporaries become combined blocks.
#include "heff_impl.hpp"

namespace c2g {

using std::abs;
using std::sqrt;

namespace {

const Blk kNo;
inline int ph(int x) { return heff_phase(x); }

// sum_l coef(l) * L_l(block) over the left (side == Lt) or right orbitals l whose irrep
// equals `ir`; invalid Blk when no orbital qualifies.
template <class Coef>
Blk lsum(HeffEmitter& h, const BoundaryOps* side, bool left, int ir, Coef coef, int n1, int s1, int i1, int n2,
         int s2, int i2, int rows, int cols) {
  thread_local std::vector<std::pair<double, Blk>> parts;  // reused: no allocation per block
  parts.clear();
  const int lo = left ? 0 : h.theindex + 2, hi = left ? h.theindex : h.L;
  for (int l = lo; l < hi; l++)
    if (h.irr(l) == ir) parts.push_back({coef(l), HeffEmitter::need(side->Lop(l).blk(n1, s1, i1, n2, s2, i2))});
  return h.combine(parts, rows, cols);
}

bool any_irrep(HeffEmitter& h, int lo, int hi, int ir) {
  for (int l = lo; l < hi; l++)
    if (h.irr(l) == ir) return true;
  return false;
}

}  // namespace

// CheMPS2/HeffDiagrams4.cpp:2334-2594
void HeffEmitter::d4D() {
  const int i = theindex;
  const int ILd = irrep_prod(IL, irr(i + 1));
  const int ir = irr(i + 1);
  if (N1 == 0 && N2 > 0) {  // 4D1A and 4D1B
    const int S2d = (N2 == 1) ? 0 : 1;
    for (int SLd = TwoSL - 1; SLd <= TwoSL + 1; SLd += 2) {
      if (abs(SLd - TwoSR) > S2d) continue;
      const int dLd = dL(NL - 1, SLd, ILd);
      if (dLd <= 0) continue;
      const Blk W = lsum(*this, Lt, true, ir, [&](int l) { return V(l, i + 1, i, i); }, NL - 1, SLd, ILd, NL, TwoSL, IL,
                         dLd, dimL);
      if (!W.valid) continue;
      double f = -1.0;
      if (N2 == 1) f = ph(TwoSR + 1 - TwoSL) * sqrt((TwoSL + 1.0) / (TwoSR + 1.0));
      const int kp = kap(NL - 1, SLd, ILd, 2, N2 - 1, S2d, NR, TwoSR, IR);
      if (kp != -1) emit(f, W, true, kp, kNo, false);
    }
  }
  if (N1 == 2 && N2 < 2) {  // 4D2A and 4D2B
    const int S2d = (N2 == 0) ? 1 : 0;
    for (int SLd = TwoSL - 1; SLd <= TwoSL + 1; SLd += 2) {
      if (abs(SLd - TwoSR) > S2d) continue;
      const int dLd = dL(NL + 1, SLd, ILd);
      if (dLd <= 0) continue;
      const Blk W = lsum(*this, Lt, true, ir, [&](int l) { return V(l, i + 1, i, i); }, NL, TwoSL, IL, NL + 1, SLd, ILd,
                         dimL, dLd);
      if (!W.valid) continue;
      double f = -1.0;
      if (N2 == 0) f = ph(TwoSR + 1 - SLd) * sqrt((SLd + 1.0) / (TwoSR + 1.0));
      const int kp = kap(NL + 1, SLd, ILd, 0, N2 + 1, S2d, NR, TwoSR, IR);
      if (kp != -1) emit(f, W, false, kp, kNo, false);
    }
  }
  if (N1 > 0 && N2 < 2) {  // 4D3A, 4D3B, 4D3C and 4D3D
    for (int SLd = TwoSL - 1; SLd <= TwoSL + 1; SLd += 2) {
      const int dLd = dL(NL - 1, SLd, ILd);
      if (dLd <= 0) continue;
      const int sum = ((N1 == 1) ? 1 : 0) + ((N2 == 0) ? 1 : 0);
      const int start = ((SLd != TwoSR) || (sum < 2)) ? sum : 0;
      for (int TJd = start; TJd <= sum; TJd += 2) {
        if (abs(SLd - TwoSR) > TJd) continue;
        double af = 0.0;
        if (N1 == 1 && N2 == 0) af = ph(SLd + TwoSR + 2) * sqrt((TwoSL + 1.0) * (TJd + 1)) * wigner6j(TJd, 1, 1, TwoSL, SLd, TwoSR);
        if (N1 == 1 && N2 == 1) af = ph(SLd + TwoSR + 3 + TwoJ) * sqrt((TwoSL + 1.0) * (TwoJ + 1)) * wigner6j(TwoSL, TwoSR, TwoJ, 1, 1, SLd);
        if (N1 == 2 && N2 == 0) af = -1.0;
        if (N1 == 2 && N2 == 1) af = ph(TwoSL + 1 - TwoSR) * sqrt((TwoSL + 1.0) / (TwoSR + 1.0));
        auto coef = [&](int l) {
          double a = 0.0;
          if (N1 == 1 && N2 == 0) a = af * (V(l, i, i, i + 1) + ((TJd == 0) ? 1 : -1) * V(l, i, i + 1, i));
          if (N1 == 1 && N2 == 1) {
            a = af * V(l, i, i + 1, i);
            if (TwoJ == 0) a += sqrt(2.0) * V(l, i, i, i + 1);
          }
          if (N1 == 2) a = af * (V(l, i, i, i + 1) - 2 * V(l, i, i + 1, i));
          return a;
        };
        const Blk W = lsum(*this, Lt, true, ir, coef, NL - 1, SLd, ILd, NL, TwoSL, IL, dLd, dimL);
        if (!W.valid) continue;
        const int kp = kap(NL - 1, SLd, ILd, N1, N2 + 1, TJd, NR, TwoSR, IR);
        if (kp != -1) emit(1.0, W, true, kp, kNo, false);
      }
    }
  }
  if (N1 > 0 && N2 > 0) {  // 4D4A, 4D4B, 4D4C and 4D4D
    for (int SLd = TwoSL - 1; SLd <= TwoSL + 1; SLd += 2) {
      const int dLd = dL(NL + 1, SLd, ILd);
      if (dLd <= 0) continue;
      const int sum = ((N1 == 1) ? 1 : 0) + ((N2 == 2) ? 1 : 0);
      const int start = ((SLd != TwoSR) || (sum < 2)) ? sum : 0;
      for (int TJd = start; TJd <= sum; TJd += 2) {
        if (abs(SLd - TwoSR) > TJd) continue;
        double af = 0.0;
        if (N1 == 1 && N2 == 1) af = ph(TwoSL + TwoSR + 2) * sqrt((SLd + 1.0) * (TwoJ + 1)) * wigner6j(TwoJ, 1, 1, SLd, TwoSL, TwoSR);
        if (N1 == 1 && N2 == 2) af = ph(TwoSL + TwoSR + 3 + TJd) * sqrt((SLd + 1.0) * (TJd + 1)) * wigner6j(SLd, TwoSR, TJd, 1, 1, TwoSL);
        if (N1 == 2 && N2 == 1) af = -1.0;
        if (N1 == 2 && N2 == 2) af = ph(SLd + 1 - TwoSR) * sqrt((SLd + 1.0) / (TwoSR + 1.0));
        auto coef = [&](int l) {
          double a = 0.0;
          if (N1 == 1 && N2 == 1) a = af * (V(l, i, i, i + 1) + ((TwoJ == 0) ? 1 : -1) * V(l, i, i + 1, i));
          if (N1 == 1 && N2 == 2) {
            a = af * V(l, i, i + 1, i);
            if (TJd == 0) a += sqrt(2.0) * V(l, i, i, i + 1);
          }
          if (N1 == 2) a = af * (V(l, i, i, i + 1) - 2 * V(l, i, i + 1, i));
          return a;
        };
        const Blk W = lsum(*this, Lt, true, ir, coef, NL, TwoSL, IL, NL + 1, SLd, ILd, dimL, dLd);
        if (!W.valid) continue;
        const int kp = kap(NL + 1, SLd, ILd, N1, N2 - 1, TJd, NR, TwoSR, IR);
        if (kp != -1) emit(1.0, W, false, kp, kNo, false);
      }
    }
  }
}

// CheMPS2/HeffDiagrams4.cpp:2596-3027. For every left orbital l_a of irrep I, a sandwich
// L_left(l_a) * X * (sum over right orbitals l_b of irrep I of c(l_a,l_b) L_right(l_b)).
void HeffEmitter::d4E() {
  const int i = theindex;
  const int S2 = (N2 == 1) ? 1 : 0;
  const int nirr = bk.getNumberOfIrreps();
  // Common driver. ldn: left creator block (down -> up, used transposed) when true,
  // else (up -> down). rdn similarly for the right creator: (down -> up) used as is.
  auto body = [&](int nld, int SLd, int nrd, int SRd, int kn1, int kn2, int ktj, double outer, bool ldn, bool rdn,
                  auto coef) {
    for (int Irrep = 0; Irrep < nirr; Irrep++) {
      const int ILd = irrep_prod(IL, Irrep), IRd = irrep_prod(IR, Irrep);
      const int dLd = dL(nld, SLd, ILd), dRd = dR(nrd, SRd, IRd);
      if (dLd <= 0 || dRd <= 0) continue;
      if (!any_irrep(*this, 0, i, Irrep) || !any_irrep(*this, i + 2, L, Irrep)) continue;
      const int kp = kap(nld, SLd, ILd, kn1, kn2, ktj, nrd, SRd, IRd);
      for (int la = 0; la < i; la++) {
        if (irr(la) != Irrep) continue;
        thread_local std::vector<std::pair<double, Blk>> parts;  // reused: no allocation per block
        parts.clear();
        for (int lb = i + 2; lb < L; lb++) {
          if (irr(lb) != Irrep) continue;
          const Blk rb = rdn ? Rt->Lop(lb).blk(nrd, SRd, IRd, NR, TwoSR, IR) : Rt->Lop(lb).blk(NR, TwoSR, IR, nrd, SRd, IRd);
          parts.push_back({coef(la, lb), need(rb)});
        }
        const Blk W = rdn ? combine(parts, dRd, dimR) : combine(parts, dimR, dRd);
        const Blk lb2 = ldn ? Lt->Lop(la).blk(nld, SLd, ILd, NL, TwoSL, IL) : Lt->Lop(la).blk(NL, TwoSL, IL, nld, SLd, ILd);
        if (kp != -1) emit(outer, need(lb2), ldn, kp, W, !rdn);
      }
    }
  };
  if (N1 == 0)  // 4E1
    for (int SLd = TwoSL - 1; SLd <= TwoSL + 1; SLd += 2)
      for (int SRd = TwoSR - 1; SRd <= TwoSR + 1; SRd += 2) {
        if (abs(SLd - SRd) > TwoJ || SLd < 0 || SRd < 0) continue;
        const double f = ph(TwoSL + TwoSR - S2) * sqrt((TwoSL + 1) * (SRd + 1.0)) * wigner6j(TwoSL, TwoSR, S2, SRd, SLd, 1);
        body(NL - 1, SLd, NR + 1, SRd, 2, N2, S2, f, true, false, [&](int la, int lb) { return V(la, lb, i, i); });
      }
  if (N1 == 2)  // 4E2
    for (int SLd = TwoSL - 1; SLd <= TwoSL + 1; SLd += 2)
      for (int SRd = TwoSR - 1; SRd <= TwoSR + 1; SRd += 2) {
        if (abs(SLd - SRd) > TwoJ || SLd < 0 || SRd < 0) continue;
        const double f = ph(SLd + SRd - S2) * sqrt((SLd + 1) * (TwoSR + 1.0)) * wigner6j(SLd, SRd, S2, TwoSR, TwoSL, 1);
        body(NL + 1, SLd, NR - 1, SRd, 0, N2, S2, f, false, true, [&](int la, int lb) { return V(la, lb, i, i); });
      }
  if (N1 == 1)  // 4E3A
    for (int SLd = TwoSL - 1; SLd <= TwoSL + 1; SLd += 2)
      for (int SRd = TwoSR - 1; SRd <= TwoSR + 1; SRd += 2) {
        const int start = ((SLd != SRd) || (S2 == 0)) ? S2 + 1 : 0;
        for (int TJd = start; TJd <= S2 + 1; TJd += 2) {
          if (abs(SLd - SRd) > TJd || SLd < 0 || SRd < 0) continue;
          const double f1 = ph(TwoSL + TwoSR + TwoJ + SLd + SRd + 1 - S2) * sqrt((TwoJ + 1) * (TJd + 1) * (TwoSL + 1) * (TwoSR + 1.0)) *
                            wigner6j(TwoSL, SRd, S2, TJd, 1, SLd) * wigner6j(TwoJ, 1, S2, SRd, TwoSL, TwoSR);
          double f2 = 0.0;
          if (TwoJ == TJd) f2 = ph(TwoSL + SRd + TwoJ + 3 + 2 * S2) * sqrt((TwoSL + 1) * (TwoSR + 1.0)) * wigner6j(SLd, SRd, TwoJ, TwoSR, TwoSL, 1);
          body(NL - 1, SLd, NR - 1, SRd, 1, N2, TJd, 1.0, true, true, [&](int la, int lb) {
            double p = f1 * V(la, i, i, lb);
            if (TwoJ == TJd) p += f2 * V(la, i, lb, i);
            return p;
          });
        }
      }
  if (N1 == 2)  // 4E3B
    for (int SLd = TwoSL - 1; SLd <= TwoSL + 1; SLd += 2)
      for (int SRd = TwoSR - 1; SRd <= TwoSR + 1; SRd += 2) {
        if (abs(SLd - SRd) > TwoJ || SLd < 0 || SRd < 0) continue;
        const double f = ph(TwoSL + SRd - S2 + 3) * sqrt((TwoSL + 1) * (TwoSR + 1.0)) * wigner6j(SLd, SRd, S2, TwoSR, TwoSL, 1);
        body(NL - 1, SLd, NR - 1, SRd, 2, N2, S2, f, true, true,
             [&](int la, int lb) { return V(la, i, i, lb) - 2 * V(la, i, lb, i); });
      }
  if (N1 == 1)  // 4E4A
    for (int SLd = TwoSL - 1; SLd <= TwoSL + 1; SLd += 2)
      for (int SRd = TwoSR - 1; SRd <= TwoSR + 1; SRd += 2) {
        const int start = ((SLd != SRd) || (S2 == 0)) ? S2 + 1 : 0;
        for (int TJd = start; TJd <= S2 + 1; TJd += 2) {
          if (abs(SLd - SRd) > TJd || SLd < 0 || SRd < 0) continue;
          const double f1 = ph(TwoSL + TwoSR + TJd + SLd + SRd + 1 - S2) * sqrt((TwoJ + 1) * (TJd + 1) * (SLd + 1) * (SRd + 1.0)) *
                            wigner6j(SLd, TwoSR, S2, TwoJ, 1, TwoSL) * wigner6j(TJd, 1, S2, TwoSR, SLd, SRd);
          double f2 = 0.0;
          if (TwoJ == TJd) f2 = ph(SLd + TwoSR + TwoJ + 3 + 2 * S2) * sqrt((SLd + 1) * (SRd + 1.0)) * wigner6j(TwoSL, TwoSR, TwoJ, SRd, SLd, 1);
          body(NL + 1, SLd, NR + 1, SRd, 1, N2, TJd, 1.0, false, false, [&](int la, int lb) {
            double p = f1 * V(la, i, i, lb);
            if (TwoJ == TJd) p += f2 * V(la, i, lb, i);
            return p;
          });
        }
      }
  if (N1 == 2)  // 4E4B
    for (int SLd = TwoSL - 1; SLd <= TwoSL + 1; SLd += 2)
      for (int SRd = TwoSR - 1; SRd <= TwoSR + 1; SRd += 2) {
        if (abs(SLd - SRd) > TwoJ || SLd < 0 || SRd < 0) continue;
        const double f = ph(SLd + TwoSR - S2 + 3) * sqrt((SLd + 1) * (SRd + 1.0)) * wigner6j(TwoSL, TwoSR, S2, SRd, SLd, 1);
        body(NL + 1, SLd, NR + 1, SRd, 2, N2, S2, f, false, false,
             [&](int la, int lb) { return V(la, i, i, lb) - 2 * V(la, i, lb, i); });
      }
}

// CheMPS2/HeffDiagrams4.cpp:3029-3295
void HeffEmitter::d4F() {
  const int i = theindex;
  const int IRd = irrep_prod(IR, irr(i + 1));
  const int ir = irr(i + 1);
  if (N1 == 2 && N2 < 2) {  // 4F1A and 4F1B
    const int S2d = (N2 == 1) ? 0 : 1;
    for (int SRd = TwoSR - 1; SRd <= TwoSR + 1; SRd += 2) {
      if (abs(TwoSL - SRd) > S2d) continue;
      const int dRd = dR(NR - 1, SRd, IRd);
      if (dRd <= 0) continue;
      const Blk W = lsum(*this, Rt, false, ir, [&](int l) { return V(i, i, i + 1, l); }, NR - 1, SRd, IRd, NR, TwoSR, IR,
                         dRd, dimR);
      if (!W.valid) continue;
      const double f = (N2 == 1) ? -sqrt((TwoSR + 1.0) / (SRd + 1.0)) : (double)ph(TwoSR + 1 - SRd);
      const int kp = kap(NL, TwoSL, IL, 0, N2 + 1, S2d, NR - 1, SRd, IRd);
      if (kp != -1) emit(f, kNo, false, kp, W, false);
    }
  }
  if (N1 == 0 && N2 > 0) {  // 4F2A and 4F2B
    const int S2d = (N2 == 1) ? 0 : 1;
    for (int SRd = TwoSR - 1; SRd <= TwoSR + 1; SRd += 2) {
      if (abs(TwoSL - SRd) > S2d) continue;
      const int dRd = dR(NR + 1, SRd, IRd);
      if (dRd <= 0) continue;
      const Blk W = lsum(*this, Rt, false, ir, [&](int l) { return V(i, i, i + 1, l); }, NR, TwoSR, IR, NR + 1, SRd, IRd,
                         dimR, dRd);
      if (!W.valid) continue;
      const double f = (N2 == 2) ? -sqrt((SRd + 1.0) / (TwoSR + 1.0)) : (double)ph(SRd + 1 - TwoSR);
      const int kp = kap(NL, TwoSL, IL, 2, N2 - 1, S2d, NR + 1, SRd, IRd);
      if (kp != -1) emit(f, kNo, false, kp, W, true);
    }
  }
  if (N1 > 0 && N2 > 0) {  // 4F3A..4F3D
    for (int SRd = TwoSR - 1; SRd <= TwoSR + 1; SRd += 2) {
      const int dRd = dR(NR - 1, SRd, IRd);
      if (dRd <= 0) continue;
      const int sum = ((N1 == 1) ? 1 : 0) + ((N2 == 2) ? 1 : 0);
      const int start = ((TwoSL != SRd) || (sum < 2)) ? sum : 0;
      for (int TJd = start; TJd <= sum; TJd += 2) {
        if (abs(TwoSL - SRd) > TJd) continue;
        double f = 0.0, f2 = 0.0;
        if (N1 == 1 && N2 == 1) f = ph(TwoSL + TwoSR + 2) * sqrt((TwoSR + 1.0) * (TwoJ + 1)) * wigner6j(TwoJ, 1, 1, SRd, TwoSR, TwoSL);
        if (N1 == 1 && N2 == 2) {
          f = ph(TwoSL + TwoSR + 3) * sqrt((TwoSR + 1.0) * (TJd + 1)) * wigner6j(TJd, 1, 1, TwoSR, SRd, TwoSL);
          f2 = (TJd == 0) ? sqrt(2.0 * (TwoSR + 1.0) / (SRd + 1.0)) : 0.0;
        }
        if (N1 == 2 && N2 == 1) f = sqrt((TwoSR + 1.0) / (SRd + 1.0));
        if (N1 == 2 && N2 == 2) f = ph(TwoSR + 1 - SRd);
        auto coef = [&](int l) {
          double p = 0.0;
          if (N1 == 1 && N2 == 1) p = f * (V(i, i + 1, i, l) + ((TwoJ == 0) ? 1 : -1) * V(i, i + 1, l, i));
          if (N1 == 1 && N2 == 2) {
            p = f * V(i, i + 1, i, l);
            if (TJd == 0) p += f2 * V(i, i + 1, l, i);
          }
          if (N1 == 2) p = f * (2 * V(i, i + 1, i, l) - V(i, i + 1, l, i));
          return p;
        };
        const Blk W = lsum(*this, Rt, false, ir, coef, NR - 1, SRd, IRd, NR, TwoSR, IR, dRd, dimR);
        if (!W.valid) continue;
        const int kp = kap(NL, TwoSL, IL, N1, N2 - 1, TJd, NR - 1, SRd, IRd);
        if (kp != -1) emit(1.0, kNo, false, kp, W, false);
      }
    }
  }
  if (N1 > 0 && N2 < 2) {  // 4F4A..4F4D
    for (int SRd = TwoSR - 1; SRd <= TwoSR + 1; SRd += 2) {
      const int dRd = dR(NR + 1, SRd, IRd);
      if (dRd <= 0) continue;
      const int sum = ((N1 == 1) ? 1 : 0) + ((N2 == 0) ? 1 : 0);
      const int start = ((TwoSL != SRd) || (sum < 2)) ? sum : 0;
      for (int TJd = start; TJd <= sum; TJd += 2) {
        if (abs(TwoSL - SRd) > TJd) continue;
        double f = 0.0, f2 = 0.0;
        if (N1 == 1 && N2 == 0) f = ph(TwoSL + SRd + 2) * sqrt((SRd + 1.0) * (TJd + 1)) * wigner6j(TJd, 1, 1, TwoSR, SRd, TwoSL);
        if (N1 == 1 && N2 == 1) {
          f = ph(TwoSL + SRd + 3) * sqrt((SRd + 1.0) * (TwoJ + 1)) * wigner6j(TwoJ, 1, 1, SRd, TwoSR, TwoSL);
          f2 = (TwoJ == 0) ? sqrt(2.0 * (SRd + 1.0) / (TwoSR + 1.0)) : 0.0;
        }
        if (N1 == 2 && N2 == 0) f = sqrt((SRd + 1.0) / (TwoSR + 1.0));
        if (N1 == 2 && N2 == 1) f = ph(SRd + 1 - TwoSR);
        auto coef = [&](int l) {
          double p = 0.0;
          if (N1 == 1 && N2 == 0) p = f * (V(i, i + 1, i, l) + ((TJd == 0) ? 1 : -1) * V(i, i + 1, l, i));
          if (N1 == 1 && N2 == 1) {
            p = f * V(i, i + 1, i, l);
            if (TwoJ == 0) p += f2 * V(i, i + 1, l, i);
          }
          if (N1 == 2) p = f * (2 * V(i, i + 1, i, l) - V(i, i + 1, l, i));
          return p;
        };
        const Blk W = lsum(*this, Rt, false, ir, coef, NR, TwoSR, IR, NR + 1, SRd, IRd, dimR, dRd);
        if (!W.valid) continue;
        const int kp = kap(NL, TwoSL, IL, N1, N2 + 1, TJd, NR + 1, SRd, IRd);
        if (kp != -1) emit(1.0, kNo, false, kp, W, true);
      }
    }
  }
}

// CheMPS2/HeffDiagrams4.cpp:3297-3561
void HeffEmitter::d4G() {
  const int i = theindex;
  const int IRd = irrep_prod(IR, irr(i));
  const int ir = irr(i);
  if (N1 < 2 && N2 == 2) {  // 4G1A and 4G1B
    const int S1d = (N1 == 1) ? 0 : 1;
    for (int SRd = TwoSR - 1; SRd <= TwoSR + 1; SRd += 2) {
      if (abs(TwoSL - SRd) > S1d) continue;
      const int dRd = dR(NR - 1, SRd, IRd);
      if (dRd <= 0) continue;
      const Blk W = lsum(*this, Rt, false, ir, [&](int l) { return V(i, l, i + 1, i + 1); }, NR - 1, SRd, IRd, NR, TwoSR,
                         IR, dRd, dimR);
      if (!W.valid) continue;
      const double f = (N1 == 1) ? -sqrt((TwoSR + 1.0) / (SRd + 1.0)) : (double)ph(TwoSR + 1 - SRd);
      const int kp = kap(NL, TwoSL, IL, N1 + 1, 0, S1d, NR - 1, SRd, IRd);
      if (kp != -1) emit(f, kNo, false, kp, W, false);
    }
  }
  if (N1 > 0 && N2 == 0) {  // 4G2A and 4G2B
    const int S1d = (N1 == 1) ? 0 : 1;
    for (int SRd = TwoSR - 1; SRd <= TwoSR + 1; SRd += 2) {
      if (abs(TwoSL - SRd) > S1d) continue;
      const int dRd = dR(NR + 1, SRd, IRd);
      if (dRd <= 0) continue;
      const Blk W = lsum(*this, Rt, false, ir, [&](int l) { return V(i, l, i + 1, i + 1); }, NR, TwoSR, IR, NR + 1, SRd,
                         IRd, dimR, dRd);
      if (!W.valid) continue;
      const double f = (N1 == 2) ? -sqrt((SRd + 1.0) / (TwoSR + 1.0)) : (double)ph(SRd + 1 - TwoSR);
      const int kp = kap(NL, TwoSL, IL, N1 - 1, 2, S1d, NR + 1, SRd, IRd);
      if (kp != -1) emit(f, kNo, false, kp, W, true);
    }
  }
  if (N1 < 2 && N2 > 0) {  // 4G3A..4G3D
    for (int SRd = TwoSR - 1; SRd <= TwoSR + 1; SRd += 2) {
      const int dRd = dR(NR + 1, SRd, IRd);
      if (dRd <= 0) continue;
      const int sum = ((N1 == 1) ? 0 : 1) + ((N2 == 1) ? 1 : 0);
      const int start = ((TwoSL != SRd) || (sum < 2)) ? sum : 0;
      for (int TJd = start; TJd <= sum; TJd += 2) {
        if (abs(TwoSL - SRd) > TJd) continue;
        double a = 0.0, a2 = 0.0;
        if (N1 == 0 && N2 == 1) a = ph(TwoSL + SRd + 2) * sqrt((TJd + 1) * (SRd + 1.0)) * wigner6j(TJd, 1, 1, TwoSR, SRd, TwoSL);
        if (N1 == 1 && N2 == 1) {
          a = ph(TwoSL + SRd + TwoJ + 3) * sqrt((TwoJ + 1) * (SRd + 1.0)) * wigner6j(TwoJ, 1, 1, SRd, TwoSR, TwoSL);
          a2 = (TwoJ == 0) ? sqrt(2.0 * (SRd + 1.0) / (TwoSR + 1.0)) : 0.0;
        }
        if (N1 == 0 && N2 == 2) a = -sqrt((SRd + 1.0) / (TwoSR + 1.0));
        if (N1 == 1 && N2 == 2) a = ph(TwoSR + 1 - SRd);
        auto coef = [&](int l) {
          double p = 0.0;
          if (N1 == 0 && N2 == 1) p = a * (V(i, i + 1, i + 1, l) + ((TJd == 0) ? 1 : -1) * V(i, i + 1, l, i + 1));
          if (N1 == 1 && N2 == 1) {
            p = a * V(i, i + 1, l, i + 1);
            if (TwoJ == 0) p += a2 * V(i, i + 1, i + 1, l);
          }
          if (N2 == 2) p = a * (V(i, i + 1, i + 1, l) - 2 * V(i, i + 1, l, i + 1));
          return p;
        };
        const Blk W = lsum(*this, Rt, false, ir, coef, NR, TwoSR, IR, NR + 1, SRd, IRd, dimR, dRd);
        if (!W.valid) continue;
        const int kp = kap(NL, TwoSL, IL, N1 + 1, N2, TJd, NR + 1, SRd, IRd);
        if (kp != -1) emit(1.0, kNo, false, kp, W, true);
      }
    }
  }
  if (N1 > 0 && N2 > 0) {  // 4G4A..4G4D
    for (int SRd = TwoSR - 1; SRd <= TwoSR + 1; SRd += 2) {
      const int dRd = dR(NR - 1, SRd, IRd);
      if (dRd <= 0) continue;
      const int sum = ((N1 == 1) ? 0 : 1) + ((N2 == 1) ? 1 : 0);
      const int start = ((TwoSL != SRd) || (sum < 2)) ? sum : 0;
      for (int TJd = start; TJd <= sum; TJd += 2) {
        if (abs(TwoSL - SRd) > TJd) continue;
        double a = 0.0, a2 = 0.0;
        if (N1 == 1 && N2 == 1) a = ph(TwoSL + TwoSR + 2) * sqrt((TwoJ + 1) * (TwoSR + 1.0)) * wigner6j(TwoJ, 1, 1, SRd, TwoSR, TwoSL);
        if (N1 == 2 && N2 == 1) {
          a = ph(TwoSL + TwoSR + TJd + 3) * sqrt((TJd + 1) * (TwoSR + 1.0)) * wigner6j(TJd, 1, 1, TwoSR, SRd, TwoSL);
          a2 = (TJd == 0) ? sqrt(2.0 * (TwoSR + 1.0) / (SRd + 1.0)) : 0.0;
        }
        if (N1 == 1 && N2 == 2) a = -sqrt((TwoSR + 1.0) / (SRd + 1.0));
        if (N1 == 2 && N2 == 2) a = ph(SRd + 1 - TwoSR);
        auto coef = [&](int l) {
          double p = 0.0;
          if (N1 == 1 && N2 == 1) p = a * (V(i, i + 1, i + 1, l) + ((TwoJ == 0) ? 1 : -1) * V(i, i + 1, l, i + 1));
          if (N1 == 2 && N2 == 1) {
            p = a * V(i, i + 1, l, i + 1);
            if (TJd == 0) p += a2 * V(i, i + 1, i + 1, l);
          }
          if (N2 == 2) p = a * (V(i, i + 1, i + 1, l) - 2 * V(i, i + 1, l, i + 1));
          return p;
        };
        const Blk W = lsum(*this, Rt, false, ir, coef, NR - 1, SRd, IRd, NR, TwoSR, IR, dRd, dimR);
        if (!W.valid) continue;
        const int kp = kap(NL, TwoSL, IL, N1 - 1, N2, TJd, NR - 1, SRd, IRd);
        if (kp != -1) emit(1.0, kNo, false, kp, W, false);
      }
    }
  }
}

// CheMPS2/HeffDiagrams4.cpp:3563-4013 (the 4E pattern with the roles of the two local
// orbitals exchanged: integrals carry theindex + 1).
void HeffEmitter::d4H() {
  const int i = theindex;
  const int S1 = (N1 == 1) ? 1 : 0;
  const int nirr = bk.getNumberOfIrreps();
  auto body = [&](int nld, int SLd, int nrd, int SRd, int kn1, int kn2, int ktj, bool ldn, bool rdn, auto coef) {
    for (int Irrep = 0; Irrep < nirr; Irrep++) {
      const int ILd = irrep_prod(IL, Irrep), IRd = irrep_prod(IR, Irrep);
      const int dLd = dL(nld, SLd, ILd), dRd = dR(nrd, SRd, IRd);
      if (dLd <= 0 || dRd <= 0) continue;
      if (!any_irrep(*this, 0, i, Irrep) || !any_irrep(*this, i + 2, L, Irrep)) continue;
      const int kp = kap(nld, SLd, ILd, kn1, kn2, ktj, nrd, SRd, IRd);
      for (int la = 0; la < i; la++) {
        if (irr(la) != Irrep) continue;
        thread_local std::vector<std::pair<double, Blk>> parts;  // reused: no allocation per block
        parts.clear();
        for (int lb = i + 2; lb < L; lb++) {
          if (irr(lb) != Irrep) continue;
          const Blk rb = rdn ? Rt->Lop(lb).blk(nrd, SRd, IRd, NR, TwoSR, IR) : Rt->Lop(lb).blk(NR, TwoSR, IR, nrd, SRd, IRd);
          parts.push_back({coef(la, lb), need(rb)});
        }
        const Blk W = rdn ? combine(parts, dRd, dimR) : combine(parts, dimR, dRd);
        const Blk lb2 = ldn ? Lt->Lop(la).blk(nld, SLd, ILd, NL, TwoSL, IL) : Lt->Lop(la).blk(NL, TwoSL, IL, nld, SLd, ILd);
        if (kp != -1) emit(1.0, need(lb2), ldn, kp, W, !rdn);
      }
    }
  };
  if (N2 == 2)  // 4H1
    for (int SRd = TwoSR - 1; SRd <= TwoSR + 1; SRd += 2)
      for (int SLd = TwoSL - 1; SLd <= TwoSL + 1; SLd += 2) {
        if (abs(SLd - SRd) > TwoJ || SLd < 0 || SRd < 0) continue;
        const double f = ph(SLd + SRd - S1) * sqrt((SLd + 1) * (TwoSR + 1.0)) * wigner6j(TwoSL, TwoSR, S1, SRd, SLd, 1);
        body(NL + 1, SLd, NR - 1, SRd, N1, 0, S1, false, true, [&](int la, int lb) { return f * V(la, lb, i + 1, i + 1); });
      }
  if (N2 == 0)  // 4H2
    for (int SRd = TwoSR - 1; SRd <= TwoSR + 1; SRd += 2)
      for (int SLd = TwoSL - 1; SLd <= TwoSL + 1; SLd += 2) {
        if (abs(SLd - SRd) > TwoJ || SLd < 0 || SRd < 0) continue;
        const double f = ph(TwoSL + TwoSR - S1) * sqrt((TwoSL + 1) * (SRd + 1.0)) * wigner6j(SLd, SRd, S1, TwoSR, TwoSL, 1);
        body(NL - 1, SLd, NR + 1, SRd, N1, 2, S1, true, false, [&](int la, int lb) { return f * V(la, lb, i + 1, i + 1); });
      }
  if (N2 == 1)  // 4H3A
    for (int SRd = TwoSR - 1; SRd <= TwoSR + 1; SRd += 2)
      for (int SLd = TwoSL - 1; SLd <= TwoSL + 1; SLd += 2) {
        const int start = ((SLd != SRd) || (S1 == 0)) ? S1 + 1 : 0;
        for (int TJd = start; TJd <= S1 + 1; TJd += 2) {
          if (abs(SLd - SRd) > TJd || SLd < 0 || SRd < 0) continue;
          const double f1 = ph(TwoSL + TwoSR + SLd + SRd + TJd + 1 - S1) * sqrt((TwoJ + 1) * (TJd + 1) * (TwoSL + 1) * (TwoSR + 1.0)) *
                            wigner6j(TwoSL, SRd, S1, TJd, 1, SLd) * wigner6j(TwoJ, 1, S1, SRd, TwoSL, TwoSR);
          double f2 = 0.0;
          if (TwoJ == TJd) f2 = ph(TwoSL + SRd + TwoJ + 3 + 2 * S1) * sqrt((TwoSL + 1) * (TwoSR + 1.0)) * wigner6j(SLd, SRd, TwoJ, TwoSR, TwoSL, 1);
          body(NL - 1, SLd, NR - 1, SRd, N1, 1, TJd, true, true, [&](int la, int lb) {
            double p = f1 * V(la, i + 1, i + 1, lb);
            if (TwoJ == TJd) p += f2 * V(la, i + 1, lb, i + 1);
            return p;
          });
        }
      }
  if (N2 == 2)  // 4H3B
    for (int SRd = TwoSR - 1; SRd <= TwoSR + 1; SRd += 2)
      for (int SLd = TwoSL - 1; SLd <= TwoSL + 1; SLd += 2) {
        if (abs(SLd - SRd) > TwoJ || SLd < 0 || SRd < 0) continue;
        const double f = ph(TwoSL + SRd + 3 - S1) * sqrt((TwoSL + 1) * (TwoSR + 1.0)) * wigner6j(SLd, SRd, S1, TwoSR, TwoSL, 1);
        body(NL - 1, SLd, NR - 1, SRd, N1, 2, S1, true, true,
             [&](int la, int lb) { return f * (V(la, i + 1, i + 1, lb) - 2 * V(la, i + 1, lb, i + 1)); });
      }
  if (N2 == 1)  // 4H4A
    for (int SRd = TwoSR - 1; SRd <= TwoSR + 1; SRd += 2)
      for (int SLd = TwoSL - 1; SLd <= TwoSL + 1; SLd += 2) {
        const int start = ((SLd != SRd) || (S1 == 0)) ? S1 + 1 : 0;
        for (int TJd = start; TJd <= S1 + 1; TJd += 2) {
          if (abs(SLd - SRd) > TJd || SLd < 0 || SRd < 0) continue;
          const double f1 = ph(TwoSL + TwoSR + SLd + SRd + TwoJ + 1 - S1) * sqrt((TwoJ + 1) * (TJd + 1) * (SLd + 1) * (SRd + 1.0)) *
                            wigner6j(SLd, TwoSR, S1, TwoJ, 1, TwoSL) * wigner6j(TJd, 1, S1, TwoSR, SLd, SRd);
          double f2 = 0.0;
          if (TwoJ == TJd) f2 = ph(SLd + TwoSR + TwoJ + 3 + 2 * S1) * sqrt((SLd + 1) * (SRd + 1.0)) * wigner6j(TwoSL, TwoSR, TwoJ, SRd, SLd, 1);
          body(NL + 1, SLd, NR + 1, SRd, N1, 1, TJd, false, false, [&](int la, int lb) {
            double p = f1 * V(la, i + 1, i + 1, lb);
            if (TwoJ == TJd) p += f2 * V(la, i + 1, lb, i + 1);
            return p;
          });
        }
      }
  if (N2 == 2)  // 4H4B
    for (int SRd = TwoSR - 1; SRd <= TwoSR + 1; SRd += 2)
      for (int SLd = TwoSL - 1; SLd <= TwoSL + 1; SLd += 2) {
        if (abs(SLd - SRd) > TwoJ || SLd < 0 || SRd < 0) continue;
        const double f = ph(SLd + TwoSR + 3 - S1) * sqrt((SLd + 1) * (SRd + 1.0)) * wigner6j(TwoSL, TwoSR, S1, SRd, SLd, 1);
        body(NL + 1, SLd, NR + 1, SRd, N1, 2, S1, false, false,
             [&](int la, int lb) { return f * (V(la, i + 1, i + 1, lb) - 2 * V(la, i + 1, lb, i + 1)); });
      }
}

// CheMPS2/HeffDiagrams4.cpp:4015-4275
void HeffEmitter::d4I() {
  const int i = theindex;
  const int ILd = irrep_prod(IL, irr(i));
  const int ir = irr(i);
  if (N1 > 0 && N2 == 0) {  // 4I1A and 4I1B
    const int TJd = (N1 == 2) ? 1 : 0;
    for (int SLd = TwoSL - 1; SLd <= TwoSL + 1; SLd += 2) {
      if (abs(SLd - TwoSR) > TJd) continue;
      const int dLd = dL(NL - 1, SLd, ILd);
      if (dLd <= 0) continue;
      const Blk W = lsum(*this, Lt, true, ir, [&](int l) { return V(l, i, i + 1, i + 1); }, NL - 1, SLd, ILd, NL, TwoSL, IL,
                         dLd, dimL);
      if (!W.valid) continue;
      double f = -1.0;
      if (N1 == 1) f = ph(TwoSR + 1 - TwoSL) * sqrt((TwoSL + 1.0) / (TwoSR + 1.0));
      const int kp = kap(NL - 1, SLd, ILd, N1 - 1, 2, TJd, NR, TwoSR, IR);
      if (kp != -1) emit(f, W, true, kp, kNo, false);
    }
  }
  if (N1 < 2 && N2 == 2) {  // 4I2A and 4I2B
    const int TJd = (N1 == 0) ? 1 : 0;
    for (int SLd = TwoSL - 1; SLd <= TwoSL + 1; SLd += 2) {
      if (abs(SLd - TwoSR) > TJd) continue;
      const int dLd = dL(NL + 1, SLd, ILd);
      if (dLd <= 0) continue;
      const Blk W = lsum(*this, Lt, true, ir, [&](int l) { return V(l, i, i + 1, i + 1); }, NL, TwoSL, IL, NL + 1, SLd, ILd,
                         dimL, dLd);
      if (!W.valid) continue;
      double f = -1.0;
      if (N1 == 0) f = ph(TwoSR + 1 - SLd) * sqrt((SLd + 1.0) / (TwoSR + 1.0));
      const int kp = kap(NL + 1, SLd, ILd, N1 + 1, 0, TJd, NR, TwoSR, IR);
      if (kp != -1) emit(f, W, false, kp, kNo, false);
    }
  }
  if (N1 < 2 && N2 > 0) {  // 4I3A..4I3D
    for (int SLd = TwoSL - 1; SLd <= TwoSL + 1; SLd += 2) {
      const int dLd = dL(NL - 1, SLd, ILd);
      if (dLd <= 0) continue;
      const int sum = ((N1 == 0) ? 1 : 0) + ((N2 == 1) ? 1 : 0);
      const int start = ((TwoSR != SLd) || (sum < 2)) ? sum : 0;
      for (int TJd = start; TJd <= sum; TJd += 2) {
        if (abs(SLd - TwoSR) > TJd) continue;
        double pf = 0.0;
        if (N1 == 0 && N2 == 1) pf = ph(SLd + TwoSR + 2) * sqrt((TwoSL + 1.0) * (TJd + 1)) * wigner6j(TJd, 1, 1, TwoSL, SLd, TwoSR);
        if (N1 == 1 && N2 == 1) pf = ph(SLd + TwoSR + 3) * sqrt((TwoJ + 1) * (TwoSL + 1.0)) * wigner6j(TwoJ, 1, 1, SLd, TwoSL, TwoSR);
        if (N1 == 0 && N2 == 2) pf = 1.0;
        if (N1 == 1 && N2 == 2) pf = ph(TwoSR + 1 - TwoSL) * sqrt((TwoSL + 1.0) / (TwoSR + 1.0));
        auto coef = [&](int l) {
          double a = 0.0;
          if (N1 == 0 && N2 == 1) a = pf * (V(l, i + 1, i, i + 1) + ((TJd == 0) ? 1 : -1) * V(l, i + 1, i + 1, i));
          if (N1 == 1 && N2 == 1) {
            a = pf * V(l, i + 1, i, i + 1);
            if (TwoJ == 0) a += sqrt(2.0) * V(l, i + 1, i + 1, i);
          }
          if (N2 == 2) a = pf * (2 * V(l, i + 1, i, i + 1) - V(l, i + 1, i + 1, i));
          return a;
        };
        const Blk W = lsum(*this, Lt, true, ir, coef, NL - 1, SLd, ILd, NL, TwoSL, IL, dLd, dimL);
        if (!W.valid) continue;
        const int kp = kap(NL - 1, SLd, ILd, N1 + 1, N2, TJd, NR, TwoSR, IR);
        if (kp != -1) emit(1.0, W, true, kp, kNo, false);
      }
    }
  }
  if (N1 > 0 && N2 > 0) {  // 4I4A..4I4D
    for (int SLd = TwoSL - 1; SLd <= TwoSL + 1; SLd += 2) {
      const int dLd = dL(NL + 1, SLd, ILd);
      if (dLd <= 0) continue;
      const int sum = ((N1 == 2) ? 1 : 0) + ((N2 == 1) ? 1 : 0);
      const int start = ((SLd != TwoSR) || (sum < 2)) ? sum : 0;
      for (int TJd = start; TJd <= sum; TJd += 2) {
        if (abs(SLd - TwoSR) > TJd) continue;
        double pf = 0.0;
        if (N1 == 1 && N2 == 1) pf = ph(TwoSL + TwoSR + 2) * sqrt((SLd + 1.0) * (TwoJ + 1)) * wigner6j(TwoJ, 1, 1, SLd, TwoSL, TwoSR);
        if (N1 == 2 && N2 == 1) pf = ph(TwoSL + TwoSR + 3) * sqrt((TJd + 1) * (SLd + 1.0)) * wigner6j(TJd, 1, 1, TwoSL, SLd, TwoSR);
        if (N1 == 1 && N2 == 2) pf = 1.0;
        if (N1 == 2 && N2 == 2) pf = ph(TwoSR + 1 - SLd) * sqrt((SLd + 1.0) / (TwoSR + 1.0));
        auto coef = [&](int l) {
          double a = 0.0;
          if (N1 == 1 && N2 == 1) a = pf * (V(l, i + 1, i, i + 1) + ((TwoJ == 0) ? 1 : -1) * V(l, i + 1, i + 1, i));
          if (N1 == 2 && N2 == 1) {
            a = pf * V(l, i + 1, i, i + 1);
            if (TJd == 0) a += sqrt(2.0) * V(l, i + 1, i + 1, i);
          }
          if (N2 == 2) a = pf * (2 * V(l, i + 1, i, i + 1) - V(l, i + 1, i + 1, i));
          return a;
        };
        const Blk W = lsum(*this, Lt, true, ir, coef, NL, TwoSL, IL, NL + 1, SLd, ILd, dimL, dLd);
        if (!W.valid) continue;
        const int kp = kap(NL + 1, SLd, ILd, N1 - 1, N2, TJd, NR, TwoSR, IR);
        if (kp != -1) emit(1.0, W, false, kp, kNo, false);
      }
    }
  }
}

}  // namespace c2g
