// Heff diagrams 4K and 4L (CheMPS2/HeffDiagrams4.cpp:4847-6518): the creator L_l of the
// left block (l left of the two sites) times a complementary pair operator of the right
// block on the orbital pair (l, theindex + 1) for 4K or (l, theindex) for 4L.
#include "heff_impl.hpp"

namespace c2g {

using std::abs;
using std::sqrt;

namespace {

inline int ph(int x) { return heff_phase(x); }
int jstart(int sl, int sr, int two_s) { return ((sl != sr) || (two_s == 0)) ? two_s + 1 : 0; }

// Y += f * op(left creator block) * X[kp] * op(right complementary block); same
// conventions as the 4B/4C helper: "down -> up" blocks are transposed on the left and
// used as stored on the right.
void lr(HeffEmitter& h, const OpT& lo, int nld, int sld, int ild, bool ldu, const OpT& ro, int nrd, int srd,
        int ird, bool rdu, double f, int kp) {
  if (kp == -1) return;
  const Blk lb = ldu ? lo.blk(nld, sld, ild, h.NL, h.TwoSL, h.IL) : lo.blk(h.NL, h.TwoSL, h.IL, nld, sld, ild);
  const Blk rb = rdu ? ro.blk(nrd, srd, ird, h.NR, h.TwoSR, h.IR) : ro.blk(h.NR, h.TwoSR, h.IR, nrd, srd, ird);
  h.emit(f, HeffEmitter::need(lb), ldu, kp, HeffEmitter::need(rb), !rdu);
}

// Shared body: for every left orbital l, the complementary right operator R(l) with the
// down sector (nrd, srd) and the left creator with down sector (nld, sld).
template <class RofL>
void over_l(HeffEmitter& h, RofL R, int nld, int sld, bool ldu, int nrd, int srd, bool rdu, int kn1, int kn2,
            int ktj, double f) {
  for (int l = 0; l < h.theindex; l++) {
    const OpT& ro = R(l);
    const int ILd = irrep_prod(h.IL, h.irr(l)), IRd = irrep_prod(h.IR, ro.irrep());
    if (h.dL(nld, sld, ILd) <= 0 || h.dR(nrd, srd, IRd) <= 0) continue;
    lr(h, h.Lt->Lop(l), nld, sld, ILd, ldu, ro, nrd, srd, IRd, rdu, f,
       h.kap(nld, sld, ILd, kn1, kn2, ktj, nrd, srd, IRd));
  }
}

}  // namespace

// CheMPS2/HeffDiagrams4.cpp:4847-5049
void HeffEmitter::d4K1and4K2spin0() {
  const int S1 = (N1 == 1) ? 1 : 0;
  auto R = [&](int l) -> const OpT& { return Rt->A[theindex + 1 - l][0]; };
  if (N2 == 1)
    for (int SLd = TwoSL - 1; SLd <= TwoSL + 1; SLd += 2) {
      if (abs(SLd - TwoSR) > S1 || SLd < 0) continue;
      const double f = ph(SLd + TwoSR + TwoJ + 1 + 2 * S1) * sqrt(0.5 * (TwoSL + 1) * (TwoJ + 1)) * wigner6j(S1, TwoJ, 1, TwoSL, SLd, TwoSR);
      over_l(*this, R, NL - 1, SLd, true, NR - 2, TwoSR, true, N1, 0, S1, f);
    }
  if (N2 == 2)
    for (int SLd = TwoSL - 1; SLd <= TwoSL + 1; SLd += 2)
      for (int TJd = jstart(SLd, TwoSR, S1); TJd <= S1 + 1; TJd += 2) {
        if (abs(SLd - TwoSR) > TJd || SLd < 0) continue;
        const double f = ph(SLd + TwoSR + TJd + 2 + 2 * S1) * sqrt(0.5 * (TwoSL + 1) * (TJd + 1)) * wigner6j(TJd, S1, 1, TwoSL, SLd, TwoSR);
        over_l(*this, R, NL - 1, SLd, true, NR - 2, TwoSR, true, N1, 1, TJd, f);
      }
  if (N2 == 0)
    for (int SLd = TwoSL - 1; SLd <= TwoSL + 1; SLd += 2)
      for (int TJd = jstart(SLd, TwoSR, S1); TJd <= S1 + 1; TJd += 2) {
        if (abs(SLd - TwoSR) > TJd || SLd < 0) continue;
        const double f = ph(TwoSL + TwoSR + TJd + 1 + 2 * S1) * sqrt(0.5 * (SLd + 1) * (TJd + 1)) * wigner6j(TJd, S1, 1, TwoSL, SLd, TwoSR);
        over_l(*this, R, NL + 1, SLd, false, NR + 2, TwoSR, false, N1, 1, TJd, f);
      }
  if (N2 == 1)
    for (int SLd = TwoSL - 1; SLd <= TwoSL + 1; SLd += 2) {
      if (abs(SLd - TwoSR) > S1 || SLd < 0) continue;
      const double f = ph(TwoSL + TwoSR + TwoJ + 2 + 2 * S1) * sqrt(0.5 * (SLd + 1) * (TwoJ + 1)) * wigner6j(TwoJ, S1, 1, SLd, TwoSL, TwoSR);
      over_l(*this, R, NL + 1, SLd, false, NR + 2, TwoSR, false, N1, 2, S1, f);
    }
}

// CheMPS2/HeffDiagrams4.cpp:5051-5257
void HeffEmitter::d4L1and4L2spin0() {
  const int S2 = (N2 == 1) ? 1 : 0;
  auto R = [&](int l) -> const OpT& { return Rt->A[theindex - l][1]; };
  if (N1 == 1)
    for (int SLd = TwoSL - 1; SLd <= TwoSL + 1; SLd += 2) {
      if (abs(SLd - TwoSR) > S2 || SLd < 0) continue;
      const double f = ph(SLd + TwoSR + 2 + S2) * sqrt(0.5 * (TwoSL + 1) * (TwoJ + 1)) * wigner6j(S2, TwoJ, 1, TwoSL, SLd, TwoSR);
      over_l(*this, R, NL - 1, SLd, true, NR - 2, TwoSR, true, 0, N2, S2, f);
    }
  if (N1 == 2)
    for (int SLd = TwoSL - 1; SLd <= TwoSL + 1; SLd += 2)
      for (int TJd = jstart(SLd, TwoSR, S2); TJd <= S2 + 1; TJd += 2) {
        if (abs(SLd - TwoSR) > TJd || SLd < 0) continue;
        const double f = ph(SLd + TwoSR + 3 + S2) * sqrt(0.5 * (TwoSL + 1) * (TJd + 1)) * wigner6j(TJd, S2, 1, TwoSL, SLd, TwoSR);
        over_l(*this, R, NL - 1, SLd, true, NR - 2, TwoSR, true, 1, N2, TJd, f);
      }
  if (N1 == 0)
    for (int SLd = TwoSL - 1; SLd <= TwoSL + 1; SLd += 2)
      for (int TJd = jstart(SLd, TwoSR, S2); TJd <= S2 + 1; TJd += 2) {
        if (abs(SLd - TwoSR) > TJd || SLd < 0) continue;
        const double f = ph(TwoSL + TwoSR + 2 + S2) * sqrt(0.5 * (SLd + 1) * (TJd + 1)) * wigner6j(TJd, S2, 1, TwoSL, SLd, TwoSR);
        over_l(*this, R, NL + 1, SLd, false, NR + 2, TwoSR, false, 1, N2, TJd, f);
      }
  if (N1 == 1)
    for (int SLd = TwoSL - 1; SLd <= TwoSL + 1; SLd += 2) {
      if (abs(SLd - TwoSR) > S2 || SLd < 0) continue;
      const double f = ph(TwoSL + TwoSR + 3 + S2) * sqrt(0.5 * (SLd + 1) * (TwoJ + 1)) * wigner6j(TwoJ, S2, 1, SLd, TwoSL, TwoSR);
      over_l(*this, R, NL + 1, SLd, false, NR + 2, TwoSR, false, 2, N2, S2, f);
    }
}

// CheMPS2/HeffDiagrams4.cpp:5259-5472
void HeffEmitter::d4K1and4K2spin1() {
  const int S1 = (N1 == 1) ? 1 : 0;
  auto R = [&](int l) -> const OpT& { return Rt->B[theindex + 1 - l][0]; };
  if (N2 == 1)
    for (int SLd = TwoSL - 1; SLd <= TwoSL + 1; SLd += 2)
      for (int SRd = TwoSR - 2; SRd <= TwoSR + 2; SRd += 2) {
        if (abs(SLd - SRd) > S1 || SLd < 0 || SRd < 0) continue;
        const double f = ((S1 == 1) ? -1 : 1) * sqrt(3.0 * (TwoSR + 1) * (TwoSL + 1) * (TwoJ + 1)) *
                         wigner9j(2, TwoSR, SRd, 1, TwoSL, SLd, 1, TwoJ, S1);
        over_l(*this, R, NL - 1, SLd, true, NR - 2, SRd, true, N1, 0, S1, f);
      }
  if (N2 == 2)
    for (int SLd = TwoSL - 1; SLd <= TwoSL + 1; SLd += 2)
      for (int SRd = TwoSR - 2; SRd <= TwoSR + 2; SRd += 2)
        for (int TJd = jstart(SLd, SRd, S1); TJd <= S1 + 1; TJd += 2) {
          if (abs(SLd - SRd) > TJd || SLd < 0 || SRd < 0) continue;
          const double f = ph(TwoSR - SRd + SLd - TwoSL + 3 + 2 * S1) * sqrt(3.0 * (TwoSR + 1) * (TwoSL + 1) * (TJd + 1)) *
                           wigner9j(2, SRd, TwoSR, 1, SLd, TwoSL, 1, TJd, S1);
          over_l(*this, R, NL - 1, SLd, true, NR - 2, SRd, true, N1, 1, TJd, f);
        }
  if (N2 == 0)
    for (int SLd = TwoSL - 1; SLd <= TwoSL + 1; SLd += 2)
      for (int SRd = TwoSR - 2; SRd <= TwoSR + 2; SRd += 2)
        for (int TJd = jstart(SLd, SRd, S1); TJd <= S1 + 1; TJd += 2) {
          if (abs(SLd - SRd) > TJd || SLd < 0 || SRd < 0) continue;
          const double f = ((S1 == 1) ? -1 : 1) * sqrt(3.0 * (SRd + 1) * (SLd + 1) * (TJd + 1)) *
                           wigner9j(2, SRd, TwoSR, 1, SLd, TwoSL, 1, TJd, S1);
          over_l(*this, R, NL + 1, SLd, false, NR + 2, SRd, false, N1, 1, TJd, f);
        }
  if (N2 == 1)
    for (int SLd = TwoSL - 1; SLd <= TwoSL + 1; SLd += 2)
      for (int SRd = TwoSR - 2; SRd <= TwoSR + 2; SRd += 2) {
        if (abs(SLd - SRd) > S1 || SLd < 0 || SRd < 0) continue;
        const double f = ph(SRd - TwoSR + TwoSL - SLd + 3 + 2 * S1) * sqrt(3.0 * (SRd + 1) * (SLd + 1) * (TwoJ + 1)) *
                         wigner9j(2, TwoSR, SRd, 1, TwoSL, SLd, 1, TwoJ, S1);
        over_l(*this, R, NL + 1, SLd, false, NR + 2, SRd, false, N1, 2, S1, f);
      }
}

// CheMPS2/HeffDiagrams4.cpp:5474-5684
void HeffEmitter::d4L1and4L2spin1() {
  const int S2 = (N2 == 1) ? 1 : 0;
  auto R = [&](int l) -> const OpT& { return Rt->B[theindex - l][1]; };
  if (N1 == 1)
    for (int SLd = TwoSL - 1; SLd <= TwoSL + 1; SLd += 2)
      for (int SRd = TwoSR - 2; SRd <= TwoSR + 2; SRd += 2) {
        if (abs(SLd - SRd) > S2 || SLd < 0 || SRd < 0) continue;
        const double f = ph(1 + S2 - TwoJ) * sqrt(3.0 * (TwoSR + 1) * (TwoSL + 1) * (TwoJ + 1)) *
                         wigner9j(2, TwoSR, SRd, 1, TwoSL, SLd, 1, TwoJ, S2);
        over_l(*this, R, NL - 1, SLd, true, NR - 2, SRd, true, 0, N2, S2, f);
      }
  if (N1 == 2)
    for (int SLd = TwoSL - 1; SLd <= TwoSL + 1; SLd += 2)
      for (int SRd = TwoSR - 2; SRd <= TwoSR + 2; SRd += 2)
        for (int TJd = jstart(SLd, SRd, S2); TJd <= S2 + 1; TJd += 2) {
          if (abs(SLd - SRd) > TJd || SLd < 0 || SRd < 0) continue;
          const double f = ph(TwoSR - SRd + SLd - TwoSL + S2 - TJd) * sqrt(3.0 * (TwoSR + 1) * (TwoSL + 1) * (TJd + 1)) *
                           wigner9j(2, SRd, TwoSR, 1, SLd, TwoSL, 1, TJd, S2);
          over_l(*this, R, NL - 1, SLd, true, NR - 2, SRd, true, 1, N2, TJd, f);
        }
  if (N1 == 0)
    for (int SLd = TwoSL - 1; SLd <= TwoSL + 1; SLd += 2)
      for (int SRd = TwoSR - 2; SRd <= TwoSR + 2; SRd += 2)
        for (int TJd = jstart(SLd, SRd, S2); TJd <= S2 + 1; TJd += 2) {
          if (abs(SLd - SRd) > TJd || SLd < 0 || SRd < 0) continue;
          const double f = ph(1 + S2 - TJd) * sqrt(3.0 * (SRd + 1) * (SLd + 1) * (TJd + 1)) *
                           wigner9j(2, SRd, TwoSR, 1, SLd, TwoSL, 1, TJd, S2);
          over_l(*this, R, NL + 1, SLd, false, NR + 2, SRd, false, 1, N2, TJd, f);
        }
  if (N1 == 1)
    for (int SLd = TwoSL - 1; SLd <= TwoSL + 1; SLd += 2)
      for (int SRd = TwoSR - 2; SRd <= TwoSR + 2; SRd += 2) {
        if (abs(SLd - SRd) > S2 || SLd < 0 || SRd < 0) continue;
        const double f = ph(SRd - TwoSR + TwoSL - SLd + S2 - TwoJ) * sqrt(3.0 * (SRd + 1) * (SLd + 1) * (TwoJ + 1)) *
                         wigner9j(2, TwoSR, SRd, 1, TwoSL, SLd, 1, TwoJ, S2);
        over_l(*this, R, NL + 1, SLd, false, NR + 2, SRd, false, 2, N2, S2, f);
      }
}

// CheMPS2/HeffDiagrams4.cpp:5686-5888
void HeffEmitter::d4K3and4K4spin0() {
  const int S1 = (N1 == 1) ? 1 : 0;
  auto R = [&](int l) -> const OpT& { return Rt->C[theindex + 1 - l][0]; };
  if (N2 == 1)
    for (int SLd = TwoSL - 1; SLd <= TwoSL + 1; SLd += 2) {
      if (abs(SLd - TwoSR) > S1 || SLd < 0) continue;
      const double f = ph(TwoSL + TwoSR + TwoJ + 2 * S1) * sqrt(0.5 * (SLd + 1) * (TwoJ + 1)) * wigner6j(TwoJ, S1, 1, SLd, TwoSL, TwoSR);
      over_l(*this, R, NL + 1, SLd, false, NR, TwoSR, false, N1, 0, S1, f);
    }
  if (N2 == 2)
    for (int SLd = TwoSL - 1; SLd <= TwoSL + 1; SLd += 2)
      for (int TJd = jstart(SLd, TwoSR, S1); TJd <= S1 + 1; TJd += 2) {
        if (abs(SLd - TwoSR) > TJd || SLd < 0) continue;
        const double f = ph(TwoSL + TwoSR + TJd + 1 + 2 * S1) * sqrt(0.5 * (SLd + 1) * (TJd + 1)) * wigner6j(TJd, S1, 1, TwoSL, SLd, TwoSR);
        over_l(*this, R, NL + 1, SLd, false, NR, TwoSR, false, N1, 1, TJd, f);
      }
  if (N2 == 0)
    for (int SLd = TwoSL - 1; SLd <= TwoSL + 1; SLd += 2)
      for (int TJd = jstart(SLd, TwoSR, S1); TJd <= S1 + 1; TJd += 2) {
        if (abs(SLd - TwoSR) > TJd || SLd < 0) continue;
        const double f = ph(SLd + TwoSR + TJd + 2 * S1) * sqrt(0.5 * (TwoSL + 1) * (TJd + 1)) * wigner6j(TJd, S1, 1, TwoSL, SLd, TwoSR);
        over_l(*this, R, NL - 1, SLd, true, NR, TwoSR, true, N1, 1, TJd, f);
      }
  if (N2 == 1)
    for (int SLd = TwoSL - 1; SLd <= TwoSL + 1; SLd += 2) {
      if (abs(SLd - TwoSR) > S1 || SLd < 0) continue;
      const double f = ph(SLd + TwoSR + 1 + TwoJ + 2 * S1) * sqrt(0.5 * (TwoSL + 1) * (TwoJ + 1)) * wigner6j(TwoJ, S1, 1, SLd, TwoSL, TwoSR);
      over_l(*this, R, NL - 1, SLd, true, NR, TwoSR, true, N1, 2, S1, f);
    }
}

// CheMPS2/HeffDiagrams4.cpp:5890-6092
void HeffEmitter::d4L3and4L4spin0() {
  const int S2 = (N2 == 1) ? 1 : 0;
  auto R = [&](int l) -> const OpT& { return Rt->C[theindex - l][1]; };
  if (N1 == 1)
    for (int SLd = TwoSL - 1; SLd <= TwoSL + 1; SLd += 2) {
      if (abs(SLd - TwoSR) > S2 || SLd < 0) continue;
      const double f = ph(TwoSL + TwoSR + 1 + S2) * sqrt(0.5 * (SLd + 1) * (TwoJ + 1)) * wigner6j(TwoJ, S2, 1, SLd, TwoSL, TwoSR);
      over_l(*this, R, NL + 1, SLd, false, NR, TwoSR, false, 0, N2, S2, f);
    }
  if (N1 == 2)
    for (int SLd = TwoSL - 1; SLd <= TwoSL + 1; SLd += 2)
      for (int TJd = jstart(SLd, TwoSR, S2); TJd <= S2 + 1; TJd += 2) {
        if (abs(SLd - TwoSR) > TJd || SLd < 0) continue;
        const double f = ph(TwoSL + TwoSR + 2 + S2) * sqrt(0.5 * (SLd + 1) * (TJd + 1)) * wigner6j(TJd, S2, 1, TwoSL, SLd, TwoSR);
        over_l(*this, R, NL + 1, SLd, false, NR, TwoSR, false, 1, N2, TJd, f);
      }
  if (N1 == 0)
    for (int SLd = TwoSL - 1; SLd <= TwoSL + 1; SLd += 2)
      for (int TJd = jstart(SLd, TwoSR, S2); TJd <= S2 + 1; TJd += 2) {
        if (abs(SLd - TwoSR) > TJd || SLd < 0) continue;
        const double f = ph(SLd + TwoSR + 1 + S2) * sqrt(0.5 * (TwoSL + 1) * (TJd + 1)) * wigner6j(TJd, S2, 1, TwoSL, SLd, TwoSR);
        over_l(*this, R, NL - 1, SLd, true, NR, TwoSR, true, 1, N2, TJd, f);
      }
  if (N1 == 1)
    for (int SLd = TwoSL - 1; SLd <= TwoSL + 1; SLd += 2) {
      if (abs(SLd - TwoSR) > S2 || SLd < 0) continue;
      const double f = ph(SLd + TwoSR + 2 + S2) * sqrt(0.5 * (TwoSL + 1) * (TwoJ + 1)) * wigner6j(TwoJ, S2, 1, SLd, TwoSL, TwoSR);
      over_l(*this, R, NL - 1, SLd, true, NR, TwoSR, true, 2, N2, S2, f);
    }
}

// CheMPS2/HeffDiagrams4.cpp:6094-6304
void HeffEmitter::d4K3and4K4spin1() {
  const int S1 = (N1 == 1) ? 1 : 0;
  auto R = [&](int l) -> const OpT& { return Rt->D[theindex + 1 - l][0]; };
  if (N2 == 1)
    for (int SLd = TwoSL - 1; SLd <= TwoSL + 1; SLd += 2)
      for (int SRd = TwoSR - 2; SRd <= TwoSR + 2; SRd += 2) {
        if (abs(SLd - SRd) > S1 || SLd < 0 || SRd < 0) continue;
        const double f = ph(TwoSL - SLd + 1 + 2 * S1) * sqrt(3.0 * (TwoSR + 1) * (SLd + 1) * (TwoJ + 1)) *
                         wigner9j(2, TwoSR, SRd, 1, TwoSL, SLd, 1, TwoJ, S1);
        over_l(*this, R, NL + 1, SLd, false, NR, SRd, false, N1, 0, S1, f);
      }
  if (N2 == 2)
    for (int SLd = TwoSL - 1; SLd <= TwoSL + 1; SLd += 2)
      for (int SRd = TwoSR - 2; SRd <= TwoSR + 2; SRd += 2)
        for (int TJd = jstart(SLd, SRd, S1); TJd <= S1 + 1; TJd += 2) {
          if (abs(SLd - SRd) > TJd || SLd < 0 || SRd < 0) continue;
          const double f = ph(TwoSR - SRd + 2 * S1) * sqrt(3.0 * (TwoSR + 1) * (SLd + 1) * (TJd + 1)) *
                           wigner9j(2, SRd, TwoSR, 1, SLd, TwoSL, 1, TJd, S1);
          over_l(*this, R, NL + 1, SLd, false, NR, SRd, false, N1, 1, TJd, f);
        }
  if (N2 == 0)
    for (int SLd = TwoSL - 1; SLd <= TwoSL + 1; SLd += 2)
      for (int SRd = TwoSR - 2; SRd <= TwoSR + 2; SRd += 2)
        for (int TJd = jstart(SLd, SRd, S1); TJd <= S1 + 1; TJd += 2) {
          if (abs(SLd - SRd) > TJd || SLd < 0 || SRd < 0) continue;
          const double f = ph(SLd + 1 - TwoSL + 2 * S1) * sqrt(3.0 * (SRd + 1) * (TwoSL + 1) * (TJd + 1)) *
                           wigner9j(2, SRd, TwoSR, 1, SLd, TwoSL, 1, TJd, S1);
          over_l(*this, R, NL - 1, SLd, true, NR, SRd, true, N1, 1, TJd, f);
        }
  if (N2 == 1)
    for (int SLd = TwoSL - 1; SLd <= TwoSL + 1; SLd += 2)
      for (int SRd = TwoSR - 2; SRd <= TwoSR + 2; SRd += 2) {
        if (abs(SLd - SRd) > S1 || SLd < 0 || SRd < 0) continue;
        const double f = ph(TwoSR - SRd + 2 * S1) * sqrt(3.0 * (SRd + 1) * (TwoSL + 1) * (TwoJ + 1)) *
                         wigner9j(2, TwoSR, SRd, 1, TwoSL, SLd, 1, TwoJ, S1);
        over_l(*this, R, NL - 1, SLd, true, NR, SRd, true, N1, 2, S1, f);
      }
}

// CheMPS2/HeffDiagrams4.cpp:6306-6518
void HeffEmitter::d4L3and4L4spin1() {
  const int S2 = (N2 == 1) ? 1 : 0;
  auto R = [&](int l) -> const OpT& { return Rt->D[theindex - l][1]; };
  if (N1 == 1)
    for (int SLd = TwoSL - 1; SLd <= TwoSL + 1; SLd += 2)
      for (int SRd = TwoSR - 2; SRd <= TwoSR + 2; SRd += 2) {
        if (abs(SLd - SRd) > S2 || SLd < 0 || SRd < 0) continue;
        const double f = ph(TwoSL - SLd + 2 + S2 - TwoJ) * sqrt(3.0 * (TwoSR + 1) * (SLd + 1) * (TwoJ + 1)) *
                         wigner9j(2, TwoSR, SRd, 1, TwoSL, SLd, 1, TwoJ, S2);
        over_l(*this, R, NL + 1, SLd, false, NR, SRd, false, 0, N2, S2, f);
      }
  if (N1 == 2)
    for (int SLd = TwoSL - 1; SLd <= TwoSL + 1; SLd += 2)
      for (int SRd = TwoSR - 2; SRd <= TwoSR + 2; SRd += 2)
        for (int TJd = jstart(SLd, SRd, S2); TJd <= S2 + 1; TJd += 2) {
          if (abs(SLd - SRd) > TJd || SLd < 0 || SRd < 0) continue;
          const double f = ph(TwoSR - SRd + 1 + S2 - TJd) * sqrt(3.0 * (TwoSR + 1) * (SLd + 1) * (TJd + 1)) *
                           wigner9j(2, SRd, TwoSR, 1, SLd, TwoSL, 1, TJd, S2);
          over_l(*this, R, NL + 1, SLd, false, NR, SRd, false, 1, N2, TJd, f);
        }
  if (N1 == 0)
    for (int SLd = TwoSL - 1; SLd <= TwoSL + 1; SLd += 2)
      for (int SRd = TwoSR - 2; SRd <= TwoSR + 2; SRd += 2)
        for (int TJd = jstart(SLd, SRd, S2); TJd <= S2 + 1; TJd += 2) {
          if (abs(SLd - SRd) > TJd || SLd < 0 || SRd < 0) continue;
          const double f = ph(SLd + 2 - TwoSL + S2 - TJd) * sqrt(3.0 * (SRd + 1) * (TwoSL + 1) * (TJd + 1)) *
                           wigner9j(2, SRd, TwoSR, 1, SLd, TwoSL, 1, TJd, S2);
          over_l(*this, R, NL - 1, SLd, true, NR, SRd, true, 1, N2, TJd, f);
        }
  if (N1 == 1)
    for (int SLd = TwoSL - 1; SLd <= TwoSL + 1; SLd += 2)
      for (int SRd = TwoSR - 2; SRd <= TwoSR + 2; SRd += 2) {
        if (abs(SLd - SRd) > S2 || SLd < 0 || SRd < 0) continue;
        const double f = ph(TwoSR - SRd + 1 + S2 - TwoJ) * sqrt(3.0 * (SRd + 1) * (TwoSL + 1) * (TwoJ + 1)) *
                         wigner9j(2, TwoSR, SRd, 1, TwoSL, SLd, 1, TwoJ, S2);
        over_l(*this, R, NL - 1, SLd, true, NR, SRd, true, 2, N2, S2, f);
      }
}

}  // namespace c2g
