// Heff diagrams 4B and 4C (CheMPS2/HeffDiagrams4.cpp:670-2332): a complementary pair
// operator of the left block (A/B/C/D on orbital pair (theindex, l) for 4B or
// (theindex + 1, l) for 4C) times the creator L_l of the right block, for every l right
// of the two sites.
#include "heff_impl.hpp"

namespace c2g {

using std::abs;
using std::sqrt;

namespace {

inline int ph(int x) { return heff_phase(x); }

// Y += f * op(left block) * X[kp] * op(right creator block).
//   ldu: left block stored (down -> up) and used transposed, else (up -> down) as is.
//   rdu: right block stored (down -> up) and used as is, else (up -> down) transposed.
void lr(HeffEmitter& h, const OpT& lo, int nld, int sld, int ild, bool ldu, const OpT& ro, int nrd, int srd,
        int ird, bool rdu, double f, int kp) {
  if (kp == -1) return;
  const Blk lb = ldu ? lo.blk(nld, sld, ild, h.NL, h.TwoSL, h.IL) : lo.blk(h.NL, h.TwoSL, h.IL, nld, sld, ild);
  const Blk rb = rdu ? ro.blk(nrd, srd, ird, h.NR, h.TwoSR, h.IR) : ro.blk(h.NR, h.TwoSR, h.IR, nrd, srd, ird);
  h.emit(f, HeffEmitter::need(lb), ldu, kp, HeffEmitter::need(rb), !rdu);
}

int jstart(int sl, int sr, int two_s) { return ((sl != sr) || (two_s == 0)) ? two_s + 1 : 0; }

// Loops of the reference: for each case the right spin SRd (outer), the left spin SLd
// (spin-1 variants only) and the coupled spin 2J (when it can change), then l.
template <class Body>
void for_l(HeffEmitter& h, Body body) {
  for (int l = h.theindex + 2; l < h.L; l++) body(l);
}

}  // namespace

// ------------------------------------------------------------------------- 4B
// CheMPS2/HeffDiagrams4.cpp:670-868
void HeffEmitter::d4B1and4B2spin0() {
  const int S2 = (N2 == 1) ? 1 : 0;
  auto Aof = [&](int l) -> const OpT& { return Lt->A[l - theindex][0]; };
  if (N1 == 0)
    for (int SRd = TwoSR - 1; SRd <= TwoSR + 1; SRd += 2)
      for (int TJd = jstart(TwoSL, SRd, S2); TJd <= S2 + 1; TJd += 2) {
        if (abs(TwoSL - SRd) > TJd || SRd < 0) continue;
        const double f = ph(TwoSR + TwoSL + 1 + TJd + 2 * S2) * sqrt(0.5 * (TwoSR + 1) * (TJd + 1)) *
                         wigner6j(TJd, S2, 1, TwoSR, SRd, TwoSL);
        for_l(*this, [&](int l) {
          const int ILd = irrep_prod(IL, Aof(l).irrep()), IRd = irrep_prod(IR, irr(l));
          lr(*this, Aof(l), NL - 2, TwoSL, ILd, true, Rt->Lop(l), NR - 1, SRd, IRd, true, f,
             kap(NL - 2, TwoSL, ILd, 1, N2, TJd, NR - 1, SRd, IRd));
        });
      }
  if (N1 == 1)
    for (int SRd = TwoSR - 1; SRd <= TwoSR + 1; SRd += 2) {
      if (abs(TwoSL - SRd) > S2 || SRd < 0) continue;
      const double f = ph(TwoSR + TwoSL + 2 + TwoJ + 2 * S2) * sqrt(0.5 * (TwoSR + 1) * (TwoJ + 1)) *
                       wigner6j(TwoJ, S2, 1, SRd, TwoSR, TwoSL);
      for_l(*this, [&](int l) {
        const int ILd = irrep_prod(IL, Aof(l).irrep()), IRd = irrep_prod(IR, irr(l));
        lr(*this, Aof(l), NL - 2, TwoSL, ILd, true, Rt->Lop(l), NR - 1, SRd, IRd, true, f,
           kap(NL - 2, TwoSL, ILd, 2, N2, S2, NR - 1, SRd, IRd));
      });
    }
  if (N1 == 1)
    for (int SRd = TwoSR - 1; SRd <= TwoSR + 1; SRd += 2) {
      if (abs(TwoSL - SRd) > S2 || SRd < 0) continue;
      const double f = ph(SRd + TwoSL + 1 + TwoJ + 2 * S2) * sqrt(0.5 * (SRd + 1) * (TwoJ + 1)) *
                       wigner6j(TwoJ, S2, 1, SRd, TwoSR, TwoSL);
      for_l(*this, [&](int l) {
        const int ILd = irrep_prod(IL, Aof(l).irrep()), IRd = irrep_prod(IR, irr(l));
        lr(*this, Aof(l), NL + 2, TwoSL, ILd, false, Rt->Lop(l), NR + 1, SRd, IRd, false, f,
           kap(NL + 2, TwoSL, ILd, 0, N2, S2, NR + 1, SRd, IRd));
      });
    }
  if (N1 == 2)
    for (int SRd = TwoSR - 1; SRd <= TwoSR + 1; SRd += 2)
      for (int TJd = jstart(TwoSL, SRd, S2); TJd <= S2 + 1; TJd += 2) {
        if (abs(TwoSL - SRd) > TJd || SRd < 0) continue;
        const double f = ph(SRd + TwoSL + 2 + TJd + 2 * S2) * sqrt(0.5 * (SRd + 1) * (TJd + 1)) *
                         wigner6j(TJd, S2, 1, TwoSR, SRd, TwoSL);
        for_l(*this, [&](int l) {
          const int ILd = irrep_prod(IL, Aof(l).irrep()), IRd = irrep_prod(IR, irr(l));
          lr(*this, Aof(l), NL + 2, TwoSL, ILd, false, Rt->Lop(l), NR + 1, SRd, IRd, false, f,
             kap(NL + 2, TwoSL, ILd, 1, N2, TJd, NR + 1, SRd, IRd));
        });
      }
}

// CheMPS2/HeffDiagrams4.cpp:870-1080
void HeffEmitter::d4B1and4B2spin1() {
  const int S2 = (N2 == 1) ? 1 : 0;
  auto Bof = [&](int l) -> const OpT& { return Lt->B[l - theindex][0]; };
  if (N1 == 0)
    for (int SRd = TwoSR - 1; SRd <= TwoSR + 1; SRd += 2)
      for (int SLd = TwoSL - 2; SLd <= TwoSL + 2; SLd += 2)
        for (int TJd = jstart(SLd, SRd, S2); TJd <= S2 + 1; TJd += 2) {
          if (abs(SLd - SRd) > TJd || SLd < 0 || SRd < 0) continue;
          const double f = ((S2 == 0) ? 1 : -1) * sqrt(3.0 * (TwoSR + 1) * (TwoSL + 1) * (TJd + 1)) *
                           wigner9j(2, SLd, TwoSL, 1, SRd, TwoSR, 1, TJd, S2);
          for_l(*this, [&](int l) {
            const int ILd = irrep_prod(IL, Bof(l).irrep()), IRd = irrep_prod(IR, irr(l));
            lr(*this, Bof(l), NL - 2, SLd, ILd, true, Rt->Lop(l), NR - 1, SRd, IRd, true, f,
               kap(NL - 2, SLd, ILd, 1, N2, TJd, NR - 1, SRd, IRd));
          });
        }
  if (N1 == 1)
    for (int SRd = TwoSR - 1; SRd <= TwoSR + 1; SRd += 2)
      for (int SLd = TwoSL - 2; SLd <= TwoSL + 2; SLd += 2) {
        if (abs(SLd - SRd) > S2 || SLd < 0 || SRd < 0) continue;
        const double f = ph(TwoSR - SRd + TwoSL + 3 - SLd + 2 * S2) * sqrt(3.0 * (TwoSR + 1) * (TwoSL + 1) * (TwoJ + 1)) *
                         wigner9j(2, TwoSL, SLd, 1, TwoSR, SRd, 1, TwoJ, S2);
        for_l(*this, [&](int l) {
          const int ILd = irrep_prod(IL, Bof(l).irrep()), IRd = irrep_prod(IR, irr(l));
          lr(*this, Bof(l), NL - 2, SLd, ILd, true, Rt->Lop(l), NR - 1, SRd, IRd, true, f,
             kap(NL - 2, SLd, ILd, 2, N2, S2, NR - 1, SRd, IRd));
        });
      }
  if (N1 == 1)
    for (int SRd = TwoSR - 1; SRd <= TwoSR + 1; SRd += 2)
      for (int SLd = TwoSL - 2; SLd <= TwoSL + 2; SLd += 2) {
        if (abs(SLd - SRd) > S2 || SLd < 0 || SRd < 0) continue;
        const double f = ((S2 == 0) ? 1 : -1) * sqrt(3.0 * (SRd + 1) * (SLd + 1) * (TwoJ + 1)) *
                         wigner9j(2, TwoSL, SLd, 1, TwoSR, SRd, 1, TwoJ, S2);
        for_l(*this, [&](int l) {
          const int ILd = irrep_prod(IL, Bof(l).irrep()), IRd = irrep_prod(IR, irr(l));
          lr(*this, Bof(l), NL + 2, SLd, ILd, false, Rt->Lop(l), NR + 1, SRd, IRd, false, f,
             kap(NL + 2, SLd, ILd, 0, N2, S2, NR + 1, SRd, IRd));
        });
      }
  if (N1 == 2)
    for (int SRd = TwoSR - 1; SRd <= TwoSR + 1; SRd += 2)
      for (int SLd = TwoSL - 2; SLd <= TwoSL + 2; SLd += 2)
        for (int TJd = jstart(SLd, SRd, S2); TJd <= S2 + 1; TJd += 2) {
          if (abs(SLd - SRd) > TJd || SLd < 0 || SRd < 0) continue;
          const double f = ph(SLd + 3 - TwoSL + SRd - TwoSR + 2 * S2) * sqrt(3.0 * (SRd + 1) * (TJd + 1) * (SLd + 1)) *
                           wigner9j(2, SLd, TwoSL, 1, SRd, TwoSR, 1, TJd, S2);
          for_l(*this, [&](int l) {
            const int ILd = irrep_prod(IL, Bof(l).irrep()), IRd = irrep_prod(IR, irr(l));
            lr(*this, Bof(l), NL + 2, SLd, ILd, false, Rt->Lop(l), NR + 1, SRd, IRd, false, f,
               kap(NL + 2, SLd, ILd, 1, N2, TJd, NR + 1, SRd, IRd));
          });
        }
}

// CheMPS2/HeffDiagrams4.cpp:1082-1284
void HeffEmitter::d4B3and4B4spin0() {
  const int S2 = (N2 == 1) ? 1 : 0;
  auto Cof = [&](int l) -> const OpT& { return Lt->C[l - theindex][0]; };
  if (N1 == 1)
    for (int SRd = TwoSR - 1; SRd <= TwoSR + 1; SRd += 2) {
      if (abs(TwoSL - SRd) > S2 || SRd < 0) continue;
      const double f = ph(TwoSR + TwoSL + TwoJ + 2 * S2) * sqrt(0.5 * (TwoSR + 1) * (TwoJ + 1)) *
                       wigner6j(TwoJ, S2, 1, SRd, TwoSR, TwoSL);
      for_l(*this, [&](int l) {
        const int ILd = irrep_prod(IL, Cof(l).irrep()), IRd = irrep_prod(IR, irr(l));
        lr(*this, Cof(l), NL, TwoSL, ILd, true, Rt->Lop(l), NR - 1, SRd, IRd, true, f,
           kap(NL, TwoSL, ILd, 0, N2, S2, NR - 1, SRd, IRd));
      });
    }
  if (N1 == 2)
    for (int SRd = TwoSR - 1; SRd <= TwoSR + 1; SRd += 2)
      for (int TJd = jstart(TwoSL, SRd, S2); TJd <= S2 + 1; TJd += 2) {
        if (abs(TwoSL - SRd) > TJd || SRd < 0) continue;
        const double f = ph(TwoSR + TwoSL + 1 + TJd + 2 * S2) * sqrt(0.5 * (TwoSR + 1) * (TJd + 1)) *
                         wigner6j(TJd, S2, 1, TwoSR, SRd, TwoSL);
        for_l(*this, [&](int l) {
          const int ILd = irrep_prod(IL, Cof(l).irrep()), IRd = irrep_prod(IR, irr(l));
          lr(*this, Cof(l), NL, TwoSL, ILd, true, Rt->Lop(l), NR - 1, SRd, IRd, true, f,
             kap(NL, TwoSL, ILd, 1, N2, TJd, NR - 1, SRd, IRd));
        });
      }
  if (N1 == 0)
    for (int SRd = TwoSR - 1; SRd <= TwoSR + 1; SRd += 2)
      for (int TJd = jstart(TwoSL, SRd, S2); TJd <= S2 + 1; TJd += 2) {
        if (abs(TwoSL - SRd) > TJd || SRd < 0) continue;
        const double f = ph(SRd + TwoSL + TJd + 2 * S2) * sqrt(0.5 * (SRd + 1) * (TJd + 1)) *
                         wigner6j(TJd, S2, 1, TwoSR, SRd, TwoSL);
        for_l(*this, [&](int l) {
          const int ILd = irrep_prod(IL, Cof(l).irrep()), IRd = irrep_prod(IR, irr(l));
          lr(*this, Cof(l), NL, TwoSL, ILd, false, Rt->Lop(l), NR + 1, SRd, IRd, false, f,
             kap(NL, TwoSL, ILd, 1, N2, TJd, NR + 1, SRd, IRd));
        });
      }
  if (N1 == 1)
    for (int SRd = TwoSR - 1; SRd <= TwoSR + 1; SRd += 2) {
      if (abs(TwoSL - SRd) > S2 || SRd < 0) continue;
      const double f = ph(SRd + TwoSL + 1 + TwoJ + 2 * S2) * sqrt(0.5 * (SRd + 1) * (TwoJ + 1)) *
                       wigner6j(TwoJ, S2, 1, SRd, TwoSR, TwoSL);
      for_l(*this, [&](int l) {
        const int ILd = irrep_prod(IL, Cof(l).irrep()), IRd = irrep_prod(IR, irr(l));
        lr(*this, Cof(l), NL, TwoSL, ILd, false, Rt->Lop(l), NR + 1, SRd, IRd, false, f,
           kap(NL, TwoSL, ILd, 2, N2, S2, NR + 1, SRd, IRd));
      });
    }
}

// CheMPS2/HeffDiagrams4.cpp:1286-1500
void HeffEmitter::d4B3and4B4spin1() {
  const int S2 = (N2 == 1) ? 1 : 0;
  auto Dof = [&](int l) -> const OpT& { return Lt->D[l - theindex][0]; };
  if (N1 == 1)
    for (int SRd = TwoSR - 1; SRd <= TwoSR + 1; SRd += 2)
      for (int SLd = TwoSL - 2; SLd <= TwoSL + 2; SLd += 2) {
        if (abs(SLd - SRd) > S2 || SLd < 0 || SRd < 0) continue;
        const double f = ph(TwoSL - SLd + TwoSR - SRd + 3 + 2 * S2) * sqrt(3.0 * (TwoSR + 1) * (TwoJ + 1) * (TwoSL + 1)) *
                         wigner9j(2, TwoSL, SLd, 1, TwoSR, SRd, 1, TwoJ, S2);
        for_l(*this, [&](int l) {
          const int ILd = irrep_prod(IL, Dof(l).irrep()), IRd = irrep_prod(IR, irr(l));
          lr(*this, Dof(l), NL, SLd, ILd, true, Rt->Lop(l), NR - 1, SRd, IRd, true, f,
             kap(NL, SLd, ILd, 0, N2, S2, NR - 1, SRd, IRd));
        });
      }
  if (N1 == 2)
    for (int SRd = TwoSR - 1; SRd <= TwoSR + 1; SRd += 2)
      for (int SLd = TwoSL - 2; SLd <= TwoSL + 2; SLd += 2)
        for (int TJd = jstart(SLd, SRd, S2); TJd <= S2 + 1; TJd += 2) {
          if (abs(SLd - SRd) > TJd || SLd < 0 || SRd < 0) continue;
          const double f = ((S2 == 0) ? -1 : 1) * sqrt(3.0 * (TwoSR + 1) * (TJd + 1) * (TwoSL + 1)) *
                           wigner9j(2, SLd, TwoSL, 1, SRd, TwoSR, 1, TJd, S2);
          for_l(*this, [&](int l) {
            const int ILd = irrep_prod(IL, Dof(l).irrep()), IRd = irrep_prod(IR, irr(l));
            lr(*this, Dof(l), NL, SLd, ILd, true, Rt->Lop(l), NR - 1, SRd, IRd, true, f,
               kap(NL, SLd, ILd, 1, N2, TJd, NR - 1, SRd, IRd));
          });
        }
  if (N1 == 0)
    for (int SRd = TwoSR - 1; SRd <= TwoSR + 1; SRd += 2)
      for (int SLd = TwoSL - 2; SLd <= TwoSL + 2; SLd += 2)
        for (int TJd = jstart(SLd, SRd, S2); TJd <= S2 + 1; TJd += 2) {
          if (abs(SLd - SRd) > TJd || SLd < 0 || SRd < 0) continue;
          const double f = ph(SRd - TwoSR + SLd - TwoSL + 3 + 2 * S2) * sqrt(3.0 * (SRd + 1) * (TJd + 1) * (SLd + 1)) *
                           wigner9j(2, SLd, TwoSL, 1, SRd, TwoSR, 1, TJd, S2);
          for_l(*this, [&](int l) {
            const int ILd = irrep_prod(IL, Dof(l).irrep()), IRd = irrep_prod(IR, irr(l));
            lr(*this, Dof(l), NL, SLd, ILd, false, Rt->Lop(l), NR + 1, SRd, IRd, false, f,
               kap(NL, SLd, ILd, 1, N2, TJd, NR + 1, SRd, IRd));
          });
        }
  if (N1 == 1)
    for (int SRd = TwoSR - 1; SRd <= TwoSR + 1; SRd += 2)
      for (int SLd = TwoSL - 2; SLd <= TwoSL + 2; SLd += 2) {
        if (abs(SLd - SRd) > S2 || SLd < 0 || SRd < 0) continue;
        const double f = ((S2 == 0) ? -1 : 1) * sqrt(3.0 * (SRd + 1) * (TwoJ + 1) * (SLd + 1)) *
                         wigner9j(2, TwoSL, SLd, 1, TwoSR, SRd, 1, TwoJ, S2);
        for_l(*this, [&](int l) {
          const int ILd = irrep_prod(IL, Dof(l).irrep()), IRd = irrep_prod(IR, irr(l));
          lr(*this, Dof(l), NL, SLd, ILd, false, Rt->Lop(l), NR + 1, SRd, IRd, false, f,
             kap(NL, SLd, ILd, 2, N2, S2, NR + 1, SRd, IRd));
        });
      }
}

// ------------------------------------------------------------------------- 4C
// CheMPS2/HeffDiagrams4.cpp:1502-1700
void HeffEmitter::d4C1and4C2spin0() {
  const int S1 = (N1 == 1) ? 1 : 0;
  auto Aof = [&](int l) -> const OpT& { return Lt->A[l - theindex - 1][1]; };
  if (N2 == 0)
    for (int SRd = TwoSR - 1; SRd <= TwoSR + 1; SRd += 2)
      for (int TJd = jstart(TwoSL, SRd, S1); TJd <= S1 + 1; TJd += 2) {
        if (abs(TwoSL - SRd) > TJd || SRd < 0) continue;
        const double f = ph(TwoSR + TwoSL + 2 + S1) * sqrt(0.5 * (TwoSR + 1) * (TJd + 1)) *
                         wigner6j(TJd, S1, 1, TwoSR, SRd, TwoSL);
        for_l(*this, [&](int l) {
          const int ILd = irrep_prod(IL, Aof(l).irrep()), IRd = irrep_prod(IR, irr(l));
          lr(*this, Aof(l), NL - 2, TwoSL, ILd, true, Rt->Lop(l), NR - 1, SRd, IRd, true, f,
             kap(NL - 2, TwoSL, ILd, N1, 1, TJd, NR - 1, SRd, IRd));
        });
      }
  if (N2 == 1)
    for (int SRd = TwoSR - 1; SRd <= TwoSR + 1; SRd += 2) {
      if (abs(TwoSL - SRd) > S1 || SRd < 0) continue;
      const double f = ph(TwoSR + TwoSL + 3 + S1) * sqrt(0.5 * (TwoSR + 1) * (TwoJ + 1)) *
                       wigner6j(TwoJ, S1, 1, SRd, TwoSR, TwoSL);
      for_l(*this, [&](int l) {
        const int ILd = irrep_prod(IL, Aof(l).irrep()), IRd = irrep_prod(IR, irr(l));
        lr(*this, Aof(l), NL - 2, TwoSL, ILd, true, Rt->Lop(l), NR - 1, SRd, IRd, true, f,
           kap(NL - 2, TwoSL, ILd, N1, 2, S1, NR - 1, SRd, IRd));
      });
    }
  if (N2 == 1)
    for (int SRd = TwoSR - 1; SRd <= TwoSR + 1; SRd += 2) {
      if (abs(TwoSL - SRd) > S1 || SRd < 0) continue;
      const double f = ph(SRd + TwoSL + 2 + S1) * sqrt(0.5 * (SRd + 1) * (TwoJ + 1)) *
                       wigner6j(TwoJ, S1, 1, SRd, TwoSR, TwoSL);
      for_l(*this, [&](int l) {
        const int ILd = irrep_prod(IL, Aof(l).irrep()), IRd = irrep_prod(IR, irr(l));
        lr(*this, Aof(l), NL + 2, TwoSL, ILd, false, Rt->Lop(l), NR + 1, SRd, IRd, false, f,
           kap(NL + 2, TwoSL, ILd, N1, 0, S1, NR + 1, SRd, IRd));
      });
    }
  if (N2 == 2)
    for (int SRd = TwoSR - 1; SRd <= TwoSR + 1; SRd += 2)
      for (int TJd = jstart(TwoSL, SRd, S1); TJd <= S1 + 1; TJd += 2) {
        if (abs(TwoSL - SRd) > TJd || SRd < 0) continue;
        const double f = ph(SRd + TwoSL + 3 + S1) * sqrt(0.5 * (SRd + 1) * (TJd + 1)) *
                         wigner6j(TJd, S1, 1, TwoSR, SRd, TwoSL);
        for_l(*this, [&](int l) {
          const int ILd = irrep_prod(IL, Aof(l).irrep()), IRd = irrep_prod(IR, irr(l));
          lr(*this, Aof(l), NL + 2, TwoSL, ILd, false, Rt->Lop(l), NR + 1, SRd, IRd, false, f,
             kap(NL + 2, TwoSL, ILd, N1, 1, TJd, NR + 1, SRd, IRd));
        });
      }
}

// CheMPS2/HeffDiagrams4.cpp:1702-1912
void HeffEmitter::d4C1and4C2spin1() {
  const int S1 = (N1 == 1) ? 1 : 0;
  auto Bof = [&](int l) -> const OpT& { return Lt->B[l - theindex - 1][1]; };
  if (N2 == 0)
    for (int SRd = TwoSR - 1; SRd <= TwoSR + 1; SRd += 2)
      for (int SLd = TwoSL - 2; SLd <= TwoSL + 2; SLd += 2)
        for (int TJd = jstart(SLd, SRd, S1); TJd <= S1 + 1; TJd += 2) {
          if (abs(SLd - SRd) > TJd || SLd < 0 || SRd < 0) continue;
          const double f = ph(1 + S1 - TJd) * sqrt(3.0 * (TwoSR + 1) * (TwoSL + 1) * (TJd + 1)) *
                           wigner9j(2, SLd, TwoSL, 1, SRd, TwoSR, 1, TJd, S1);
          for_l(*this, [&](int l) {
            const int ILd = irrep_prod(IL, Bof(l).irrep()), IRd = irrep_prod(IR, irr(l));
            lr(*this, Bof(l), NL - 2, SLd, ILd, true, Rt->Lop(l), NR - 1, SRd, IRd, true, f,
               kap(NL - 2, SLd, ILd, N1, 1, TJd, NR - 1, SRd, IRd));
          });
        }
  if (N2 == 1)
    for (int SRd = TwoSR - 1; SRd <= TwoSR + 1; SRd += 2)
      for (int SLd = TwoSL - 2; SLd <= TwoSL + 2; SLd += 2) {
        if (abs(SLd - SRd) > S1 || SLd < 0 || SRd < 0) continue;
        const double f = ph(TwoSR - SRd + TwoSL - SLd + S1 - TwoJ) * sqrt(3.0 * (TwoSR + 1) * (TwoSL + 1) * (TwoJ + 1)) *
                         wigner9j(2, TwoSL, SLd, 1, TwoSR, SRd, 1, TwoJ, S1);
        for_l(*this, [&](int l) {
          const int ILd = irrep_prod(IL, Bof(l).irrep()), IRd = irrep_prod(IR, irr(l));
          lr(*this, Bof(l), NL - 2, SLd, ILd, true, Rt->Lop(l), NR - 1, SRd, IRd, true, f,
             kap(NL - 2, SLd, ILd, N1, 2, S1, NR - 1, SRd, IRd));
        });
      }
  if (N2 == 1)
    for (int SRd = TwoSR - 1; SRd <= TwoSR + 1; SRd += 2)
      for (int SLd = TwoSL - 2; SLd <= TwoSL + 2; SLd += 2) {
        if (abs(SLd - SRd) > S1 || SLd < 0 || SRd < 0) continue;
        const double f = ph(1 + S1 - TwoJ) * sqrt(3.0 * (SRd + 1) * (SLd + 1) * (TwoJ + 1)) *
                         wigner9j(2, TwoSL, SLd, 1, TwoSR, SRd, 1, TwoJ, S1);
        for_l(*this, [&](int l) {
          const int ILd = irrep_prod(IL, Bof(l).irrep()), IRd = irrep_prod(IR, irr(l));
          lr(*this, Bof(l), NL + 2, SLd, ILd, false, Rt->Lop(l), NR + 1, SRd, IRd, false, f,
             kap(NL + 2, SLd, ILd, N1, 0, S1, NR + 1, SRd, IRd));
        });
      }
  if (N2 == 2)
    for (int SRd = TwoSR - 1; SRd <= TwoSR + 1; SRd += 2)
      for (int SLd = TwoSL - 2; SLd <= TwoSL + 2; SLd += 2)
        for (int TJd = jstart(SLd, SRd, S1); TJd <= S1 + 1; TJd += 2) {
          if (abs(SLd - SRd) > TJd || SLd < 0 || SRd < 0) continue;
          const double f = ph(SLd - TwoSL + SRd - TwoSR + S1 - TJd) * sqrt(3.0 * (SRd + 1) * (TJd + 1) * (SLd + 1)) *
                           wigner9j(2, SLd, TwoSL, 1, SRd, TwoSR, 1, TJd, S1);
          for_l(*this, [&](int l) {
            const int ILd = irrep_prod(IL, Bof(l).irrep()), IRd = irrep_prod(IR, irr(l));
            lr(*this, Bof(l), NL + 2, SLd, ILd, false, Rt->Lop(l), NR + 1, SRd, IRd, false, f,
               kap(NL + 2, SLd, ILd, N1, 1, TJd, NR + 1, SRd, IRd));
          });
        }
}

// CheMPS2/HeffDiagrams4.cpp:1914-2116
void HeffEmitter::d4C3and4C4spin0() {
  const int S1 = (N1 == 1) ? 1 : 0;
  auto Cof = [&](int l) -> const OpT& { return Lt->C[l - theindex - 1][1]; };
  if (N2 == 1)
    for (int SRd = TwoSR - 1; SRd <= TwoSR + 1; SRd += 2) {
      if (abs(TwoSL - SRd) > S1 || SRd < 0) continue;
      const double f = ph(TwoSR + TwoSL + 1 + S1) * sqrt(0.5 * (TwoSR + 1) * (TwoJ + 1)) *
                       wigner6j(TwoJ, S1, 1, SRd, TwoSR, TwoSL);
      for_l(*this, [&](int l) {
        const int ILd = irrep_prod(IL, Cof(l).irrep()), IRd = irrep_prod(IR, irr(l));
        lr(*this, Cof(l), NL, TwoSL, ILd, true, Rt->Lop(l), NR - 1, SRd, IRd, true, f,
           kap(NL, TwoSL, ILd, N1, 0, S1, NR - 1, SRd, IRd));
      });
    }
  if (N2 == 2)
    for (int SRd = TwoSR - 1; SRd <= TwoSR + 1; SRd += 2)
      for (int TJd = jstart(TwoSL, SRd, S1); TJd <= S1 + 1; TJd += 2) {
        if (abs(TwoSL - SRd) > TJd || SRd < 0) continue;
        const double f = ph(TwoSR + TwoSL + 2 + S1) * sqrt(0.5 * (TwoSR + 1) * (TJd + 1)) *
                         wigner6j(TJd, S1, 1, TwoSR, SRd, TwoSL);
        for_l(*this, [&](int l) {
          const int ILd = irrep_prod(IL, Cof(l).irrep()), IRd = irrep_prod(IR, irr(l));
          lr(*this, Cof(l), NL, TwoSL, ILd, true, Rt->Lop(l), NR - 1, SRd, IRd, true, f,
             kap(NL, TwoSL, ILd, N1, 1, TJd, NR - 1, SRd, IRd));
        });
      }
  if (N2 == 0)
    for (int SRd = TwoSR - 1; SRd <= TwoSR + 1; SRd += 2)
      for (int TJd = jstart(TwoSL, SRd, S1); TJd <= S1 + 1; TJd += 2) {
        if (abs(TwoSL - SRd) > TJd || SRd < 0) continue;
        const double f = ph(SRd + TwoSL + 1 + S1) * sqrt(0.5 * (SRd + 1) * (TJd + 1)) *
                         wigner6j(TJd, S1, 1, TwoSR, SRd, TwoSL);
        for_l(*this, [&](int l) {
          const int ILd = irrep_prod(IL, Cof(l).irrep()), IRd = irrep_prod(IR, irr(l));
          lr(*this, Cof(l), NL, TwoSL, ILd, false, Rt->Lop(l), NR + 1, SRd, IRd, false, f,
             kap(NL, TwoSL, ILd, N1, 1, TJd, NR + 1, SRd, IRd));
        });
      }
  if (N2 == 1)
    for (int SRd = TwoSR - 1; SRd <= TwoSR + 1; SRd += 2) {
      if (abs(TwoSL - SRd) > S1 || SRd < 0) continue;
      const double f = ph(SRd + TwoSL + 2 + S1) * sqrt(0.5 * (SRd + 1) * (TwoJ + 1)) *
                       wigner6j(TwoJ, S1, 1, SRd, TwoSR, TwoSL);
      for_l(*this, [&](int l) {
        const int ILd = irrep_prod(IL, Cof(l).irrep()), IRd = irrep_prod(IR, irr(l));
        lr(*this, Cof(l), NL, TwoSL, ILd, false, Rt->Lop(l), NR + 1, SRd, IRd, false, f,
           kap(NL, TwoSL, ILd, N1, 2, S1, NR + 1, SRd, IRd));
      });
    }
}

// CheMPS2/HeffDiagrams4.cpp:2118-2332
void HeffEmitter::d4C3and4C4spin1() {
  const int S1 = (N1 == 1) ? 1 : 0;
  auto Dof = [&](int l) -> const OpT& { return Lt->D[l - theindex - 1][1]; };
  if (N2 == 1)
    for (int SRd = TwoSR - 1; SRd <= TwoSR + 1; SRd += 2)
      for (int SLd = TwoSL - 2; SLd <= TwoSL + 2; SLd += 2) {
        if (abs(SLd - SRd) > S1 || SLd < 0 || SRd < 0) continue;
        const double f = ph(TwoSL - SLd + TwoSR - SRd + S1 - TwoJ) * sqrt(3.0 * (TwoSR + 1) * (TwoJ + 1) * (TwoSL + 1)) *
                         wigner9j(2, TwoSL, SLd, 1, TwoSR, SRd, 1, TwoJ, S1);
        for_l(*this, [&](int l) {
          const int ILd = irrep_prod(IL, Dof(l).irrep()), IRd = irrep_prod(IR, irr(l));
          lr(*this, Dof(l), NL, SLd, ILd, true, Rt->Lop(l), NR - 1, SRd, IRd, true, f,
             kap(NL, SLd, ILd, N1, 0, S1, NR - 1, SRd, IRd));
        });
      }
  if (N2 == 2)
    for (int SRd = TwoSR - 1; SRd <= TwoSR + 1; SRd += 2)
      for (int SLd = TwoSL - 2; SLd <= TwoSL + 2; SLd += 2)
        for (int TJd = jstart(SLd, SRd, S1); TJd <= S1 + 1; TJd += 2) {
          if (abs(SLd - SRd) > TJd || SLd < 0 || SRd < 0) continue;
          const double f = ph(3 + S1 - TJd) * sqrt(3.0 * (TwoSR + 1) * (TJd + 1) * (TwoSL + 1)) *
                           wigner9j(2, SLd, TwoSL, 1, SRd, TwoSR, 1, TJd, S1);
          for_l(*this, [&](int l) {
            const int ILd = irrep_prod(IL, Dof(l).irrep()), IRd = irrep_prod(IR, irr(l));
            lr(*this, Dof(l), NL, SLd, ILd, true, Rt->Lop(l), NR - 1, SRd, IRd, true, f,
               kap(NL, SLd, ILd, N1, 1, TJd, NR - 1, SRd, IRd));
          });
        }
  if (N2 == 0)
    for (int SRd = TwoSR - 1; SRd <= TwoSR + 1; SRd += 2)
      for (int SLd = TwoSL - 2; SLd <= TwoSL + 2; SLd += 2)
        for (int TJd = jstart(SLd, SRd, S1); TJd <= S1 + 1; TJd += 2) {
          if (abs(SLd - SRd) > TJd || SLd < 0 || SRd < 0) continue;
          const double f = ph(SRd - TwoSR + SLd - TwoSL + S1 - TJd) * sqrt(3.0 * (SRd + 1) * (TJd + 1) * (SLd + 1)) *
                           wigner9j(2, SLd, TwoSL, 1, SRd, TwoSR, 1, TJd, S1);
          for_l(*this, [&](int l) {
            const int ILd = irrep_prod(IL, Dof(l).irrep()), IRd = irrep_prod(IR, irr(l));
            lr(*this, Dof(l), NL, SLd, ILd, false, Rt->Lop(l), NR + 1, SRd, IRd, false, f,
               kap(NL, SLd, ILd, N1, 1, TJd, NR + 1, SRd, IRd));
          });
        }
  if (N2 == 1)
    for (int SRd = TwoSR - 1; SRd <= TwoSR + 1; SRd += 2)
      for (int SLd = TwoSL - 2; SLd <= TwoSL + 2; SLd += 2) {
        if (abs(SLd - SRd) > S1 || SLd < 0 || SRd < 0) continue;
        const double f = ph(3 + S1 - TwoJ) * sqrt(3.0 * (SRd + 1) * (TwoJ + 1) * (SLd + 1)) *
                         wigner9j(2, TwoSL, SLd, 1, TwoSR, SRd, 1, TwoJ, S1);
        for_l(*this, [&](int l) {
          const int ILd = irrep_prod(IL, Dof(l).irrep()), IRd = irrep_prod(IR, irr(l));
          lr(*this, Dof(l), NL, SLd, ILd, false, Rt->Lop(l), NR + 1, SRd, IRd, false, f,
             kap(NL, SLd, ILd, N1, 2, S1, NR + 1, SRd, IRd));
        });
      }
}

}  // namespace c2g
