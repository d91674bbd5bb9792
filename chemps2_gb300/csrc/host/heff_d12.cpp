// Heff diagram groups 1 and 2 as contraction tasks.
// Each function records the contractions of the reference function of the same name
// (CheMPS2/HeffDiagrams1.cpp, CheMPS2/HeffDiagrams2.cpp) for the current block.
#include "heff_impl.hpp"

namespace c2g {

using std::abs;
using std::sqrt;

#define need HeffEmitter::need
static const Blk kNo;

// CheMPS2/HeffDiagrams1.cpp:26-34
void HeffEmitter::d1A() {
  const Blk Xb = need(Lt->X.blk(NL, TwoSL, IL, NL, TwoSL, IL));
  emit(1.0, Xb, false, ik, kNo, false);
}
// CheMPS2/HeffDiagrams1.cpp:36-45
void HeffEmitter::d1B() {
  const Blk Xb = need(Rt->X.blk(NR, TwoSR, IR, NR, TwoSR, IR));
  emit(1.0, kNo, false, ik, Xb, true);
}
// CheMPS2/HeffDiagrams1.cpp:47-54
void HeffEmitter::d1C() {
  if (N1 == 2) emit_scalar(V(theindex, theindex, theindex, theindex), ik);
}
// CheMPS2/HeffDiagrams1.cpp:56-63
void HeffEmitter::d1D() {
  if (N2 == 2) emit_scalar(V(theindex + 1, theindex + 1, theindex + 1, theindex + 1), ik);
}

// CheMPS2/HeffDiagrams2.cpp:28-127
void HeffEmitter::d2a1spin0() {
  if (theindex < L * 0.5) {
    for (int la = 0; la < theindex; la++)
      for (int lb = la; lb < theindex; lb++) {
        const OpT& s0 = Lt->S0[lb - la][theindex - 1 - lb];
        const OpT& a = Rt->A[lb - la][theindex + 1 - lb];
        const int ILd = irrep_prod(IL, s0.irrep()), IRd = irrep_prod(IR, a.irrep());
        const int kp = kap(NL - 2, TwoSL, ILd, N1, N2, TwoJ, NR - 2, TwoSR, IRd);
        if (kp == -1) continue;
        emit(1.0, need(s0.blk(NL - 2, TwoSL, ILd, NL, TwoSL, IL)), true, kp,
             need(a.blk(NR - 2, TwoSR, IRd, NR, TwoSR, IR)), false);
      }
  } else {
    for (int lg = theindex + 2; lg < L; lg++)
      for (int ld = lg; ld < L; ld++) {
        const OpT& a = Lt->A[ld - lg][lg - theindex];
        const OpT& s0 = Rt->S0[ld - lg][lg - theindex - 2];
        const int ILd = irrep_prod(IL, a.irrep()), IRd = irrep_prod(IR, s0.irrep());
        const int kp = kap(NL - 2, TwoSL, ILd, N1, N2, TwoJ, NR - 2, TwoSR, IRd);
        if (kp == -1) continue;
        emit(1.0, need(a.blk(NL - 2, TwoSL, ILd, NL, TwoSL, IL)), true, kp,
             need(s0.blk(NR - 2, TwoSR, IRd, NR, TwoSR, IR)), false);
      }
  }
}

// CheMPS2/HeffDiagrams2.cpp:129-228
void HeffEmitter::d2a2spin0() {
  if (theindex < L * 0.5) {
    for (int la = 0; la < theindex; la++)
      for (int lb = la; lb < theindex; lb++) {
        const OpT& s0 = Lt->S0[lb - la][theindex - 1 - lb];
        const OpT& a = Rt->A[lb - la][theindex + 1 - lb];
        const int ILd = irrep_prod(IL, s0.irrep()), IRd = irrep_prod(IR, a.irrep());
        const int kp = kap(NL + 2, TwoSL, ILd, N1, N2, TwoJ, NR + 2, TwoSR, IRd);
        if (kp == -1) continue;
        emit(1.0, need(s0.blk(NL, TwoSL, IL, NL + 2, TwoSL, ILd)), false, kp,
             need(a.blk(NR, TwoSR, IR, NR + 2, TwoSR, IRd)), true);
      }
  } else {
    for (int lg = theindex + 2; lg < L; lg++)
      for (int ld = lg; ld < L; ld++) {
        const OpT& a = Lt->A[ld - lg][lg - theindex];
        const OpT& s0 = Rt->S0[ld - lg][lg - theindex - 2];
        const int ILd = irrep_prod(IL, a.irrep()), IRd = irrep_prod(IR, s0.irrep());
        const int kp = kap(NL + 2, TwoSL, ILd, N1, N2, TwoJ, NR + 2, TwoSR, IRd);
        if (kp == -1) continue;
        emit(1.0, need(a.blk(NL, TwoSL, IL, NL + 2, TwoSL, ILd)), false, kp,
             need(s0.blk(NR, TwoSR, IR, NR + 2, TwoSR, IRd)), true);
      }
  }
}

// CheMPS2/HeffDiagrams2.cpp:230-351
void HeffEmitter::d2a1spin1() {
  for (int SLd = TwoSL - 2; SLd <= TwoSL + 2; SLd += 2)
    for (int SRd = TwoSR - 2; SRd <= TwoSR + 2; SRd += 2) {
      if (SLd < 0 || SRd < 0 || abs(SLd - SRd) > TwoJ) continue;
      const double f = heff_phase(SRd + TwoSL + TwoJ + 2) * sqrt((TwoSR + 1) * (TwoSL + 1.0)) *
                       wigner6j(SLd, SRd, TwoJ, TwoSR, TwoSL, 2);
      if (theindex < L * 0.5) {
        for (int la = 0; la < theindex; la++)
          for (int lb = la + 1; lb < theindex; lb++) {
            const OpT& s1 = Lt->S1[lb - la][theindex - 1 - lb];
            const OpT& b = Rt->B[lb - la][theindex + 1 - lb];
            const int ILd = irrep_prod(IL, s1.irrep()), IRd = irrep_prod(IR, b.irrep());
            const int kp = kap(NL - 2, SLd, ILd, N1, N2, TwoJ, NR - 2, SRd, IRd);
            if (kp == -1) continue;
            emit(f, need(s1.blk(NL - 2, SLd, ILd, NL, TwoSL, IL)), true, kp,
                 need(b.blk(NR - 2, SRd, IRd, NR, TwoSR, IR)), false);
          }
      } else {
        for (int lg = theindex + 2; lg < L; lg++)
          for (int ld = lg + 1; ld < L; ld++) {
            const OpT& b = Lt->B[ld - lg][lg - theindex];
            const OpT& s1 = Rt->S1[ld - lg][lg - theindex - 2];
            const int ILd = irrep_prod(IL, b.irrep()), IRd = irrep_prod(IR, s1.irrep());
            const int kp = kap(NL - 2, SLd, ILd, N1, N2, TwoJ, NR - 2, SRd, IRd);
            if (kp == -1) continue;
            emit(f, need(b.blk(NL - 2, SLd, ILd, NL, TwoSL, IL)), true, kp,
                 need(s1.blk(NR - 2, SRd, IRd, NR, TwoSR, IR)), false);
          }
      }
    }
}

// CheMPS2/HeffDiagrams2.cpp:353-474
void HeffEmitter::d2a2spin1() {
  for (int SLd = TwoSL - 2; SLd <= TwoSL + 2; SLd += 2)
    for (int SRd = TwoSR - 2; SRd <= TwoSR + 2; SRd += 2) {
      if (SLd < 0 || SRd < 0 || abs(SLd - SRd) > TwoJ) continue;
      const double f = heff_phase(SLd + TwoSR + TwoJ + 2) * sqrt((SRd + 1) * (SLd + 1.0)) *
                       wigner6j(SLd, SRd, TwoJ, TwoSR, TwoSL, 2);
      if (theindex < L * 0.5) {
        for (int la = 0; la < theindex; la++)
          for (int lb = la + 1; lb < theindex; lb++) {
            const OpT& s1 = Lt->S1[lb - la][theindex - 1 - lb];
            const OpT& b = Rt->B[lb - la][theindex + 1 - lb];
            const int ILd = irrep_prod(IL, s1.irrep()), IRd = irrep_prod(IR, b.irrep());
            const int kp = kap(NL + 2, SLd, ILd, N1, N2, TwoJ, NR + 2, SRd, IRd);
            if (kp == -1) continue;
            emit(f, need(s1.blk(NL, TwoSL, IL, NL + 2, SLd, ILd)), false, kp,
                 need(b.blk(NR, TwoSR, IR, NR + 2, SRd, IRd)), true);
          }
      } else {
        for (int lg = theindex + 2; lg < L; lg++)
          for (int ld = lg + 1; ld < L; ld++) {
            const OpT& b = Lt->B[ld - lg][lg - theindex];
            const OpT& s1 = Rt->S1[ld - lg][lg - theindex - 2];
            const int ILd = irrep_prod(IL, b.irrep()), IRd = irrep_prod(IR, s1.irrep());
            const int kp = kap(NL + 2, SLd, ILd, N1, N2, TwoJ, NR + 2, SRd, IRd);
            if (kp == -1) continue;
            emit(f, need(b.blk(NL, TwoSL, IL, NL + 2, SLd, ILd)), false, kp,
                 need(s1.blk(NR, TwoSR, IR, NR + 2, SRd, IRd)), true);
          }
      }
    }
}

// CheMPS2/HeffDiagrams2.cpp:476-649
void HeffEmitter::d2a3spin0() {
  if (theindex < L * 0.5) {
    for (int lg = 0; lg < theindex; lg++)
      for (int la = lg + 1; la < theindex; la++) {
        const OpT& f0 = Lt->F0[la - lg][theindex - 1 - la];
        const OpT& c = Rt->C[la - lg][theindex + 1 - la];
        const int ILd = irrep_prod(IL, f0.irrep()), IRd = irrep_prod(IR, c.irrep());
        const int kp = kap(NL, TwoSL, ILd, N1, N2, TwoJ, NR, TwoSR, IRd);
        if (kp == -1) continue;
        emit(1.0, need(f0.blk(NL, TwoSL, IL, NL, TwoSL, ILd)), false, kp,
             need(c.blk(NR, TwoSR, IR, NR, TwoSR, IRd)), true);
      }
    for (int la = 0; la < theindex; la++)
      for (int lg = la; lg < theindex; lg++) {
        const OpT& f0 = Lt->F0[lg - la][theindex - 1 - lg];
        const OpT& c = Rt->C[lg - la][theindex + 1 - lg];
        const int ILd = irrep_prod(IL, f0.irrep()), IRd = irrep_prod(IR, c.irrep());
        const int kp = kap(NL, TwoSL, ILd, N1, N2, TwoJ, NR, TwoSR, IRd);
        if (kp == -1) continue;
        emit(1.0, need(f0.blk(NL, TwoSL, ILd, NL, TwoSL, IL)), true, kp,
             need(c.blk(NR, TwoSR, IRd, NR, TwoSR, IR)), false);
      }
  } else {
    for (int ld = theindex + 2; ld < L; ld++)
      for (int lb = ld + 1; lb < L; lb++) {
        const OpT& c = Lt->C[lb - ld][ld - theindex];
        const OpT& f0 = Rt->F0[lb - ld][ld - theindex - 2];
        const int ILd = irrep_prod(IL, c.irrep()), IRd = irrep_prod(IR, f0.irrep());
        const int kp = kap(NL, TwoSL, ILd, N1, N2, TwoJ, NR, TwoSR, IRd);
        if (kp == -1) continue;
        emit(1.0, need(c.blk(NL, TwoSL, IL, NL, TwoSL, ILd)), false, kp,
             need(f0.blk(NR, TwoSR, IR, NR, TwoSR, IRd)), true);
      }
    for (int lb = theindex + 2; lb < L; lb++)
      for (int ld = lb; ld < L; ld++) {
        const OpT& c = Lt->C[ld - lb][lb - theindex];
        const OpT& f0 = Rt->F0[ld - lb][lb - theindex - 2];
        const int ILd = irrep_prod(IL, c.irrep()), IRd = irrep_prod(IR, f0.irrep());
        const int kp = kap(NL, TwoSL, ILd, N1, N2, TwoJ, NR, TwoSR, IRd);
        if (kp == -1) continue;
        emit(1.0, need(c.blk(NL, TwoSL, ILd, NL, TwoSL, IL)), true, kp,
             need(f0.blk(NR, TwoSR, IRd, NR, TwoSR, IR)), false);
      }
  }
}

// CheMPS2/HeffDiagrams2.cpp:651-848
void HeffEmitter::d2a3spin1() {
  for (int SLd = TwoSL - 2; SLd <= TwoSL + 2; SLd += 2)
    for (int SRd = TwoSR - 2; SRd <= TwoSR + 2; SRd += 2) {
      if (SLd < 0 || SRd < 0 || abs(SLd - SRd) > TwoJ) continue;
      const double w = wigner6j(SLd, SRd, TwoJ, TwoSR, TwoSL, 2);
      const double p1 = heff_phase(SLd + SRd + TwoJ + 2) * sqrt((TwoSR + 1) * (SLd + 1.0)) * w;
      const double p2 = heff_phase(TwoSL + TwoSR + TwoJ + 2) * sqrt((SRd + 1) * (TwoSL + 1.0)) * w;
      if (theindex < L * 0.5) {
        for (int lg = 0; lg < theindex; lg++)
          for (int la = lg + 1; la < theindex; la++) {
            const OpT& f1 = Lt->F1[la - lg][theindex - 1 - la];
            const OpT& d = Rt->D[la - lg][theindex + 1 - la];
            const int ILd = irrep_prod(IL, f1.irrep()), IRd = irrep_prod(IR, d.irrep());
            const int kp = kap(NL, SLd, ILd, N1, N2, TwoJ, NR, SRd, IRd);
            if (kp == -1) continue;
            emit(p1, need(f1.blk(NL, TwoSL, IL, NL, SLd, ILd)), false, kp,
                 need(d.blk(NR, TwoSR, IR, NR, SRd, IRd)), true);
          }
        for (int la = 0; la < theindex; la++)
          for (int lg = la; lg < theindex; lg++) {
            const OpT& f1 = Lt->F1[lg - la][theindex - 1 - lg];
            const OpT& d = Rt->D[lg - la][theindex + 1 - lg];
            const int ILd = irrep_prod(IL, f1.irrep()), IRd = irrep_prod(IR, d.irrep());
            const int kp = kap(NL, SLd, ILd, N1, N2, TwoJ, NR, SRd, IRd);
            if (kp == -1) continue;
            emit(p2, need(f1.blk(NL, SLd, ILd, NL, TwoSL, IL)), true, kp,
                 need(d.blk(NR, SRd, IRd, NR, TwoSR, IR)), false);
          }
      } else {
        for (int ld = theindex + 2; ld < L; ld++)
          for (int lb = ld + 1; lb < L; lb++) {
            const OpT& d = Lt->D[lb - ld][ld - theindex];
            const OpT& f1 = Rt->F1[lb - ld][ld - theindex - 2];
            const int ILd = irrep_prod(IL, d.irrep()), IRd = irrep_prod(IR, f1.irrep());
            const int kp = kap(NL, SLd, ILd, N1, N2, TwoJ, NR, SRd, IRd);
            if (kp == -1) continue;
            emit(p1, need(d.blk(NL, TwoSL, IL, NL, SLd, ILd)), false, kp,
                 need(f1.blk(NR, TwoSR, IR, NR, SRd, IRd)), true);
          }
        for (int lb = theindex + 2; lb < L; lb++)
          for (int ld = lb; ld < L; ld++) {
            const OpT& d = Lt->D[ld - lb][lb - theindex];
            const OpT& f1 = Rt->F1[ld - lb][lb - theindex - 2];
            const int ILd = irrep_prod(IL, d.irrep()), IRd = irrep_prod(IR, f1.irrep());
            const int kp = kap(NL, SLd, ILd, N1, N2, TwoJ, NR, SRd, IRd);
            if (kp == -1) continue;
            emit(p2, need(d.blk(NL, SLd, ILd, NL, TwoSL, IL)), true, kp,
                 need(f1.blk(NR, SRd, IRd, NR, TwoSR, IR)), false);
          }
      }
    }
}

// CheMPS2/HeffDiagrams2.cpp:850-921
void HeffEmitter::d2b1and2b2() {
  const OpT& a = Lt->A[0][0];
  if (N1 == 0 && dL(NL - 2, TwoSL, IL) > 0) {
    const int kp = kap(NL - 2, TwoSL, IL, 2, N2, TwoJ, NR, TwoSR, IR);
    if (kp != -1) emit(sqrt(2.0), need(a.blk(NL - 2, TwoSL, IL, NL, TwoSL, IL)), true, kp, kNo, false);
  }
  if (N1 == 2 && dL(NL + 2, TwoSL, IL) > 0) {
    const int kp = kap(NL + 2, TwoSL, IL, 0, N2, TwoJ, NR, TwoSR, IR);
    if (kp != -1) emit(sqrt(2.0), need(a.blk(NL, TwoSL, IL, NL + 2, TwoSL, IL)), false, kp, kNo, false);
  }
}

// CheMPS2/HeffDiagrams2.cpp:923-994
void HeffEmitter::d2c1and2c2() {
  const OpT& a = Lt->A[0][1];
  if (N2 == 0 && dL(NL - 2, TwoSL, IL) > 0) {
    const int kp = kap(NL - 2, TwoSL, IL, N1, 2, TwoJ, NR, TwoSR, IR);
    if (kp != -1) emit(sqrt(2.0), need(a.blk(NL - 2, TwoSL, IL, NL, TwoSL, IL)), true, kp, kNo, false);
  }
  if (N2 == 2 && dL(NL + 2, TwoSL, IL) > 0) {
    const int kp = kap(NL + 2, TwoSL, IL, N1, 0, TwoJ, NR, TwoSR, IR);
    if (kp != -1) emit(sqrt(2.0), need(a.blk(NL, TwoSL, IL, NL + 2, TwoSL, IL)), false, kp, kNo, false);
  }
}

// CheMPS2/HeffDiagrams2.cpp:996-1058
void HeffEmitter::d2dall() {
  const int i = theindex;
  if (N1 == 2 && N2 == 0) {
    const int kp = kap(NL, TwoSL, IL, 0, 2, 0, NR, TwoSR, IR);
    if (kp != -1) emit_scalar(V(i, i, i + 1, i + 1), kp);
  }
  if (N1 == 0 && N2 == 2) {
    const int kp = kap(NL, TwoSL, IL, 2, 0, 0, NR, TwoSR, IR);
    if (kp != -1) emit_scalar(V(i, i, i + 1, i + 1), kp);
  }
  if (N1 == 2 && N2 == 2) emit_scalar(4 * V(i, i + 1, i, i + 1) - 2 * V(i, i + 1, i + 1, i), ik);
  if (N1 == 1 && N2 == 1) {
    const int fase = (TwoJ == 0) ? 1 : -1;
    emit_scalar(V(i, i + 1, i, i + 1) + fase * V(i, i + 1, i + 1, i), ik);
  }
  if (N1 == 2 && N2 == 1) emit_scalar(2 * V(i, i + 1, i, i + 1) - V(i, i + 1, i + 1, i), ik);
  if (N1 == 1 && N2 == 2) emit_scalar(2 * V(i, i + 1, i, i + 1) - V(i, i + 1, i + 1, i), ik);
}

// CheMPS2/HeffDiagrams2.cpp:1060-1121
void HeffEmitter::d2e1and2e2() {
  const OpT& a = Rt->A[0][1];
  if (N1 == 2) {
    const int kp = kap(NL, TwoSL, IL, 0, N2, TwoJ, NR - 2, TwoSR, IR);
    if (kp != -1) emit(sqrt(2.0), kNo, false, kp, need(a.blk(NR - 2, TwoSR, IR, NR, TwoSR, IR)), false);
  }
  if (N1 == 0) {
    const int kp = kap(NL, TwoSL, IL, 2, N2, TwoJ, NR + 2, TwoSR, IR);
    if (kp != -1) emit(sqrt(2.0), kNo, false, kp, need(a.blk(NR, TwoSR, IR, NR + 2, TwoSR, IR)), true);
  }
}

// CheMPS2/HeffDiagrams2.cpp:1123-1184
void HeffEmitter::d2f1and2f2() {
  const OpT& a = Rt->A[0][0];
  if (N2 == 2) {
    const int kp = kap(NL, TwoSL, IL, N1, 0, TwoJ, NR - 2, TwoSR, IR);
    if (kp != -1) emit(sqrt(2.0), kNo, false, kp, need(a.blk(NR - 2, TwoSR, IR, NR, TwoSR, IR)), false);
  }
  if (N2 == 0) {
    const int kp = kap(NL, TwoSL, IL, N1, 2, TwoJ, NR + 2, TwoSR, IR);
    if (kp != -1) emit(sqrt(2.0), kNo, false, kp, need(a.blk(NR, TwoSR, IR, NR + 2, TwoSR, IR)), true);
  }
}

// CheMPS2/HeffDiagrams2.cpp:1186-1212
void HeffEmitter::d2b3spin0() {
  if (N1 == 0) return;
  const Blk c = need(Lt->C[0][0].blk(NL, TwoSL, IL, NL, TwoSL, IL));
  emit(((N1 == 2) ? 1.0 : 0.5) * sqrt(2.0), c, true, ik, kNo, false);
}
// CheMPS2/HeffDiagrams2.cpp:1214-1240
void HeffEmitter::d2c3spin0() {
  if (N2 == 0) return;
  const Blk c = need(Lt->C[0][1].blk(NL, TwoSL, IL, NL, TwoSL, IL));
  emit(((N2 == 2) ? 1.0 : 0.5) * sqrt(2.0), c, true, ik, kNo, false);
}
// CheMPS2/HeffDiagrams2.cpp:1242-1267
void HeffEmitter::d2e3spin0() {
  if (N1 == 0) return;
  const Blk c = need(Rt->C[0][1].blk(NR, TwoSR, IR, NR, TwoSR, IR));
  emit(((N1 == 2) ? 1.0 : 0.5) * sqrt(2.0), kNo, false, ik, c, false);
}
// CheMPS2/HeffDiagrams2.cpp:1269-1294
void HeffEmitter::d2f3spin0() {
  if (N2 == 0) return;
  const Blk c = need(Rt->C[0][0].blk(NR, TwoSR, IR, NR, TwoSR, IR));
  emit(((N2 == 2) ? 1.0 : 0.5) * sqrt(2.0), kNo, false, ik, c, false);
}

// CheMPS2/HeffDiagrams2.cpp:1296-1348 (2b3spin1) and :1350-1402 (2c3spin1): the D
// operator of orbital theindex (2b) or theindex + 1 (2c) acting from the left.
namespace {
void d2bc3spin1_impl(HeffEmitter& h, const OpT& D, bool is_b) {
  const int Nme = is_b ? h.N1 : h.N2;
  if (Nme != 1) return;
  const int Nother = is_b ? h.N2 : h.N1;
  for (int SLd = h.TwoSL - 2; SLd <= h.TwoSL + 2; SLd += 2) {
    if (h.dL(h.NL, SLd, h.IL) <= 0) continue;
    const Blk Db = HeffEmitter::need(D.blk(h.NL, SLd, h.IL, h.NL, h.TwoSL, h.IL));
    const int TwoSo = (Nother == 1) ? 1 : 0;
    const int TwoJstart = ((h.TwoSR != SLd) || (TwoSo == 0)) ? 1 + TwoSo : 0;
    for (int TJd = TwoJstart; TJd <= 1 + TwoSo; TJd += 2) {
      if (abs(SLd - h.TwoSR) > TJd) continue;
      const int kp = h.kap(h.NL, SLd, h.IL, h.N1, h.N2, TJd, h.NR, h.TwoSR, h.IR);
      if (kp == -1) continue;
      const int fase = is_b ? heff_phase(SLd + h.TwoSR + h.TwoJ + TwoSo + TJd - 1)
                            : heff_phase(SLd + h.TwoSR + 2 * h.TwoJ + TwoSo - 1);
      const double alpha = fase * sqrt(3.0 * (h.TwoJ + 1) * (TJd + 1) * (h.TwoSL + 1)) *
                           wigner6j(TJd, h.TwoJ, 2, 1, 1, TwoSo) *
                           wigner6j(TJd, h.TwoJ, 2, h.TwoSL, SLd, h.TwoSR);
      h.emit(alpha, Db, true, kp, kNo, false);
    }
  }
}
// CheMPS2/HeffDiagrams2.cpp:1404-1455 (2e3spin1) and :1457-1509 (2f3spin1)
void d2ef3spin1_impl(HeffEmitter& h, const OpT& D, bool is_e) {
  const int Nme = is_e ? h.N1 : h.N2;
  if (Nme != 1) return;
  const int Nother = is_e ? h.N2 : h.N1;
  for (int SRd = h.TwoSR - 2; SRd <= h.TwoSR + 2; SRd += 2) {
    if (h.dR(h.NR, SRd, h.IR) <= 0) continue;
    const Blk Db = HeffEmitter::need(D.blk(h.NR, SRd, h.IR, h.NR, h.TwoSR, h.IR));
    const int TwoSo = (Nother == 1) ? 1 : 0;
    const int TwoJstart = ((SRd != h.TwoSL) || (TwoSo == 0)) ? 1 + TwoSo : 0;
    for (int TJd = TwoJstart; TJd <= 1 + TwoSo; TJd += 2) {
      if (abs(h.TwoSL - SRd) > TJd) continue;
      const int kp = h.kap(h.NL, h.TwoSL, h.IL, h.N1, h.N2, TJd, h.NR, SRd, h.IR);
      if (kp == -1) continue;
      const int fase = is_e ? heff_phase(SRd + h.TwoSL + 2 * h.TwoJ + TwoSo + 1)
                            : heff_phase(SRd + h.TwoSL + h.TwoJ + TwoSo + TJd + 1);
      const double alpha = fase * sqrt(3.0 * (h.TwoJ + 1) * (TJd + 1) * (SRd + 1)) *
                           wigner6j(TJd, h.TwoJ, 2, 1, 1, TwoSo) *
                           wigner6j(TJd, h.TwoJ, 2, h.TwoSR, SRd, h.TwoSL);
      h.emit(alpha, kNo, false, kp, Db, false);
    }
  }
}
}  // namespace

void HeffEmitter::d2b3spin1() { d2bc3spin1_impl(*this, Lt->D[0][0], true); }
void HeffEmitter::d2c3spin1() { d2bc3spin1_impl(*this, Lt->D[0][1], false); }
void HeffEmitter::d2e3spin1() { d2ef3spin1_impl(*this, Rt->D[0][1], true); }
void HeffEmitter::d2f3spin1() { d2ef3spin1_impl(*this, Rt->D[0][0], false); }

#undef need

}  // namespace c2g
