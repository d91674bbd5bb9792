// Heff diagrams 4A (complementary pair operators of the two sites on the left, acting
// with the two local sites) and 4J (the same on the right), CheMPS2/HeffDiagrams4.cpp.
// Notation of the helpers, for an operator block on the left (L*) or right (R*):
//   LT: Y += f * O(down -> up)^T * X[kp]      LN: Y += f * O(up -> down) * X[kp]
//   RN: Y += f * X[kp] * O(down -> up)        RT: Y += f * X[kp] * O(up -> down)^T
#include "heff_impl.hpp"

namespace c2g {

using std::abs;
using std::sqrt;

namespace {
const Blk kNo;
struct H4 {
  HeffEmitter& h;
  void LT(const OpT& o, int n, int s, int i, double f, int kp) {
    if (kp == -1) return;
    h.emit(f, HeffEmitter::need(o.blk(n, s, i, h.NL, h.TwoSL, h.IL)), true, kp, kNo, false);
  }
  void LN(const OpT& o, int n, int s, int i, double f, int kp) {
    if (kp == -1) return;
    h.emit(f, HeffEmitter::need(o.blk(h.NL, h.TwoSL, h.IL, n, s, i)), false, kp, kNo, false);
  }
  void RN(const OpT& o, int n, int s, int i, double f, int kp) {
    if (kp == -1) return;
    h.emit(f, kNo, false, kp, HeffEmitter::need(o.blk(n, s, i, h.NR, h.TwoSR, h.IR)), false);
  }
  void RT(const OpT& o, int n, int s, int i, double f, int kp) {
    if (kp == -1) return;
    h.emit(f, kNo, false, kp, HeffEmitter::need(o.blk(h.NR, h.TwoSR, h.IR, n, s, i)), true);
  }
};
inline int ph(int x) { return heff_phase(x); }
}  // namespace

// CheMPS2/HeffDiagrams4.cpp:28-167
void HeffEmitter::d4A1and4A2spin0() {
  H4 e{*this};
  const OpT& A = Lt->A[1][0];
  const int ILd = irrep_prod(IL, A.irrep());
  auto k = [&](int nl, int n1, int n2, int tj) { return kap(nl, TwoSL, ILd, n1, n2, tj, NR, TwoSR, IR); };
  if (N1 == 0 && N2 == 0) e.LT(A, NL - 2, TwoSL, ILd, 1.0, k(NL - 2, 1, 1, 0));
  if (N1 == 1 && N2 == 0) e.LT(A, NL - 2, TwoSL, ILd, -sqrt(0.5), k(NL - 2, 2, 1, 1));
  if (N1 == 0 && N2 == 1) e.LT(A, NL - 2, TwoSL, ILd, -sqrt(0.5), k(NL - 2, 1, 2, 1));
  if (N1 == 1 && N2 == 1 && TwoJ == 0) {
    e.LT(A, NL - 2, TwoSL, ILd, -1.0, k(NL - 2, 2, 2, 0));
    e.LN(A, NL + 2, TwoSL, ILd, 1.0, k(NL + 2, 0, 0, 0));
  }
  if (N1 == 2 && N2 == 1) e.LN(A, NL + 2, TwoSL, ILd, -sqrt(0.5), k(NL + 2, 1, 0, 1));
  if (N1 == 1 && N2 == 2) e.LN(A, NL + 2, TwoSL, ILd, -sqrt(0.5), k(NL + 2, 0, 1, 1));
  if (N1 == 2 && N2 == 2) e.LN(A, NL + 2, TwoSL, ILd, -1.0, k(NL + 2, 1, 1, 0));
}

// CheMPS2/HeffDiagrams4.cpp:169-342
void HeffEmitter::d4A1and4A2spin1() {
  H4 e{*this};
  const OpT& B = Lt->B[1][0];
  const int ILd = irrep_prod(IL, B.irrep());
  auto k = [&](int nl, int sl, int n1, int n2, int tj) { return kap(nl, sl, ILd, n1, n2, tj, NR, TwoSR, IR); };
  if (N1 == 0 && N2 == 0)
    for (int s = TwoSL - 2; s <= TwoSL + 2; s += 2)
      if (s >= 0) e.LT(B, NL - 2, s, ILd, 1.0, k(NL - 2, s, 1, 1, 2));
  if (N1 == 1 && N2 == 0)
    for (int s = TwoSL - 2; s <= TwoSL + 2; s += 2)
      if (abs(s - TwoSR) <= 1 && s >= 0)
        e.LT(B, NL - 2, s, ILd, ph(s + TwoSR + 1) * sqrt(3.0 * (TwoSL + 1)) * wigner6j(1, 1, 2, TwoSL, s, TwoSR),
             k(NL - 2, s, 2, 1, 1));
  if (N1 == 0 && N2 == 1)
    for (int s = TwoSL - 2; s <= TwoSL + 2; s += 2)
      if (abs(s - TwoSR) <= 1 && s >= 0)
        e.LT(B, NL - 2, s, ILd, ph(s + TwoSR + 3) * sqrt(3.0 * (TwoSL + 1)) * wigner6j(1, 1, 2, TwoSL, s, TwoSR),
             k(NL - 2, s, 1, 2, 1));
  if (N1 == 1 && N2 == 1 && TwoJ == 2) {
    const int s = TwoSR;
    e.LT(B, NL - 2, s, ILd, ph(s - TwoSL) * sqrt((TwoSL + 1.0) / (s + 1.0)), k(NL - 2, s, 2, 2, 0));
    e.LN(B, NL + 2, s, ILd, 1.0, k(NL + 2, s, 0, 0, 0));
  }
  if (N1 == 2 && N2 == 1)
    for (int s = TwoSL - 2; s <= TwoSL + 2; s += 2)
      if (abs(s - TwoSR) <= 1 && s >= 0)
        e.LN(B, NL + 2, s, ILd, ph(TwoSL + TwoSR + 1) * sqrt(3.0 * (s + 1)) * wigner6j(1, 1, 2, TwoSL, s, TwoSR),
             k(NL + 2, s, 1, 0, 1));
  if (N1 == 1 && N2 == 2)
    for (int s = TwoSL - 2; s <= TwoSL + 2; s += 2)
      if (abs(s - TwoSR) <= 1 && s >= 0)
        e.LN(B, NL + 2, s, ILd, ph(TwoSL + TwoSR + 3) * sqrt(3.0 * (s + 1)) * wigner6j(1, 1, 2, TwoSL, s, TwoSR),
             k(NL + 2, s, 0, 1, 1));
  if (N1 == 2 && N2 == 2)
    for (int s = TwoSL - 2; s <= TwoSL + 2; s += 2)
      if (s >= 0) e.LN(B, NL + 2, s, ILd, ph(s - TwoSL) * sqrt((s + 1.0) / (TwoSL + 1.0)), k(NL + 2, s, 1, 1, 2));
}

// CheMPS2/HeffDiagrams4.cpp:344-488
void HeffEmitter::d4A3and4A4spin0() {
  H4 e{*this};
  const OpT& C = Lt->C[1][0];
  const int ILd = irrep_prod(IL, C.irrep());
  auto k = [&](int n1, int n2, int tj) { return kap(NL, TwoSL, ILd, n1, n2, tj, NR, TwoSR, IR); };
  if (N1 == 1 && N2 == 0) e.LT(C, NL, TwoSL, ILd, sqrt(0.5), k(0, 1, 1));
  if (N1 == 1 && N2 == 1 && TwoJ == 0) e.LT(C, NL, TwoSL, ILd, 1.0, k(0, 2, 0));
  if (N1 == 2 && N2 == 0) e.LT(C, NL, TwoSL, ILd, 1.0, k(1, 1, 0));
  if (N1 == 2 && N2 == 1) e.LT(C, NL, TwoSL, ILd, -sqrt(0.5), k(1, 2, 1));
  if (N1 == 0 && N2 == 1) e.LN(C, NL, TwoSL, ILd, sqrt(0.5), k(1, 0, 1));
  if (N1 == 0 && N2 == 2) e.LN(C, NL, TwoSL, ILd, 1.0, k(1, 1, 0));
  if (N1 == 1 && N2 == 1 && TwoJ == 0) e.LN(C, NL, TwoSL, ILd, 1.0, k(2, 0, 0));
  if (N1 == 1 && N2 == 2) e.LN(C, NL, TwoSL, ILd, -sqrt(0.5), k(2, 1, 1));
}

// CheMPS2/HeffDiagrams4.cpp:490-668
void HeffEmitter::d4A3and4A4spin1() {
  H4 e{*this};
  const OpT& D = Lt->D[1][0];
  const int ILd = irrep_prod(IL, D.irrep());
  auto k = [&](int s, int n1, int n2, int tj) { return kap(NL, s, ILd, n1, n2, tj, NR, TwoSR, IR); };
  auto f6 = [&](int s) { return sqrt(3.0 * (TwoSL + 1)) * wigner6j(1, 1, 2, TwoSL, s, TwoSR); };
  auto g6 = [&](int s) { return sqrt(3.0 * (s + 1)) * wigner6j(1, 1, 2, TwoSL, s, TwoSR); };
  if (N1 == 1 && N2 == 0)
    for (int s = TwoSL - 2; s <= TwoSL + 2; s += 2)
      if (abs(s - TwoSR) <= 1 && s >= 0) e.LT(D, NL, s, ILd, ph(s + TwoSR + 1) * f6(s), k(s, 0, 1, 1));
  if (N1 == 1 && N2 == 1 && TwoJ == 2) {
    const int s = TwoSR;
    e.LT(D, NL, s, ILd, ph(s - TwoSL) * sqrt((TwoSL + 1.0) / (s + 1.0)), k(s, 0, 2, 0));
  }
  if (N1 == 2 && N2 == 0)
    for (int s = TwoSL - 2; s <= TwoSL + 2; s += 2)
      if (s >= 0) e.LT(D, NL, s, ILd, -1.0, k(s, 1, 1, 2));
  if (N1 == 2 && N2 == 1)
    for (int s = TwoSL - 2; s <= TwoSL + 2; s += 2)
      if (abs(s - TwoSR) <= 1 && s >= 0) e.LT(D, NL, s, ILd, ph(s + TwoSR + 1) * f6(s), k(s, 1, 2, 1));
  if (N1 == 0 && N2 == 1)
    for (int s = TwoSL - 2; s <= TwoSL + 2; s += 2)
      if (abs(s - TwoSR) <= 1 && s >= 0) e.LN(D, NL, s, ILd, ph(TwoSL + TwoSR + 1) * g6(s), k(s, 1, 0, 1));
  if (N1 == 0 && N2 == 2)
    for (int s = TwoSL - 2; s <= TwoSL + 2; s += 2)
      if (s >= 0) e.LN(D, NL, s, ILd, ph(TwoSL - s) * sqrt((s + 1.0) / (TwoSL + 1.0)), k(s, 1, 1, 2));
  if (N1 == 1 && N2 == 1 && TwoJ == 2) e.LN(D, NL, TwoSR, ILd, -1.0, k(TwoSR, 2, 0, 0));
  if (N1 == 1 && N2 == 2)
    for (int s = TwoSL - 2; s <= TwoSL + 2; s += 2)
      if (abs(s - TwoSR) <= 1 && s >= 0) e.LN(D, NL, s, ILd, ph(TwoSL + TwoSR + 1) * g6(s), k(s, 2, 1, 1));
}

// CheMPS2/HeffDiagrams4.cpp:4277-4415
void HeffEmitter::d4J1and4J2spin0() {
  H4 e{*this};
  const OpT& A = Rt->A[1][0];
  const int IRd = irrep_prod(IR, A.irrep());
  auto k = [&](int n1, int n2, int tj, int nr) { return kap(NL, TwoSL, IL, n1, n2, tj, nr, TwoSR, IRd); };
  const bool up = dR(NR + 2, TwoSR, IRd) > 0, dn = dR(NR - 2, TwoSR, IRd) > 0;
  if (N1 == 0 && N2 == 0 && up) e.RT(A, NR + 2, TwoSR, IRd, 1.0, k(1, 1, 0, NR + 2));
  if (N1 == 1 && N2 == 0 && up) e.RT(A, NR + 2, TwoSR, IRd, -sqrt(0.5), k(2, 1, 1, NR + 2));
  if (N1 == 0 && N2 == 1 && up) e.RT(A, NR + 2, TwoSR, IRd, -sqrt(0.5), k(1, 2, 1, NR + 2));
  if (N1 == 1 && N2 == 1 && TwoJ == 0) {
    if (up) e.RT(A, NR + 2, TwoSR, IRd, -1.0, k(2, 2, 0, NR + 2));
    if (dn) e.RN(A, NR - 2, TwoSR, IRd, 1.0, k(0, 0, 0, NR - 2));
  }
  if (N1 == 2 && N2 == 1 && dn) e.RN(A, NR - 2, TwoSR, IRd, -sqrt(0.5), k(1, 0, 1, NR - 2));
  if (N1 == 1 && N2 == 2 && dn) e.RN(A, NR - 2, TwoSR, IRd, -sqrt(0.5), k(0, 1, 1, NR - 2));
  if (N1 == 2 && N2 == 2 && dn) e.RN(A, NR - 2, TwoSR, IRd, -1.0, k(1, 1, 0, NR - 2));
}

// CheMPS2/HeffDiagrams4.cpp:4417-4586
void HeffEmitter::d4J1and4J2spin1() {
  H4 e{*this};
  const OpT& B = Rt->B[1][0];
  const int IRd = irrep_prod(IR, B.irrep());
  auto k = [&](int n1, int n2, int tj, int nr, int s) { return kap(NL, TwoSL, IL, n1, n2, tj, nr, s, IRd); };
  if (N1 == 0 && N2 == 0)
    for (int s = TwoSR - 2; s <= TwoSR + 2; s += 2)
      if (dR(NR + 2, s, IRd) > 0) e.RT(B, NR + 2, s, IRd, sqrt((s + 1.0) / (TwoSR + 1.0)), k(1, 1, 2, NR + 2, s));
  if (N1 == 1 && N2 == 0)
    for (int s = TwoSR - 2; s <= TwoSR + 2; s += 2)
      if (abs(TwoSL - s) <= 1 && dR(NR + 2, s, IRd) > 0)
        e.RT(B, NR + 2, s, IRd, ph(TwoSL + s + 3) * sqrt(3.0 * (s + 1)) * wigner6j(1, 1, 2, TwoSR, s, TwoSL),
             k(2, 1, 1, NR + 2, s));
  if (N1 == 0 && N2 == 1)
    for (int s = TwoSR - 2; s <= TwoSR + 2; s += 2)
      if (abs(TwoSL - s) <= 1 && dR(NR + 2, s, IRd) > 0)
        e.RT(B, NR + 2, s, IRd, ph(TwoSL + s + 1) * sqrt(3.0 * (s + 1)) * wigner6j(1, 1, 2, TwoSR, s, TwoSL),
             k(1, 2, 1, NR + 2, s));
  if (N1 == 1 && N2 == 1 && TwoJ == 2) {
    const int s = TwoSL;
    if (dR(NR + 2, s, IRd) > 0) e.RT(B, NR + 2, s, IRd, ph(TwoSR - s), k(2, 2, 0, NR + 2, s));
    if (dR(NR - 2, s, IRd) > 0) e.RN(B, NR - 2, s, IRd, sqrt((TwoSR + 1.0) / (s + 1.0)), k(0, 0, 0, NR - 2, s));
  }
  if (N1 == 2 && N2 == 1)
    for (int s = TwoSR - 2; s <= TwoSR + 2; s += 2)
      if (abs(TwoSL - s) <= 1 && dR(NR - 2, s, IRd) > 0)
        e.RN(B, NR - 2, s, IRd, ph(TwoSL + TwoSR + 3) * sqrt(3.0 * (TwoSR + 1)) * wigner6j(1, 1, 2, s, TwoSR, TwoSL),
             k(1, 0, 1, NR - 2, s));
  if (N1 == 1 && N2 == 2)
    for (int s = TwoSR - 2; s <= TwoSR + 2; s += 2)
      if (abs(TwoSL - s) <= 1 && dR(NR - 2, s, IRd) > 0)
        e.RN(B, NR - 2, s, IRd, ph(TwoSL + TwoSR + 1) * sqrt(3.0 * (TwoSR + 1)) * wigner6j(1, 1, 2, s, TwoSR, TwoSL),
             k(0, 1, 1, NR - 2, s));
  if (N1 == 2 && N2 == 2)
    for (int s = TwoSR - 2; s <= TwoSR + 2; s += 2)
      if (dR(NR - 2, s, IRd) > 0) e.RN(B, NR - 2, s, IRd, ph(TwoSR - s), k(1, 1, 2, NR - 2, s));
}

// CheMPS2/HeffDiagrams4.cpp:4588-4712
void HeffEmitter::d4J3and4J4spin0() {
  H4 e{*this};
  const OpT& C = Rt->C[1][0];
  const int IRd = irrep_prod(IR, C.irrep());
  if (dR(NR, TwoSR, IRd) <= 0) return;
  auto k = [&](int n1, int n2, int tj) { return kap(NL, TwoSL, IL, n1, n2, tj, NR, TwoSR, IRd); };
  if (N1 == 1 && N2 == 0) e.RN(C, NR, TwoSR, IRd, sqrt(0.5), k(0, 1, 1));
  if (N1 == 2 && N2 == 0) e.RN(C, NR, TwoSR, IRd, 1.0, k(1, 1, 0));
  if (N1 == 1 && N2 == 1 && TwoJ == 0) e.RN(C, NR, TwoSR, IRd, 1.0, k(0, 2, 0));
  if (N1 == 2 && N2 == 1) e.RN(C, NR, TwoSR, IRd, -sqrt(0.5), k(1, 2, 1));
  if (N1 == 0 && N2 == 1) e.RT(C, NR, TwoSR, IRd, sqrt(0.5), k(1, 0, 1));
  if (N1 == 1 && N2 == 1 && TwoJ == 0) e.RT(C, NR, TwoSR, IRd, 1.0, k(2, 0, 0));
  if (N1 == 0 && N2 == 2) e.RT(C, NR, TwoSR, IRd, 1.0, k(1, 1, 0));
  if (N1 == 1 && N2 == 2) e.RT(C, NR, TwoSR, IRd, -sqrt(0.5), k(2, 1, 1));
}

// CheMPS2/HeffDiagrams4.cpp:4714-4845
void HeffEmitter::d4J3and4J4spin1() {
  H4 e{*this};
  const OpT& D = Rt->D[1][0];
  const int IRd = irrep_prod(IR, D.irrep());
  for (int s = TwoSR - 2; s <= TwoSR + 2; s += 2) {
    if (dR(NR, s, IRd) <= 0) continue;
    auto k = [&](int n1, int n2, int tj) { return kap(NL, TwoSL, IL, n1, n2, tj, NR, s, IRd); };
    const double fa = sqrt(3.0 * (s + 1)) * wigner6j(1, 1, 2, TwoSR, s, TwoSL);
    const double fb = sqrt(3.0 * (TwoSR + 1)) * wigner6j(1, 1, 2, TwoSR, s, TwoSL);
    if (N1 == 1 && N2 == 0 && abs(TwoSL - s) <= 1) e.RN(D, NR, s, IRd, ph(TwoSL + s + 3) * fa, k(0, 1, 1));
    if (N1 == 2 && N2 == 0) e.RN(D, NR, s, IRd, -sqrt((s + 1.0) / (TwoSR + 1.0)), k(1, 1, 2));
    if (N1 == 1 && N2 == 1 && TwoJ == 2 && TwoSL == s) e.RN(D, NR, s, IRd, ph(TwoSR - s), k(0, 2, 0));
    if (N1 == 2 && N2 == 1 && abs(TwoSL - s) <= 1) e.RN(D, NR, s, IRd, ph(TwoSL + s + 3) * fa, k(1, 2, 1));
    if (N1 == 0 && N2 == 1 && abs(TwoSL - s) <= 1) e.RT(D, NR, s, IRd, ph(TwoSL + TwoSR + 3) * fb, k(1, 0, 1));
    if (N1 == 1 && N2 == 1 && TwoJ == 2 && TwoSL == s) e.RT(D, NR, s, IRd, -sqrt((TwoSR + 1.0) / (s + 1.0)), k(2, 0, 0));
    if (N1 == 0 && N2 == 2) e.RT(D, NR, s, IRd, ph(TwoSR - s), k(1, 1, 2));
    if (N1 == 1 && N2 == 2 && abs(TwoSL - s) <= 1) e.RT(D, NR, s, IRd, ph(TwoSL + TwoSR + 3) * fb, k(2, 1, 1));
  }
}

}  // namespace c2g
