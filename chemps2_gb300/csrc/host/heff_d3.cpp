// Heff diagram group 3 as contraction tasks (CheMPS2/HeffDiagrams3.cpp). The
// "dcopy Q; daxpy V*L" temporaries of the reference become combined blocks.
#include "heff_impl.hpp"

namespace c2g {

using std::abs;
using std::sqrt;

static const Blk kNo;

// Q block of `q` plus sum_l V(l) * (creator on l), l over `sites` with orbital irrep `ir`.
static Blk q_plus_l(HeffEmitter& h, const OpT& q, const BoundaryOps* side, const std::vector<int>& sites,
                    int ir, double (*coef)(HeffEmitter&, int), int n1, int s1, int i1, int n2, int s2, int i2,
                    int rows, int cols) {
  thread_local std::vector<std::pair<double, Blk>> parts;  // reused: no allocation per block
  parts.assign(1, {1.0, HeffEmitter::need(q.blk(n1, s1, i1, n2, s2, i2))});
  for (int l : sites)
    if (h.irr(l) == ir) parts.push_back({coef(h, l), HeffEmitter::need(side->Lop(l).blk(n1, s1, i1, n2, s2, i2))});
  return h.combine(parts, rows, cols);
}

static std::vector<int> range(int a, int b) {
  std::vector<int> v;
  for (int i = a; i < b; i++) v.push_back(i);
  return v;
}

// CheMPS2/HeffDiagrams3.cpp:28-159
void HeffEmitter::d3Aand3D() {
  const OpT& Q = Lt->Q[0];
  const int ILd = irrep_prod(IL, irr(theindex));
  const int TwoS2 = (N2 == 1) ? 1 : 0;
  const std::vector<int> left = range(0, theindex);
  auto coef = [](HeffEmitter& h, int l) { return h.V(l, h.theindex, h.theindex, h.theindex); };
  if (N1 == 2) {  // 3A1A and 3D1
    for (int SLd = TwoSL - 1; SLd <= TwoSL + 1; SLd += 2) {
      const int dLd = dL(NL + 1, SLd, ILd);
      if (dLd <= 0) continue;
      const int start = ((TwoSR != SLd) || (TwoS2 == 0)) ? 1 + TwoS2 : 0;
      for (int TJd = start; TJd <= 1 + TwoS2; TJd += 2) {
        if (abs(SLd - TwoSR) > TJd) continue;
        const int kp = kap(NL + 1, SLd, ILd, 1, N2, TJd, NR, TwoSR, IR);
        if (kp == -1) continue;
        const double f = sqrt((TJd + 1) * (SLd + 1.0)) * heff_phase(TwoSL + TwoSR + 2 + TwoS2) *
                         wigner6j(TJd, TwoS2, 1, TwoSL, SLd, TwoSR);
        const Blk W = q_plus_l(*this, Q, Lt, left, irr(theindex), coef, NL, TwoSL, IL, NL + 1, SLd, ILd, dimL, dLd);
        emit(f, W, false, kp, kNo, false);
      }
    }
  }
  if (N1 == 1) {  // 3A1B
    for (int SLd = TwoSL - 1; SLd <= TwoSL + 1; SLd += 2) {
      if (abs(SLd - TwoSR) > TwoS2 || SLd < 0) continue;
      const int kp = kap(NL + 1, SLd, ILd, 0, N2, TwoS2, NR, TwoSR, IR);
      if (kp == -1) continue;
      const double f = sqrt((SLd + 1) * (TwoJ + 1.0)) * heff_phase(TwoSL + TwoSR + 1 + TwoS2) *
                       wigner6j(TwoS2, TwoJ, 1, TwoSL, SLd, TwoSR);
      emit(f, need(Q.blk(NL, TwoSL, IL, NL + 1, SLd, ILd)), false, kp, kNo, false);
    }
  }
  if (N1 == 0) {  // 3A2A
    for (int SLd = TwoSL - 1; SLd <= TwoSL + 1; SLd += 2) {
      if (dL(NL - 1, SLd, ILd) <= 0) continue;
      const int start = ((TwoSR != SLd) || (TwoS2 == 0)) ? 1 + TwoS2 : 0;
      for (int TJd = start; TJd <= 1 + TwoS2; TJd += 2) {
        if (abs(SLd - TwoSR) > TJd) continue;
        const int kp = kap(NL - 1, SLd, ILd, 1, N2, TJd, NR, TwoSR, IR);
        if (kp == -1) continue;
        const double f = heff_phase(SLd + TwoSR + 1 + TwoS2) * sqrt((TwoSL + 1) * (TJd + 1.0)) *
                         wigner6j(TJd, TwoS2, 1, TwoSL, SLd, TwoSR);
        emit(f, need(Q.blk(NL - 1, SLd, ILd, NL, TwoSL, IL)), true, kp, kNo, false);
      }
    }
  }
  if (N1 == 1) {  // 3A2B and 3D2
    for (int SLd = TwoSL - 1; SLd <= TwoSL + 1; SLd += 2) {
      if (abs(SLd - TwoSR) > TwoS2 || SLd < 0) continue;
      const int kp = kap(NL - 1, SLd, ILd, 2, N2, TwoS2, NR, TwoSR, IR);
      if (kp == -1) continue;
      const double f = heff_phase(SLd + TwoSR + 2 + TwoS2) * sqrt((TwoSL + 1) * (TwoJ + 1.0)) *
                       wigner6j(TwoS2, TwoJ, 1, TwoSL, SLd, TwoSR);
      const int dLd = dL(NL - 1, SLd, ILd);
      const Blk W = q_plus_l(*this, Q, Lt, left, irr(theindex), coef, NL - 1, SLd, ILd, NL, TwoSL, IL, dLd, dimL);
      emit(f, W, true, kp, kNo, false);
    }
  }
}

// CheMPS2/HeffDiagrams3.cpp:161-292
void HeffEmitter::d3Band3I() {
  const OpT& Q = Lt->Q[1];
  const int ILd = irrep_prod(IL, irr(theindex + 1));
  const int TwoS1 = (N1 == 1) ? 1 : 0;
  const std::vector<int> left = range(0, theindex);
  auto coef = [](HeffEmitter& h, int l) { return h.V(l, h.theindex + 1, h.theindex + 1, h.theindex + 1); };
  if (N2 == 2) {  // 3B1A and 3I2
    for (int SLd = TwoSL - 1; SLd <= TwoSL + 1; SLd += 2) {
      const int dLd = dL(NL + 1, SLd, ILd);
      if (dLd <= 0) continue;
      const int start = ((TwoSR != SLd) || (TwoS1 == 0)) ? 1 + TwoS1 : 0;
      for (int TJd = start; TJd <= 1 + TwoS1; TJd += 2) {
        if (abs(SLd - TwoSR) > TJd) continue;
        const int kp = kap(NL + 1, SLd, ILd, N1, 1, TJd, NR, TwoSR, IR);
        if (kp == -1) continue;
        const double f = sqrt((TJd + 1) * (SLd + 1.0)) * heff_phase(TwoSL + TwoSR + 3 - TJd) *
                         wigner6j(TJd, TwoS1, 1, TwoSL, SLd, TwoSR);
        const Blk W = q_plus_l(*this, Q, Lt, left, irr(theindex + 1), coef, NL, TwoSL, IL, NL + 1, SLd, ILd, dimL, dLd);
        emit(f, W, false, kp, kNo, false);
      }
    }
  }
  if (N2 == 1) {  // 3B1B
    for (int SLd = TwoSL - 1; SLd <= TwoSL + 1; SLd += 2) {
      if (abs(SLd - TwoSR) > TwoS1 || SLd < 0) continue;
      const int kp = kap(NL + 1, SLd, ILd, N1, 0, TwoS1, NR, TwoSR, IR);
      if (kp == -1) continue;
      const double f = sqrt((SLd + 1) * (TwoJ + 1.0)) * heff_phase(TwoSL + TwoSR + 2 - TwoJ) *
                       wigner6j(TwoS1, TwoJ, 1, TwoSL, SLd, TwoSR);
      emit(f, need(Q.blk(NL, TwoSL, IL, NL + 1, SLd, ILd)), false, kp, kNo, false);
    }
  }
  if (N2 == 0) {  // 3B2A
    for (int SLd = TwoSL - 1; SLd <= TwoSL + 1; SLd += 2) {
      if (dL(NL - 1, SLd, ILd) <= 0) continue;
      const int start = ((TwoSR != SLd) || (TwoS1 == 0)) ? 1 + TwoS1 : 0;
      for (int TJd = start; TJd <= 1 + TwoS1; TJd += 2) {
        if (abs(SLd - TwoSR) > TJd) continue;
        const int kp = kap(NL - 1, SLd, ILd, N1, 1, TJd, NR, TwoSR, IR);
        if (kp == -1) continue;
        const double f = heff_phase(SLd + TwoSR + 2 - TJd) * sqrt((TwoSL + 1) * (TJd + 1.0)) *
                         wigner6j(TJd, TwoS1, 1, TwoSL, SLd, TwoSR);
        emit(f, need(Q.blk(NL - 1, SLd, ILd, NL, TwoSL, IL)), true, kp, kNo, false);
      }
    }
  }
  if (N2 == 1) {  // 3B2B and 3I1
    for (int SLd = TwoSL - 1; SLd <= TwoSL + 1; SLd += 2) {
      if (abs(SLd - TwoSR) > TwoS1 || SLd < 0) continue;
      const int kp = kap(NL - 1, SLd, ILd, N1, 2, TwoS1, NR, TwoSR, IR);
      if (kp == -1) continue;
      const double f = heff_phase(SLd + TwoSR + 3 - TwoJ) * sqrt((TwoSL + 1) * (TwoJ + 1.0)) *
                       wigner6j(TwoS1, TwoJ, 1, TwoSL, SLd, TwoSR);
      const int dLd = dL(NL - 1, SLd, ILd);
      const Blk W = q_plus_l(*this, Q, Lt, left, irr(theindex + 1), coef, NL - 1, SLd, ILd, NL, TwoSL, IL, dLd, dimL);
      emit(f, W, true, kp, kNo, false);
    }
  }
}

// CheMPS2/HeffDiagrams3.cpp:294-397
void HeffEmitter::d3C() {
  const int e1 = ((N1 == 1) ? 2 : 0) + ((N2 == 1) ? 2 : 0);
  for (int SLd = TwoSL - 1; SLd <= TwoSL + 1; SLd += 2)  // 3C1
    for (int SRd = TwoSR - 1; SRd <= TwoSR + 1; SRd += 2) {
      if (abs(SLd - SRd) > TwoJ || SLd < 0 || SRd < 0) continue;
      const double f = heff_phase(SLd + TwoSR + TwoJ + 1 + e1) * sqrt((SLd + 1) * (SRd + 1.0)) *
                       wigner6j(TwoSL, TwoSR, TwoJ, SRd, SLd, 1);
      for (int l = theindex + 2; l < L; l++) {
        const int ILd = irrep_prod(IL, irr(l)), IRd = irrep_prod(IR, irr(l));
        const int kp = kap(NL + 1, SLd, ILd, N1, N2, TwoJ, NR + 1, SRd, IRd);
        if (kp == -1) continue;
        emit(f, need(Lt->Qop(l).blk(NL, TwoSL, IL, NL + 1, SLd, ILd)), false, kp,
             need(Rt->Lop(l).blk(NR, TwoSR, IR, NR + 1, SRd, IRd)), true);
      }
    }
  for (int SLd = TwoSL - 1; SLd <= TwoSL + 1; SLd += 2)  // 3C2
    for (int SRd = TwoSR - 1; SRd <= TwoSR + 1; SRd += 2) {
      if (abs(SLd - SRd) > TwoJ || SLd < 0 || SRd < 0) continue;
      const double f = heff_phase(TwoSL + SRd + TwoJ + 1 + e1) * sqrt((TwoSL + 1) * (TwoSR + 1.0)) *
                       wigner6j(TwoSL, TwoSR, TwoJ, SRd, SLd, 1);
      for (int l = theindex + 2; l < L; l++) {
        const int ILd = irrep_prod(IL, irr(l)), IRd = irrep_prod(IR, irr(l));
        const int kp = kap(NL - 1, SLd, ILd, N1, N2, TwoJ, NR - 1, SRd, IRd);
        if (kp == -1) continue;
        emit(f, need(Lt->Qop(l).blk(NL - 1, SLd, ILd, NL, TwoSL, IL)), true, kp,
             need(Rt->Lop(l).blk(NR - 1, SRd, IRd, NR, TwoSR, IR)), false);
      }
    }
}

// CheMPS2/HeffDiagrams3.cpp:399-474
void HeffEmitter::d3Eand3H() {
  if (irr(theindex) != irr(theindex + 1)) return;
  const int i = theindex;
  if (N1 == 2 && N2 == 0) {
    const int kp = kap(NL, TwoSL, IL, 1, 1, 0, NR, TwoSR, IR);
    if (kp != -1) emit_scalar(sqrt(2.0) * V(i, i, i, i + 1), kp);
  }
  if (N1 == 2 && N2 == 1) {
    const int kp = kap(NL, TwoSL, IL, 1, 2, 1, NR, TwoSR, IR);
    if (kp != -1) emit_scalar(-(V(i, i, i, i + 1) + V(i, i + 1, i + 1, i + 1)), kp);
  }
  if (N1 == 1 && N2 == 1 && TwoJ == 0) {
    int kp = kap(NL, TwoSL, IL, 2, 0, 0, NR, TwoSR, IR);
    if (kp != -1) emit_scalar(sqrt(2.0) * V(i, i, i, i + 1), kp);
    kp = kap(NL, TwoSL, IL, 0, 2, 0, NR, TwoSR, IR);
    if (kp != -1) emit_scalar(sqrt(2.0) * V(i, i + 1, i + 1, i + 1), kp);
  }
  if (N1 == 1 && N2 == 2) {
    const int kp = kap(NL, TwoSL, IL, 2, 1, 1, NR, TwoSR, IR);
    if (kp != -1) emit_scalar(-(V(i, i, i, i + 1) + V(i, i + 1, i + 1, i + 1)), kp);
  }
  if (N1 == 0 && N2 == 2) {
    const int kp = kap(NL, TwoSL, IL, 1, 1, 0, NR, TwoSR, IR);
    if (kp != -1) emit_scalar(sqrt(2.0) * V(i, i + 1, i + 1, i + 1), kp);
  }
}

// CheMPS2/HeffDiagrams3.cpp:476-607
void HeffEmitter::d3Kand3F() {
  const OpT& Q = Rt->Q[1];
  const int IRd = irrep_prod(IR, irr(theindex));
  const int TwoS2 = (N2 == 1) ? 1 : 0;
  const std::vector<int> right = range(theindex + 2, L);
  auto coef = [](HeffEmitter& h, int l) { return h.V(h.theindex, h.theindex, h.theindex, l); };
  if (N1 == 1) {  // 3K1A
    for (int SRd = TwoSR - 1; SRd <= TwoSR + 1; SRd += 2) {
      if (abs(TwoSL - SRd) > TwoS2 || SRd < 0) continue;
      const int kp = kap(NL, TwoSL, IL, 0, N2, TwoS2, NR - 1, SRd, IRd);
      if (kp == -1) continue;
      const double f = sqrt((TwoJ + 1) * (TwoSR + 1.0)) * heff_phase(TwoSL + TwoSR + TwoJ + 2 * TwoS2) *
                       wigner6j(TwoS2, TwoJ, 1, TwoSR, SRd, TwoSL);
      emit(f, kNo, false, kp, need(Q.blk(NR - 1, SRd, IRd, NR, TwoSR, IR)), false);
    }
  }
  if (N1 == 2) {  // 3K1B and 3F1
    for (int SRd = TwoSR - 1; SRd <= TwoSR + 1; SRd += 2) {
      const int dRd = dR(NR - 1, SRd, IRd);
      if (dRd <= 0) continue;
      const int start = ((SRd != TwoSL) || (TwoS2 == 0)) ? 1 + TwoS2 : 0;
      for (int TJd = start; TJd <= 1 + TwoS2; TJd += 2) {
        if (abs(TwoSL - SRd) > TJd) continue;
        const int kp = kap(NL, TwoSL, IL, 1, N2, TJd, NR - 1, SRd, IRd);
        if (kp == -1) continue;
        const double f = sqrt((TJd + 1) * (TwoSR + 1.0)) * heff_phase(TwoSL + TwoSR + TJd + 1 + 2 * TwoS2) *
                         wigner6j(TJd, TwoS2, 1, TwoSR, SRd, TwoSL);
        const Blk W = q_plus_l(*this, Q, Rt, right, irr(theindex), coef, NR - 1, SRd, IRd, NR, TwoSR, IR, dRd, dimR);
        emit(f, kNo, false, kp, W, false);
      }
    }
  }
  if (N1 == 0) {  // 3K2A
    for (int SRd = TwoSR - 1; SRd <= TwoSR + 1; SRd += 2) {
      if (dR(NR + 1, SRd, IRd) <= 0) continue;
      const int start = ((SRd != TwoSL) || (TwoS2 == 0)) ? 1 + TwoS2 : 0;
      for (int TJd = start; TJd <= 1 + TwoS2; TJd += 2) {
        if (abs(TwoSL - SRd) > TJd) continue;
        const int kp = kap(NL, TwoSL, IL, 1, N2, TJd, NR + 1, SRd, IRd);
        if (kp == -1) continue;
        const double f = sqrt((TJd + 1) * (SRd + 1.0)) * heff_phase(TwoSL + SRd + TJd + 2 * TwoS2) *
                         wigner6j(TJd, TwoS2, 1, TwoSR, SRd, TwoSL);
        emit(f, kNo, false, kp, need(Q.blk(NR, TwoSR, IR, NR + 1, SRd, IRd)), true);
      }
    }
  }
  if (N1 == 1) {  // 3K2B and 3F2
    for (int SRd = TwoSR - 1; SRd <= TwoSR + 1; SRd += 2) {
      if (abs(TwoSL - SRd) > TwoS2 || SRd < 0) continue;
      const int kp = kap(NL, TwoSL, IL, 2, N2, TwoS2, NR + 1, SRd, IRd);
      if (kp == -1) continue;
      const double f = sqrt((TwoJ + 1) * (SRd + 1.0)) * heff_phase(TwoSL + SRd + TwoJ + 1 + 2 * TwoS2) *
                       wigner6j(TwoS2, TwoJ, 1, TwoSR, SRd, TwoSL);
      const int dRd = dR(NR + 1, SRd, IRd);
      const Blk W = q_plus_l(*this, Q, Rt, right, irr(theindex), coef, NR, TwoSR, IR, NR + 1, SRd, IRd, dimR, dRd);
      emit(f, kNo, false, kp, W, true);
    }
  }
}

// CheMPS2/HeffDiagrams3.cpp:609-740
void HeffEmitter::d3Land3G() {
  const OpT& Q = Rt->Q[0];
  const int IRd = irrep_prod(IR, irr(theindex + 1));
  const int TwoS1 = (N1 == 1) ? 1 : 0;
  const std::vector<int> right = range(theindex + 2, L);
  auto coef = [](HeffEmitter& h, int l) { return h.V(h.theindex + 1, h.theindex + 1, h.theindex + 1, l); };
  if (N2 == 1) {  // 3L1A
    for (int SRd = TwoSR - 1; SRd <= TwoSR + 1; SRd += 2) {
      if (abs(TwoSL - SRd) > TwoS1 || SRd < 0) continue;
      const int kp = kap(NL, TwoSL, IL, N1, 0, TwoS1, NR - 1, SRd, IRd);
      if (kp == -1) continue;
      const double f = sqrt((TwoJ + 1) * (TwoSR + 1.0)) * heff_phase(TwoSL + TwoSR + TwoS1 + 1) *
                       wigner6j(TwoS1, TwoJ, 1, TwoSR, SRd, TwoSL);
      emit(f, kNo, false, kp, need(Q.blk(NR - 1, SRd, IRd, NR, TwoSR, IR)), false);
    }
  }
  if (N2 == 2) {  // 3L1B and 3G1
    for (int SRd = TwoSR - 1; SRd <= TwoSR + 1; SRd += 2) {
      const int dRd = dR(NR - 1, SRd, IRd);
      if (dRd <= 0) continue;
      const int start = ((SRd != TwoSL) || (TwoS1 == 0)) ? 1 + TwoS1 : 0;
      for (int TJd = start; TJd <= 1 + TwoS1; TJd += 2) {
        if (abs(TwoSL - SRd) > TJd) continue;
        const int kp = kap(NL, TwoSL, IL, N1, 1, TJd, NR - 1, SRd, IRd);
        if (kp == -1) continue;
        const double f = sqrt((TJd + 1) * (TwoSR + 1.0)) * heff_phase(TwoSL + TwoSR + TwoS1 + 2) *
                         wigner6j(TJd, TwoS1, 1, TwoSR, SRd, TwoSL);
        const Blk W = q_plus_l(*this, Q, Rt, right, irr(theindex + 1), coef, NR - 1, SRd, IRd, NR, TwoSR, IR, dRd, dimR);
        emit(f, kNo, false, kp, W, false);
      }
    }
  }
  if (N2 == 0) {  // 3L2A
    for (int SRd = TwoSR - 1; SRd <= TwoSR + 1; SRd += 2) {
      if (dR(NR + 1, SRd, IRd) <= 0) continue;
      const int start = ((SRd != TwoSL) || (TwoS1 == 0)) ? 1 + TwoS1 : 0;
      for (int TJd = start; TJd <= 1 + TwoS1; TJd += 2) {
        if (abs(TwoSL - SRd) > TJd) continue;
        const int kp = kap(NL, TwoSL, IL, N1, 1, TJd, NR + 1, SRd, IRd);
        if (kp == -1) continue;
        const double f = sqrt((TJd + 1) * (SRd + 1.0)) * heff_phase(TwoSL + SRd + TwoS1 + 1) *
                         wigner6j(TJd, TwoS1, 1, TwoSR, SRd, TwoSL);
        emit(f, kNo, false, kp, need(Q.blk(NR, TwoSR, IR, NR + 1, SRd, IRd)), true);
      }
    }
  }
  if (N2 == 1) {  // 3L2B and 3G2
    for (int SRd = TwoSR - 1; SRd <= TwoSR + 1; SRd += 2) {
      if (abs(TwoSL - SRd) > TwoS1 || SRd < 0) continue;
      const int kp = kap(NL, TwoSL, IL, N1, 2, TwoS1, NR + 1, SRd, IRd);
      if (kp == -1) continue;
      const double f = sqrt((TwoJ + 1) * (SRd + 1.0)) * heff_phase(TwoSL + SRd + TwoS1 + 2) *
                       wigner6j(TwoS1, TwoJ, 1, TwoSR, SRd, TwoSL);
      const int dRd = dR(NR + 1, SRd, IRd);
      const Blk W = q_plus_l(*this, Q, Rt, right, irr(theindex + 1), coef, NR, TwoSR, IR, NR + 1, SRd, IRd, dimR, dRd);
      emit(f, kNo, false, kp, W, true);
    }
  }
}

// CheMPS2/HeffDiagrams3.cpp:742-848
void HeffEmitter::d3J() {
  const int e1 = ((N1 == 1) ? 2 : 0) + ((N2 == 1) ? 2 : 0);
  for (int SLd = TwoSL - 1; SLd <= TwoSL + 1; SLd += 2)  // 3J2
    for (int SRd = TwoSR - 1; SRd <= TwoSR + 1; SRd += 2) {
      if (abs(SLd - SRd) > TwoJ || SLd < 0 || SRd < 0) continue;
      const double f = heff_phase(SLd + TwoSR + TwoJ + 1 + e1) * sqrt((SLd + 1) * (SRd + 1.0)) *
                       wigner6j(TwoSL, TwoSR, TwoJ, SRd, SLd, 1);
      for (int l = 0; l < theindex; l++) {
        const int ILd = irrep_prod(IL, irr(l)), IRd = irrep_prod(IR, irr(l));
        const int kp = kap(NL + 1, SLd, ILd, N1, N2, TwoJ, NR + 1, SRd, IRd);
        if (kp == -1) continue;
        emit(f, need(Lt->Lop(l).blk(NL, TwoSL, IL, NL + 1, SLd, ILd)), false, kp,
             need(Rt->Qop(l).blk(NR, TwoSR, IR, NR + 1, SRd, IRd)), true);
      }
    }
  for (int SLd = TwoSL - 1; SLd <= TwoSL + 1; SLd += 2)  // 3J1
    for (int SRd = TwoSR - 1; SRd <= TwoSR + 1; SRd += 2) {
      if (abs(SLd - SRd) > TwoJ || SLd < 0 || SRd < 0) continue;
      const double f = heff_phase(TwoSL + SRd + TwoJ + 1 + e1) * sqrt((TwoSL + 1) * (TwoSR + 1.0)) *
                       wigner6j(TwoSL, TwoSR, TwoJ, SRd, SLd, 1);
      for (int l = 0; l < theindex; l++) {
        const int ILd = irrep_prod(IL, irr(l)), IRd = irrep_prod(IR, irr(l));
        const int kp = kap(NL - 1, SLd, ILd, N1, N2, TwoJ, NR - 1, SRd, IRd);
        if (kp == -1) continue;
        emit(f, need(Lt->Lop(l).blk(NL - 1, SLd, ILd, NL, TwoSL, IL)), true, kp,
             need(Rt->Qop(l).blk(NR - 1, SRd, IRd, NR, TwoSR, IR)), false);
      }
    }
}

}  // namespace c2g
