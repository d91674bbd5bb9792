#include "correlations.hpp"

#include <cmath>
#include <stdexcept>

#include "chemps2/Correlations.h"
#include "symm.hpp"

namespace c2g {

namespace {

inline int64_t align4(int64_t x) { return (x + 3) & ~int64_t(3); }

OpT corr_op(CorrTensors& c, int two_j, int n_elec, int irrep, int64_t& off) {
  OpT t;
  t.lay = c.layouts->get(c.boundary, two_j, n_elec, irrep);
  t.base = make_ref(c.slot, off);
  t.moving_right = true;
  t.prime_last = true;
  t.jw_phase = false;
  off = align4(off + t.lay->size());
  return t;
}

Blk need(const Blk& b) {
  if (!b.valid) throw std::logic_error("correlations: a block of nonzero dimensions is missing");
  return b;
}

// Pass 1 records the products P = Op * T_b into the work slot, pass 2 the Frobenius
// products factor * < T_dot, P > into slot Y.
struct CorrSink {
  TaskBuilder* tb = nullptr;
  int pass = 1;
  int64_t woff = 0;
  void product(const Blk& Tdot, const Blk& Op, const Blk& Tb, int value, double factor) {
    const int m = Tdot.rows, n = Tdot.cols;
    if (m <= 0 || n <= 0) return;
    const int64_t K = static_cast<int64_t>(m) * n;
    if (pass == 1) {
      tb->contract(Blk::make(make_ref(kSlotWork, woff), m, n), 1.0, Op, false, Tb, false, Blk(), false);
    } else {
      tb->contract(Blk::make(make_ref(kSlotY, value), 1, 1), factor, Blk::make(Tdot.ref, 1, static_cast<int>(K), 1),
                   false, Blk::make(make_ref(kSlotWork, woff), static_cast<int>(K), 1, static_cast<int>(K)), false,
                   Blk(), false);
    }
    woff += K;
  }
};

class CorrEmitter {
 public:
  CorrEmitter(const CheMPS2::SyBookkeeper& bk, int site, const MpsT& T, CorrSink& s)
      : bk_(bk), s_(site), T_(T), sink_(s), nirr_(bk.getNumberOfIrreps()) {}

  template <class F>
  void for_right(F f) const {
    for (int NR = bk_.gNmin(s_ + 1); NR <= bk_.gNmax(s_ + 1); NR++)
      for (int SR = bk_.gTwoSmin(s_ + 1, NR); SR <= bk_.gTwoSmax(s_ + 1, NR); SR += 2)
        for (int IR = 0; IR < nirr_; IR++) f(NR, SR, IR);
  }
  int dim(int b, int N, int S, int I) const { return (N < 0 || S < 0) ? 0 : bk_.gCurrentDim(b, N, S, I); }

  // CheMPS2/Correlations.cpp:353-387
  void diagram1(const OpT& O, int v) {
    for_right([&](int NR, int SR, int IR) {
      if (dim(s_, NR, SR, IR) > 0 && dim(s_ + 1, NR, SR, IR) > 0) {
        const Blk t = need(T_.blk(NR, SR, IR, NR, SR, IR));
        sink_.product(t, need(O.blk(NR, SR, IR, NR, SR, IR)), t, v, SR + 1.0);
      }
    });
  }
  // :389-423
  void diagram2(const OpT& O, int v) {
    for_right([&](int NR, int SR, int IR) {
      if (dim(s_, NR - 2, SR, IR) > 0 && dim(s_ + 1, NR, SR, IR) > 0) {
        const Blk t = need(T_.blk(NR - 2, SR, IR, NR, SR, IR));
        sink_.product(t, need(O.blk(NR - 2, SR, IR, NR - 2, SR, IR)), t, v, SR + 1.0);
      }
    });
  }
  // :425-467
  void diagram3(const OpT& O, int v) {
    for_right([&](int NR, int SR, int IR) {
      if (dim(s_ + 1, NR, SR, IR) <= 0) return;
      const int IL = irrep_prod(IR, bk_.gIrrep(s_));
      for (int SL = SR - 1; SL <= SR + 1; SL += 2) {
        if (dim(s_, NR - 1, SL, IL) <= 0) continue;
        const Blk t = need(T_.blk(NR - 1, SL, IL, NR, SR, IR));
        sink_.product(t, need(O.blk(NR - 1, SL, IL, NR - 1, SL, IL)), t, v, SR + 1.0);
      }
    });
  }
  // :469-513
  void diagram4(const OpT& O, int v) {
    for_right([&](int NR, int SR, int IR) {
      if (!(dim(s_ + 1, NR, SR, IR) > 0 && dim(s_, NR, SR, IR) > 0)) return;
      const int ILd = irrep_prod(IR, bk_.gIrrep(s_));
      for (int SLd = SR - 1; SLd <= SR + 1; SLd += 2) {
        if (dim(s_, NR - 1, SLd, ILd) <= 0) continue;
        sink_.product(need(T_.blk(NR - 1, SLd, ILd, NR, SR, IR)), need(O.blk(NR - 1, SLd, ILd, NR, SR, IR)),
                      need(T_.blk(NR, SR, IR, NR, SR, IR)), v, SR + 1.0);
      }
    });
  }
  // :515-560
  void diagram5(const OpT& O, int v) {
    for_right([&](int NR, int SR, int IR) {
      if (!(dim(s_ + 1, NR, SR, IR) > 0 && dim(s_, NR - 2, SR, IR) > 0)) return;
      const int ILu = irrep_prod(IR, bk_.gIrrep(s_));
      for (int SLu = SR - 1; SLu <= SR + 1; SLu += 2) {
        if (dim(s_, NR - 1, SLu, ILu) <= 0) continue;
        const double f = phase(SLu + 1 - SR) * std::sqrt((SLu + 1.0) * (SR + 1));
        sink_.product(need(T_.blk(NR - 2, SR, IR, NR, SR, IR)), need(O.blk(NR - 2, SR, IR, NR - 1, SLu, ILu)),
                      need(T_.blk(NR - 1, SLu, ILu, NR, SR, IR)), v, f);
      }
    });
  }

 private:
  const CheMPS2::SyBookkeeper& bk_;
  const int s_;
  const MpsT& T_;
  CorrSink& sink_;
  const int nirr_;
};

}  // namespace

void allocate_corr(CorrTensors& c, const CheMPS2::SyBookkeeper& bk, int boundary, int slot) {
  c.boundary = boundary;
  c.slot = slot;
  c.layouts = std::make_unique<OpLayoutCache>(&bk);
  c.G.clear();
  c.Y.clear();
  c.Z.clear();
  c.K.clear();
  c.M.clear();
  int64_t off = 0;
  for (int p = 0; p < boundary; p++) {
    c.G.push_back(corr_op(c, 0, 0, 0, off));
    c.Y.push_back(corr_op(c, 0, 0, 0, off));
    c.Z.push_back(corr_op(c, 0, 0, 0, off));
    c.K.push_back(corr_op(c, 1, 1, bk.gIrrep(p), off));
    c.M.push_back(corr_op(c, 1, 1, bk.gIrrep(p), off));
  }
  c.size = off;
}

void compile_corr_update(TaskBuilder& tb, const CheMPS2::SyBookkeeper& bk, const CheMPS2::Problem& prob, int L,
                         int site, const CorrTensors* prev, const CorrTensors& next, const MpsT& T) {
  auto dim = [&](int b, int N, int S, int I) { return (N < 0 || S < 0) ? 0 : bk.gCurrentDim(b, N, S, I); };
  for (int p = 0; p + 1 < site; p++) {
    if (!prev) throw std::logic_error("correlations: previous tensors missing");
    for (auto member : {&CorrTensors::G, &CorrTensors::Y, &CorrTensors::Z, &CorrTensors::K, &CorrTensors::M})
      emit_generic_update(tb, bk, prob, T, L, (next.*member)[p], (prev->*member)[p]);
  }
  const int p = site - 1;
  const int Ip = bk.gIrrep(p);
  // TensorGYZ::construct (CheMPS2/TensorGYZ.cpp:35-99)
  for (int which = 0; which < 3; which++) {
    const OpT& O = (which == 0) ? next.G[p] : (which == 1) ? next.Y[p] : next.Z[p];
    for (int ik = 0; ik < O.lay->nkappa; ik++) {
      const Blk ob = O.blk_k(ik);
      tb.declare_output(ob);
      const int N = O.lay->n_up[ik], S = O.lay->spin_up[ik], I = O.lay->irrep_up[ik];
      if (which == 0) {  // G: NL = N - 1, S_L = S -+ 1, IL = I x I_p, alpha = sqrt(1/2)
        for (int SL = S - 1; SL <= S + 1; SL += 2)
          if (dim(site - 1, N - 1, SL, irrep_prod(I, Ip)) > 0) {
            const Blk t = need(T.blk(N - 1, SL, irrep_prod(I, Ip), N, S, I));
            tb.contract(ob, std::sqrt(0.5), t, true, t, false, Blk(), false);
          }
      } else {
        const int NL = (which == 1) ? N : N - 2;
        if (dim(site - 1, NL, S, I) > 0) {
          const Blk t = need(T.blk(NL, S, I, N, S, I));
          tb.contract(ob, 1.0, t, true, t, false, Blk(), false);
        }
      }
    }
  }
  // TensorKM::construct (CheMPS2/TensorKM.cpp:35-96)
  for (int which = 0; which < 2; which++) {
    const OpT& O = (which == 0) ? next.K[p] : next.M[p];
    for (int ik = 0; ik < O.lay->nkappa; ik++) {
      const Blk ob = O.blk_k(ik);
      tb.declare_output(ob);
      const int N = O.lay->n_up[ik], S = O.lay->spin_up[ik], I = O.lay->irrep_up[ik];
      const int Sd = O.lay->spin_down[ik], IDR = irrep_prod(O.lay->n_irrep, I);
      if (which == 0) {
        if (dim(site - 1, N, S, I) > 0)
          tb.contract(ob, 1.0, need(T.blk(N, S, I, N, S, I)), true, need(T.blk(N, S, I, N + 1, Sd, IDR)), false, Blk(),
                      false);
      } else {
        if (dim(site - 1, N - 1, Sd, IDR) > 0) {
          const double alpha = phase(Sd - S + 1) * std::sqrt((S + 1.0) / (Sd + 1));
          tb.contract(ob, alpha, need(T.blk(N - 1, Sd, IDR, N, S, I)), true, need(T.blk(N - 1, Sd, IDR, N + 1, Sd, IDR)),
                      false, Blk(), false);
        }
      }
    }
  }
}

int64_t compile_corr_fill(TaskBuilder& tb, const CheMPS2::SyBookkeeper& bk, int site, const MpsT& T,
                          const CorrTensors& c) {
  CorrSink sink;
  sink.tb = &tb;
  CorrEmitter e(bk, site, T, sink);
  for (int pass = 1; pass <= 2; pass++) {
    sink.pass = pass;
    sink.woff = 0;
    if (pass == 2) tb.next_stage("correlations.dots");
    for (int p = 0; p < site; p++) {
      const bool eq = bk.gIrrep(p) == bk.gIrrep(site);
      const int v = p * kCorrValues;
      e.diagram3(c.G[p], v + 0);
      e.diagram1(c.Y[p], v + 1);
      e.diagram2(c.Z[p], v + 2);
      e.diagram1(c.G[p], v + 3);
      e.diagram3(c.Y[p], v + 4);
      if (eq) e.diagram4(c.K[p], v + 5);
      e.diagram2(c.G[p], v + 6);
      e.diagram3(c.Z[p], v + 7);
      if (eq) e.diagram5(c.M[p], v + 8);
      e.diagram1(c.Z[p], v + 9);
      if (eq) e.diagram5(c.K[p], v + 10);
      if (eq) e.diagram4(c.M[p], v + 11);
      e.diagram2(c.Y[p], v + 12);
    }
  }
  for (int v = 0; v < site * kCorrValues; v++) tb.declare_output(Blk::make(make_ref(kSlotY, v), 1, 1));
  return sink.woff;
}

}  // namespace c2g

namespace CheMPS2 {

namespace {
constexpr double kDiscardEig = 1e-100;  // CORRELATIONS_discardEig (CheMPS2/include/chemps2/Options.h)

// eigenvalues of a symmetric n x n matrix (cyclic Jacobi)
std::vector<double> sym_eigenvalues(std::vector<double> a, int n) {
  for (int sweep = 0; sweep < 100; sweep++) {
    double off = 0.0;
    for (int i = 0; i < n; i++)
      for (int j = 0; j < n; j++)
        if (i != j) off += a[i + n * j] * a[i + n * j];
    if (off < 1e-32) break;
    for (int p = 0; p < n; p++)
      for (int q = p + 1; q < n; q++) {
        const double apq = a[p + n * q];
        if (apq == 0.0) continue;
        const double tau = (a[q + n * q] - a[p + n * p]) / (2 * apq);
        const double t = (tau >= 0 ? 1.0 : -1.0) / (std::fabs(tau) + std::sqrt(1 + tau * tau));
        const double c = 1 / std::sqrt(1 + t * t), s = t * c;
        for (int j = 0; j < n; j++) {
          const double x = a[p + n * j], y = a[q + n * j];
          a[p + n * j] = c * x - s * y;
          a[q + n * j] = s * x + c * y;
        }
        for (int i = 0; i < n; i++) {
          const double x = a[i + n * p], y = a[i + n * q];
          a[i + n * p] = c * x - s * y;
          a[i + n * q] = s * x + c * y;
        }
      }
  }
  std::vector<double> ev(n);
  for (int i = 0; i < n; i++) ev[i] = a[i + n * i];
  return ev;
}
}  // namespace

// CheMPS2/Correlations.cpp:40-103
Correlations::Correlations(const Problem* prob, const TwoDM* dm) : prob_(prob), dm_(dm), L_(dm->gL()) {
  const size_t n = static_cast<size_t>(L_) * L_;
  Cspin_.assign(n, 0.0);
  Cdens_.assign(n, 0.0);
  Cspinflip_.assign(n, 0.0);
  Cdirad_.assign(n, 0.0);
  MutInfo_.assign(n, 0.0);
  for (int r = 0; r < L_; r++) {
    for (int c = 0; c < L_; c++) {
      Cspin_[r + L_ * c] = dm->getTwoDMB_DMRG(r, c, r, c);
      Cdens_[r + L_ * c] = dm->getTwoDMA_DMRG(r, c, r, c) - dm->get1RDM_DMRG(r, r) * dm->get1RDM_DMRG(c, c);
      Cspinflip_[r + L_ * c] = 0.5 * (dm->getTwoDMB_DMRG(r, c, c, r) - dm->getTwoDMA_DMRG(r, c, c, r));
      Cdirad_[r + L_ * c] = -0.5 * (dm->get1RDM_DMRG(r, r) - dm->getTwoDMA_DMRG(r, r, r, r)) *
                            (dm->get1RDM_DMRG(c, c) - dm->getTwoDMA_DMRG(c, c, c, c));
    }
    Cspin_[r + L_ * r] += dm->get1RDM_DMRG(r, r);
    Cdens_[r + L_ * r] += dm->get1RDM_DMRG(r, r);
    Cspinflip_[r + L_ * r] += dm->get1RDM_DMRG(r, r);
  }
}

double Correlations::SingleOrbitalEntropy_DMRG(int i) const {
  const double val4 = 0.5 * dm_->getTwoDMA_DMRG(i, i, i, i);
  const double val23 = 0.5 * (dm_->get1RDM_DMRG(i, i) - dm_->getTwoDMA_DMRG(i, i, i, i));
  const double val1 = 1.0 - val4 - 2 * val23;
  double e = 0.0;
  if (val1 > kDiscardEig) e -= val1 * std::log(val1);
  if (val23 > kDiscardEig) e -= 2 * val23 * std::log(val23);
  if (val4 > kDiscardEig) e -= val4 * std::log(val4);
  return e;
}

double Correlations::MutualInformationDistance(double power) const {
  double d = 0.0;
  for (int r = 0; r < L_; r++)
    for (int c = 0; c < L_; c++)
      if (r != c) d += MutInfo_[r + L_ * c] * std::pow(std::abs(r - c), power);
  return d;
}

// CheMPS2/Correlations.cpp:212-351
void Correlations::fill_pair(int p, int s, const double* v) {
  const double pS = 1.0 / (prob_->gTwoS() + 1.0);
  const double r12 = std::sqrt(0.5);
  const bool eq = prob_->gIrrep(p) == prob_->gIrrep(s);
  const double diag1 = v[0] * pS * 0.5 * r12;
  const double diag2 = 0.125 * (dm_->getTwoDMB_DMRG(p, s, s, p) - dm_->getTwoDMA_DMRG(p, s, s, p));
  const double val1 = v[1] * pS, val2 = v[2] * pS, val3 = diag1 + diag2;
  const double val4 = v[3] * pS * r12, val5 = v[4] * pS * 0.5, val6 = eq ? v[5] * pS * 0.5 : 0.0;
  const double val7 = v[6] * pS * r12, val8 = v[7] * pS * 0.5, val9 = eq ? v[8] * pS * 0.5 : 0.0;
  const double alpha = v[12] * pS, beta = diag1 - diag2, gamma = v[9] * pS, lambda = 2 * diag2;
  const double delta = eq ? -v[10] * pS * 0.5 : 0.0, epsilon = eq ? v[11] * pS * 0.5 : 0.0;
  const double kappa = 0.5 * dm_->getTwoDMA_DMRG(p, p, s, s);
  const int n = 16;
  std::vector<double> R(n * n, 0.0);
  auto set = [&](int i, int j, double x) { R[i + n * j] = x; };
  set(0, 0, val1);
  set(15, 15, val2);
  set(5, 5, val3);
  set(10, 10, val3);
  set(1, 1, val4);
  set(3, 3, val4);
  set(2, 2, val5);
  set(4, 4, val5);
  set(1, 2, val6); set(2, 1, val6); set(3, 4, val6); set(4, 3, val6);
  set(11, 11, val7);
  set(13, 13, val7);
  set(12, 12, val8);
  set(14, 14, val8);
  set(11, 12, val9); set(12, 11, val9); set(13, 14, val9); set(14, 13, val9);
  set(6, 6, alpha);
  set(7, 7, beta);
  set(8, 8, beta);
  set(9, 9, gamma);
  set(6, 7, delta); set(7, 6, delta);
  set(6, 8, -delta); set(8, 6, -delta);
  set(7, 9, epsilon); set(9, 7, epsilon);
  set(8, 9, -epsilon); set(9, 8, -epsilon);
  set(6, 9, kappa); set(9, 6, kappa);
  set(7, 8, lambda); set(8, 7, lambda);
  double entropy = 0.0;
  for (double e : sym_eigenvalues(R, n))
    if (e > kDiscardEig) entropy -= e * std::log(e);
  const double mi = 0.5 * (SingleOrbitalEntropy_DMRG(p) + SingleOrbitalEntropy_DMRG(s) - entropy);
  MutInfo_[p + L_ * s] = MutInfo_[s + L_ * p] = mi;
  Cdirad_[p + L_ * s] += 2 * beta;
  Cdirad_[s + L_ * p] += 2 * beta;
}

}  // namespace CheMPS2
