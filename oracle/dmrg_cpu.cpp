// ORACLE (test infrastructure, not product code): the two-site DMRG sweep on the CPU.
//
// A restatement of CheMPS2's ground-state DMRG for the tests and the CPU baseline:
//   * sweep control, solve_site, PreSolve        CheMPS2/DMRG.cpp:36-452
//   * random initial MPS + Householder QR        CheMPS2/DMRG.cpp:159-170, CheMPS2/TensorT.cpp:167-289
//   * Davidson, problem type 'E'                 CheMPS2/Davidson.cpp:31-536 (one modified
//                                                Gram-Schmidt pass, Jacobi instead of dsyev)
//   * Split truncation rule and discarded weight CheMPS2/Sobject.cpp:260-621 (Gram matrix
//                                                and cyclic Jacobi instead of dgesdd)
// The contractions (Join, Heff, its diagonal, the Split block copies and the operator
// updates) are the task programs of the product's host compiler, executed by the CPU
// executor of this directory, which also checks every program's memory accesses.
//
// Exposed through a C API (oracle_*), loaded by the tests and the benchmark's CPU
// baseline with ctypes.
#include <algorithm>
#include <array>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "chemps2/ConvergenceScheme.h"
#include "chemps2/Hamiltonian.h"
#include "chemps2/Problem.h"
#include "chemps2/SyBookkeeper.h"
#include "compile.hpp"
#include "exec_cpu.hpp"
#include "fcicoef.hpp"
#include "gauge.hpp"
#include "heff.hpp"
#include "layout.hpp"
#include "operators.hpp"
#include "chemps2/Correlations.h"
#include "correlations.hpp"
#include "sobject.hpp"
#include "twodm.hpp"
#include "symm.hpp"

namespace oracle {

using namespace c2g;
using CheMPS2::SyBookkeeper;

// Cyclic Jacobi eigensolver of a symmetric n x n matrix (column major, ld n). On return
// `w` holds the eigenvalues ascending and the columns of `v` the eigenvectors.
void jacobi_eigh(std::vector<double>& a, int n, std::vector<double>& w, std::vector<double>& v) {
  v.assign(size_t(n) * n, 0.0);
  for (int i = 0; i < n; i++) v[i + size_t(n) * i] = 1.0;
  auto A = [&](int i, int j) -> double& { return a[i + size_t(n) * j]; };
  for (int sweep = 0; sweep < 60; sweep++) {
    double off = 0.0, tot = 0.0;
    for (int j = 0; j < n; j++)
      for (int i = 0; i < n; i++) {
        tot += A(i, j) * A(i, j);
        if (i != j) off += A(i, j) * A(i, j);
      }
    if (!(off > 1e-30 * tot)) break;
    for (int p = 0; p < n; p++)
      for (int q = p + 1; q < n; q++) {
        const double apq = A(p, q);
        if (apq == 0.0) continue;
        const double tau = (A(q, q) - A(p, p)) / (2.0 * apq);
        const double t = (tau >= 0.0 ? 1.0 : -1.0) / (std::fabs(tau) + std::sqrt(1.0 + tau * tau));
        const double c = 1.0 / std::sqrt(1.0 + t * t), s = t * c;
        for (int j = 0; j < n; j++) {
          const double x = A(p, j), y = A(q, j);
          A(p, j) = c * x - s * y;
          A(q, j) = s * x + c * y;
        }
        for (int i = 0; i < n; i++) {
          const double x = A(i, p), y = A(i, q);
          A(i, p) = c * x - s * y;
          A(i, q) = s * x + c * y;
          const double vx = v[i + size_t(n) * p], vy = v[i + size_t(n) * q];
          v[i + size_t(n) * p] = c * vx - s * vy;
          v[i + size_t(n) * q] = s * vx + c * vy;
        }
      }
  }
  std::vector<int> order(n);
  for (int i = 0; i < n; i++) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return A(x, x) < A(y, y); });
  w.resize(n);
  std::vector<double> vs(size_t(n) * n);
  for (int j = 0; j < n; j++) {
    w[j] = A(order[j], order[j]);
    for (int i = 0; i < n; i++) vs[i + size_t(n) * j] = v[i + size_t(n) * order[j]];
  }
  v.swap(vs);
}

// CheMPS2::Davidson, problem type 'E' (CheMPS2/Davidson.cpp).
struct Davidson {
  int64_t n;
  int MAX, KEEP;
  double RTOL, CUTOFF;
  int n_matvec = 0;
  template <class MV>
  double solve(std::vector<double>& x, const std::vector<double>& diag, MV matvec) {
    std::vector<std::vector<double>> vecs, Hvecs;
    std::vector<double> mxM(size_t(MAX) * MAX, 0.0), evals, evecs;
    std::vector<double> t(x), u(n), work(n);
    auto dot = [&](const std::vector<double>& a, const std::vector<double>& b) {
      double s = 0.0;
      for (int64_t i = 0; i < n; i++) s += a[i] * b[i];
      return s;
    };
    auto nrm = [&](const std::vector<double>& a) { return std::sqrt(dot(a, a)); };
    if (nrm(t) == 0.0)
      for (int64_t i = 0; i < n; i++) t[i] = static_cast<double>(std::rand()) / RAND_MAX;
    int num_vec = 0;
    auto add_new_vec = [&]() {
      for (int c = 0; c < num_vec; c++) {
        const double ov = -dot(t, vecs[c]);
        for (int64_t i = 0; i < n; i++) t[i] += ov * vecs[c][i];
      }
      const double a = 1.0 / nrm(t);
      for (auto& e : t) e *= a;
      if (static_cast<int>(vecs.size()) <= num_vec) {
        vecs.push_back(t);
        Hvecs.emplace_back(n);
      } else {
        vecs[num_vec] = t;
      }
    };
    add_new_vec();
    matvec(vecs[num_vec].data(), Hvecs[num_vec].data());
    n_matvec++;
    for (;;) {
      for (int c = 0; c < num_vec; c++) {
        mxM[c + size_t(MAX) * num_vec] = dot(vecs[num_vec], Hvecs[c]);
        mxM[num_vec + size_t(MAX) * c] = mxM[c + size_t(MAX) * num_vec];
      }
      mxM[num_vec + size_t(MAX) * num_vec] = dot(vecs[num_vec], Hvecs[num_vec]);
      num_vec++;
      std::vector<double> sm(size_t(num_vec) * num_vec);
      for (int j = 0; j < num_vec; j++)
        for (int i = 0; i < num_vec; i++) sm[i + size_t(num_vec) * j] = mxM[i + size_t(MAX) * j];
      jacobi_eigh(sm, num_vec, evals, evecs);
      std::fill(t.begin(), t.end(), 0.0);
      std::fill(u.begin(), u.end(), 0.0);
      for (int c = 0; c < num_vec; c++) {
        const double a = evecs[c];
        for (int64_t i = 0; i < n; i++) {
          t[i] += a * Hvecs[c][i];
          u[i] += a * vecs[c][i];
        }
      }
      for (int64_t i = 0; i < n; i++) t[i] -= evals[0] * u[i];
      const double rnorm = nrm(t);
      if (!(rnorm > RTOL)) break;
      const double shift = evals[0];
      for (int64_t i = 0; i < n; i++) {
        const double d = diag[i] - shift;
        work[i] = u[i] / ((std::fabs(d) > CUTOFF) ? d : CUTOFF);
      }
      const double alpha = -dot(work, t) / dot(work, u);
      for (int64_t i = 0; i < n; i++) t[i] += alpha * u[i];
      for (int64_t i = 0; i < n; i++) {
        const double d = diag[i] - shift;
        t[i] = -t[i] / ((std::fabs(d) > CUTOFF) ? d : CUTOFF);
      }
      if (num_vec == MAX) {
        std::vector<std::vector<double>> E(KEEP, std::vector<double>(n, 0.0));
        E[0] = u;
        for (int c = 1; c < KEEP; c++)
          for (int iv = 0; iv < MAX; iv++) {
            const double a = evecs[iv + size_t(num_vec) * c];
            for (int64_t i = 0; i < n; i++) E[c][i] += vecs[iv][i] * a;
          }
        std::vector<double> S(size_t(KEEP) * KEEP), sw, sv;
        for (int a = 0; a < KEEP; a++)
          for (int b = 0; b < KEEP; b++) S[a + size_t(KEEP) * b] = dot(E[a], E[b]);
        jacobi_eigh(S, KEEP, sw, sv);
        std::vector<double> Lw(size_t(KEEP) * KEEP, 0.0);
        for (int a = 0; a < KEEP; a++)
          for (int b = 0; b < KEEP; b++)
            for (int l = 0; l < KEEP; l++)
              Lw[a + size_t(KEEP) * b] += sv[a + size_t(KEEP) * l] * std::pow(sw[l], -0.5) * sv[b + size_t(KEEP) * l];
        for (int iv = 0; iv < KEEP; iv++) {
          std::fill(vecs[iv].begin(), vecs[iv].end(), 0.0);
          for (int iv2 = 0; iv2 < KEEP; iv2++) {
            const double a = Lw[iv2 + size_t(KEEP) * iv];
            for (int64_t i = 0; i < n; i++) vecs[iv][i] += a * E[iv2][i];
          }
        }
        for (int iv = 0; iv < KEEP; iv++) {
          matvec(vecs[iv].data(), Hvecs[iv].data());
          n_matvec++;
        }
        num_vec = KEEP;
        for (int a = 0; a < KEEP; a++)
          for (int b = a; b < KEEP; b++) {
            mxM[a + size_t(MAX) * b] = dot(vecs[a], Hvecs[b]);
            mxM[b + size_t(MAX) * a] = mxM[a + size_t(MAX) * b];
          }
      }
      add_new_vec();
      matvec(vecs[num_vec].data(), Hvecs[num_vec].data());
      n_matvec++;
    }
    x = u;
    return evals[0];
  }
};

struct OracleDMRG {
  CheMPS2::Problem* Prob;
  CheMPS2::ConvergenceScheme* Opt;
  int L;
  std::unique_ptr<SyBookkeeper> bk;
  std::vector<std::unique_ptr<MpsLayout>> mps_lay;
  std::vector<std::vector<double>> mps;
  std::vector<std::unique_ptr<BoundaryOps>> ops;
  std::vector<std::vector<double>> ops_mem;
  std::vector<int> isAllocated;
  CpuExecutor ex;
  double TotalMinEnergy = 1e8, MaxDisc = 0.0;
  std::vector<double> step_energies;
  long long n_matvec = 0;
  double t_matvec = 0.0;
  bool check = true;
  std::vector<double> ones;
  int left_upto_ = -1;

  // dims (optional): rows (boundary, N, 2S, I, dim) that replace the bookkeeper's scaled
  // dimensions (every sector not listed gets 0), for a state with given sector dimensions;
  // left_upto: the left operators are built for the first left_upto boundaries only (all
  // when negative).
  OracleDMRG(CheMPS2::Problem* p, CheMPS2::ConvergenceScheme* o, bool check_programs,
             const std::vector<std::array<int, 5>>* dims = nullptr, int left_upto = -1)
      : Prob(p), Opt(o), L(p->gL()), ex(c2g::num_slots(p->gL()) + 8), check(check_programs) {
    Prob->construct_mxelem();
    bk = std::make_unique<SyBookkeeper>(Prob, Opt->get_D(0));
    if (!bk->IsPossible()) throw std::invalid_argument("impossible symmetry sector");
    if (dims) {
      for (int b = 0; b <= L; b++)
        for (int id = 0; id < bk->num_sectors(b); id++) {
          int n, s2, i;
          bk->sector_labels(b, id, &n, &s2, &i);
          bk->SetDim(b, n, s2, i, 0);
        }
      for (const auto& r : *dims) {
        if (r[0] < 0 || r[0] > L) throw std::invalid_argument("dims: boundary out of range");
        if (r[4] > bk->gFCIdim(r[0], r[1], r[2], r[3])) throw std::invalid_argument("dims: above the FCI dimension");
        bk->SetDim(r[0], r[1], r[2], r[3], r[4]);
      }
    }
    left_upto_ = left_upto;
    mps_lay.resize(L);
    mps.resize(L);
    ops.resize(L - 1);
    ops_mem.resize(L - 1);
    isAllocated.assign(L - 1, 0);
    for (int site = 0; site < L; site++) {
      mps_lay[site] = std::make_unique<MpsLayout>();
      mps_lay[site]->build(*bk, site);
      mps[site].resize(mps_lay[site]->size());
      for (auto& v : mps[site]) v = (2 * static_cast<double>(std::rand()) / RAND_MAX) - 1.0;
      qr(site);
      bind_mps(site);
    }
    presolve();
  }

  void bind_mps(int site) { ex.bind(kSlotMpsBase + site, mps[site].data(), static_cast<int64_t>(mps[site].size())); }
  MpsT mpsT(int site) const {
    MpsT t;
    t.lay = mps_lay[site].get();
    t.base = make_ref(kSlotMpsBase + site, 0);
    return t;
  }

  void exec(const Program& p, double* x, int64_t nx, double* y, int64_t ny) {
    ex.prepare_scratch(p);
    ex.bind(kSlotX, x, x ? nx : 0);
    ex.bind(kSlotY, y, y ? ny : 0);
    if (check) ex.check(p);
    ex.run(p, true, true);
  }

  // Left normalisation by Householder QR per right sector (CheMPS2/TensorT.cpp:188-289).
  void qr(int site) {
    const MpsLayout& lay = *mps_lay[site];
    std::vector<double>& data = mps[site];
    for (int NR = bk->gNmin(site + 1); NR <= bk->gNmax(site + 1); NR++)
      for (int TwoSR = bk->gTwoSmin(site + 1, NR); TwoSR <= bk->gTwoSmax(site + 1, NR); TwoSR += 2)
        for (int IR = 0; IR < bk->getNumberOfIrreps(); IR++) {
          const int n = bk->gCurrentDim(site + 1, NR, TwoSR, IR);
          if (n <= 0) continue;
          std::vector<int> blocks;
          int m = 0;
          for (int k = 0; k < lay.nkappa; k++)
            if (lay.NR[k] == NR && lay.TwoSR[k] == TwoSR && lay.IR[k] == IR && lay.rows[k] > 0) {
              blocks.push_back(k);
              m += lay.rows[k];
            }
          if (m == 0) continue;
          std::vector<double> a(size_t(m) * n);
          int r0 = 0;
          for (int k : blocks) {
            for (int l = 0; l < lay.rows[k]; l++)
              for (int r = 0; r < n; r++) a[r0 + l + size_t(m) * r] = data[lay.k2i[k] + l + lay.rows[k] * r];
            r0 += lay.rows[k];
          }
          // Householder QR (LAPACK dgeqr2 conventions) and Q = H_1 ... H_kk I (dorg2r)
          const int kk = std::min(m, n);
          std::vector<double> tau(kk, 0.0);
          for (int j = 0; j < kk; j++) {
            double* x = &a[j + size_t(m) * j];
            const int len = m - j;
            double xn = 0.0;
            for (int i = 1; i < len; i++) xn += x[i] * x[i];
            xn = std::sqrt(xn);
            if (xn == 0.0) continue;
            const double alpha = x[0];
            const double beta = -std::copysign(std::hypot(alpha, xn), alpha);
            tau[j] = (beta - alpha) / beta;
            for (int i = 1; i < len; i++) x[i] /= (alpha - beta);
            x[0] = beta;
            for (int c = j + 1; c < n; c++) {
              double* y = &a[j + size_t(m) * c];
              double sdot = y[0];
              for (int i = 1; i < len; i++) sdot += x[i] * y[i];
              sdot *= tau[j];
              y[0] -= sdot;
              for (int i = 1; i < len; i++) y[i] -= sdot * x[i];
            }
          }
          std::vector<double> q(size_t(m) * n, 0.0);
          for (int c = 0; c < kk; c++) q[c + size_t(m) * c] = 1.0;
          for (int j = kk - 1; j >= 0; j--) {
            const double* v = &a[j + size_t(m) * j];
            const int len = m - j;
            for (int c = j; c < kk; c++) {
              double* y = &q[j + size_t(m) * c];
              double sdot = y[0];
              for (int i = 1; i < len; i++) sdot += v[i] * y[i];
              sdot *= tau[j];
              y[0] -= sdot;
              for (int i = 1; i < len; i++) y[i] -= sdot * v[i];
            }
          }
          r0 = 0;
          for (int k : blocks) {
            for (int l = 0; l < lay.rows[k]; l++)
              for (int r = 0; r < n; r++) data[lay.k2i[k] + l + lay.rows[k] * r] = q[r0 + l + size_t(m) * r];
            r0 += lay.rows[k];
          }
        }
  }

  void update(int index, bool mr) {
    ops[index] = std::make_unique<BoundaryOps>();
    allocate_ops(*ops[index], *bk, L, index, mr, slot_ops(L, index));
    ops_mem[index].assign(std::max<int64_t>(ops[index]->size, 1), 0.0);
    ex.bind(slot_ops(L, index), ops_mem[index].data(), ops[index]->size);
    isAllocated[index] = mr ? 1 : 2;
    UpdateContext ctx;
    ctx.bk = bk.get();
    ctx.prob = Prob;
    ctx.L = L;
    ctx.index = index;
    ctx.moving_right = mr;
    if (mr)
      ctx.prev = (index > 0) ? ops[index - 1].get() : nullptr;
    else
      ctx.prev = (index + 1 < L - 1) ? ops[index + 1].get() : nullptr;
    ctx.next = ops[index].get();
    ctx.mps = mr ? mpsT(index) : mpsT(index + 1);
    exec(compile_update_program(ctx).program, nullptr, 0, nullptr, 0);
  }

  void presolve() {
    for (int b = 0; b < L - 1; b++) {
      ops[b].reset();
      ops_mem[b].clear();
      ex.bind(slot_ops(L, b), nullptr, 0);
      isAllocated[b] = 0;
    }
    const int upto = (left_upto_ >= 0) ? std::min(left_upto_, L - 2) : L - 2;
    for (int c = 0; c < upto; c++) update(c, true);
    TotalMinEnergy = 1e8;
    MaxDisc = 0.0;
  }

  // The 2-RDM pass of DMRG::calc2DMandCorrelations (CheMPS2/DMRGtechnics.cpp:40-120) with
  // the product's host parts: gauge changes (host/gauge.cpp), operator updates and the
  // 2-RDM programs (host/twodm.cpp), run on this executor. Leaves the state as the pass
  // leaves it (site 0 the orthogonality centre, right operators of every boundary).
  std::unique_ptr<CheMPS2::TwoDM> two_dm;
  void calc_2dm() {
    c2g::left_normalize(*bk, L - 2, *mps_lay[L - 2], mps[L - 2], mps_lay[L - 1].get(), &mps[L - 1]);
    c2g::left_normalize(*bk, L - 1, *mps_lay[L - 1], mps[L - 1]);
    update(L - 2, true);
    two_dm = std::make_unique<CheMPS2::TwoDM>(Prob, L);
    for (int site = L - 1; site >= 0; site--) {
      c2g::TwoDMContext ctx;
      ctx.bk = bk.get();
      ctx.L = L;
      ctx.site = site;
      ctx.T = mpsT(site);
      ctx.left = (site > 0) ? ops[site - 1].get() : nullptr;
      ctx.right = (site < L - 1) ? ops[site].get() : nullptr;
      if (site > 0 && isAllocated[site - 1] != 1) throw std::logic_error("2-RDM: left operators missing");
      if (site < L - 1 && isAllocated[site] != 2) throw std::logic_error("2-RDM: right operators missing");
      const std::vector<c2g::TwoDMInstance> inst = c2g::twodm_instances(ctx);
      const int nv = inst.back().value0 + c2g::twodm_num_values(inst.back().kind);
      int64_t work = 0;
      for (const auto& in : inst) work += in.work;
      std::vector<double> values(nv, 0.0), wmem(std::max<int64_t>(work, 1), 0.0);
      TaskBuilder tb;
      c2g::compile_twodm(tb, ctx, inst, 0, inst.size());
      ex.bind(kSlotWork, wmem.data(), work);
      exec(tb.finalize(), nullptr, 0, values.data(), nv);
      ex.bind(kSlotWork, nullptr, 0);
      c2g::twodm_assemble(*two_dm, site, inst, values);
      if (site > 0) {
        c2g::right_normalize(*bk, site, *mps_lay[site], mps[site], mps_lay[site - 1].get(), &mps[site - 1]);
        update(site - 1, false);
      }
    }
    two_dm->correct_higher_multiplicities();
  }

  // The correlation pass that follows the 2-RDM pass (CheMPS2/DMRGtechnics.cpp:157-176)
  // with the product's host parts: left normalisation site by site, the G/Y/Z/K/M tensors
  // (host/correlations.cpp programs) and Correlations::fill_pair.
  std::unique_ptr<CheMPS2::Correlations> corr;
  void calc_corr() {
    if (!two_dm) throw std::logic_error("correlations: no 2-RDM");
    corr = std::make_unique<CheMPS2::Correlations>(Prob, two_dm.get());
    std::unique_ptr<c2g::CorrTensors> cprev;
    std::vector<double> mprev;
    for (int site = 0; site < L - 1; site++) {
      c2g::left_normalize(*bk, site, *mps_lay[site], mps[site], mps_lay[site + 1].get(), &mps[site + 1]);
      const int s = site + 1;
      auto cnext = std::make_unique<c2g::CorrTensors>();
      const int slot = (s % 2 == 0) ? kSlotCorr0 : kSlotCorr1;
      c2g::allocate_corr(*cnext, *bk, s, slot);
      std::vector<double> mnext(std::max<int64_t>(cnext->size, 1), 0.0);
      ex.bind(slot, mnext.data(), cnext->size);
      {
        TaskBuilder tb;
        c2g::compile_corr_update(tb, *bk, *Prob, L, s, cprev.get(), *cnext, mpsT(site));
        exec(tb.finalize(), nullptr, 0, nullptr, 0);
      }
      {
        TaskBuilder tb;
        const int64_t work = c2g::compile_corr_fill(tb, *bk, s, mpsT(s), *cnext);
        const int nv = s * c2g::kCorrValues;
        std::vector<double> values(nv, 0.0), wmem(std::max<int64_t>(work, 1), 0.0);
        ex.bind(kSlotWork, wmem.data(), work);
        exec(tb.finalize(), nullptr, 0, values.data(), nv);
        ex.bind(kSlotWork, nullptr, 0);
        for (int q = 0; q < s; q++) corr->fill_pair(q, s, values.data() + q * c2g::kCorrValues);
      }
      if (cprev) ex.bind(cprev->slot, nullptr, 0);
      cprev = std::move(cnext);
      mprev = std::move(mnext);
      if (site <= L - 3) update(site, true);
    }
    if (cprev) ex.bind(cprev->slot, nullptr, 0);
  }

  HeffContext heff_ctx(const TwoSiteLayout& S, int index) {
    HeffContext ctx;
    ctx.bk = bk.get();
    ctx.prob = Prob;
    ctx.S = &S;
    ctx.left = (index > 0) ? ops[index - 1].get() : nullptr;
    ctx.right = (index + 1 < L - 1) ? ops[index + 1].get() : nullptr;
    return ctx;
  }

  std::vector<double> join(const TwoSiteLayout& S, int index) {
    std::vector<double> s(std::max<int64_t>(S.size(), 1), 0.0);
    TaskBuilder tb;
    compile_join(tb, *bk, S, mpsT(index), mpsT(index + 1));
    exec(tb.finalize(), nullptr, 0, s.data(), S.size());
    return s;
  }

  double solve_site(int index, double rtol, double noise, int D, bool mr, bool change) {
    TwoSiteLayout S;
    S.build(*bk, index);
    const int64_t n = S.size();
    std::vector<double> s = join(S, index);
    const HeffContext ctx = heff_ctx(S, index);
    int maxdim = 1;
    for (int k = 0; k < S.nkappa; k++) maxdim = std::max(maxdim, std::max(S.rows[k], S.cols[k]));
    ones.assign(maxdim, 1.0);
    ex.bind(kSlotOnes, ones.data(), maxdim);
    std::vector<double> diag(n, 0.0);
    exec(compile_heff_diag_program(ctx).program, nullptr, 0, diag.data(), n);
    const Program ph = compile_heff_program(ctx).program;
    ex.prepare_scratch(ph);
    if (check) {
      std::vector<double> dx(n, 0.0), dy(n, 0.0);
      ex.bind(kSlotX, dx.data(), n);
      ex.bind(kSlotY, dy.data(), n);
      ex.check(ph);
    }
    ex.run(ph, true, false);
    Davidson dv{n, 32, 3, rtol, 1e-12};
    const auto t0 = std::chrono::steady_clock::now();
    const double e = dv.solve(s, diag, [&](double* x, double* y) {
      ex.bind(kSlotX, x, n);
      ex.bind(kSlotY, y, n);
      ex.run(ph, false, true);
    });
    t_matvec += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    n_matvec += dv.n_matvec;
    const double energy = e + Prob->gEconst();
    if (noise > 0.0)
      for (int k = 0; k < S.nkappa; k++) {
        const double f = std::sqrt(S.TwoSR[k] + 1.0);
        for (int64_t c = S.k2i[k]; c < S.k2i[k + 1]; c++)
          s[c] += f * noise * (static_cast<double>(std::rand()) / RAND_MAX - 0.5);
      }
    MaxDisc = std::max(MaxDisc, split(S, s, index, D, mr, change));
    return energy;
  }

  double split(const TwoSiteLayout& S, std::vector<double>& s, int index, int D, bool mr, bool change) {
    const SplitPlan plan = plan_split(*bk, index, mr);
    std::vector<double> work(std::max<int64_t>(plan.work_size, 1), 0.0);
    ex.bind(kSlotWork, work.data(), plan.work_size);
    {
      TaskBuilder tb;
      compile_split_assemble(tb, *bk, S, plan);
      exec(tb.finalize(), s.data(), S.size(), nullptr, 0);
    }
    const int nC = static_cast<int>(plan.centers.size());
    std::vector<std::vector<double>> lambdas(nC);
    for (int ic = 0; ic < nC; ic++) {
      const SplitCenter& c = plan.centers[ic];
      if (c.cd <= 0) continue;
      std::vector<double> G(work.begin() + c.offG, work.begin() + c.offG + int64_t(c.g) * c.g), w, v;
      jacobi_eigh(G, c.g, w, v);
      for (int j = 0; j < c.g; j++) {
        // eigenvector gauge: largest-magnitude entry (first on ties) positive
        const double* col = &v[size_t(c.g) * (c.g - 1 - j)];
        int bi = 0;
        for (int i = 1; i < c.g; i++)
          if (std::fabs(col[i]) > std::fabs(col[bi])) bi = i;
        const double sgn = (col[bi] < 0.0) ? -1.0 : 1.0;
        for (int i = 0; i < c.g; i++) work[c.offU + i + int64_t(c.g) * j] = sgn * col[i];
      }
      lambdas[ic].resize(c.cd);
      for (int i = 0; i < c.cd; i++) lambdas[ic][i] = std::sqrt(std::max(w[c.g - 1 - i], 0.0));
    }
    double disc = 0.0;
    bool upd = false;
    std::vector<int> NewDims(nC);
    if (change) {
      int tot = 0;
      for (int ic = 0; ic < nC; ic++) {
        NewDims[ic] = plan.centers[ic].cd;
        tot += NewDims[ic];
      }
      if (tot > D) {
        std::vector<double> values;
        for (int ic = 0; ic < nC; ic++)
          for (int i = 0; i < NewDims[ic]; i++) values.push_back(lambdas[ic][i]);
        std::sort(values.begin(), values.end(), std::greater<double>());
        const double lb = values[D];
        for (int ic = 0; ic < nC; ic++)
          for (int cnt = 0; cnt < NewDims[ic]; cnt++)
            if (lambdas[ic][cnt] <= lb) NewDims[ic] = cnt;
        double ts = 0.0, ds = 0.0;
        for (int ic = 0; ic < nC; ic++)
          for (int i = 0; i < plan.centers[ic].cd; i++) {
            const double tmp = (plan.centers[ic].TwoSM + 1) * lambdas[ic][i] * lambdas[ic][i];
            ts += tmp;
            if (lambdas[ic][i] <= lb) ds += tmp;
          }
        disc = ds / ts;
      }
      for (int ic = 0; ic < nC; ic++) {
        const auto& c = plan.centers[ic];
        if (NewDims[ic] != bk->gCurrentDim(index + 1, c.NM, c.TwoSM, c.IM)) upd = true;
      }
    }
    if (upd)
      for (int ic = 0; ic < nC; ic++) {
        const auto& c = plan.centers[ic];
        bk->SetDim(index + 1, c.NM, c.TwoSM, c.IM, NewDims[ic]);
      }
    std::vector<int> dims_m(nC);
    for (int ic = 0; ic < nC; ic++) {
      const auto& c = plan.centers[ic];
      dims_m[ic] = bk->gCurrentDim(index + 1, c.NM, c.TwoSM, c.IM);
    }
    for (int site = index; site <= index + 1; site++) {
      mps_lay[site] = std::make_unique<MpsLayout>();
      mps_lay[site]->build(*bk, site);
      mps[site].assign(std::max<int64_t>(mps_lay[site]->size(), 1), 0.0);
      bind_mps(site);
    }
    {
      TaskBuilder tb;
      compile_split_copy(tb, plan, dims_m, mpsT(index), mpsT(index + 1));
      exec(tb.finalize(), nullptr, 0, nullptr, 0);
    }
    ex.bind(kSlotWork, nullptr, 0);
    return disc;
  }

  double sweep(bool mr, bool change, int instr) {
    const double noise = std::fabs(Opt->get_noise_prefactor(instr)) * MaxDisc;
    const double rtol = Opt->get_dvdson_rtol(instr);
    const int D = Opt->get_D(instr);
    MaxDisc = 0.0;
    double E = 0.0;
    if (mr) {
      for (int index = 0; index < L - 2; index++) {
        E = solve_site(index, rtol, noise, D, true, change);
        TotalMinEnergy = std::min(TotalMinEnergy, E);
        step_energies.push_back(E);
        update(index, true);
      }
    } else {
      for (int index = L - 2; index > 0; index--) {
        E = solve_site(index, rtol, noise, D, false, change);
        TotalMinEnergy = std::min(TotalMinEnergy, E);
        step_energies.push_back(E);
        update(index, false);
      }
    }
    return E;
  }

  double solve() {
    bool change = (TotalMinEnergy < 1e8);
    double E = 0.0;
    for (int instr = 0; instr < Opt->get_number(); instr++) {
      int it = 0;
      double Eprev = E + 10 * Opt->get_energy_conv(instr);
      while (std::fabs(E - Eprev) > Opt->get_energy_conv(instr) && it < Opt->get_max_sweeps(instr)) {
        Eprev = E;
        E = sweep(false, change, instr);
        change = true;
        E = sweep(true, change, instr);
        it++;
      }
    }
    return TotalMinEnergy;
  }
};

}  // namespace oracle

// ------------------------------------------------------------------------------ C API
namespace {
thread_local std::string g_err;

struct OracleHandle {
  std::unique_ptr<CheMPS2::Hamiltonian> ham;
  std::unique_ptr<CheMPS2::Problem> prob;
  std::unique_ptr<CheMPS2::ConvergenceScheme> opt;
  std::unique_ptr<oracle::OracleDMRG> dmrg;
};

template <class F>
int guard(F&& f) {
  try {
    f();
    return 0;
  } catch (const std::exception& e) {
    g_err = e.what();
    return -1;
  }
}
}  // namespace

extern "C" {

const char* oracle_last_error() { return g_err.c_str(); }

// Host threads of the task-program executor (groups of a stage run in parallel).
int oracle_set_threads(int n) {
  oracle::CpuExecutor::set_threads(n);
  return 0;
}

// Builds a Hamiltonian (tmat L x L, vmat L^4 in physics notation, element (i,j,k,l) at
// i + L*(j + L*(k + L*l))) or reads an FCIDUMP when fcidump is non-null, the Problem, the
// ConvergenceScheme and the CPU DMRG (random MPS from the C generator, PreSolve).
// reorder: 0 none, 1 SetupReorderD2h, 2 SetupReorderC2v.
int oracle_dmrg_create(const char* fcidump, int L, int group, const int* irreps, const double* tmat,
                       const double* vmat, double econst, int two_s, int n, int irrep, int reorder, int ninstr,
                       const int* D, const double* econv, const int* maxsweeps, const double* noise,
                       const double* rtol, int check_programs, void** out) {
  return guard([&] {
    auto h = std::make_unique<OracleHandle>();
    if (fcidump) {
      h->ham = std::make_unique<CheMPS2::Hamiltonian>(std::string(fcidump), group);
    } else {
      h->ham = std::make_unique<CheMPS2::Hamiltonian>(L, group, irreps);
      for (int i = 0; i < L; i++)
        for (int j = 0; j < L; j++)
          if (tmat[i + L * j] != 0.0) h->ham->setTmat(i, j, tmat[i + L * j]);
      for (int i = 0; i < L; i++)
        for (int j = 0; j < L; j++)
          for (int k = 0; k < L; k++)
            for (int l = 0; l < L; l++) {
              const double v = vmat[i + size_t(L) * (j + size_t(L) * (k + size_t(L) * l))];
              if (v != 0.0) h->ham->setVmat(i, j, k, l, v);
            }
      h->ham->setEconst(econst);
    }
    h->prob = std::make_unique<CheMPS2::Problem>(h->ham.get(), two_s, n, irrep);
    if (reorder == 1) h->prob->SetupReorderD2h();
    if (reorder == 2) h->prob->SetupReorderC2v();
    h->opt = std::make_unique<CheMPS2::ConvergenceScheme>(ninstr);
    for (int i = 0; i < ninstr; i++) h->opt->set_instruction(i, D[i], econv[i], maxsweeps[i], noise[i], rtol[i]);
    h->dmrg = std::make_unique<oracle::OracleDMRG>(h->prob.get(), h->opt.get(), check_programs != 0);
    *out = h.release();
  });
}

// As oracle_dmrg_create (no FCIDUMP) with the sector dimensions given: ndims rows of
// (boundary, N, 2S, I, dim) in `dims`; left operators for the first left_upto boundaries.
int oracle_dmrg_create_dims(int L, int group, const int* irreps, const double* tmat, const double* vmat,
                            double econst, int two_s, int n, int irrep, int D, int ndims, const int* dims,
                            int left_upto, void** out) {
  return guard([&] {
    auto h = std::make_unique<OracleHandle>();
    h->ham = std::make_unique<CheMPS2::Hamiltonian>(L, group, irreps);
    for (int i = 0; i < L; i++)
      for (int j = 0; j < L; j++)
        if (tmat[i + L * j] != 0.0) h->ham->setTmat(i, j, tmat[i + L * j]);
    for (int i = 0; i < L; i++)
      for (int j = 0; j < L; j++)
        for (int k = 0; k < L; k++)
          for (int l = 0; l < L; l++) {
            const double v = vmat[i + size_t(L) * (j + size_t(L) * (k + size_t(L) * l))];
            if (v != 0.0) h->ham->setVmat(i, j, k, l, v);
          }
    h->ham->setEconst(econst);
    h->prob = std::make_unique<CheMPS2::Problem>(h->ham.get(), two_s, n, irrep);
    h->opt = std::make_unique<CheMPS2::ConvergenceScheme>(1);
    h->opt->set_instruction(0, D, 1e-10, 1, 0.0, 1e-8);
    std::vector<std::array<int, 5>> rows(ndims);
    for (int r = 0; r < ndims; r++)
      for (int c = 0; c < 5; c++) rows[r][c] = dims[5 * r + c];
    h->dmrg = std::make_unique<oracle::OracleDMRG>(h->prob.get(), h->opt.get(), false, &rows, left_upto);
    *out = h.release();
  });
}

int oracle_dmrg_destroy(void* h) {
  delete static_cast<OracleHandle*>(h);
  return 0;
}

int oracle_dmrg_solve(void* h, double* energy) {
  return guard([&] { *energy = static_cast<OracleHandle*>(h)->dmrg->solve(); });
}

int oracle_dmrg_presolve(void* h) {
  return guard([&] { static_cast<OracleHandle*>(h)->dmrg->presolve(); });
}

int oracle_set_mx_element(void* h, int a, int b, int c, int d, double v) {
  return guard([&] { static_cast<OracleHandle*>(h)->prob->setMxElement(a, b, c, d, v); });
}

int oracle_dmrg_step_energies(void* h, double* out, int cap, int* count) {
  return guard([&] {
    auto& e = static_cast<OracleHandle*>(h)->dmrg->step_energies;
    *count = static_cast<int>(e.size());
    for (int i = 0; i < cap && i < static_cast<int>(e.size()); i++) out[i] = e[i];
  });
}

int oracle_dmrg_solve_site(void* h, int index, double rtol, double noise, int D, int mr, int change, double* energy) {
  return guard([&] {
    auto* d = static_cast<OracleHandle*>(h)->dmrg.get();
    *energy = d->solve_site(index, rtol, noise, D, mr != 0, change != 0);
  });
}

int oracle_dmrg_update(void* h, int index, int mr) {
  return guard([&] { static_cast<OracleHandle*>(h)->dmrg->update(index, mr != 0); });
}

int oracle_dmrg_sobject_size(void* h, int index, int64_t* n) {
  return guard([&] {
    auto* d = static_cast<OracleHandle*>(h)->dmrg.get();
    c2g::TwoSiteLayout S;
    S.build(*d->bk, index);
    *n = S.size();
  });
}

// y = Heff x at sites (index, index + 1) on the current state (symmetric convention); when
// join_into_x is set, x is first overwritten by the joined two-site object. nx is the
// length of x as bound for the program check (y must hold the two-site object).
int oracle_dmrg_heff_apply(void* h, int index, int join_into_x, double* x, int64_t nx, double* y, double* diag) {
  return guard([&] {
    auto* d = static_cast<OracleHandle*>(h)->dmrg.get();
    c2g::TwoSiteLayout S;
    S.build(*d->bk, index);
    const int64_t n = S.size();
    if (join_into_x) {
      auto s = d->join(S, index);
      std::copy(s.begin(), s.begin() + n, x);
    }
    const c2g::HeffContext ctx = d->heff_ctx(S, index);
    int maxdim = 1;
    for (int k = 0; k < S.nkappa; k++) maxdim = std::max(maxdim, std::max(S.rows[k], S.cols[k]));
    d->ones.assign(maxdim, 1.0);
    d->ex.bind(c2g::kSlotOnes, d->ones.data(), maxdim);
    d->exec(c2g::compile_heff_program(ctx).program, x, join_into_x ? n : nx, y, n);
    if (diag) d->exec(c2g::compile_heff_diag_program(ctx).program, nullptr, 0, diag, n);
  });
}

int oracle_dmrg_stats(void* h, double* out) {
  return guard([&] {
    auto* d = static_cast<OracleHandle*>(h)->dmrg.get();
    out[0] = static_cast<double>(d->n_matvec);
    out[1] = d->t_matvec;
    out[2] = static_cast<double>(d->ex.flops_done);
  });
}

// The MPS tensor of `site` (TensorT block order, column-major); *n receives its length.
int oracle_dmrg_get_mps(void* h, int site, double* out, int64_t cap, int64_t* n) {
  return guard([&] {
    auto* d = static_cast<OracleHandle*>(h)->dmrg.get();
    if (site < 0 || site >= d->L) throw std::out_of_range("site");
    const int64_t len = d->mps_lay[site]->size();
    *n = len;
    if (cap <= 0) return;
    if (cap < len) throw std::invalid_argument("buffer shorter than the tensor");
    std::copy(d->mps[site].begin(), d->mps[site].begin() + len, out);
  });
}

// Rows (N, 2S, I, FCI dim, current dim) of the oracle's bookkeeper at `boundary`.
int oracle_dmrg_sectors(void* h, int boundary, int* out, int cap, int* count) {
  return guard([&] {
    auto* d = static_cast<OracleHandle*>(h)->dmrg.get();
    const CheMPS2::SyBookkeeper& bk = *d->bk;
    if (boundary < 0 || boundary > bk.gL()) throw std::out_of_range("boundary");
    const int ns = bk.num_sectors(boundary);
    *count = ns;
    for (int id = 0; id < ns && id < cap; id++) {
      int n, s2, i;
      bk.sector_labels(boundary, id, &n, &s2, &i);
      out[5 * id + 0] = n;
      out[5 * id + 1] = s2;
      out[5 * id + 2] = i;
      out[5 * id + 3] = bk.fci_dim_by_id(boundary, id);
      out[5 * id + 4] = bk.cur_dim_by_id(boundary, id);
    }
  });
}

// The gauge changes of the 2-RDM pass (CheMPS2/DMRGtechnics.cpp:276-322) on the oracle's
// MPS, with the product's host routines (chemps2_gb300/csrc/host/gauge.cpp): kind 0
// left-normalises `site` and multiplies R into site + 1 (nothing at the last site), kind 1
// right-normalises `site` and multiplies L into site - 1. The operators are not updated.
int oracle_dmrg_gauge(void* h, int site, int kind) {
  return guard([&] {
    auto* d = static_cast<OracleHandle*>(h)->dmrg.get();
    if (site < 0 || site >= d->L) throw std::out_of_range("site");
    if (kind == 0) {
      if (site + 1 < d->L)
        c2g::left_normalize(*d->bk, site, *d->mps_lay[site], d->mps[site], d->mps_lay[site + 1].get(),
                            &d->mps[site + 1]);
      else
        c2g::left_normalize(*d->bk, site, *d->mps_lay[site], d->mps[site]);
    } else if (kind == 1) {
      if (site < 1) throw std::out_of_range("right normalisation needs a previous site");
      c2g::right_normalize(*d->bk, site, *d->mps_lay[site], d->mps[site], d->mps_lay[site - 1].get(),
                           &d->mps[site - 1]);
    } else {
      throw std::invalid_argument("gauge kind must be 0 (left) or 1 (right)");
    }
  });
}

// The 2-RDM of the current state (OracleDMRG::calc_2dm); A and B (L^4 each, element
// (a, b, c, d) at a + L (b + L (c + L d)), DMRG orbital order), its trace and energy.
int oracle_dmrg_calc_2dm(void* h, double* A, double* B, double* trace, double* energy) {
  return guard([&] {
    auto* d = static_cast<OracleHandle*>(h)->dmrg.get();
    d->calc_2dm();
    const CheMPS2::TwoDM& dm = *d->two_dm;
    const int L = d->L;
    for (int a = 0; a < L; a++)
      for (int b = 0; b < L; b++)
        for (int c = 0; c < L; c++)
          for (int e = 0; e < L; e++) {
            const size_t at = a + size_t(L) * (b + size_t(L) * (c + size_t(L) * e));
            if (A) A[at] = dm.getTwoDMA_DMRG(a, b, c, e);
            if (B) B[at] = dm.getTwoDMB_DMRG(a, b, c, e);
          }
    *trace = dm.trace();
    *energy = dm.energy();
  });
}

// The correlation pass after oracle_dmrg_calc_2dm: mutual information (L x L, DMRG order,
// element (r, c) at r + L c) and single-orbital entropies (L).
int oracle_dmrg_calc_correlations(void* h, double* mutinfo, double* entropy) {
  return guard([&] {
    auto* d = static_cast<OracleHandle*>(h)->dmrg.get();
    d->calc_corr();
    const int L = d->L;
    for (int r = 0; r < L; r++) {
      entropy[r] = d->corr->SingleOrbitalEntropy_DMRG(r);
      for (int c = 0; c < L; c++) mutinfo[r + size_t(L) * c] = d->corr->getMutualInformation_DMRG(r, c);
    }
  });
}

// DMRG::getFCIcoefficient on the oracle's MPS with the product's host routine
// (chemps2_gb300/csrc/host/fcicoef.cpp).
int oracle_dmrg_fci_coefficient(void* h, const int* alpha, const int* beta, double* coeff) {
  return guard([&] {
    auto* d = static_cast<OracleHandle*>(h)->dmrg.get();
    std::vector<const c2g::MpsLayout*> lay(d->L);
    std::vector<const double*> T(d->L);
    for (int k = 0; k < d->L; k++) {
      lay[k] = d->mps_lay[k].get();
      T[k] = d->mps[k].data();
    }
    *coeff = c2g::fci_coefficient(*d->bk, *d->Prob, lay, T, alpha, beta);
  });
}

int oracle_dmrg_num_orbitals(void* h, int* L) {
  return guard([&] { *L = static_cast<OracleHandle*>(h)->dmrg->L; });
}

int oracle_dmrg_num_mps_var(void* h, int* n) {
  return guard([&] {
    auto* d = static_cast<OracleHandle*>(h)->dmrg.get();
    int s = 0;
    for (int i = 0; i < d->L; i++) s += static_cast<int>(d->mps_lay[i]->size());
    *n = s;
  });
}

}  // extern "C"
