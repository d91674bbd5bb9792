#include "gauge.hpp"

#include <algorithm>
#include <atomic>
#include <array>
#include <cmath>
#include <thread>

namespace c2g {

namespace {
// Calls f(k) for k in [0, n) on up to 16 host threads (the sectors of a gauge change touch
// disjoint blocks of both tensors).
template <class F>
void parallel_sectors(size_t n, F f) {
  const size_t nt = std::min<size_t>(n, std::min(16u, std::max(1u, std::thread::hardware_concurrency())));
  if (nt <= 1) {
    for (size_t k = 0; k < n; k++) f(k);
    return;
  }
  std::atomic<size_t> next{0};
  auto work = [&] {
    for (size_t k = next++; k < n; k = next++) f(k);
  };
  std::vector<std::thread> pool;
  for (size_t t = 1; t < nt; t++) pool.emplace_back(work);
  work();
  for (auto& t : pool) t.join();
}
}  // namespace

void householder_qr(int m, int n, const std::vector<double>& ain, std::vector<double>& q, std::vector<double>& r) {
  std::vector<double> a(ain);
  const int kk = std::min(m, n);
  std::vector<double> tau(kk, 0.0);
  // dgeqr2: reflector j zeroes column j below the diagonal and is applied to the trailing
  // columns
  for (int j = 0; j < kk; j++) {
    double* x = &a[j + static_cast<size_t>(m) * j];
    const int len = m - j;
    double xnorm = 0.0;
    for (int i = 1; i < len; i++) xnorm += x[i] * x[i];
    xnorm = std::sqrt(xnorm);
    if (xnorm == 0.0) {
      tau[j] = 0.0;
      continue;
    }
    const double alpha = x[0];
    const double beta = -std::copysign(std::hypot(alpha, xnorm), alpha);
    tau[j] = (beta - alpha) / beta;
    const double scal = 1.0 / (alpha - beta);
    for (int i = 1; i < len; i++) x[i] *= scal;
    x[0] = beta;
    for (int c = j + 1; c < n; c++) {
      double* y = &a[j + static_cast<size_t>(m) * c];
      double s = y[0];
      for (int i = 1; i < len; i++) s += x[i] * y[i];
      s *= tau[j];
      y[0] -= s;
      for (int i = 1; i < len; i++) y[i] -= s * x[i];
    }
  }
  r.assign(static_cast<size_t>(n) * n, 0.0);
  for (int i = 0; i < kk; i++)
    for (int c = i; c < n; c++) r[i + static_cast<size_t>(n) * c] = a[i + static_cast<size_t>(m) * c];
  // dorg2r: Q = H_1 ... H_kk applied to the first kk columns of the identity
  q.assign(static_cast<size_t>(m) * n, 0.0);
  for (int c = 0; c < kk; c++) q[c + static_cast<size_t>(m) * c] = 1.0;
  for (int j = kk - 1; j >= 0; j--) {
    const double* v = &a[j + static_cast<size_t>(m) * j];
    const int len = m - j;
    for (int c = j; c < kk; c++) {
      double* y = &q[j + static_cast<size_t>(m) * c];
      double s = y[0];
      for (int i = 1; i < len; i++) s += v[i] * y[i];
      s *= tau[j];
      y[0] -= s;
      for (int i = 1; i < len; i++) y[i] -= s * v[i];
    }
  }
}

void left_normalize(const CheMPS2::SyBookkeeper& bk, int site, const MpsLayout& lay, std::vector<double>& data,
                    const MpsLayout* next_lay, std::vector<double>* next) {
  std::vector<std::array<int, 3>> sectors;
  for (int NR = bk.gNmin(site + 1); NR <= bk.gNmax(site + 1); NR++)
    for (int TwoSR = bk.gTwoSmin(site + 1, NR); TwoSR <= bk.gTwoSmax(site + 1, NR); TwoSR += 2)
      for (int IR = 0; IR < bk.getNumberOfIrreps(); IR++)
        if (bk.gCurrentDim(site + 1, NR, TwoSR, IR) > 0) sectors.push_back({NR, TwoSR, IR});
  parallel_sectors(sectors.size(), [&](size_t sec) {
    const int NR = sectors[sec][0], TwoSR = sectors[sec][1], IR = sectors[sec][2];
    const int n = bk.gCurrentDim(site + 1, NR, TwoSR, IR);
    std::vector<int> blocks;
    int m = 0;
    for (int k = 0; k < lay.nkappa; k++)
      if (lay.NR[k] == NR && lay.TwoSR[k] == TwoSR && lay.IR[k] == IR && lay.rows[k] > 0) {
        blocks.push_back(k);
        m += lay.rows[k];
      }
    if (m == 0) {
      // A right sector that no block of this site feeds holds states without a left
      // history (a virtual dimension kept fixed through a sweep can leave such
      // states): they are zero vectors, and R is zero there, so the next site's
      // blocks of that left sector vanish. (The reference leaves this R block
      // uninitialised, CheMPS2/TensorT.cpp:209 with CheMPS2/TensorOperator.cpp:100.)
      if (next)
        for (int k = 0; k < next_lay->nkappa; k++)
          if (next_lay->NL[k] == NR && next_lay->TwoSL[k] == TwoSR && next_lay->IL[k] == IR)
            std::fill_n(next->data() + next_lay->k2i[k], static_cast<size_t>(n) * next_lay->cols[k], 0.0);
      return;
    }
    std::vector<double> a(static_cast<size_t>(m) * n), q, r;
    int r0 = 0;
    for (int k : blocks) {
      for (int l = 0; l < lay.rows[k]; l++)
        for (int c = 0; c < n; c++) a[r0 + l + static_cast<size_t>(m) * c] = data[lay.k2i[k] + l + lay.rows[k] * c];
      r0 += lay.rows[k];
    }
    householder_qr(m, n, a, q, r);
    r0 = 0;
    for (int k : blocks) {
      for (int l = 0; l < lay.rows[k]; l++)
        for (int c = 0; c < n; c++) data[lay.k2i[k] + l + lay.rows[k] * c] = q[r0 + l + static_cast<size_t>(m) * c];
      r0 += lay.rows[k];
    }
    if (!next) return;
    // TensorT::LeftMultiply: next blocks with left sector (NR, TwoSR, IR) <- R * block
    for (int k = 0; k < next_lay->nkappa; k++) {
      if (next_lay->NL[k] != NR || next_lay->TwoSL[k] != TwoSR || next_lay->IL[k] != IR) continue;
      const int cols = next_lay->cols[k];
      double* blk = next->data() + next_lay->k2i[k];
      std::vector<double> tmp(static_cast<size_t>(n) * cols, 0.0);
      for (int c = 0; c < cols; c++)
        for (int p = 0; p < n; p++) {
          const double b = blk[p + static_cast<size_t>(n) * c];
          for (int i = 0; i <= p; i++) tmp[i + static_cast<size_t>(n) * c] += r[i + static_cast<size_t>(n) * p] * b;
        }
      std::copy(tmp.begin(), tmp.end(), blk);
    }
  });
}

void right_normalize(const CheMPS2::SyBookkeeper& bk, int site, const MpsLayout& lay, std::vector<double>& data,
                     const MpsLayout* prev_lay, std::vector<double>* prev) {
  std::vector<std::array<int, 3>> sectors;
  for (int NL = bk.gNmin(site); NL <= bk.gNmax(site); NL++)
    for (int TwoSL = bk.gTwoSmin(site, NL); TwoSL <= bk.gTwoSmax(site, NL); TwoSL += 2)
      for (int IL = 0; IL < bk.getNumberOfIrreps(); IL++)
        if (bk.gCurrentDim(site, NL, TwoSL, IL) > 0) sectors.push_back({NL, TwoSL, IL});
  parallel_sectors(sectors.size(), [&](size_t sec) {
    const int NL = sectors[sec][0], TwoSL = sectors[sec][1], IL = sectors[sec][2];
    const int dimL = bk.gCurrentDim(site, NL, TwoSL, IL);
    std::vector<int> blocks;
    int ntot = 0;
    for (int k = 0; k < lay.nkappa; k++)
      if (lay.NL[k] == NL && lay.TwoSL[k] == TwoSL && lay.IL[k] == IL && lay.cols[k] > 0) {
        blocks.push_back(k);
        ntot += lay.cols[k];
      }
    if (ntot == 0) {
      // A left sector without any block to its right holds states without a right
      // completion: L is zero there, so the previous site's blocks of that right
      // sector vanish (left uninitialised by the reference, CheMPS2/TensorT.cpp:312).
      if (prev)
        for (int k = 0; k < prev_lay->nkappa; k++)
          if (prev_lay->NR[k] == NL && prev_lay->TwoSR[k] == TwoSL && prev_lay->IR[k] == IL)
            std::fill_n(prev->data() + prev_lay->k2i[k], static_cast<size_t>(prev_lay->rows[k]) * dimL, 0.0);
      return;
    }
    // M^T (ntot x dimL), blocks scaled by sqrt((2 S_R + 1) / (2 S_L + 1))
    std::vector<double> mt(static_cast<size_t>(ntot) * dimL), q, r;
    int c0 = 0;
    for (int k : blocks) {
      const double f = std::sqrt((lay.TwoSR[k] + 1.0) / (TwoSL + 1.0));
      for (int l = 0; l < dimL; l++)
        for (int c = 0; c < lay.cols[k]; c++)
          mt[c0 + c + static_cast<size_t>(ntot) * l] = f * data[lay.k2i[k] + l + dimL * c];
      c0 += lay.cols[k];
    }
    // M = L Q with L = R^T (dimL x dimL) and Q = Q'^T (dimL x ntot)
    householder_qr(ntot, dimL, mt, q, r);
    c0 = 0;
    for (int k : blocks) {
      const double f = std::sqrt((TwoSL + 1.0) / (lay.TwoSR[k] + 1.0));
      for (int l = 0; l < dimL; l++)
        for (int c = 0; c < lay.cols[k]; c++)
          data[lay.k2i[k] + l + dimL * c] = f * q[c0 + c + static_cast<size_t>(ntot) * l];
      c0 += lay.cols[k];
    }
    if (!prev) return;
    // TensorT::RightMultiply: prev blocks with right sector (NL, TwoSL, IL) <- block * L
    for (int k = 0; k < prev_lay->nkappa; k++) {
      if (prev_lay->NR[k] != NL || prev_lay->TwoSR[k] != TwoSL || prev_lay->IR[k] != IL) continue;
      const int rows = prev_lay->rows[k];
      double* blk = prev->data() + prev_lay->k2i[k];
      std::vector<double> tmp(static_cast<size_t>(rows) * dimL, 0.0);
      // (block * L)(i, c) = sum_p block(i, p) L(p, c), L(p, c) = R(c, p), nonzero for c <= p
      for (int c = 0; c < dimL; c++)
        for (int p = c; p < dimL; p++) {
          const double lpc = r[c + static_cast<size_t>(dimL) * p];
          if (lpc == 0.0) continue;
          for (int i = 0; i < rows; i++)
            tmp[i + static_cast<size_t>(rows) * c] += blk[i + static_cast<size_t>(rows) * p] * lpc;
        }
      std::copy(tmp.begin(), tmp.end(), blk);
    }
  });
}

}  // namespace c2g
