// ORACLE (test infrastructure, not product code): full configuration interaction in the
// determinant basis, for small systems, as an independent check of DMRG energies.
//
// Plays the role of CheMPS2::FCI (CheMPS2/include/chemps2/FCI.h:43,100,110) in the
// reference's DMRG-versus-FCI tests (tests/test1-4.cpp.in): the Hamiltonian
//   H = sum_ij T_ij E_ij + 1/2 sum_ijkl V_ijkl sum_st a+_is a+_jt a_lt a_ks
// (V in physics notation, V_ijkl = (ik|jl)) is applied in the space of determinants with
// N_up = (N + 2S)/2 up and N_down = (N - 2S)/2 down electrons whose irrep product equals
// the target, and its lowest eigenvalue is found by Davidson iteration. This space holds
// every spin >= S; the tests use systems whose lowest state in it has spin S.
#include <algorithm>
#include <cmath>
#include <functional>
#include <map>
#include <cstdint>
#include <cstring>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

#include "exec_cpu.hpp"

namespace {

thread_local std::string g_fci_err;

int popcount(uint64_t x) { return __builtin_popcountll(x); }

struct Strings {
  std::vector<uint64_t> str;
  std::vector<int> irrep;
  std::vector<int> index_of;  // dense over 2^L, -1 when absent (L <= 24)
};

Strings make_strings(int L, int ne, const int* orb_irrep) {
  Strings s;
  s.index_of.assign(size_t(1) << L, -1);
  for (uint64_t m = 0; m < (uint64_t(1) << L); m++) {
    if (popcount(m) != ne) continue;
    int ir = 0;
    for (int i = 0; i < L; i++)
      if (m >> i & 1) ir ^= orb_irrep[i];
    s.index_of[m] = static_cast<int>(s.str.size());
    s.str.push_back(m);
    s.irrep.push_back(ir);
  }
  return s;
}

// a+_i a_j |m>: returns the sign (0 if the result vanishes) and the new string.
inline int excite(uint64_t m, int i, int j, uint64_t& out) {
  if (!(m >> j & 1)) return 0;
  uint64_t t = m & ~(uint64_t(1) << j);
  if (t >> i & 1) return 0;
  int sgn = (popcount(m & ((uint64_t(1) << j) - 1)) & 1) ? -1 : 1;
  sgn *= (popcount(t & ((uint64_t(1) << i) - 1)) & 1) ? -1 : 1;
  out = t | (uint64_t(1) << i);
  return sgn;
}

struct FCI {
  int L;
  std::vector<double> T, V;  // V physics notation
  Strings A, B;
  std::vector<int64_t> det_of;  // [ia * nb + ib] -> det index or -1
  std::vector<std::pair<int, int>> dets;
  struct Exc {
    int to;
    int sign;
  };
  std::vector<std::vector<std::vector<Exc>>> exA, exB;  // [string][ij] (ij = i + L j)

  void build_exc(const Strings& S, std::vector<std::vector<std::vector<Exc>>>& ex) {
    ex.assign(S.str.size(), std::vector<std::vector<Exc>>(size_t(L) * L));
    for (size_t k = 0; k < S.str.size(); k++)
      for (int i = 0; i < L; i++)
        for (int j = 0; j < L; j++) {
          uint64_t o;
          const int sg = excite(S.str[k], i, j, o);
          if (sg) ex[k][i + size_t(L) * j].push_back({S.index_of[o], sg});
        }
  }

  // D[ij][det] = <det| E_ij |c>
  void apply_E(int i, int j, const std::vector<double>& c, std::vector<double>& out) {
    const size_t nb = B.str.size();
    std::fill(out.begin(), out.end(), 0.0);
    for (size_t d = 0; d < dets.size(); d++) {
      const double cd = c[d];
      if (cd == 0.0) continue;
      const int ia = dets[d].first, ib = dets[d].second;
      for (const Exc& e : exA[ia][i + size_t(L) * j]) {
        const int64_t t = det_of[size_t(e.to) * nb + ib];
        if (t >= 0) out[t] += e.sign * cd;
      }
      for (const Exc& e : exB[ib][i + size_t(L) * j]) {
        const int64_t t = det_of[size_t(ia) * nb + e.to];
        if (t >= 0) out[t] += e.sign * cd;
      }
    }
  }

  // sigma = H c, with H = sum_ij k_ij E_ij + 1/2 sum_ijkl (ij|kl) E_ij E_kl,
  // k_ij = T_ij - 1/2 sum_k (ik|kj), (ij|kl) = V_ikjl. The E_kl c and the (i, j) terms
  // run on the oracle's host threads (each thread sums its (i, j) terms into its own
  // vector; the vectors are added in thread order, so the result does not depend on the
  // scheduling).
  void sigma(const std::vector<double>& c, std::vector<double>& s) {
    const size_t n = dets.size();
    const size_t L2 = size_t(L) * L;
    const int nt = std::max(1, std::min<int>(oracle::CpuExecutor::threads(), static_cast<int>(L2)));
    auto parallel = [&](const std::function<void(int)>& f) {
      std::vector<std::thread> pool;
      for (int t = 1; t < nt; t++) pool.emplace_back(f, t);
      f(0);
      for (auto& th : pool) th.join();
    };
    std::vector<std::vector<double>> D(L2, std::vector<double>(n));
    parallel([&](int t) {
      for (size_t kl = t; kl < L2; kl += nt) apply_E(static_cast<int>(kl % L), static_cast<int>(kl / L), c, D[kl]);
    });
    auto chem = [&](int i, int j, int k, int l) { return V[i + size_t(L) * (k + size_t(L) * (j + size_t(L) * l))]; };
    std::vector<std::vector<double>> part(nt, std::vector<double>(n, 0.0));
    parallel([&](int t) {
      std::vector<double> G(n), tmp(n);
      std::vector<double>& acc = part[t];
      for (size_t ij = t; ij < L2; ij += nt) {
        const int i = static_cast<int>(ij % L), j = static_cast<int>(ij / L);
        double kij = T[i + size_t(L) * j];
        for (int k = 0; k < L; k++) kij -= 0.5 * chem(i, k, k, j);
        for (size_t d = 0; d < n; d++) G[d] = kij * c[d];
        for (int k = 0; k < L; k++)
          for (int l = 0; l < L; l++) {
            const double v = 0.5 * chem(i, j, k, l);
            if (v == 0.0) continue;
            const std::vector<double>& Dkl = D[k + size_t(L) * l];
            for (size_t d = 0; d < n; d++) G[d] += v * Dkl[d];
          }
        apply_E(i, j, G, tmp);
        for (size_t d = 0; d < n; d++) acc[d] += tmp[d];
      }
    });
    std::fill(s.begin(), s.end(), 0.0);
    for (int t = 0; t < nt; t++)
      for (size_t d = 0; d < n; d++) s[d] += part[t][d];
  }

  double diag_element(size_t d) {
    const uint64_t a = A.str[dets[d].first], b = B.str[dets[d].second];
    double e = 0.0;
    auto occ = [&](uint64_t m, int i) { return int(m >> i & 1); };
    for (int i = 0; i < L; i++) e += (occ(a, i) + occ(b, i)) * T[i + size_t(L) * i];
    auto Vp = [&](int i, int j, int k, int l) { return V[i + size_t(L) * (j + size_t(L) * (k + size_t(L) * l))]; };
    for (int i = 0; i < L; i++)
      for (int j = 0; j < L; j++) {
        const int ni = occ(a, i) + occ(b, i);
        const int nj = occ(a, j) + occ(b, j);
        double coul = 0.5 * Vp(i, j, i, j) * ni * nj;
        if (i == j) coul -= 0.5 * Vp(i, i, i, i) * (occ(a, i) + occ(b, i));  // remove self pairs
        const int same = occ(a, i) * occ(a, j) + occ(b, i) * occ(b, j);
        const double exch = (i == j) ? 0.0 : 0.5 * Vp(i, j, j, i) * same;
        e += coul - exch;
      }
    return e;
  }
};

}  // namespace

extern "C" {

const char* oracle_fci_last_error() { return g_fci_err.c_str(); }

// Lowest eigenvalue of H (plus econst) in the (N_up, N_down, irrep) determinant space.
// tmat: L x L; vmat: L^4 physics notation, (i,j,k,l) at i + L*(j + L*(k + L*l)).
// With A / B non-null, also the spin-summed 2-RDMs of that eigenvector
// (CheMPS2/include/chemps2/TwoDM.h definitions, same index layout as vmat):
//   A_ijkl = sum_st <a+_is a+_jt a_lt a_ks>,
//   B_ijkl = sum_s (<a+_is a+_js a_ls a_ks> - <a+_is a+_j-s a_l-s a_ks>),
// from <a+_is a+_jt a_lt a_ks> = <E^s_ik E^t_jl> - delta_jk delta_st <E^s_il> with
// E^s_pq = a+_ps a_qs.
int oracle_fci_state(int L, const int* orb_irrep, const double* tmat, const double* vmat, double econst, int n_up,
                     int n_down, int irrep, double tol, int max_iter, double* energy, int64_t* dim, double* A,
                     double* B);

int oracle_fci_ground_state(int L, const int* orb_irrep, const double* tmat, const double* vmat, double econst,
                            int n_up, int n_down, int irrep, double tol, int max_iter, double* energy, int64_t* dim) {
  return oracle_fci_state(L, orb_irrep, tmat, vmat, econst, n_up, n_down, irrep, tol, max_iter, energy, dim, nullptr,
                          nullptr);
}

}  // extern "C"

namespace {
// The ground state of the determinant space; `extra` sees the solver and the normalised
// eigenvector.
int fci_core(int L, const int* orb_irrep, const double* tmat, const double* vmat, double econst, int n_up,
             int n_down, int irrep, double tol, int max_iter, double* energy, int64_t* dim, double* A, double* B,
             const std::function<void(FCI&, const std::vector<double>&)>& extra) {
  try {
    if (L > 24) throw std::invalid_argument("FCI oracle: at most 24 orbitals");
    FCI f;
    f.L = L;
    f.T.assign(tmat, tmat + size_t(L) * L);
    f.V.assign(vmat, vmat + size_t(L) * L * L * L);
    f.A = make_strings(L, n_up, orb_irrep);
    f.B = make_strings(L, n_down, orb_irrep);
    const size_t na = f.A.str.size(), nb = f.B.str.size();
    f.det_of.assign(na * nb, -1);
    // All (N_up, N_down) determinants: the intermediate vectors E_kl |c> of the sigma
    // build leave the target irrep. The iterates are kept in the target irrep by masking.
    std::vector<char> target;
    for (size_t ia = 0; ia < na; ia++)
      for (size_t ib = 0; ib < nb; ib++) {
        f.det_of[ia * nb + ib] = static_cast<int64_t>(f.dets.size());
        f.dets.push_back({static_cast<int>(ia), static_cast<int>(ib)});
        target.push_back((f.A.irrep[ia] ^ f.B.irrep[ib]) == irrep);
      }
    const size_t n = f.dets.size();
    size_t ntarget = 0;
    for (char c : target) ntarget += c;
    *dim = static_cast<int64_t>(ntarget);
    if (ntarget == 0) throw std::invalid_argument("FCI oracle: empty determinant space");
    f.build_exc(f.A, f.exA);
    f.build_exc(f.B, f.exB);
    std::vector<double> hd(n);
    for (size_t d = 0; d < n; d++) hd[d] = f.diag_element(d);
    // Davidson with diagonal preconditioner, restart at 24 vectors.
    size_t best = n;
    for (size_t d = 0; d < n; d++)
      if (target[d] && (best == n || hd[d] < hd[best])) best = d;
    std::vector<std::vector<double>> vs, hv;
    std::vector<double> t(n, 0.0);
    t[best] = 1.0;
    for (size_t d = 0; d < n; d++)
      if (target[d]) t[d] += 1e-3 * std::sin(1.0 + d);  // break symmetry ties
    double theta = 0.0;
    auto dot = [&](const std::vector<double>& x, const std::vector<double>& y) {
      double s = 0.0;
      for (size_t i = 0; i < n; i++) s += x[i] * y[i];
      return s;
    };
    std::vector<double> ritz(n), hritz(n);
    for (int it = 0; it < max_iter; it++) {
      for (size_t d = 0; d < n; d++)
        if (!target[d]) t[d] = 0.0;
      for (int pass = 0; pass < 2; pass++)
        for (auto& v : vs) {
          const double o = dot(v, t);
          for (size_t i = 0; i < n; i++) t[i] -= o * v[i];
        }
      const double nt = std::sqrt(dot(t, t));
      if (nt < 1e-14) break;
      for (auto& e : t) e /= nt;
      vs.push_back(t);
      hv.emplace_back(n);
      f.sigma(vs.back(), hv.back());
      const int m = static_cast<int>(vs.size());
      std::vector<double> Hm(size_t(m) * m);
      for (int a = 0; a < m; a++)
        for (int b = 0; b < m; b++) Hm[a + size_t(m) * b] = dot(vs[a], hv[b]);
      // Jacobi on the small matrix
      std::vector<double> Vm(size_t(m) * m, 0.0);
      for (int a = 0; a < m; a++) Vm[a + size_t(m) * a] = 1.0;
      for (int sw = 0; sw < 100; sw++) {
        double off = 0.0;
        for (int a = 0; a < m; a++)
          for (int b = 0; b < m; b++)
            if (a != b) off += Hm[a + size_t(m) * b] * Hm[a + size_t(m) * b];
        if (off < 1e-28) break;
        for (int p = 0; p < m; p++)
          for (int q = p + 1; q < m; q++) {
            const double apq = Hm[p + size_t(m) * q];
            if (apq == 0.0) continue;
            const double tau = (Hm[q + size_t(m) * q] - Hm[p + size_t(m) * p]) / (2 * apq);
            const double tt = (tau >= 0 ? 1.0 : -1.0) / (std::fabs(tau) + std::sqrt(1 + tau * tau));
            const double c = 1 / std::sqrt(1 + tt * tt), s = tt * c;
            for (int j = 0; j < m; j++) {
              const double x = Hm[p + size_t(m) * j], y = Hm[q + size_t(m) * j];
              Hm[p + size_t(m) * j] = c * x - s * y;
              Hm[q + size_t(m) * j] = s * x + c * y;
            }
            for (int i = 0; i < m; i++) {
              const double x = Hm[i + size_t(m) * p], y = Hm[i + size_t(m) * q];
              Hm[i + size_t(m) * p] = c * x - s * y;
              Hm[i + size_t(m) * q] = s * x + c * y;
              const double vx = Vm[i + size_t(m) * p], vy = Vm[i + size_t(m) * q];
              Vm[i + size_t(m) * p] = c * vx - s * vy;
              Vm[i + size_t(m) * q] = s * vx + c * vy;
            }
          }
      }
      int lo = 0;
      for (int a = 1; a < m; a++)
        if (Hm[a + size_t(m) * a] < Hm[lo + size_t(m) * lo]) lo = a;
      theta = Hm[lo + size_t(m) * lo];
      std::fill(ritz.begin(), ritz.end(), 0.0);
      std::fill(hritz.begin(), hritz.end(), 0.0);
      for (int a = 0; a < m; a++) {
        const double y = Vm[a + size_t(m) * lo];
        for (size_t i = 0; i < n; i++) {
          ritz[i] += y * vs[a][i];
          hritz[i] += y * hv[a][i];
        }
      }
      double rn = 0.0;
      for (size_t i = 0; i < n; i++) {
        const double r = hritz[i] - theta * ritz[i];
        rn += r * r;
        const double den = hd[i] - theta;
        t[i] = -r / ((std::fabs(den) > 1e-10) ? den : 1e-10);
      }
      if (std::sqrt(rn) < tol) break;
      if (m >= 24) {  // restart with the Ritz vector
        vs.clear();
        hv.clear();
        vs.push_back(ritz);
        hv.push_back(hritz);
      }
    }
    *energy = theta + econst;
    if (A || B) {
      double nr = 0.0;
      for (double x : ritz) nr += x * x;
      nr = std::sqrt(nr);
      for (double& x : ritz) x /= nr;
      // Es[s][p + L q] = E^s_pq |c>, s = 0 up, 1 down
      const size_t nb = f.B.str.size();
      std::vector<std::vector<double>> Es[2];
      for (int sp = 0; sp < 2; sp++) Es[sp].assign(size_t(L) * L, std::vector<double>(n, 0.0));
      for (size_t d = 0; d < n; d++) {
        const double cd = ritz[d];
        if (cd == 0.0) continue;
        const int ia = f.dets[d].first, ib = f.dets[d].second;
        for (int p = 0; p < L; p++)
          for (int q = 0; q < L; q++) {
            for (const auto& e : f.exA[ia][p + size_t(L) * q]) {
              const int64_t t = f.det_of[size_t(e.to) * nb + ib];
              if (t >= 0) Es[0][p + size_t(L) * q][t] += e.sign * cd;
            }
            for (const auto& e : f.exB[ib][p + size_t(L) * q]) {
              const int64_t t = f.det_of[size_t(ia) * nb + e.to];
              if (t >= 0) Es[1][p + size_t(L) * q][t] += e.sign * cd;
            }
          }
      }
      auto dot = [&](const std::vector<double>& x, const std::vector<double>& y) {
        double s = 0.0;
        for (size_t q = 0; q < n; q++) s += x[q] * y[q];
        return s;
      };
      // one-body <E^s_il> = c . E^s_il c
      std::vector<double> one[2];
      for (int sp = 0; sp < 2; sp++) {
        one[sp].assign(size_t(L) * L, 0.0);
        for (int p = 0; p < L; p++)
          for (int q = 0; q < L; q++) one[sp][p + size_t(L) * q] = dot(ritz, Es[sp][p + size_t(L) * q]);
      }
      for (int i = 0; i < L; i++)
        for (int j = 0; j < L; j++)
          for (int k = 0; k < L; k++)
            for (int l = 0; l < L; l++) {
              double g[2][2];
              for (int s1 = 0; s1 < 2; s1++)
                for (int s2 = 0; s2 < 2; s2++) {
                  // <E^s1_ik E^s2_jl> = (E^s1_ki c) . (E^s2_jl c)
                  double v = dot(Es[s1][k + size_t(L) * i], Es[s2][j + size_t(L) * l]);
                  if (j == k && s1 == s2) v -= one[s1][i + size_t(L) * l];
                  g[s1][s2] = v;
                }
              const size_t at = i + size_t(L) * (j + size_t(L) * (k + size_t(L) * l));
              if (A) A[at] = g[0][0] + g[0][1] + g[1][0] + g[1][1];
              if (B) B[at] = g[0][0] + g[1][1] - g[0][1] - g[1][0];
            }
    }
    if (extra) {
      double nr = 0.0;
      for (double x : ritz) nr += x * x;
      nr = std::sqrt(nr);
      std::vector<double> v(ritz);
      for (double& x : v) x /= nr;
      extra(f, v);
    }
    return 0;
  } catch (const std::exception& e) {
    g_fci_err = e.what();
    return -1;
  }
}

// Eigenvalues of a symmetric n x n matrix (cyclic Jacobi).
std::vector<double> sym_eig(std::vector<double> a, int n) {
  for (int sw = 0; sw < 100; sw++) {
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
        const double c = 1 / std::sqrt(1 + t * t), sn = t * c;
        for (int j = 0; j < n; j++) {
          const double x = a[p + n * j], y = a[q + n * j];
          a[p + n * j] = c * x - sn * y;
          a[q + n * j] = sn * x + c * y;
        }
        for (int i = 0; i < n; i++) {
          const double x = a[i + n * p], y = a[i + n * q];
          a[i + n * p] = c * x - sn * y;
          a[i + n * q] = sn * x + c * y;
        }
      }
  }
  std::vector<double> ev(n);
  for (int i = 0; i < n; i++) ev[i] = a[i + n * i];
  return ev;
}

double entropy_of(const std::vector<double>& ev) {
  double e = 0.0;
  for (double x : ev)
    if (x > 1e-100) e -= x * std::log(x);
  return e;
}

// Reduced density matrix of a set of spin orbitals ("modes", global index o for up and
// L + o for down; the fermionic order is all up modes, then all down modes), in the basis
// c+_i |vac> with c+_i the product of the creators of configuration i in ascending mode
// order: rho_ij = <psi| c+_i P_vac c_j |psi>, P_vac the projector on the empty modes.
std::vector<double> mode_rdm(FCI& f, const std::vector<double>& psi, const std::vector<int>& modes) {
  const int L = f.L, nm = static_cast<int>(modes.size()), dim = 1 << nm;
  const size_t nb = f.B.str.size();
  std::vector<double> rho(size_t(dim) * dim, 0.0);
  auto det_mask = [&](size_t d) {
    return f.A.str[f.dets[d].first] | (f.B.str[f.dets[d].second] << L);
  };
  auto find = [&](uint64_t m) -> int64_t {
    const uint64_t a = m & ((uint64_t(1) << L) - 1), b = m >> L;
    const int ia = f.A.index_of[a], ib = f.B.index_of[b];
    if (ia < 0 || ib < 0) return -1;
    return f.det_of[size_t(ia) * nb + ib];
  };
  auto sign_before = [](uint64_t m, int k) { return (__builtin_popcountll(m & ((uint64_t(1) << k) - 1)) & 1) ? -1 : 1; };
  for (size_t d = 0; d < f.dets.size(); d++) {
    const double cd = psi[d];
    if (cd == 0.0) continue;
    const uint64_t m0 = det_mask(d);
    // configuration j of the modes in this determinant; c_j = (c+_j)^+ applies the
    // annihilator of the lowest mode first
    int j = 0;
    for (int t = 0; t < nm; t++)
      if (m0 >> modes[t] & 1) j |= 1 << t;
    int sgn = 1;
    uint64_t m = m0;
    for (int t = 0; t < nm; t++)
      if (j >> t & 1) {
        sgn *= sign_before(m, modes[t]);
        m &= ~(uint64_t(1) << modes[t]);
      }
    // c+_i creates configuration i in ascending order applied right to left: the last
    // creator acts first
    for (int i = 0; i < dim; i++) {
      int s2 = sgn;
      uint64_t mm = m;
      for (int t = nm - 1; t >= 0; t--)
        if (i >> t & 1) {
          s2 *= sign_before(mm, modes[t]);
          mm |= uint64_t(1) << modes[t];
        }
      const int64_t e = find(mm);
      if (e < 0) continue;
      rho[i + size_t(dim) * j] += psi[e] * s2 * cd;
    }
  }
  return rho;
}
}  // namespace

extern "C" {

int oracle_fci_state(int L, const int* orb_irrep, const double* tmat, const double* vmat, double econst, int n_up,
                     int n_down, int irrep, double tol, int max_iter, double* energy, int64_t* dim, double* A,
                     double* B) {
  return fci_core(L, orb_irrep, tmat, vmat, econst, n_up, n_down, irrep, tol, max_iter, energy, dim, A, B, nullptr);
}

// Two-orbital density matrix of orbitals p < q as the plain partial trace in the orbital
// tensor-product basis: amplitudes in the orbital-major fermionic order (0 up, 0 down,
// 1 up, ...) grouped by the configuration of the other orbitals, with no Jordan-Wigner
// string for the orbitals between p and q.
std::vector<double> orbital_pair_rdm(FCI& f, const std::vector<double>& psi, int p, int q) {
  const int L = f.L;
  std::map<std::pair<uint64_t, uint64_t>, std::vector<std::pair<int, double>>> env;
  for (size_t d = 0; d < f.dets.size(); d++) {
    if (psi[d] == 0.0) continue;
    const uint64_t a = f.A.str[f.dets[d].first], b = f.B.str[f.dets[d].second];
    // sign of reordering all-up-then-all-down into orbital-major order
    int swaps = 0;
    for (int i = 0; i < L; i++)
      if (b >> i & 1) swaps += __builtin_popcountll(a >> (i + 1));
    const double amp = (swaps & 1) ? -psi[d] : psi[d];
    const int cfg = int(a >> p & 1) + 2 * int(b >> p & 1) + 4 * int(a >> q & 1) + 8 * int(b >> q & 1);
    const uint64_t clear = ~((uint64_t(1) << p) | (uint64_t(1) << q));
    env[{a & clear, b & clear}].push_back({cfg, amp});
  }
  std::vector<double> rho(256, 0.0);
  for (const auto& kv : env)
    for (const auto& x : kv.second)
      for (const auto& y : kv.second) rho[x.first + 16 * y.first] += x.second * y.second;
  return rho;
}

// Single-orbital entropies s1[L] and the mutual information mi[L*L] (row + L col):
// I_pq = (s_p + s_q - s_pq) / 2 from the one- and two-orbital reduced density matrices
// of the FCI ground state (the quantities of CheMPS2/Correlations.cpp:165-351), averaged
// over the spin multiplet like the reference's (its density matrices carry the factor
// 1 / (2S + 1)): for n_up != n_down the density matrices of the state and of its spin
// partner with n_up and n_down exchanged are averaged, which is the multiplet average
// for a doublet (the case this oracle covers besides singlets).
// jw != 0: the fermionic two-orbital RDM (mode operators, the parity of the orbitals
// between p and q included); jw == 0: the tensor-product partial trace without it, the
// definition the reference's correlation tensors follow (TensorGYZ / TensorKM are
// updated without the Jordan-Wigner phase, CheMPS2/TensorKM.cpp:27-30).
int oracle_fci_mutual_information(int L, const int* orb_irrep, const double* tmat, const double* vmat,
                                  double econst, int n_up, int n_down, int irrep, double tol, int max_iter, int jw,
                                  double* energy, double* s1, double* mi) {
  if (std::abs(n_up - n_down) > 1) {
    g_fci_err = "FCI oracle: mutual information only for singlets and doublets";
    return -1;
  }
  std::vector<std::vector<double>> r1(L, std::vector<double>(16, 0.0));
  std::vector<std::vector<double>> r2(size_t(L) * L, std::vector<double>(256, 0.0));
  const int nstates = (n_up == n_down) ? 1 : 2;
  for (int st = 0; st < nstates; st++) {
    const int nu = st == 0 ? n_up : n_down, nd = st == 0 ? n_down : n_up;
    int64_t dim = 0;
    double e = 0.0;
    const int rc = fci_core(L, orb_irrep, tmat, vmat, econst, nu, nd, irrep, tol, max_iter, &e, &dim, nullptr, nullptr,
                            [&](FCI& f, const std::vector<double>& psi) {
                              for (int p = 0; p < L; p++) {
                                const std::vector<double> r = mode_rdm(f, psi, {p, L + p});
                                for (int k = 0; k < 16; k++) r1[p][k] += r[k] / nstates;
                                for (int q = p + 1; q < L; q++) {
                                  const std::vector<double> rr =
                                      jw ? mode_rdm(f, psi, {p, q, L + p, L + q}) : orbital_pair_rdm(f, psi, p, q);
                                  for (int k = 0; k < 256; k++) r2[p + size_t(L) * q][k] += rr[k] / nstates;
                                }
                              }
                            });
    if (rc != 0) return rc;
    if (st == 0) *energy = e;
  }
  std::vector<double> s(L);
  for (int p = 0; p < L; p++) s[p] = entropy_of(sym_eig(r1[p], 4));
  for (int p = 0; p < L; p++) {
    s1[p] = s[p];
    mi[p + size_t(L) * p] = 0.0;
    for (int q = p + 1; q < L; q++) {
      const double spq = entropy_of(sym_eig(r2[p + size_t(L) * q], 16));
      mi[p + size_t(L) * q] = mi[q + size_t(L) * p] = 0.5 * (s[p] + s[q] - spq);
    }
  }
  return 0;
}

}  // extern "C"
