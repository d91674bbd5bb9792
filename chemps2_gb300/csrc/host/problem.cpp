// Hamiltonian, Problem and ConvergenceScheme: the host side of the drop-in API.
// Behaviour follows CheMPS2/Hamiltonian.cpp, CheMPS2/Problem.cpp and
// CheMPS2/ConvergenceScheme.cpp; the storage is dense instead of irrep-blocked.
#include <cassert>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <sstream>
#include <stdexcept>
#include <string>

#include "chemps2/ConvergenceScheme.h"
#include "chemps2/Hamiltonian.h"
#include "chemps2/Problem.h"
#include "symm.hpp"

namespace CheMPS2 {

// ---------------------------------------------------------------- Hamiltonian ----

Hamiltonian::Hamiltonian(const int Norbitals, const int nGroup, const int* OrbIrreps)
    : L(Norbitals), group(nGroup), Econst(0.0) {
  if (nGroup < 0 || nGroup > 7) throw std::invalid_argument("Hamiltonian: group must be 0..7");
  const int nirr = c2g::num_irreps(nGroup);
  orb2irrep.assign(OrbIrreps, OrbIrreps + L);
  for (int o = 0; o < L; o++) {
    if (orb2irrep[o] < 0 || orb2irrep[o] >= nirr)
      throw std::invalid_argument("Hamiltonian: orbital irrep out of range");
  }
  allocate();
}

void Hamiltonian::allocate() {
  tmat.assign(static_cast<size_t>(L) * L, 0.0);
  vmat.assign(static_cast<size_t>(L) * L * L * L, 0.0);
}

void Hamiltonian::setTmat(const int i, const int j, const double val) {
  // CheMPS2/Hamiltonian.cpp:104-109: only same-irrep elements exist.
  if (orb2irrep[i] != orb2irrep[j]) throw std::invalid_argument("setTmat: irreps differ");
  tmat[i + L * j] = val;
  tmat[j + L * i] = val;
}

void Hamiltonian::set_all_vmat(int i, int j, int k, int l, double val, bool add) {
  if (c2g::irrep_prod(orb2irrep[i], orb2irrep[j]) != c2g::irrep_prod(orb2irrep[k], orb2irrep[l]))
    throw std::invalid_argument("setVmat: I_i x I_j != I_k x I_l");
  // The 8 physics-notation permutations of (ik|jl): the slots the reference's
  // FourIndex container maps onto one storage element.
  const int perm[8][4] = {{i, j, k, l}, {k, j, i, l}, {i, l, k, j}, {k, l, i, j},
                          {j, i, l, k}, {l, i, j, k}, {j, k, l, i}, {l, k, j, i}};
  if (add) {
    // addToVmat adds once to the shared element; every slot gets the same new value.
    const double nv = getVmat(i, j, k, l) + val;
    for (auto& p : perm) vmat[p[0] + L * (p[1] + L * (p[2] + static_cast<size_t>(L) * p[3]))] = nv;
  } else {
    for (auto& p : perm) vmat[p[0] + L * (p[1] + L * (p[2] + static_cast<size_t>(L) * p[3]))] = val;
  }
}

void Hamiltonian::setVmat(const int i, const int j, const int k, const int l, const double val) {
  set_all_vmat(i, j, k, l, val, false);
}

void Hamiltonian::addToVmat(const int i, const int j, const int k, const int l, const double val) {
  set_all_vmat(i, j, k, l, val, true);
}

namespace {
// psi4 -> molpro irrep numbers (CheMPS2/Irreps.cpp:184-214).
void psi2molpro(int group, int* map) {
  switch (group) {
    case 0: map[0] = 1; break;
    case 1: case 2: case 3: map[0] = 1; map[1] = 2; break;
    case 4: map[0] = 1; map[1] = 4; map[2] = 3; map[3] = 2; break;
    case 5: case 6: map[0] = 1; map[1] = 4; map[2] = 2; map[3] = 3; break;
    case 7: {
      const int m[8] = {1, 4, 6, 7, 8, 5, 3, 2};
      for (int i = 0; i < 8; i++) map[i] = m[i];
      break;
    }
    default: break;
  }
}

std::string upper(std::string s) {
  for (auto& c : s) c = static_cast<char>(toupper(static_cast<unsigned char>(c)));
  return s;
}
}  // namespace

Hamiltonian::Hamiltonian(const std::string& fcidumpfile, const int psi4groupnumber)
    : L(0), group(psi4groupnumber), Econst(0.0) {
  std::ifstream in(fcidumpfile);
  if (!in) throw std::runtime_error("Hamiltonian: unable to open FCIDUMP " + fcidumpfile);
  // Header: everything up to the terminating "/" or "&END" line.
  std::string header, line;
  while (std::getline(in, line)) {
    const std::string u = upper(line);
    header += u + " ";
    if (u.find("&END") != std::string::npos || u.find('/') != std::string::npos) break;
  }
  auto find_int = [&](const char* key) {
    const size_t p = header.find(key);
    if (p == std::string::npos) throw std::runtime_error(std::string("FCIDUMP: no ") + key);
    return std::atoi(header.c_str() + header.find('=', p) + 1);
  };
  L = find_int("NORB");
  const int nirr = c2g::num_irreps(group);
  int map[8] = {0};
  psi2molpro(group, map);
  orb2irrep.assign(L, 0);
  {
    size_t p = header.find("ORBSYM");
    if (p == std::string::npos) throw std::runtime_error("FCIDUMP: no ORBSYM");
    p = header.find('=', p) + 1;
    for (int o = 0; o < L; o++) {
      while (p < header.size() && !isdigit(static_cast<unsigned char>(header[p]))) p++;
      const int molpro = std::atoi(header.c_str() + p);
      while (p < header.size() && isdigit(static_cast<unsigned char>(header[p]))) p++;
      int psi = -1;
      for (int ir = 0; ir < nirr; ir++)
        if (map[ir] == molpro) psi = ir;
      if (psi < 0) throw std::runtime_error("FCIDUMP: ORBSYM not in the point group");
      orb2irrep[o] = psi;
    }
  }
  allocate();
  double value;
  int i1, i2, i3, i4;
  while (in >> value >> i1 >> i2 >> i3 >> i4) {
    if (i4 != 0) {
      setVmat(i1 - 1, i3 - 1, i2 - 1, i4 - 1, value);  // chemists' -> physics notation
    } else if (i2 != 0) {
      setTmat(i1 - 1, i2 - 1, value);
    } else {
      Econst = value;
    }
  }
}

void Hamiltonian::writeFCIDUMP(const std::string& fcidumpfile, const int Nelec, const int TwoS,
                               const int TargetIrrep) const {
  int map[8] = {0};
  psi2molpro(group, map);
  FILE* f = std::fopen(fcidumpfile.c_str(), "w");
  if (!f) throw std::runtime_error("writeFCIDUMP: unable to open " + fcidumpfile);
  std::fprintf(f, " &FCI NORB= %d,NELEC= %d,MS2= %d,\n  ORBSYM=", L, Nelec, TwoS);
  for (int o = 0; o < L; o++) std::fprintf(f, "%d,", map[orb2irrep[o]]);
  std::fprintf(f, "\n  ISYM=%d,\n /\n", map[TargetIrrep]);
  auto line = [&](double v, int a, int b, int c, int d) { std::fprintf(f, " % 23.16E %3d %3d %3d %3d\n", v, a, b, c, d); };
  // (pq|rs) = V_prqs in physics notation
  for (int p = 0; p < L; p++)
    for (int q = 0; q <= p; q++)
      for (int r = 0; r <= p; r++)
        for (int s = 0; s <= r; s++) {
          if ((orb2irrep[p] ^ orb2irrep[q]) != (orb2irrep[r] ^ orb2irrep[s])) continue;
          if (p == r && q < s) continue;
          line(getVmat(p, r, q, s), p + 1, q + 1, r + 1, s + 1);
        }
  for (int p = 0; p < L; p++)
    for (int q = 0; q <= p; q++)
      if (orb2irrep[p] == orb2irrep[q]) line(getTmat(p, q), p + 1, q + 1, 0, 0);
  std::fprintf(f, " % 23.16E %3d %3d %3d %3d", Econst, 0, 0, 0, 0);
  std::fclose(f);
}

// ---------------------------------------------------------------- Problem --------

Problem::Problem(const Hamiltonian* Hamin, const int TwoSin, const int Nin, const int Irrepin)
    : Ham(Hamin), L(Hamin->getL()), TwoS(TwoSin), N(Nin), Irrep(Irrepin), bReorder(false) {}

int Problem::gIrrep(const int nOrb) const {
  return Ham->getOrbitalIrrep(bReorder ? f2[nOrb] : nOrb);
}

void Problem::construct_mxelem() {
  // CheMPS2/Problem.cpp:363-384
  mx_elem.assign(static_cast<size_t>(L) * L * L * L, 0.0);
  const double prefact = 1.0 / (N - 1);
  for (int o1 = 0; o1 < L; o1++) {
    const int m1 = bReorder ? f2[o1] : o1;
    for (int o2 = 0; o2 < L; o2++) {
      const int m2 = bReorder ? f2[o2] : o2;
      for (int o3 = 0; o3 < L; o3++) {
        const int m3 = bReorder ? f2[o3] : o3;
        for (int o4 = 0; o4 < L; o4++) {
          const int m4 = bReorder ? f2[o4] : o4;
          setMxElement(o1, o2, o3, o4,
                       Ham->getVmat(m1, m2, m3, m4) +
                           prefact * ((o1 == o3) ? Ham->getTmat(m2, m4) : 0) +
                           prefact * ((o2 == o4) ? Ham->getTmat(m1, m3) : 0));
        }
      }
    }
  }
}

bool Problem::check_rohf_occ(const int* occupancies) const {
  // CheMPS2/Problem.cpp:422-451
  int n = 0, two_s = 0, irrep = 0;
  for (int k = 0; k < L; k++) {
    if (occupancies[k] < 0 || occupancies[k] > 2) return false;
    n += occupancies[k];
    if (occupancies[k] == 1) {
      two_s += 1;
      irrep ^= gIrrep(k);
    }
  }
  return n == N && two_s == TwoS && irrep == Irrep;
}

bool Problem::checkConsistency() const {
  // CheMPS2/Problem.cpp:386-421
  const int nirr = c2g::num_irreps(gSy());
  if (Irrep < 0 || Irrep >= nirr) return false;
  if (TwoS < 0 || N < 0 || L < 0) return false;
  if (N > 2 * L) return false;
  if ((N % 2) != (TwoS % 2)) return false;
  if (TwoS > L - std::abs(N - L)) return false;
  return true;
}

void Problem::SetupReorderD2h() {
  // CheMPS2/Problem.cpp:57-94: Ag, B1u, B3u, B2g, B2u, B3g, B1g, Au
  bReorder = false;
  if (gSy() != 7) return;
  const int order[8] = {0, 5, 7, 2, 6, 3, 1, 4};
  f1.assign(L, 0);
  f2.assign(L, 0);
  int d = 0;
  for (int ir = 0; ir < 8; ir++)
    for (int h = 0; h < L; h++)
      if (Ham->getOrbitalIrrep(h) == order[ir]) { f1[h] = d; f2[d] = h; d++; }
  bReorder = true;
}

void Problem::SetupReorderC2v() {
  // CheMPS2/Problem.cpp:96-147: A1 reversed, then B1, B2, A2
  bReorder = false;
  if (gSy() != 5) return;
  const int order[4] = {0, 2, 3, 1};
  f1.assign(L, 0);
  f2.assign(L, 0);
  int d = 0;
  for (int h = L - 1; h >= 0; h--)
    if (Ham->getOrbitalIrrep(h) == order[0]) { f1[h] = d; f2[d] = h; d++; }
  for (int ir = 1; ir < 4; ir++)
    for (int h = 0; h < L; h++)
      if (Ham->getOrbitalIrrep(h) == order[ir]) { f1[h] = d; f2[d] = h; d++; }
  bReorder = true;
}

void Problem::setup_reorder_custom(int* dmrg2ham) {
  // CheMPS2/Problem.cpp:149-170
  f1.assign(L, -2);
  f2.assign(L, 0);
  for (int d = 0; d < L; d++) {
    if (dmrg2ham[d] < 0 || dmrg2ham[d] >= L) throw std::invalid_argument("reorder out of range");
    f2[d] = dmrg2ham[d];
    f1[dmrg2ham[d]] = d;
  }
  for (int h = 0; h < L; h++)
    if (f1[h] < 0) throw std::invalid_argument("reorder is not a permutation");
  bReorder = true;
}

// ---------------------------------------------------------------- ConvergenceScheme

ConvergenceScheme::ConvergenceScheme(const int n)
    : D(n, 0), maxsweeps(n, 0), econv(n, 0.0), noise(n, 0.0), rtol(n, 0.0) {
  if (n <= 0) throw std::invalid_argument("ConvergenceScheme: need >= 1 instruction");
}

void ConvergenceScheme::set_instruction(const int i, const int d, const double ec,
                                        const int ms, const double nz, const double rt) {
  // CheMPS2/ConvergenceScheme.cpp:50-62 asserts, turned into exceptions.
  if (i < 0 || i >= get_number()) throw std::invalid_argument("instruction out of range");
  if (d <= 0 || !(ec > 0.0) || ms <= 0 || !(rt > 0.0))
    throw std::invalid_argument("set_instruction: D, Econv, maxSweeps and rtol must be > 0");
  D[i] = d;
  econv[i] = ec;
  maxsweeps[i] = ms;
  noise[i] = nz;
  rtol[i] = rt;
}

}  // namespace CheMPS2
