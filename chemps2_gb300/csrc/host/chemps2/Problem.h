// Drop-in replacement for CheMPS2::Problem (CheMPS2/include/chemps2/Problem.h).
//
// Holds the targeted symmetry sector (2S, N, irrep) and the DMRG matrix elements
//   h_{abcd} = V_{abcd} + (delta_ac T_bd + delta_bd T_ac) / (N - 1)
// built by construct_mxelem() (CheMPS2/Problem.cpp:363-384) in DMRG orbital order, plus
// the orbital reorderings (CheMPS2/Problem.cpp:57-335). As in the reference, the DMRG
// constructor calls construct_mxelem(); a caller that overwrites elements with
// setMxElement() afterwards must call DMRG::PreSolve() (tests/test12.cpp.in:67-80).
#pragma once

#include <vector>

#include "Hamiltonian.h"

namespace CheMPS2 {

class Problem {
 public:
  Problem(const Hamiltonian* Hamin, const int TwoSin, const int Nin, const int Irrepin);

  int gL() const { return L; }
  int gSy() const { return Ham->getNGroup(); }
  int gIrrep(const int nOrb) const;
  int gTwoS() const { return TwoS; }
  int gN() const { return N; }
  int gIrrep() const { return Irrep; }
  double gEconst() const { return Ham->getEconst(); }
  const Hamiltonian* gHamiltonian() const { return Ham; }

  double gMxElement(const int a, const int b, const int c, const int d) const {
    return mx_elem[a + L * (b + L * (c + static_cast<size_t>(L) * d))];
  }
  void setMxElement(const int a, const int b, const int c, const int d, const double value) {
    mx_elem[a + L * (b + L * (c + static_cast<size_t>(L) * d))] = value;
  }
  void construct_mxelem();
  bool has_mxelem() const { return !mx_elem.empty(); }
  const double* mxelem_data() const { return mx_elem.data(); }

  bool checkConsistency() const;
  // Whether occupations (0, 1, 2 per DMRG site) give the targeted (N, 2S, irrep) with the
  // singly occupied sites high-spin coupled (CheMPS2/Problem.cpp:422-451).
  bool check_rohf_occ(const int* occupancies) const;

  bool gReorder() const { return bReorder; }
  int gf1(const int HamOrb) const { return bReorder ? f1[HamOrb] : -1; }
  int gf2(const int DMRGOrb) const { return bReorder ? f2[DMRGOrb] : -1; }
  void SetupReorderD2h();
  void SetupReorderC2v();
  void setup_reorder_custom(int* dmrg2ham);

 private:
  const Hamiltonian* Ham;
  int L, TwoS, N, Irrep;
  bool bReorder;
  std::vector<int> f1, f2;  // ham -> dmrg, dmrg -> ham
  std::vector<double> mx_elem;
};

}  // namespace CheMPS2
