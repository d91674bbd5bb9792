// Drop-in replacement for CheMPS2::TwoDM (CheMPS2/include/chemps2/TwoDM.h): the spin-summed
// two-particle density matrices of a DMRG state,
//   A_{ab;cd} = sum_{st} < a+_{a s} a+_{b t} a_{d t} a_{c s} >,
//   B_{ab;cd} = sum_s ( < a+_{a s} a+_{b s} a_{d s} a_{c s} > - < a+_{a s} a+_{b -s} a_{d -s} a_{c s} > ),
// averaged over the spin multiplet, stored as L^4 arrays (a + L (b + L (c + L d))) in the
// DMRG orbital order. DMRG::calc2DMandCorrelations fills them (CheMPS2/TwoDM.cpp:445-640).
#pragma once

#include <vector>

#include "Problem.h"

namespace CheMPS2 {

class TwoDM {
 public:
  TwoDM(const Problem* prob, int L);

  // 2-RDM elements in the DMRG orbital order (zero unless the irreps allow them)
  double getTwoDMA_DMRG(int a, int b, int c, int d) const;
  double getTwoDMB_DMRG(int a, int b, int c, int d) const;
  // 1-RDM from A: sum_r A_{ar;br} / (N - 1)
  double get1RDM_DMRG(int a, int b) const;
  // spin density (CheMPS2/TwoDM.cpp:144-163)
  double spin_density_dmrg(int a, int b) const;
  // The same in the Hamiltonian's orbital order (Problem reordering undone)
  double getTwoDMA_HAM(int a, int b, int c, int d) const;
  double getTwoDMB_HAM(int a, int b, int c, int d) const;
  double get1RDM_HAM(int a, int b) const;
  double spin_density_ham(int a, int b) const;
  // sum_ab A_{ab;ab} = N (N - 1)
  double trace() const;
  // Econst + 1/2 sum_abcd A_{ab;cd} h_{abcd}: the energy of the state
  double energy() const;
  int gL() const { return L_; }

  // Writers used while the density matrices are assembled: each sets the element and its
  // three images under (a b)(c d) and (a c)(b d) exchange.
  void set_A(int a, int b, int c, int d, double v);
  void set_B(int a, int b, int c, int d, double v);
  // Divides both arrays by 2S + 1 (CheMPS2/TwoDM.cpp:630-640)
  void correct_higher_multiplicities();
  const std::vector<double>& A() const { return A_; }
  const std::vector<double>& B() const { return B_; }

 private:
  const Problem* prob_;
  int L_;
  std::vector<double> A_, B_;
  size_t at(int a, int b, int c, int d) const {
    return static_cast<size_t>(a) + L_ * (static_cast<size_t>(b) + L_ * (static_cast<size_t>(c) + L_ * static_cast<size_t>(d)));
  }
  bool allowed(int a, int b, int c, int d) const;
  int ham2dmrg(int a) const;
};

}  // namespace CheMPS2
