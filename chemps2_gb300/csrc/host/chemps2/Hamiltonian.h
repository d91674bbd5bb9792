// Drop-in replacement for CheMPS2::Hamiltonian (CheMPS2/include/chemps2/Hamiltonian.h:61-107).
//
// Same constructor and accessors: L orbitals, a psi4 point group number (0..7) and one
// irrep per orbital. One-body elements T_ij are symmetric and only non-zero between
// orbitals of equal irrep (asserted as in CheMPS2/Hamiltonian.cpp:106). Two-body elements
// are in physics notation, V_ijkl = (ik|jl) in chemists' notation, with the 8-fold
// permutation symmetry of real orbitals (CheMPS2/include/chemps2/FourIndex.h:30-32) and
// non-zero only when I_i x I_j = I_k x I_l (asserted as in CheMPS2/Hamiltonian.cpp:125).
// Storage is dense (L^2 and L^4 doubles): a setter writes every symmetry-equivalent slot,
// so a getter is a single load.
#pragma once

#include <string>
#include <vector>

namespace CheMPS2 {

class Hamiltonian {
 public:
  Hamiltonian(const int Norbitals, const int nGroup, const int* OrbIrreps);
  // FCIDUMP reader: chemists' integrals are swapped to physics notation on input
  // (CheMPS2/Hamiltonian.cpp:296-424, swap at :405); ORBSYM uses molpro numbering.
  Hamiltonian(const std::string& fcidumpfile, const int psi4groupnumber);

  int getL() const { return L; }
  int getNGroup() const { return group; }
  int getOrbitalIrrep(const int nOrb) const { return orb2irrep[nOrb]; }

  void setEconst(const double val) { Econst = val; }
  double getEconst() const { return Econst; }

  void setTmat(const int i, const int j, const double val);
  double getTmat(const int i, const int j) const { return tmat[i + L * j]; }

  void setVmat(const int i, const int j, const int k, const int l, const double val);
  void addToVmat(const int i, const int j, const int k, const int l, const double val);
  // Writes the Hamiltonian as an FCIDUMP file (CheMPS2/Hamiltonian.cpp:539-582): the
  // header with Molpro irrep numbers, every symmetry-allowed two-electron integral (pq|rs)
  // with p >= q, r >= s and (p, q) >= (r, s), the one-electron integrals h_pq (p >= q,
  // same irrep), then the constant.
  void writeFCIDUMP(const std::string& fcidumpfile, const int Nelec, const int TwoS, const int TargetIrrep) const;
  double getVmat(const int i, const int j, const int k, const int l) const {
    return vmat[i + L * (j + L * (k + static_cast<size_t>(L) * l))];
  }

 private:
  int L;
  int group;
  double Econst;
  std::vector<int> orb2irrep;
  std::vector<double> tmat;
  std::vector<double> vmat;
  void allocate();
  void set_all_vmat(int i, int j, int k, int l, double val, bool add);
};

}  // namespace CheMPS2
