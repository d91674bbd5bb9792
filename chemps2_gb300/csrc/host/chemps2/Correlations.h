// Drop-in replacement for CheMPS2::Correlations (CheMPS2/include/chemps2/Correlations.h):
// spin, density, spin-flip and singlet-diradical correlation functions, single-orbital
// entropies and the two-orbital mutual information of a DMRG state
// (CheMPS2/Correlations.cpp). Tables are L x L (row + L col) in the DMRG orbital order.
#pragma once

#include <vector>

#include "Problem.h"
#include "TwoDM.h"

namespace CheMPS2 {

class Correlations {
 public:
  // Fills the spin, density, spin-flip and the 2-RDM part of the diradical tables from the
  // 2-RDM (CheMPS2/Correlations.cpp:69-103). The mutual information and the rest of the
  // diradical table come from DMRG::calc2DMandCorrelations.
  Correlations(const Problem* prob, const TwoDM* dm);

  double getCspin_DMRG(int r, int c) const { return Cspin_[r + L_ * c]; }
  double getCdens_DMRG(int r, int c) const { return Cdens_[r + L_ * c]; }
  double getCspinflip_DMRG(int r, int c) const { return Cspinflip_[r + L_ * c]; }
  double getCdirad_DMRG(int r, int c) const { return Cdirad_[r + L_ * c]; }
  double getMutualInformation_DMRG(int r, int c) const { return MutInfo_[r + L_ * c]; }
  double getCspin_HAM(int r, int c) const { return getCspin_DMRG(h(r), h(c)); }
  double getCdens_HAM(int r, int c) const { return getCdens_DMRG(h(r), h(c)); }
  double getCspinflip_HAM(int r, int c) const { return getCspinflip_DMRG(h(r), h(c)); }
  double getCdirad_HAM(int r, int c) const { return getCdirad_DMRG(h(r), h(c)); }
  double getMutualInformation_HAM(int r, int c) const { return getMutualInformation_DMRG(h(r), h(c)); }
  // CheMPS2/Correlations.cpp:165-186
  double SingleOrbitalEntropy_DMRG(int i) const;
  double SingleOrbitalEntropy_HAM(int i) const { return SingleOrbitalEntropy_DMRG(h(i)); }
  // sum_{r != c} I(r, c) |r - c|^power (CheMPS2/Correlations.cpp:188-201)
  double MutualInformationDistance(double power) const;
  int gL() const { return L_; }

  // The two-orbital density matrix of orbitals (prev, site) from the 13 diagram values of
  // the correlation pass (in the order of compile_corr_fill), its entropy, the mutual
  // information and the diradical update (CheMPS2/Correlations.cpp:212-351).
  void fill_pair(int prev, int site, const double* v);

 private:
  const Problem* prob_;
  const TwoDM* dm_;
  int L_;
  std::vector<double> Cspin_, Cdens_, Cspinflip_, Cdirad_, MutInfo_;
  int h(int a) const { return prob_->gReorder() ? prob_->gf1(a) : a; }
};

}  // namespace CheMPS2
