// The coefficient of one determinant in the MPS (CheMPS2/DMRGtechnics.cpp:324-470,
// DMRG::getFCIcoefficient and getSpecificCoefficient).
#pragma once

#include <vector>

#include "chemps2/Problem.h"
#include "chemps2/SyBookkeeper.h"
#include "layout.hpp"

namespace c2g {

// alpha[h], beta[h] in {0, 1}: the occupations of Hamiltonian orbital h (the Problem's
// reordering maps DMRG site k to orbital f2(k)). The MPS tensors of every site are given
// in MpsLayout storage. Returns the coefficient of that determinant (its 2Sz component of
// the spin multiplet), or 0 when its particle number, 2Sz or irrep cannot occur in the
// targeted sector (the reference prints a message and returns 0 there).
double fci_coefficient(const CheMPS2::SyBookkeeper& bk, const CheMPS2::Problem& prob,
                       const std::vector<const MpsLayout*>& lay, const std::vector<const double*>& T,
                       const int* alpha, const int* beta);

}  // namespace c2g
