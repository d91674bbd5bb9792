// Drop-in replacement for CheMPS2::ConvergenceScheme
// (CheMPS2/include/chemps2/ConvergenceScheme.h, CheMPS2/ConvergenceScheme.cpp:50-77).
// Each instruction holds the reduced virtual dimension D, the energy convergence
// threshold (> 0), the maximum number of left+right sweeps (> 0), the noise prefactor and
// the Davidson residual tolerance (> 0, default 1e-5 via setInstruction).
#pragma once

#include <vector>

namespace CheMPS2 {

class ConvergenceScheme {
 public:
  explicit ConvergenceScheme(const int num_instructions);
  int get_number() const { return static_cast<int>(D.size()); }
  void set_instruction(const int instruction, const int D, const double energy_conv,
                       const int max_sweeps, const double noise_prefactor,
                       const double davidson_rtol);
  void setInstruction(const int instruction, const int D, const double energy_conv,
                      const int max_sweeps, const double noise_prefactor) {
    set_instruction(instruction, D, energy_conv, max_sweeps, noise_prefactor, 1e-5);
  }
  int get_D(const int i) const { return D[i]; }
  double get_energy_conv(const int i) const { return econv[i]; }
  int get_max_sweeps(const int i) const { return maxsweeps[i]; }
  double get_noise_prefactor(const int i) const { return noise[i]; }
  double get_dvdson_rtol(const int i) const { return rtol[i]; }

 private:
  std::vector<int> D, maxsweeps;
  std::vector<double> econv, noise, rtol;
};

}  // namespace CheMPS2
