// Symmetry helpers shared by the host task compiler: abelian irreps, spin phases,
// triangle-index inversion and Wigner 6j / 9j symbols.
//
// Reference behaviour followed:
//   * irrep products are a bitwise XOR in psi4's numbering
//     (CheMPS2/include/chemps2/Irreps.h:123);
//   * phase(2p) = (-1)^p for an integer p (CheMPS2/include/chemps2/Special.h);
//   * the 6j symbol is the Racah single sum over square roots of factorials, and the
//     9j symbol the sum over products of three 6j symbols (CheMPS2/Wigner.cpp:294-370).
//     The square-root-factorial table is generated at full precision by
//     gen_sqrt_fact.py, so both symbols agree with the reference to rounding.
#pragma once

#include <cstdlib>

namespace c2g {

inline int irrep_prod(int a, int b) { return a ^ b; }

// Number of irreps of the psi4 point groups c1, ci, c2, cs, d2, c2v, c2h, d2h.
inline int num_irreps(int group) {
  if (group < 0 || group > 7) return -1;
  if (group == 0) return 1;
  if (group <= 3) return 2;
  if (group <= 6) return 4;
  return 8;
}

// (-1)^(two_p / 2)
inline int phase(int two_p) { return (((two_p / 2) % 2) != 0) ? -1 : 1; }

// global = i + j(j+1)/2 with i <= j  ->  (i, j)
inline void invert_triangle_two(int global, int* result) {
  int j = 0;
  while ((j + 1) * (j + 2) <= 2 * global) j++;
  result[1] = j;
  result[0] = global - (j * (j + 1)) / 2;
}

constexpr int kWignerFactorialMax = 191;
constexpr int kWignerMax2j = 95;

// 3j symbol (ja jb jc; ma mb mc), arguments twice the (half-)integer values; zero unless
// ma + mb + mc = 0, |m| <= j with j + m integer, and the triangle rule holds. Racah's
// single sum over the same square-root-factorial table.
double wigner3j(int two_ja, int two_jb, int two_jc, int two_ma, int two_mb, int two_mc);
double wigner6j(int two_ja, int two_jb, int two_jc, int two_jd, int two_je, int two_jf);
double wigner9j(int two_ja, int two_jb, int two_jc, int two_jd, int two_je, int two_jf,
                int two_jg, int two_jh, int two_ji);

}  // namespace c2g
