// Wigner 6j / 9j symbols for the SU(2) prefactors of the task compiler.
// Racah formula as in CheMPS2/Wigner.cpp:294-339 (6j) and :341-370 (9j): same
// summation order, same square-root-factorial products, so that the host-side
// prefactors match the reference to the last bits.
#include "symm.hpp"

#include <algorithm>
#include <stdexcept>
#include <string>
#include <cstdlib>

namespace c2g {

namespace {

const double kSqrtFact[kWignerFactorialMax + 1] = {
#include "sqrt_fact.inc"
};

bool triangle_fails(int a, int b, int c) {
  return ((a + b + c) % 2 != 0) || (a + b < c) || (std::abs(a - b) > c);
}

double sqrt_delta(int a, int b, int c) {
  return kSqrtFact[(a + b - c) / 2] * kSqrtFact[(a - b + c) / 2] *
         kSqrtFact[(-a + b + c) / 2] / kSqrtFact[(a + b + c) / 2 + 1];
}

}  // namespace

double wigner6j(int ja, int jb, int jc, int jd, int je, int jf) {
  if (ja < 0 || jb < 0 || jc < 0 || jd < 0 || je < 0 || jf < 0 || ja > kWignerMax2j || jb > kWignerMax2j ||
      jc > kWignerMax2j || jd > kWignerMax2j || je > kWignerMax2j || jf > kWignerMax2j)
    throw std::logic_error("wigner6j: argument out of range (" + std::to_string(ja) + "," + std::to_string(jb) + "," +
                           std::to_string(jc) + "," + std::to_string(jd) + "," + std::to_string(je) + "," +
                           std::to_string(jf) + ")");
  if (triangle_fails(ja, jb, jc) || triangle_fails(jd, je, jc) ||
      triangle_fails(ja, je, jf) || triangle_fails(jd, jb, jf))
    return 0.0;

  const int a1 = (ja + jb + jc) / 2;
  const int a2 = (jd + je + jc) / 2;
  const int a3 = (ja + je + jf) / 2;
  const int a4 = (jd + jb + jf) / 2;
  const int b1 = (ja + jb + jd + je) / 2;
  const int b2 = (ja + jc + jd + jf) / 2;
  const int b3 = (jb + jc + je + jf) / 2;

  const int kmin = std::max(a1, std::max(a2, std::max(a3, a4)));
  const int kmax = std::min(b1, std::min(b2, b3));
  if (kmax < kmin) return 0.0;

  const double pref = sqrt_delta(ja, jb, jc) * sqrt_delta(jd, je, jc) *
                      sqrt_delta(ja, je, jf) * sqrt_delta(jd, jb, jf);
  double sum = 0.0;
  double sgn_pref = ((kmin % 2 == 0) ? 1 : -1) * pref;
  for (int k = kmin; k <= kmax; k++) {
    const double t = kSqrtFact[k + 1] /
                     (kSqrtFact[k - a1] * kSqrtFact[k - a2] * kSqrtFact[k - a3] *
                      kSqrtFact[k - a4] * kSqrtFact[b1 - k] * kSqrtFact[b2 - k] *
                      kSqrtFact[b3 - k]);
    sum += sgn_pref * t * t;
    sgn_pref = -sgn_pref;
  }
  return sum;
}

double wigner3j(int ja, int jb, int jc, int ma, int mb, int mc) {
  if (ja < 0 || jb < 0 || jc < 0 || ja > kWignerMax2j || jb > kWignerMax2j || jc > kWignerMax2j)
    throw std::logic_error("wigner3j: argument out of range (" + std::to_string(ja) + "," + std::to_string(jb) + "," +
                           std::to_string(jc) + ")");
  if (triangle_fails(ja, jb, jc) || ma + mb + mc != 0) return 0.0;
  if (std::abs(ma) > ja || std::abs(mb) > jb || std::abs(mc) > jc) return 0.0;
  if ((ja + ma) % 2 != 0 || (jb + mb) % 2 != 0 || (jc + mc) % 2 != 0) return 0.0;
  // integer arguments of the factorials
  const int c1 = (jc - jb + ma) / 2;       // k + c1 >= 0
  const int c2 = (jc - ja - mb) / 2;       // k + c2 >= 0
  const int d1 = (ja + jb - jc) / 2;       // d1 - k >= 0
  const int d2 = (ja - ma) / 2;            // d2 - k >= 0
  const int d3 = (jb + mb) / 2;            // d3 - k >= 0
  const int kmin = std::max(0, std::max(-c1, -c2));
  const int kmax = std::min(d1, std::min(d2, d3));
  if (kmax < kmin) return 0.0;
  const double pref = sqrt_delta(ja, jb, jc) * kSqrtFact[(ja + ma) / 2] * kSqrtFact[(ja - ma) / 2] *
                      kSqrtFact[(jb + mb) / 2] * kSqrtFact[(jb - mb) / 2] * kSqrtFact[(jc + mc) / 2] *
                      kSqrtFact[(jc - mc) / 2];
  double sum = 0.0;
  for (int k = kmin; k <= kmax; k++) {
    const double den = kSqrtFact[k] * kSqrtFact[k + c1] * kSqrtFact[k + c2] * kSqrtFact[d1 - k] *
                       kSqrtFact[d2 - k] * kSqrtFact[d3 - k];
    sum += ((k % 2 == 0) ? 1.0 : -1.0) / (den * den);
  }
  return phase(ja - jb - mc) * pref * sum;
}

double wigner9j(int ja, int jb, int jc, int jd, int je, int jf, int jg, int jh, int ji) {
  if (triangle_fails(ja, jb, jc) || triangle_fails(jd, je, jf) ||
      triangle_fails(jg, jh, ji) || triangle_fails(ja, jd, jg) ||
      triangle_fails(jb, je, jh) || triangle_fails(jc, jf, ji))
    return 0.0;
  const int lo = std::max(std::abs(ja - ji), std::max(std::abs(jh - jd), std::abs(jb - jf)));
  const int hi = std::min(ja + ji, std::min(jh + jd, jb + jf));
  double value = 0.0;
  for (int x = lo; x <= hi; x += 2) {
    value += (x + 1) * wigner6j(ja, jb, jc, jf, ji, x) * wigner6j(jd, je, jf, jb, x, jh) *
             wigner6j(jg, jh, ji, x, ja, jd);
  }
  return ((lo % 2 == 0) ? 1 : -1) * value;
}

}  // namespace c2g
