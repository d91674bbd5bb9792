"""Generate the table sqrt(n!) for n = 0..191 as correctly rounded doubles.

The Racah formulas for the Wigner 6j symbol need square roots of factorials up to
(4j+1)! for 2j <= 95 (CheMPS2/include/chemps2/Wigner.h:22-23 fixes the same bounds).
The values are mathematical constants: they are computed here with Python's decimal
module at 80 significant digits and printed with 20 significant digits, which the C++
compiler rounds to the nearest double.

Run:  python gen_sqrt_fact.py > sqrt_fact.inc
"""
from decimal import Decimal, getcontext

FACTORIAL_MAX = 191


def main() -> None:
    getcontext().prec = 80
    fact = Decimal(1)
    lines = []
    for n in range(FACTORIAL_MAX + 1):
        if n > 0:
            fact *= n
        root = fact.sqrt()
        lines.append(f"   {root:.19E},  // sqrt({n}!)")
    print("// Generated by gen_sqrt_fact.py: sqrt(n!) for n = 0..%d" % FACTORIAL_MAX)
    print("\n".join(lines))


if __name__ == "__main__":
    main()
