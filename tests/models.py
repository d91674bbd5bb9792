"""Seeded model Hamiltonians (re-exported from the package for the tests)."""
from chemps2_gb300.models import NIRREPS, Model, bcs, hubbard, synthetic_ab_initio  # noqa: F401

import math

import numpy as np


def hubbard_3x3_site_and_momentum(U=5.0, T=-1.0, N=9):
    """The reference's tests/test9.cpp.in: the 3 x 3 Hubbard model with periodic boundaries
    (C1) as a Model in the site basis, and the matrix elements of the same model in the
    momentum basis (orbital k = kx + 3 ky). Those have only fourfold permutation symmetry:
    U / 9 where crystal momentum is conserved, plus the one-body part folded in as
    (eps(k1) + eps(k2)) / (N - 1) on (k1 k2 | k1 k2), eps(k) = 2T (cos 2pi kx/3 + cos 2pi ky/3).
    Returns (site model, {(o1, o2, o3, o4): value} of the nonzero momentum elements)."""
    Ll = 3
    L = Ll * Ll
    tm = np.zeros((L, L))
    vm = np.zeros((L, L, L, L))
    for c in range(L):
        vm[c, c, c, c] = U
    for ix in range(Ll):
        for iy in range(Ll):
            i1 = ix + Ll * iy
            for i2 in ((ix + 1) % Ll + Ll * iy, ix + Ll * ((iy + 1) % Ll)):
                tm[i1, i2] = tm[i2, i1] = T
    site = Model(L, 0, np.zeros(L, dtype=np.int32), tm, vm)
    eps = [2 * T * (math.cos(2 * math.pi * (o % Ll) / Ll) + math.cos(2 * math.pi * (o // Ll) / Ll)) for o in range(L)]
    mom = {}
    for o1 in range(L):
        for o2 in range(L):
            for o3 in range(L):
                for o4 in range(L):
                    v = 0.0
                    if ((o1 % Ll + o2 % Ll) % Ll == (o3 % Ll + o4 % Ll) % Ll
                            and (o1 // Ll + o2 // Ll) % Ll == (o3 // Ll + o4 // Ll) % Ll):
                        v += U / L
                    if o1 == o3 and o2 == o4:
                        v += (eps[o1] + eps[o2]) / (N - 1)
                    if v != 0.0:
                        mom[(o1, o2, o3, o4)] = v
    return site, mom
