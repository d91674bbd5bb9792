"""Seeded model Hamiltonians of the benchmark configurations (also used by the tests).

synthetic_ab_initio() follows the generator of the benchmark configurations: L orbitals,
irreps assigned round robin (psi4 numbering), a symmetric symmetry-blocked one-body
matrix with sorted uniform diagonal in [-2, 1] and N(0, 0.1) exp(-|i-j|/4) off-diagonal,
and two-electron integrals (ij|kl) = sum_P L^P_ij L^P_kl over 3L Cholesky-like vectors
L^P_ij ~ N(0, 0.15) exp(-|i-j|/6), each vector carrying one irrep so the integrals are
8-fold symmetric, symmetry-blocked and positive semidefinite.
"""
from __future__ import annotations

import numpy as np

NIRREPS = {0: 1, 1: 2, 2: 2, 3: 2, 4: 4, 5: 4, 6: 4, 7: 8}


class Model:
    """tmat (L x L) and vmat (L^4, physics notation V_ijkl = (ik|jl)) as numpy arrays."""

    def __init__(self, L, group, irreps, tmat, vmat, econst=0.0):
        self.L = int(L)
        self.group = int(group)
        self.irreps = np.ascontiguousarray(irreps, dtype=np.int32)
        self.tmat = np.array(tmat, dtype=np.float64)
        self.vmat = np.array(vmat, dtype=np.float64)
        self.econst = float(econst)

    def tflat(self):
        return np.ascontiguousarray(self.tmat.ravel(order="F"))

    def vflat(self):
        return np.ascontiguousarray(self.vmat.ravel(order="F"))


def hubbard(L, U, t=-1.0):
    T = np.zeros((L, L))
    for i in range(L - 1):
        T[i, i + 1] = T[i + 1, i] = t
    V = np.zeros((L, L, L, L))
    for i in range(L):
        V[i, i, i, i] = U
    return Model(L, 0, np.zeros(L, dtype=np.int32), T, V)


def synthetic_ab_initio(L, group, seed):
    rng = np.random.default_rng(seed)
    nirr = NIRREPS[group]
    irreps = np.array([i % nirr for i in range(L)], dtype=np.int32)
    idx = np.arange(L)
    dist = np.abs(idx[:, None] - idx[None, :])
    same = irreps[:, None] == irreps[None, :]
    h = rng.normal(0.0, 0.1, size=(L, L)) * np.exp(-dist / 4.0)
    h = 0.5 * (h + h.T)
    h[~same] = 0.0
    np.fill_diagonal(h, np.sort(rng.uniform(-2.0, 1.0, size=L)))
    nvec = 3 * L
    chol = np.zeros((nvec, L, L))
    for P in range(nvec):
        gam = P % nirr
        m = rng.normal(0.0, 0.15, size=(L, L)) * np.exp(-dist / 6.0)
        m = 0.5 * (m + m.T)
        mask = (irreps[:, None] ^ irreps[None, :]) == gam
        chol[P] = np.where(mask, m, 0.0)
    eri = np.einsum("pij,pkl->ijkl", chol, chol)  # chemists' (ij|kl)
    vphys = eri.transpose(0, 2, 1, 3).copy()       # V_ikjl = (ij|kl)
    return Model(L, group, irreps, h, vphys)


def bcs(eps, g, power):
    """Model of tests/test12.cpp.in: written with Problem::setMxElement after construction."""
    L = len(eps)
    return L, [(o1, o2, g * abs(eps[o1] * eps[o2]) ** power, (eps[o1] + eps[o2]) / (L - 1))
               for o1 in range(L) for o2 in range(L)]


BATCH_BOND_DIMS = (64, 128, 256, 512)


def batch_members(count=64, seed=2024):
    """The independent problems of the batching workload: L uniform in {8..20}, N = L,
    half Hubbard chains (t = 1, U uniform in [1, 8], C1) and half synthetic_ab_initio (D2h,
    irreps round robin), D drawn from BATCH_BOND_DIMS. The spin is drawn from {0, 1} for
    even N; odd N cannot have integer spin, so it takes 2S from {1, 3} there. Target irrep
    0. Returns dicts with the model, two_s, n, irrep, D, kind and a per-problem seed."""
    rng = np.random.default_rng(seed)
    kinds = np.array(["hubbard"] * (count // 2) + ["abinit"] * (count - count // 2))
    rng.shuffle(kinds)
    out = []
    for k in range(count):
        L = int(rng.integers(8, 21))
        spin_bit = int(rng.integers(0, 2))
        D = int(rng.choice(BATCH_BOND_DIMS))
        n = L
        two_s = (n % 2) + 2 * spin_bit
        if kinds[k] == "hubbard":
            U = float(rng.uniform(1.0, 8.0))
            model = hubbard(L, U)
        else:
            model = synthetic_ab_initio(L, 7, int(rng.integers(0, 2**31 - 1)))
        out.append({"model": model, "two_s": two_s, "n": n, "irrep": 0, "D": D, "kind": str(kinds[k]),
                    "seed": int(rng.integers(1, 2**31 - 1))})
    return out
