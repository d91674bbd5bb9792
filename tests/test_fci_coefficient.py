"""DMRG::getFCIcoefficient (CheMPS2/DMRGtechnics.cpp:324-470): the product's host routine
(chemps2_gb300/csrc/host/fcicoef.cpp) run on the CPU oracle's MPS, against the Fock-space
checker (oracle/fock.py), which builds the many-electron state of the same MPS with
Clebsch-Gordan couplings of its own, and against the exact eigenvector.

Right after Solve, the M = S component carries the two-site object's symmetric
normalisation (squared norm 1 / (2S + 1)). The gauge changes of the 2-RDM pass normalise
the last site and drop its 1 x 1 R factor, as the reference's do. That is why the
reference's tests/test1.cpp.in compares getFCIcoefficient after calc2DMandCorrelations
with the normalised FCI vector. Both states are checked here. Tolerances: 1e-12 against
the Fock-space amplitudes of the same MPS (rounding only); 1e-7 against the exact
eigenvector (the DMRG is converged to a 1e-10 residual at a D above the FCI space)."""
from __future__ import annotations

import itertools

import numpy as np
import pytest

import fock_checks as fc
import models
import oracle_lib as ol
from oracle import fock

# name, model, 2S, N, irrep (each the ground multiplet of its particle number)
CASES = [
    ("abinit6_c2v_singlet", lambda: models.synthetic_ab_initio(6, 5, 31), 0, 6, 0),
    ("abinit5_c2v_doublet", lambda: models.synthetic_ab_initio(5, 5, 3), 1, 5, 2),
    ("abinit7_c1_n6_triplet", lambda: models.synthetic_ab_initio(7, 0, 11), 2, 6, 0),
]


def _determinants(m, n, two_s, irrep):
    """(alpha, beta, configuration index of the Fock-space checker) of every determinant
    with M_S = S in the targeted irrep; site k's code is alpha + 2 beta, the first site
    the most significant base-4 digit."""
    L = m.L
    n_up, n_dn = (n + two_s) // 2, (n - two_s) // 2
    out = []
    for ups in itertools.combinations(range(L), n_up):
        for dns in itertools.combinations(range(L), n_dn):
            a = np.zeros(L, dtype=np.int32)
            b = np.zeros(L, dtype=np.int32)
            a[list(ups)] = 1
            b[list(dns)] = 1
            ir = 0
            for k in range(L):
                if a[k] + b[k] == 1:
                    ir ^= int(m.irreps[k])
            if ir != irrep:
                continue
            conf = sum(int(a[k] + 2 * b[k]) * 4 ** (L - 1 - k) for k in range(L))
            out.append((a, b, conf))
    return out


def _exact_ground_state(m, dets):
    H = fock.FockHamiltonian(m.tmat, m.vmat, m.econst)
    confs = [c for _, _, c in dets]
    dim = 4 ** m.L
    cols = []
    for c in confs:
        e = np.zeros(dim)
        e[c] = 1.0
        cols.append(H.apply(e)[confs])
    w, v = np.linalg.eigh(np.array(cols).T)
    return w[0], v[:, 0]


@pytest.mark.parametrize("name,make,two_s,n,irrep", CASES)
def test_fci_coefficients_against_fock_space_and_exact_state(name, make, two_s, n, irrep):
    m = make()
    ol.srand(2)
    d = ol.OracleDMRG(m, two_s, n, irrep, [(200, 1e-11, 4, 0.0, 1e-10)])
    e = d.solve()
    dets = _determinants(m, n, two_s, irrep)
    # right after the sweeps: the Fock-space amplitudes of the same MPS, norm 1 / (2S + 1)
    psi = fc.chain_of(d, m, (n, two_s, irrep)).state()
    c = np.array([d.fci_coefficient(a, b) for a, b, _ in dets])
    assert np.max(np.abs(c - psi[[x for _, _, x in dets]])) < 1e-12
    assert abs(c @ c - 1.0 / (two_s + 1)) < 1e-10
    # after the 2-RDM pass: normalised, and the exact eigenvector up to its global sign
    d.calc_2dm()
    c = np.array([d.fci_coefficient(a, b) for a, b, _ in dets])
    psi = fc.chain_of(d, m, (n, two_s, irrep)).state()
    assert np.max(np.abs(c - psi[[x for _, _, x in dets]])) < 1e-12
    assert abs(c @ c - 1.0) < 1e-10
    w0, v0 = _exact_ground_state(m, dets)
    assert abs(w0 - e) < 1e-9, (w0, e)
    sign = 1.0 if c @ v0 >= 0 else -1.0
    assert np.max(np.abs(c - sign * v0)) < 1e-7


def test_fci_coefficient_outside_the_sector_is_zero():
    """The reference returns 0 for a determinant of another particle number, 2S_z or
    irrep (CheMPS2/DMRGtechnics.cpp:346-371)."""
    m = models.synthetic_ab_initio(5, 5, 3)
    ol.srand(2)
    d = ol.OracleDMRG(m, 1, 5, 2, [(64, 1e-10, 2, 0.0, 1e-10)])
    d.solve()
    up = np.array([1, 1, 1, 0, 0], dtype=np.int32)
    # orbital irreps 0 1 2 3 0: the singly occupied orbital 2 gives the target irrep 2
    assert d.fci_coefficient(up, np.array([1, 1, 0, 0, 0])) != 0.0
    assert d.fci_coefficient(up, np.array([1, 0, 1, 0, 0])) == 0.0  # irrep 1
    assert d.fci_coefficient(up, np.array([1, 1, 1, 0, 0])) == 0.0  # N = 6
    assert d.fci_coefficient(np.array([1, 1, 1, 1, 0]), np.array([1, 0, 0, 0, 0])) == 0.0  # 2S_z = 3 > 2S
