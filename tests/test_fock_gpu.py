"""The product's two-site DMRG on the GPU against the Fock-space checker (oracle/fock.py),
which shares no code with the product's task compiler: at every step of a left and a
right sweep, Join, Heff (random vectors, sampled columns and their diagonal entries),
Split (energy and norm of the new MPS, canonical forms) and, through every later Heff,
the operator updates (checks in tests/fock_checks.py). Chains of 6 to 8 sites: C1
Hubbard, C2v and D2h synthetic ab initio Hamiltonians, singlet, doublet and triplet, with
and without truncation."""
from __future__ import annotations

import numpy as np
import pytest

import chemps2_gb300 as c2g
import fock_checks as fc
import models

pytestmark = pytest.mark.gpu

CASES = [
    # name, model, 2S, N, irrep, D, exact (D keeps every state)
    ("hubbard8", lambda: models.hubbard(8, 4.0), 0, 8, 0, 256, True),
    ("hubbard8_truncated", lambda: models.hubbard(8, 4.0), 0, 8, 0, 24, False),
    ("abinit7_c2v", lambda: models.synthetic_ab_initio(7, 5, 31), 0, 6, 0, 128, True),
    ("abinit7_d2h_doublet", lambda: models.synthetic_ab_initio(7, 7, 22), 1, 7, 3, 128, True),
    ("abinit6_c2v_triplet", lambda: models.synthetic_ab_initio(6, 5, 23), 2, 6, 0, 64, True),
]


def gpu_dmrg(m, two_s, n, irrep, D):
    ham = c2g.Hamiltonian(m.L, m.group, m.irreps)
    for i in range(m.L):
        for j in range(i, m.L):
            if m.tmat[i, j] != 0.0:
                ham.setTmat(i, j, float(m.tmat[i, j]))
    for i, j, k, l in np.argwhere(m.vmat != 0.0):
        if i <= j and i <= k:
            ham.setVmat(int(i), int(j), int(k), int(l), float(m.vmat[i, j, k, l]))
    ham.setEconst(m.econst)
    prob = c2g.Problem(ham, two_s, n, irrep)
    scheme = c2g.ConvergenceScheme(1)
    scheme.set_instruction(0, D, 1e-10, 1, 0.0, 1e-9)
    c2g.srand(5)
    return ham, prob, scheme, c2g.DMRG(prob, scheme)


@pytest.mark.parametrize("name,make,two_s,n,irrep,D,exact", CASES)
def test_gpu_steps_against_fock_checker(name, make, two_s, n, irrep, D, exact):
    m = make()
    ham, prob, scheme, d = gpu_dmrg(m, two_s, n, irrep, D)
    try:
        fc.check_sweeps(d, m, (n, two_s, irrep), D, exact=exact)
    finally:
        d.close()
