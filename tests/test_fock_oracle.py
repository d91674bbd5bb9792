"""The Fock-space checker (oracle/fock.py) pinned against the CPU oracle's DMRG: the same
step-by-step checks the GPU parity tests run (tests/fock_checks.py), on short chains where
the CPU oracle is itself pinned to FCI and the reference's golden energies. Also that the
checker's Hamiltonian reproduces the determinant FCI ground state energy. No GPU needed."""
from __future__ import annotations

import numpy as np
import pytest

import fock_checks as fc
import models
import oracle_lib as ol
from oracle import fock

CASES = [
    # name, model, 2S, N, irrep, D, exact (D keeps every state)
    ("hubbard6", lambda: models.hubbard(6, 4.0), 0, 6, 0, 64, True),
    ("hubbard6_truncated", lambda: models.hubbard(6, 4.0), 0, 6, 0, 12, False),
    ("abinit6_c2v", lambda: models.synthetic_ab_initio(6, 5, 21), 0, 6, 0, 64, True),
    ("abinit7_d2h_doublet", lambda: models.synthetic_ab_initio(7, 7, 22), 1, 7, 3, 128, True),
    ("abinit6_c2v_triplet", lambda: models.synthetic_ab_initio(6, 5, 23), 2, 6, 0, 64, True),
    # the remaining point groups: Ci, C2, Cs, D2, C2h (psi4 numbering 1, 2, 3, 4, 6)
    ("abinit6_ci", lambda: models.synthetic_ab_initio(6, 1, 24), 0, 6, 1, 64, True),
    ("abinit7_c2_doublet", lambda: models.synthetic_ab_initio(7, 2, 25), 1, 7, 1, 128, True),
    ("abinit6_cs_truncated", lambda: models.synthetic_ab_initio(6, 3, 26), 0, 6, 0, 10, False),
    ("abinit7_d2_quartet", lambda: models.synthetic_ab_initio(7, 4, 27), 3, 7, 2, 128, True),
    ("abinit6_c2h", lambda: models.synthetic_ab_initio(6, 6, 28), 0, 6, 3, 64, True),
]


@pytest.mark.parametrize("name,make,two_s,n,irrep,D,exact", CASES)
def test_fock_checker_against_cpu_oracle(name, make, two_s, n, irrep, D, exact):
    m = make()
    ol.srand(5)
    cpu = ol.OracleDMRG(m, two_s, n, irrep, [(D, 1e-10, 1, 0.0, 1e-9)])
    fc.check_sweeps(cpu, m, (n, two_s, irrep), D, exact=exact)


def test_fock_hamiltonian_ground_state_matches_fci():
    import scipy.sparse.linalg as sla

    m = models.synthetic_ab_initio(6, 5, 21)
    H = fock.FockHamiltonian(m.tmat, m.vmat, m.econst)
    L = m.L
    # restrict to N = 6, Sz = 0 and irrep 0
    conf = np.arange(4 ** L)
    digits = np.stack([(conf // 4 ** (L - 1 - k)) % 4 for k in range(L)], axis=1)
    nup = (digits & 1).sum(1)
    ndn = ((digits >> 1) & 1).sum(1)
    irr = np.zeros(conf.size, dtype=np.int64)
    for k in range(L):
        single = (digits[:, k] == 1) | (digits[:, k] == 2)
        irr ^= np.where(single, m.irreps[k], 0)
    sel = np.flatnonzero((nup == 3) & (ndn == 3) & (irr == 0))

    def mv(v):
        full = np.zeros(conf.size)
        full[sel] = v
        return H.apply(full)[sel]

    op = sla.LinearOperator((sel.size, sel.size), matvec=mv, dtype=np.float64)
    e = sla.eigsh(op, k=1, which="SA", tol=1e-12)[0][0]
    assert abs(e - ol.fci_energy(m, 3, 3, 0)) < 1e-9
