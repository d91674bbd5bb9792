"""The two-particle density matrix and the correlation pass (DMRG::calc2DMandCorrelations,
CheMPS2/TwoDM.cpp, CheMPS2/Correlations.cpp) of a converged GPU DMRG state against the
oracle's FCI 2-RDM and FCI two-orbital mutual information, and its own identities
(CheMPS2/DMRGtechnics.cpp:105-110 prints the same checks): trace A = N(N-1) and
Econst + 1/2 sum A h = E. The DMRG runs at a virtual dimension that holds the FCI space,
so the density matrices agree with FCI up to the Davidson tolerance (1e-10 residual; the
2-RDM error is O(residual), asserted at 1e-9)."""
from __future__ import annotations

import numpy as np
import pytest

import chemps2_gb300 as c2g
import models
import oracle_lib as ol

pytestmark = pytest.mark.gpu


def _objects(m, two_s, n, irrep, D=128, sweeps=6):
    ham = c2g.Hamiltonian(m.L, m.group, m.irreps)
    for i in range(m.L):
        for j in range(i, m.L):
            if m.tmat[i, j] != 0.0:
                ham.setTmat(i, j, m.tmat[i, j])
    for i, j, k, l in np.argwhere(m.vmat != 0.0):
        ham.setVmat(int(i), int(j), int(k), int(l), float(m.vmat[i, j, k, l]))
    ham.setEconst(m.econst)
    prob = c2g.Problem(ham, two_s, n, irrep)
    scheme = c2g.ConvergenceScheme(1)
    scheme.set_instruction(0, D, 1e-11, sweeps, 0.0, 1e-10)
    return ham, prob, scheme


CASES = [
    ("hubbard6", lambda: models.hubbard(6, 4.0), 0, 6, 0),
    ("abinit6_c2v", lambda: models.synthetic_ab_initio(6, 5, 3), 0, 6, 0),
    ("abinit7_d2h_doublet", lambda: models.synthetic_ab_initio(7, 7, 12), 1, 7, 3),
]


@pytest.mark.parametrize("name,make,two_s,n,irrep", CASES)
def test_2rdm_matches_fci(name, make, two_s, n, irrep):
    m = make()
    ham, prob, scheme = _objects(m, two_s, n, irrep)
    c2g.srand(3)
    d = c2g.DMRG(prob, scheme)
    try:
        E = d.Solve()
        n_up, n_down = (n + two_s) // 2, (n - two_s) // 2
        Efci, A_fci, B_fci = ol.fci_2rdm(m, n_up, n_down, irrep)
        assert abs(E - Efci) < 1e-8, (E, Efci)
        d.calc2DMandCorrelations()
        dm = d.get2DM()
        assert abs(dm.trace() - n * (n - 1)) < 1e-8
        assert abs(dm.energy() - E) < 1e-8, (dm.energy(), E)
        assert np.max(np.abs(dm.A - A_fci)) < 1e-9, np.max(np.abs(dm.A - A_fci))
        assert np.max(np.abs(dm.B - B_fci)) < 1e-9, np.max(np.abs(dm.B - B_fci))
        # correlation pass: mutual information and single-orbital entropies against FCI. The
        # reference's two-orbital density matrices are partial traces in the orbital
        # tensor-product basis without the Jordan-Wigner string of the orbitals between
        # the pair (its G/Y/Z/K/M tensors are updated with jw_phase false,
        # CheMPS2/TensorKM.cpp:27-30), which the oracle computes with jw=False.
        _, s1_fci, mi_fci = ol.fci_mutual_information(m, n_up, n_down, irrep, jw=False)
        corr = d.getCorrelations()
        assert np.max(np.abs(corr["SingleOrbitalEntropy"] - s1_fci)) < 1e-9
        assert np.max(np.abs(corr["MutInfo"] - mi_fci)) < 1e-9, np.max(np.abs(corr["MutInfo"] - mi_fci))
        # PyDMRG's element accessors, Hamiltonian order (no reordering here)
        assert d.get2DMA(0, 1, 0, 1) == dm.A[0, 1, 0, 1] and d.get2DMB(1, 0, 0, 1) == dm.B[1, 0, 0, 1]
        assert d.get2DMenergy() == dm.energy() and d.getDoubleTrace2DMA() == dm.trace()
        assert d.getMutInfo(0, 2) == corr["MutInfo"][0, 2]
        assert d.getSingleOrbEntropy(1) == corr["SingleOrbitalEntropy"][1]
        assert d.getCspin(0, 1) == corr["Cspin"][0, 1] and d.getCdirad(1, 2) == corr["Cdirad"][1, 2]
        L = m.L
        ref = sum(corr["MutInfo"][r, c] * abs(r - c) ** 2 for r in range(L) for c in range(L) if r != c)
        assert abs(d.getMutInfoDistance(2) - ref) < 1e-12
        with pytest.raises(NotImplementedError):
            d.calc_rdms_and_correlations(True)
        # the state and the operators are left as after a right sweep: Solve continues
        E2 = d.Solve()
        assert abs(E2 - E) < 1e-8
    finally:
        d.close()
