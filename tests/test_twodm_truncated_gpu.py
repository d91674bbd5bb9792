"""The 2-RDM (DMRG::calc2DMandCorrelations, CheMPS2/TwoDM.cpp) of truncated states, where
the virtual dimension is below the FCI space: against the 2-RDM A computed in Fock space
from the product's own MPS (oracle/fock.py; independent of the product's diagrams), and
its identities trace A = N(N-1) and Econst + 1/2 sum A h = <H> of the MPS.

A truncated state can hold dead sectors: states at a boundary whose every connecting
sector on the other side was truncated to dimension zero by a later Split of the same
sweep (a left state without a right completion), or the mirror case. They are zero
vectors of the many-electron space, so the QR and LQ gauge changes of the 2-RDM pass
must drop the neighbouring site's weight on them (R or L is zero there). The case marked
`dead` is known to hold such a sector and asserts it.

Tolerances: 1e-8 (FP64 throughout; the MPS is the same object on both sides)."""
from __future__ import annotations

import numpy as np
import pytest

import chemps2_gb300 as c2g
import fock_checks as fc
import models
from oracle import fock

pytestmark = pytest.mark.gpu

# name, model, 2S, N, irrep, D, sweeps, srand seed, holds a dead sector
CASES = [
    ("hubbard8_d16", lambda: models.hubbard(8, 4.0), 0, 8, 0, 16, 2, 3, False),
    ("abinit8_c2v_d16", lambda: models.synthetic_ab_initio(8, 5, 41), 0, 8, 0, 16, 2, 3, False),
    ("abinit7_d2h_doublet_d12", lambda: models.synthetic_ab_initio(7, 7, 42), 1, 7, 3, 12, 2, 3, False),
    ("abinit8_c2v_d4_one_sweep", lambda: models.synthetic_ab_initio(8, 5, 8), 0, 8, 0, 4, 1, 1, True),
    ("abinit8_c2v_d16_one_sweep", lambda: models.synthetic_ab_initio(8, 5, 8), 0, 8, 0, 16, 1, 1, False),
    ("abinit10_d2h_d6_one_sweep", lambda: models.synthetic_ab_initio(10, 7, 9), 0, 10, 0, 6, 1, 2, False),
]


def _objects(m, two_s, n, irrep, D, sweeps):
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
    scheme.set_instruction(0, D, 1e-30, sweeps, 0.0, 1e-10)
    return ham, prob, scheme


@pytest.mark.parametrize("name,make,two_s,n,irrep,D,sweeps,seed,dead", CASES)
def test_2rdm_of_truncated_state_against_fock_space(name, make, two_s, n, irrep, D, sweeps, seed, dead):
    m = make()
    ham, prob, scheme = _objects(m, two_s, n, irrep, D, sweeps)
    c2g.srand(seed)
    d = c2g.DMRG(prob, scheme)
    try:
        d.Solve()
        if dead:
            assert fc.dead_sectors(d, m), "the state holds no dead sector"
        ch = fc.chain_of(d, m, (n, two_s, irrep))
        psi = ch.state()
        H = fock.FockHamiltonian(m.tmat, m.vmat, m.econst)
        e_mps = float(psi @ H.apply(psi)) / float(psi @ psi)
        A_fock = fock.two_rdm_a(H, psi / np.sqrt(psi @ psi))
        d.calc2DMandCorrelations()
        dm = d.get2DM()
        assert abs(dm.trace() - n * (n - 1)) < 1e-8, (dm.trace(), n * (n - 1))
        assert abs(dm.energy() - e_mps) < 1e-8, (dm.energy(), e_mps)
        assert np.max(np.abs(dm.A - A_fock)) < 1e-8, np.max(np.abs(dm.A - A_fock))
    finally:
        d.close()


_CHUNK_SCRIPT = """
import sys
import numpy as np
import chemps2_gb300 as c2g
import models
from test_twodm_truncated_gpu import _objects
m = models.synthetic_ab_initio(8, 5, 41)
ham, prob, scheme = _objects(m, 0, 8, 0, 16, 2)
c2g.srand(3)
d = c2g.DMRG(prob, scheme)
d.Solve()
d.calc2DMandCorrelations()
dm = d.get2DM()
np.savez(sys.argv[1], A=np.array(dm.A), B=np.array(dm.B))
d.close()
"""


def test_2rdm_in_many_programs_per_site(tmp_path):
    """The 2-RDM pass splits the products of a site into programs under a work budget
    (C2G_TWODM_BUDGET doubles, read once per process). With a budget of 2048 doubles every
    site runs many programs; the 2-RDM equals the one of the default budget to rounding
    (the same seeded solve on both sides)."""
    import os
    import subprocess
    import sys
    from pathlib import Path

    root = Path(__file__).resolve().parents[1]
    env = dict(os.environ, PYTHONPATH=os.pathsep.join([str(root), str(root / "tests")]))
    out = {}
    for name, budget in (("default", None), ("small", "2048")):
        e = dict(env)
        if budget:
            e["C2G_TWODM_BUDGET"] = budget
        else:
            e.pop("C2G_TWODM_BUDGET", None)
        path = tmp_path / f"{name}.npz"
        subprocess.run([sys.executable, "-c", _CHUNK_SCRIPT, str(path)], cwd=root, env=e, check=True, timeout=600)
        out[name] = np.load(path)
    assert np.max(np.abs(out["small"]["A"] - out["default"]["A"])) < 1e-10
    assert np.max(np.abs(out["small"]["B"] - out["default"]["B"])) < 1e-10
