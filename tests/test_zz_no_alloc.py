"""The allocation-free host-buffer matvec (c2g_dmrg_heff_apply_noalloc) against the
allocating one (c2g_dmrg_heff_apply) on the same DMRG state, over two calls with
different vectors: both run the same device program, so the results are identical."""
from __future__ import annotations

import numpy as np
import pytest

import chemps2_gb300 as c2g
import models

pytestmark = pytest.mark.gpu


def _dmrg(model, two_s, n, irrep):
    ham = c2g.Hamiltonian(model.L, model.group, model.irreps)
    L = model.L
    for i in range(L):
        for j in range(i, L):
            if model.tmat[i, j] != 0.0:
                ham.setTmat(i, j, model.tmat[i, j])
    for i, j, k, l in np.argwhere(model.vmat != 0.0):
        ham.setVmat(int(i), int(j), int(k), int(l), float(model.vmat[i, j, k, l]))
    prob = c2g.Problem(ham, two_s, n, irrep)
    scheme = c2g.ConvergenceScheme(1)
    scheme.set_instruction(0, 64, 1e-10, 1, 0.0, 1e-8)
    c2g.srand(7)
    return ham, prob, scheme, c2g.DMRG(prob, scheme)


def test_noalloc_matches_heff_apply_on_two_calls():
    m = models.synthetic_ab_initio(8, 5, 11)
    ham, prob, scheme, d = _dmrg(m, 0, 8, 0)
    try:
        index = m.L - 2
        n = d.sobject_size(index)
        rng = np.random.default_rng(3)
        for call in range(2):
            x = rng.standard_normal(n)
            _, y_ref, _ = d.heff_apply(index, x)
            y = d.heff_apply_noalloc(index, x)
            assert np.array_equal(y, y_ref), f"call {call}: max diff {np.max(np.abs(y - y_ref))}"
            assert np.max(np.abs(y)) > 0.0
    finally:
        d.close()


def test_noalloc_needs_a_prepared_program():
    m = models.hubbard(6, 4.0)
    ham, prob, scheme, d = _dmrg(m, 0, 6, 0)
    try:
        index = m.L - 2
        n = d.sobject_size(index)
        with pytest.raises(c2g.Chemps2Error):
            d.heff_apply_noalloc(index, np.ones(n))
        d.heff_apply(index, np.ones(n))
        with pytest.raises(c2g.Chemps2Error):
            d.heff_apply_noalloc(index, np.ones(n + 1))
    finally:
        d.close()
