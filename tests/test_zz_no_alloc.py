"""The allocation-free host-buffer matvec (c2g_dmrg_heff_apply_noalloc) against the
allocating one (c2g_dmrg_heff_apply) on the same DMRG state.

The entry point exists for callers that cannot allocate device memory while they run (a
program whose device memory is all handed out by its own allocator, or one that must not
call cudaMalloc / cudaFree because those calls can synchronise the device). It stages x
and y through one file-scope device array. These tests check that it gives the same
result as the allocating entry point on two calls in a row, that those calls leave the
device's free memory and the stream-ordered pool untouched, and that a two-site object too
large for the array is rejected with C2G_ERR_INVALID.

This file is collected last, so that a run which stops at its first failure has already
run every other test."""
from __future__ import annotations

import numpy as np
import pytest

import chemps2_gb300 as c2g
import models

pytestmark = pytest.mark.gpu


def _dmrg(model, two_s, n, irrep, D=64):
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
    scheme.set_instruction(0, D, 1e-10, 1, 0.0, 1e-8)
    c2g.srand(7)
    return ham, prob, scheme, c2g.DMRG(prob, scheme)


def test_noalloc_matches_heff_apply_on_two_calls():
    m = models.synthetic_ab_initio(8, 5, 11)
    ham, prob, scheme, d = _dmrg(m, 0, 8, 0)
    try:
        index = m.L - 2
        n = d.sobject_size(index)
        rng = np.random.default_rng(3)
        xs = [rng.standard_normal(n) for _ in range(3)]
        refs = [d.heff_apply(index, x)[1] for x in xs]
        # the first call on the device looks up the array's address (and may load the
        # library's module that holds it); the two calls after it must not allocate
        y0 = d.heff_apply_noalloc(index, xs[0])
        np.testing.assert_allclose(y0, refs[0], rtol=0, atol=1e-12 * max(1.0, np.max(np.abs(refs[0]))))
        free0, used0 = c2g.device_memory_info()
        for call in (1, 2):
            y = d.heff_apply_noalloc(index, xs[call])
            assert np.max(np.abs(y)) > 0.0
            np.testing.assert_allclose(y, refs[call], rtol=0, atol=1e-12 * max(1.0, np.max(np.abs(refs[call]))),
                                       err_msg=f"call {call}")
        free1, used1 = c2g.device_memory_info()
        assert used1 == used0, f"stream-ordered pool use changed by {used1 - used0} bytes"
        assert free1 == free0, f"free device memory changed by {free0 - free1} bytes"
    finally:
        d.close()


def test_noalloc_needs_a_prepared_program():
    m = models.hubbard(6, 4.0)
    ham, prob, scheme, d = _dmrg(m, 0, 6, 0)
    try:
        index = m.L - 2
        n = d.sobject_size(index)
        with pytest.raises(c2g.Chemps2Error) as e:
            d.heff_apply_noalloc(index, np.ones(n))
        assert e.value.code == -1
        d.heff_apply(index, np.ones(n))
        with pytest.raises(c2g.Chemps2Error) as e:
            d.heff_apply_noalloc(index, np.ones(n + 1))
        assert e.value.code == -1
    finally:
        d.close()


def test_noalloc_rejects_a_two_site_object_beyond_the_array():
    # Hubbard L=14 C1 at D=1500: the two-site object at sites (6, 7) has 2 170 742
    # amplitudes, more than the 1 048 544 the array takes; rejected before any device work
    m = models.hubbard(14, 4.0)
    ham, prob, scheme, d = _dmrg(m, 0, 14, 0, D=1500)
    try:
        n = d.sobject_size(6)
        assert n > 1048544
        with pytest.raises(c2g.Chemps2Error, match="too large") as e:
            d.heff_apply_noalloc(6, np.zeros(n))
        assert e.value.code == -1
    finally:
        d.close()
