"""The tensor-core form of the mixed-precision matvec (tcgen05 split-BF16 products for the
two-pass large-block groups, sandwich_tc.cu) against the FP64 matvec and in a full
mixed-precision solve.

Tolerances: a split-BF16 three-term product keeps ~16 significant bits of each factor
(relative error ~2^-16 ~ 1.5e-5 per product), sums accumulate in FP32, so the matvec is
checked to 1e-4 relative to its largest element; the mixed solve refines with FP64
products, so its energy must equal the FP64 run's to 1e-8 Ha.
"""
from __future__ import annotations

import numpy as np
import pytest

import chemps2_gb300 as c2g
import models

pytestmark = pytest.mark.gpu


def hubbard_objects(L, D, U=4.0, sweeps=1):
    m = models.hubbard(L, U)
    ham = c2g.Hamiltonian(L, 0, m.irreps)
    for i in range(L - 1):
        ham.setTmat(i, i + 1, -1.0)
    for i in range(L):
        ham.setVmat(i, i, i, i, U)
    prob = c2g.Problem(ham, 0, L, 0)
    scheme = c2g.ConvergenceScheme(1)
    scheme.set_instruction(0, D, 1e-10, sweeps, 0.0, 1e-8)
    return ham, prob, scheme


def rel(a, b):
    return float(np.max(np.abs(a - b))) / max(1.0, float(np.max(np.abs(b))))


@pytest.mark.parametrize("L,D,sweep", [(12, 256, False), (16, 512, True)])
def test_tensor_core_matvec_close_to_fp64(L, D, sweep):
    """C1 Hubbard chains whose middle blocks are large (tens of rows): the two-pass groups
    run on the tensor cores. The result is within split-BF16 rounding of FP64, and differs
    from the all-FP32 matvec (the tensor-core kernels did the large groups)."""
    ham, prob, scheme = hubbard_objects(L, D)
    c2g.srand(9)
    d = c2g.DMRG(prob, scheme)
    try:
        if sweep:
            d.Solve()
        mid = L // 2 - 1
        for index in range(L - 2, mid, -1):
            d.update(index, False)
        x, _, _ = d.heff_apply(mid)
        rng = np.random.default_rng(3)
        for trial in range(2):
            xr = x if trial == 0 else rng.standard_normal(x.size)
            _, y64, _ = d.heff_apply(mid, xr)
            ytc = d.heff_apply_precision(mid, xr, "tc")
            y32 = d.heff_apply_precision(mid, xr, "fp32")
            assert rel(ytc, y64) < 1e-4, rel(ytc, y64)
            assert rel(y32, y64) < 1e-5
            assert not np.array_equal(ytc, y32)
        # repeated calls give identical results (fixed summation order)
        assert np.array_equal(d.heff_apply_precision(mid, x, "tc"), d.heff_apply_precision(mid, x, "tc"))
    finally:
        d.close()


def test_mixed_tensor_core_solve_matches_fp64():
    """Mixed Davidson with tensor-core matvecs reaches the FP64 energy (1e-8 Ha) and used
    reduced-precision matvecs."""
    energies = {}
    for mode in ("fp64", "mixed_tc"):
        ham, prob, scheme = hubbard_objects(12, 256, sweeps=2)
        c2g.srand(2)
        d = c2g.DMRG(prob, scheme)
        d.set_precision(mode)
        energies[mode] = d.Solve()
        st = d.stats()
        if mode == "mixed_tc":
            assert st["n_matvec_fp32"] > 0
        d.close()
    assert abs(energies["mixed_tc"] - energies["fp64"]) < 1e-8


def test_two_pass_chunks_give_identical_products(monkeypatch):
    """The large groups run in chunks of whole groups whose pass-1 intermediates fit a
    byte budget (default 8 GB; C2G_INTER_BUDGET_KB, read at each program upload). With a
    64 KB budget the groups of this state run chunk by chunk (more launches per matvec),
    and every product is bit-identical to the one-chunk run in all three arithmetics: a
    group's items keep their order and their intermediates."""
    L, D = 12, 256
    ys, launches = {}, {}
    for budget in (None, "64"):
        if budget:
            monkeypatch.setenv("C2G_INTER_BUDGET_KB", budget)
        else:
            monkeypatch.delenv("C2G_INTER_BUDGET_KB", raising=False)
        ham, prob, scheme = hubbard_objects(L, D)
        c2g.srand(9)
        d = c2g.DMRG(prob, scheme)
        try:
            mid = L // 2 - 1
            for index in range(L - 2, mid, -1):
                d.update(index, False)
            x = np.random.default_rng(4).standard_normal(d.sobject_size(mid))
            out = {}
            for prec in ("fp64", "fp32", "tc"):
                out[prec] = d.heff_apply_precision(mid, x, prec)
            n0 = c2g.kernel_launches()
            d.heff_apply_precision(mid, x, "tc")
            launches[budget] = c2g.kernel_launches() - n0
            ys[budget] = out
        finally:
            d.close()
    assert launches["64"] > launches[None], launches
    for prec in ("fp64", "fp32", "tc"):
        assert np.array_equal(ys["64"][prec], ys[None][prec]), prec


def test_mixed_solve_of_a_hard_step_finds_the_ground_state():
    """Synthetic ab initio L=40 C2v, D=1000, from the seeded random start: at the fifth step
    of the first left half-sweep the FP64 solver needs 43 products, with plateaus of the
    residual. The reduced-precision phase must not end on such a plateau: an unconverged
    Ritz vector handed to the refinement cycles, whose single-vector restarts converge to
    the nearest eigenpair, gave an excited state 5.6 Ha above the FP64 one. The first six
    step energies of the mixed tensor-core solve equal the FP64 ones to 1e-8."""
    from chemps2_gb300.models import synthetic_ab_initio

    m = synthetic_ab_initio(40, 5, 1234)
    energies = {}
    for mode in ("fp64", "mixed_tc"):
        ham = c2g.Hamiltonian(m.L, m.group, m.irreps)
        for i in range(m.L):
            for j in range(i, m.L):
                if m.tmat[i, j] != 0.0:
                    ham.setTmat(i, j, float(m.tmat[i, j]))
        for i, j, k, l in np.argwhere(m.vmat != 0.0):
            if i <= j and i <= k:
                ham.setVmat(int(i), int(j), int(k), int(l), float(m.vmat[i, j, k, l]))
        prob = c2g.Problem(ham, 0, m.L, 0)
        scheme = c2g.ConvergenceScheme(1)
        scheme.set_instruction(0, 1000, 1e-10, 1, 0.0, 1e-8)
        c2g.srand(1234)
        d = c2g.DMRG(prob, scheme)
        try:
            d.set_precision(mode)
            es = []
            for index in range(m.L - 2, m.L - 8, -1):
                es.append(d.solve_site(index, 1e-8, 0.0, 1000, False, False))
                d.update(index, False)
            energies[mode] = np.array(es)
        finally:
            d.close()
    assert np.max(np.abs(energies["mixed_tc"] - energies["fp64"])) < 1e-8, energies
