"""GPU tests of the batch entry point (c2g_batch_solve / CheMPS2::SolveBatch): several
independent problems of uneven size solved concurrently on one GPU give the energies that
the same problems give when each is solved alone after srand(seed), and a half-filled
Hubbard member (singlet ground state) equals the oracle's FCI energy.

Tolerances: 1e-9 Ha between batch and single solves (the same arithmetic; only the
number of task-compiler shards, and with it the summation order inside the programs,
differs), 1e-8 Ha against FCI as in the reference's own tests (tests/test4.cpp.in:103).
"""
from __future__ import annotations

import pytest

import chemps2_gb300 as c2g
import models
import oracle_lib as ol
from test_gpu_parity import gpu_objects

pytestmark = pytest.mark.gpu

MEMBERS = [
    # (model, two_s, n, irrep, D, seed)
    (lambda: models.hubbard(8, 3.0), 0, 8, 0, 64, 11),
    (lambda: models.synthetic_ab_initio(7, 7, 5), 1, 7, 0, 48, 12),
    (lambda: models.hubbard(9, 6.5), 3, 9, 0, 32, 13),
    (lambda: models.synthetic_ab_initio(8, 7, 6), 2, 8, 0, 40, 14),
    (lambda: models.hubbard(6, 1.5), 2, 6, 0, 24, 15),
    (lambda: models.synthetic_ab_initio(10, 7, 9), 0, 10, 0, 64, 16),
]


def build_members():
    keep, probs, schemes, seeds = [], [], [], []
    for make, two_s, n, irrep, D, seed in MEMBERS:
        m = make()
        ham, prob, scheme = gpu_objects(m, two_s, n, irrep, [(D, 1e-10, 3, 0.0, 1e-8)])
        keep.append((m, ham))
        probs.append(prob)
        schemes.append(scheme)
        seeds.append(seed)
    return keep, probs, schemes, seeds


def test_batch_equals_single_solves_and_fci():
    keep, probs, schemes, seeds = build_members()
    res = c2g.solve_batch(probs, schemes, seeds, workers=3)
    assert all(r["status"] == 0 for r in res)
    assert all(r["matvecs"] > 0 for r in res)
    for i, (make, two_s, n, irrep, D, seed) in enumerate(MEMBERS):
        m = keep[i][0]
        ham, prob, scheme = gpu_objects(m, two_s, n, irrep, [(D, 1e-10, 3, 0.0, 1e-8)])
        c2g.srand(seed)
        d = c2g.DMRG(prob, scheme)
        e = d.Solve()
        d.close()
        assert abs(res[i]["energy"] - e) < 1e-9, (i, res[i]["energy"], e)
    e_fci = ol.fci_energy(keep[0][0], 4, 4, 0)
    assert abs(res[0]["energy"] - e_fci) < 1e-8


def test_batch_sequential_and_concurrent_agree():
    _, probs, schemes, seeds = build_members()
    seq = c2g.solve_batch(probs, schemes, seeds, workers=1)
    _, probs2, schemes2, seeds2 = build_members()
    con = c2g.solve_batch(probs2, schemes2, seeds2, workers=6)
    for a, b in zip(seq, con):
        assert abs(a["energy"] - b["energy"]) < 1e-9


def test_batch_reports_a_failing_member_and_solves_the_rest():
    keep, probs, schemes, seeds = build_members()
    # a member whose symmetry sector is impossible: 2S = 9 with 3 electrons
    m = models.hubbard(6, 2.0)
    ham, bad_prob, bad_scheme = gpu_objects(m, 9, 3, 0, [(16, 1e-10, 1, 0.0, 1e-8)])
    probs.insert(1, bad_prob)
    schemes.insert(1, bad_scheme)
    seeds.insert(1, 3)
    with pytest.raises(c2g.Chemps2Error) as err:
        c2g.solve_batch(probs, schemes, seeds, workers=3)
    assert "problem 1" in str(err.value)
    keep, probs, schemes, seeds = build_members()
    probs.insert(1, bad_prob)
    schemes.insert(1, bad_scheme)
    seeds.insert(1, 3)
    res = c2g.solve_batch(probs, schemes, seeds, workers=3, raise_on_error=False)
    assert res[1]["status"] == c2g.C2G_ERR_INVALID
    assert all(r["status"] == 0 and r["matvecs"] > 0 for k, r in enumerate(res) if k != 1)


def test_truncation_eig_against_numpy():
    """The truncation's batched Jacobi eigensolvers (orders up to 32 in one kernel, 33 to
    128 in the other) against LAPACK through numpy: eigenvalues ascending to 1e-12
    relative to the spectrum, eigenvectors in descending order with the sign gauge."""
    import ctypes as C

    import numpy as np

    rng = np.random.default_rng(4)
    orders = [1, 2, 7, 32, 33, 48, 64, 65, 97, 128]
    mats, ref = [], []
    for n in orders:
        X = rng.standard_normal((n, n + 3))
        G = X @ X.T  # a Gram matrix, as in the truncation
        mats.append(G.ravel(order="F"))
        ref.append(np.linalg.eigh(G))
    ns = np.array(orders, dtype=np.int32)
    allm = np.concatenate(mats)
    ev = np.zeros(sum(orders))
    vecs = np.zeros(allm.size)
    c2g._check(c2g.load().c2g_truncation_eig(len(orders), ns.ctypes.data_as(C.POINTER(C.c_int)),
                                             c2g._dp(allm), c2g._dp(ev), c2g._dp(vecs)))
    oe = ov = 0
    for n, (w, V) in zip(orders, ref):
        got = ev[oe:oe + n]
        U = vecs[ov:ov + n * n].reshape((n, n), order="F")
        scale = max(1.0, float(np.max(np.abs(w))))
        assert np.max(np.abs(got - w)) / scale < 1e-12, n
        for j in range(n):
            u = U[:, j]
            v = V[:, n - 1 - j]
            assert abs(abs(u @ v) - 1.0) < 1e-9, (n, j)
            k = int(np.argmax(np.abs(u)))
            assert u[k] > 0.0
        oe += n
        ov += n * n
