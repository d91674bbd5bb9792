"""Checks of a two-site DMRG (the product on the GPU, or the CPU oracle) against the
Fock-space checker oracle/fock.py, which shares no code with either: the MPS is expanded
into many-electron states with Clebsch-Gordan couplings and the Hamiltonian is applied as
second-quantised operators.

At every two-site step of a left sweep and a right sweep (each step: Join, Davidson,
Split, then the operator update):
  * left renormalised states orthonormal, right completions orthogonal with squared norm
    2SR + 1 (the canonical forms that Split and the initial QR produce);
  * Join: the joined two-site object embeds to the MPS's own many-electron state;
  * Heff on random vectors, and a sample of its columns with their diagonal entries,
    equal the projection Q^T H Q (blocks whose spins break the triangle rule carry no
    state and must stay decoupled: Heff maps the physical entries to zero there);
  * Split: after the step, the new MPS's energy <Psi|H|Psi> / <Psi|Psi> equals the step's
    Davidson energy and its norm is 1 when nothing is truncated; with truncation the
    energy lies above the Davidson energy and the norm is the kept weight (<= 1);
  * the operator updates are exercised by every Heff check after the first step.

Tolerances: 1e-10 relative to the largest element for Heff and Join (FP64 throughout, the
checker's own rounding is ~1e-14); 1e-9 for energies (the Davidson residual <= 1e-9 gives
an energy error O(1e-18), the rest is rounding).
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

sys.path.insert(0, str(Path(__file__).resolve().parents[1]))
from oracle import fock  # noqa: E402


def chain_of(d, model, total):
    L = model.L
    secs = [fock.sector_dims(d.sectors(b)) for b in range(L + 1)]
    return fock.FockChain(L, model.irreps, secs, [d.get_mps(k) for k in range(L)], total)


def dead_sectors(d, model):
    """[(site, side, (N, 2S, I))] of sectors that hold states without a left history
    ("right": a right sector of the site no block feeds) or without a right completion
    ("left": a left sector with no block to its right). A virtual dimension kept fixed
    through a sweep (the first sweep of a solve) can leave them."""
    L = model.L
    secs = [fock.sector_dims(d.sectors(b)) for b in range(L + 1)]
    out = []
    for s in range(L):
        T = fock.mps_blocks(secs[s], secs[s + 1], model.irreps[s], np.asarray(d.get_mps(s)))
        lefts = {k[:3] for k in T}
        rights = {k[3:] for k in T}
        out += [(s, "left", k) for k in secs[s] if k not in lefts]
        out += [(s, "right", k) for k in secs[s + 1] if k not in rights]
    return out


def rel(a, b):
    return float(np.max(np.abs(a - b))) / max(1.0, float(np.max(np.abs(b))))


def check_canonical(ch, upto_left, from_right, tol=1e-11):
    for b in range(1, upto_left + 1):
        for key, v in ch.left(b).items():
            G = np.einsum("amc,bmc->ab", v, v) / v.shape[1]
            assert np.max(np.abs(G - np.eye(G.shape[0]))) < tol, ("left", b, key)
    for b in range(from_right, ch.L):
        for key, v in ch.right(b).items():
            G = np.einsum("amc,bmc->ab", v, v)
            assert np.max(np.abs(G - (key[1] + 1) * np.eye(G.shape[0]))) < tol * (key[1] + 1), ("right", b, key)


def check_site(d, ch, H, index, rng, ncols=24):
    ts = fock.TwoSite(ch, index)
    assert ts.size == d.sobject_size(index)
    phys = ts.physical
    # Join
    x, _, diag = d.heff_apply(index, None, True)
    psi = ch.state(all_m=True)
    assert rel(fock.joined_state(ts, x), psi) < 1e-10, ("join", index)
    assert np.all(x[~phys] == 0.0), ("join leaves unphysical blocks empty", index)
    # Heff on random vectors over the physical entries
    for _ in range(2):
        xr = np.where(phys, rng.standard_normal(ts.size), 0.0)
        _, y, _ = d.heff_apply(index, xr)
        yf = fock.heff(ts, H, xr)
        assert rel(y[phys], yf[phys]) < 1e-10, ("heff", index, rel(y[phys], yf[phys]))
        if not phys.all():
            assert np.max(np.abs(y[~phys])) <= 1e-12 * max(1.0, np.max(np.abs(y))), ("decoupled", index)
    # a sample of columns, with the diagonal
    pidx = np.flatnonzero(phys)
    cols = pidx if pidx.size <= ncols else rng.choice(pidx, size=ncols, replace=False)
    F = fock.heff_columns(ts, H, cols)
    for c, j in enumerate(cols):
        e = np.zeros(ts.size)
        e[j] = 1.0
        _, y, _ = d.heff_apply(index, e)
        assert rel(y[phys], F[phys, c]) < 1e-10, ("column", index, int(j))
        assert abs(diag[j] - F[j, c]) < 1e-10 * max(1.0, abs(F[j, c])), ("diagonal", index, int(j), diag[j], F[j, c])


def check_sweeps(d, model, total, D, rtol=1e-9, seed=3, exact=True):
    """A left sweep then a right sweep of `d`, checked step by step. exact: D keeps every
    state, so the new MPS's energy equals the Davidson energy; otherwise (truncation) it
    can only lie above it."""
    L = model.L
    H = fock.FockHamiltonian(model.tmat, model.vmat, model.econst)
    rng = np.random.default_rng(seed)
    ch = chain_of(d, model, total)
    check_canonical(ch, L - 1, L)
    steps = [(i, False, False) for i in range(L - 2, 0, -1)] + [(i, True, True) for i in range(0, L - 2)]
    for index, moving_right, change in steps:
        check_site(d, ch, H, index, rng)
        e = d.solve_site(index, rtol, 0.0, D, moving_right, change)
        ch = chain_of(d, model, total)
        psi = ch.state()  # the M = S component
        # norm of the whole multiplet (every M component has the norm of M = S): the
        # normalised two-site vector Split starts from gives 1 without truncation
        nrm = float(psi @ psi) * (total[1] + 1)
        e_mps = float(psi @ H.apply(psi)) / float(psi @ psi)
        if exact:
            assert abs(e_mps - e) < 1e-9, ("split energy", index, e_mps, e)
            assert abs(nrm - 1.0) < 1e-10, ("split norm", index)
        else:
            assert e_mps > e - 1e-9, ("split energy below the two-site minimum", index, e_mps, e)
        assert 0.0 < nrm <= 1.0 + 1e-12
        d.update(index, moving_right)
        ch = chain_of(d, model, total)
        if moving_right:
            check_canonical(ch, index + 1, L)
        else:
            check_canonical(ch, index, index + 1)
