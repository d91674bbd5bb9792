"""The gauge changes of the 2-RDM pass (host/gauge.cpp: QR left normalisation with R into
the next site, LQ right normalisation with L into the previous one; CheMPS2/TensorT.cpp:
188-389, CheMPS2/DMRGtechnics.cpp:276-322) on a truncated state that holds dead sectors,
run on the CPU through the oracle (which links the product's host code) and checked in
Fock space (oracle/fock.py).

The state: synthetic ab initio L=8 C2v, D=4, one sweep from srand(1). The right
half-sweep truncated every boundary-3 sector that the boundary-2 states (3,1,0) connect
to, and the same holds for (5,1,2) at boundary 3. Those states have no right completion.
Right-normalising a site must leave the previous site's blocks on such states zero, or the
2-RDM diagrams count that weight (trace 108 instead of 56 on this state). The gauge
changes must not change the many-electron state either, up to its global sign (1e-12): the
last site's left normalisation drops its 1 x 1 R factor, which is -|a| in the Householder
convention (as in LAPACK's dgeqrf)."""
from __future__ import annotations

import numpy as np

import fock_checks as fc
import models
import oracle_lib as ol
from oracle import fock


def _state_with_dead_sectors():
    m = models.synthetic_ab_initio(8, 5, 8)
    ol.srand(1)
    d = ol.OracleDMRG(m, 0, 8, 0, [(4, 1e-10, 1, 0.0, 1e-8)], check=False)
    d.solve()
    return m, d


def _blocks(d, m, site):
    L = m.L
    secs = [fock.sector_dims(d.sectors(b)) for b in range(L + 1)]
    return secs, fock.mps_blocks(secs[site], secs[site + 1], m.irreps[site], np.asarray(d.get_mps(site)))


def test_gauge_changes_drop_the_weight_on_dead_states():
    m, d = _state_with_dead_sectors()
    L = m.L
    dead = fc.dead_sectors(d, m)
    assert (2, "left", (3, 1, 0)) in dead and (3, "left", (5, 1, 2)) in dead, dead
    psi0 = fc.chain_of(d, m, (8, 0, 0)).state()
    # before the pass, the state's tensors hold weight on the dead states (else this test
    # would not exercise them)
    weight = 0.0
    for site, side, key in dead:
        if side == "left" and site > 0:
            _, T = _blocks(d, m, site - 1)
            weight += sum(float(np.sum(b ** 2)) for k, b in T.items() if k[3:] == key)
    assert weight > 1e-6, weight
    # the gauge changes of the 2-RDM pass: the whole MPS left-canonical, then right
    # normalisation from the last site down to site 1
    d.gauge(L - 2, False)
    d.gauge(L - 1, False)
    for site in range(L - 1, 0, -1):
        d.gauge(site, True)
        secs, T = _blocks(d, m, site)
        lefts = {k[:3] for k in T}
        dead_here = [k for k in secs[site] if k not in lefts]
        _, P = _blocks(d, m, site - 1)
        for key in dead_here:
            for k, b in P.items():
                if k[3:] == key:
                    assert np.max(np.abs(b)) == 0.0, (site, key, np.max(np.abs(b)))
    psi1 = fc.chain_of(d, m, (8, 0, 0)).state()
    err = min(np.max(np.abs(psi1 - psi0)), np.max(np.abs(psi1 + psi0)))
    assert err < 1e-12, err


def test_2rdm_pass_of_the_state_with_dead_sectors():
    """The whole 2-RDM pass on that state (gauge changes, updates and the 2-RDM programs on
    the CPU executor): trace N(N-1) = 56, the 2-RDM energy equals <H> of the MPS, and A
    equals the 2-RDM of the MPS in Fock space, all to 1e-10. Before the gauge changes
    dropped the weight on dead states, the trace was 108."""
    m, d = _state_with_dead_sectors()
    psi = fc.chain_of(d, m, (8, 0, 0)).state()
    H = fock.FockHamiltonian(m.tmat, m.vmat, m.econst)
    e_mps = float(psi @ H.apply(psi)) / float(psi @ psi)
    A_fock = fock.two_rdm_a(H, psi / np.sqrt(psi @ psi))
    A, _, trace, energy = d.calc_2dm()
    assert abs(trace - 56.0) < 1e-10, trace
    assert abs(energy - e_mps) < 1e-10, (energy, e_mps)
    assert np.max(np.abs(A - A_fock)) < 1e-10, np.max(np.abs(A - A_fock))
