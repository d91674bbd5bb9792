"""GPU parity tests: the product path (C-ABI -> device kernels) against the CPU oracle and
the reference's golden energies. Every test here runs the CUDA library on cuda:0.

Tolerances (FP64 throughout): element-wise Heff / diagonal / joined-state parity 1e-10
relative to the largest element; per-step Davidson energies 1e-8 (both solvers stop at a
residual norm <= rtol, the energy error is O(rtol^2)); converged energies 1e-8 Ha against
FCI and the reference's goldens, the bar the reference's own tests use
(tests/test4.cpp.in:103, tests/test12.cpp.in:99, tests/test5.cpp.in:83).
"""
from __future__ import annotations

import json
from pathlib import Path

import numpy as np
import pytest

import chemps2_gb300 as c2g
import models
import oracle_lib as ol

pytestmark = pytest.mark.gpu

GOLDEN_DIR = Path(__file__).parent / "golden"
GOLDEN = json.loads((GOLDEN_DIR / "golden.json").read_text())


def gpu_objects(model: models.Model, two_s, n, irrep, schedule):
    ham = c2g.Hamiltonian(model.L, model.group, model.irreps)
    L = model.L
    for i in range(L):
        for j in range(i, L):
            if model.tmat[i, j] != 0.0:
                ham.setTmat(i, j, model.tmat[i, j])
    nz = np.argwhere(model.vmat != 0.0)
    for i, j, k, l in nz:
        ham.setVmat(int(i), int(j), int(k), int(l), float(model.vmat[i, j, k, l]))
    ham.setEconst(model.econst)
    prob = c2g.Problem(ham, two_s, n, irrep)
    scheme = c2g.ConvergenceScheme(len(schedule))
    for i, s in enumerate(schedule):
        scheme.set_instruction(i, *s)
    return ham, prob, scheme


def rel_err(a, b):
    scale = max(1.0, float(np.max(np.abs(b))) if b.size else 1.0)
    return float(np.max(np.abs(a - b))) / scale if a.size else 0.0


CASES = [
    ("hubbard8", lambda: models.hubbard(8, 4.0), 0, 8, 0),
    ("abinit8_c2v", lambda: models.synthetic_ab_initio(8, 5, 11), 0, 8, 0),
    ("abinit9_d2h_doublet", lambda: models.synthetic_ab_initio(9, 7, 12), 1, 9, 3),
]


@pytest.mark.parametrize("name,make,two_s,n,irrep", CASES)
def test_heff_matches_oracle_on_fresh_state(name, make, two_s, n, irrep):
    """Heff, its diagonal and Join at sites (L-2, L-1) right after construction: the GPU
    and the oracle start from the same random MPS, so the results agree element-wise."""
    m = make()
    sched = [(64, 1e-10, 1, 0.0, 1e-8)]
    ham, prob, scheme = gpu_objects(m, two_s, n, irrep, sched)
    c2g.srand(5)
    gpu = c2g.DMRG(prob, scheme)
    ol.srand(5)
    cpu = ol.OracleDMRG(m, two_s, n, irrep, sched)
    L = m.L
    xg, yg, dg = gpu.heff_apply(L - 2, None, True)
    xc, yc, dc = cpu.heff_apply(L - 2, None, True)
    assert xg.shape == xc.shape
    assert rel_err(xg, xc) < 1e-10
    assert rel_err(yg, yc) < 1e-10
    assert rel_err(dg, dc) < 1e-10
    # a random vector too
    rng = np.random.default_rng(1)
    x = rng.standard_normal(xg.size)
    _, yg2, _ = gpu.heff_apply(L - 2, x)
    _, yc2, _ = cpu.heff_apply(L - 2, x)
    assert rel_err(yg2, yc2) < 1e-10
    gpu.close()


@pytest.mark.parametrize("one_pass", [False, True])
def test_heff_large_blocks_match_oracle(one_pass, monkeypatch):
    """Heff at the middle of a C1 Hubbard chain whose sector blocks are large (the two-pass
    large-block path: intermediates once, then split item sums), and with C2G_LARGE=tile
    the one-pass cooperative kernel, element-wise against the oracle; the FP32 variant of
    the same program within FP32 rounding."""
    if one_pass:
        monkeypatch.setenv("C2G_LARGE", "tile")
    else:
        monkeypatch.delenv("C2G_LARGE", raising=False)
    m = models.hubbard(12, 4.0)
    sched = [(256, 1e-10, 1, 0.0, 1e-8)]
    ham, prob, scheme = gpu_objects(m, 0, 12, 0, sched)
    c2g.srand(9)
    gpu = c2g.DMRG(prob, scheme)
    ol.srand(9)
    cpu = ol.OracleDMRG(m, 0, 12, 0, sched)
    mid = m.L // 2 - 1
    for index in range(m.L - 2, mid, -1):
        gpu.update(index, False)
        cpu.update(index, False)
    xg, yg, _ = gpu.heff_apply(mid)
    rng = np.random.default_rng(3)
    x = rng.standard_normal(xg.size)
    _, yg, _ = gpu.heff_apply(mid, x)
    _, yc, _ = cpu.heff_apply(mid, x)
    assert rel_err(yg, yc) < 1e-10
    y32 = gpu.heff_apply_fp32(mid, x)
    assert rel_err(y32, yc) < 1e-4
    gpu.close()


@pytest.mark.parametrize("name,make,two_s,n,irrep", CASES)
def test_sweep_steps_match_oracle(name, make, two_s, n, irrep):
    """One left and one right sweep step by step: per-step energies, then Heff at every
    interior site (all five diagram groups active) against the oracle."""
    m = make()
    L = m.L
    D = 48
    sched = [(D, 1e-10, 1, 0.0, 1e-9)]
    ham, prob, scheme = gpu_objects(m, two_s, n, irrep, sched)
    c2g.srand(9)
    gpu = c2g.DMRG(prob, scheme)
    ol.srand(9)
    cpu = ol.OracleDMRG(m, two_s, n, irrep, sched)
    for change, mr, rng_ in ((False, False, range(L - 2, 0, -1)), (True, True, range(0, L - 2))):
        for index in rng_:
            eg = gpu.solve_site(index, 1e-9, 0.0, D, mr, change)
            ec = cpu.solve_site(index, 1e-9, 0.0, D, mr, change)
            assert abs(eg - ec) < 1e-8, (index, eg, ec)
            gpu.update(index, mr)
            cpu.update(index, mr)
    # after the right sweep, boundaries are moving right up to L-3; re-sweep left to get
    # right operators everywhere, checking Heff on the way
    for index in range(L - 2, 0, -1):
        if 0 < index < L - 2:
            xg, yg, _ = gpu.heff_apply(index, None, False)
            xc, yc, _ = cpu.heff_apply(index, None, False)
            # The Rayleigh quotient and the norms are invariant under the orthogonal gauge
            # freedom of the renormalized bases (degenerate singular values).
            assert abs(xg @ yg / (xg @ xg) - xc @ yc / (xc @ xc)) < 1e-8
            assert abs(np.linalg.norm(yg) - np.linalg.norm(yc)) < 1e-8 * max(1.0, np.linalg.norm(yc))
        eg = gpu.solve_site(index, 1e-9, 0.0, D, False, True)
        ec = cpu.solve_site(index, 1e-9, 0.0, D, False, True)
        assert abs(eg - ec) < 1e-8, (index, eg, ec)
        gpu.update(index, False)
        cpu.update(index, False)
    gpu.close()


def test_solve_hubbard_of_reference_test4_against_fci():
    m = models.hubbard(10, 2.0)
    sched = [(30, 1e-10, 3, 0.1, 1e-5), (1000, 1e-10, 10, 0.0, 1e-5)]
    ham, prob, scheme = gpu_objects(m, 5, 9, 0, sched)
    c2g.srand(1)
    gpu = c2g.DMRG(prob, scheme)
    e = gpu.Solve()
    gpu.close()
    assert abs(e - ol.fci_energy(m, 7, 2, 0)) < 1e-8


def test_solve_synthetic_d2h_against_oracle_and_fci():
    m = models.synthetic_ab_initio(10, 7, 21)
    sched = [(300, 1e-10, 4, 0.0, 1e-8)]
    ham, prob, scheme = gpu_objects(m, 0, 10, 0, sched)
    c2g.srand(2)
    gpu = c2g.DMRG(prob, scheme)
    e = gpu.Solve()
    gpu.close()
    ol.srand(2)
    cpu = ol.OracleDMRG(m, 0, 10, 0, sched)
    e_cpu = cpu.solve()
    assert abs(e - e_cpu) < 1e-8
    e_fci = ol.fci_energy(m, 5, 5, 0)
    assert e >= e_fci - 1e-8
    assert abs(e - e_fci) < 1e-6 or e_fci < e  # the lowest Sz=0 state may be a higher spin


def test_bcs_golden_of_reference_test12():
    g = GOLDEN["bcs_l8"]
    L = len(g["eps"])
    ham = c2g.Hamiltonian(L, 0, np.zeros(L, dtype=np.int32))
    prob = c2g.Problem(ham, g["two_s"], g["n"], g["irrep"])
    scheme = c2g.ConvergenceScheme(len(g["schedule"]))
    for i, s in enumerate(g["schedule"]):
        scheme.set_instruction(i, *s)
    c2g.srand(1)
    gpu = c2g.DMRG(prob, scheme)  # constructs the matrix elements, then they are overwritten
    _, elems = models.bcs(g["eps"], g["g"], g["power"])
    for o1, o2, eri, oei in elems:
        if o1 == o2:
            prob.setMxElement(o1, o1, o2, o2, eri + oei)
        else:
            prob.setMxElement(o1, o1, o2, o2, eri)
            prob.setMxElement(o1, o2, o1, o2, oei)
    gpu.PreSolve()
    e = gpu.Solve()
    gpu.close()
    assert abs(e - g["energy"]) < g["tolerance"]


def test_n2_sto3g_golden_of_reference_test5():
    g = GOLDEN["n2_sto3g"]
    ham = c2g.Hamiltonian(0, g["group"], [], filename=str(GOLDEN_DIR / g["fcidump"]))
    prob = c2g.Problem(ham, g["two_s"], g["n"], g["irrep"])
    prob.SetupReorderD2h()
    scheme = c2g.ConvergenceScheme(1)
    scheme.set_instruction(0, *g["schedule"][0])
    c2g.srand(1)
    gpu = c2g.DMRG(prob, scheme)
    e = gpu.Solve()
    gpu.close()
    assert abs(e - g["energy"]) < g["tolerance"]


def test_ch4_sto3g_against_fci_of_reference_test3():
    """The reference's tests/test3.cpp.in: CH4 STO-3G (C2v, N = 10, singlet A1) with its
    two-instruction schedule (D = 30 with noise, then D = 1000); the GPU energy equals the
    oracle's determinant FCI energy to 1e-8."""
    g = GOLDEN["ch4_sto3g"]
    path = GOLDEN_DIR / g["fcidump"]
    efci = ol.fci_energy(ol.fcidump_model(path, g["group"]), (g["n"] + g["two_s"]) // 2,
                         (g["n"] - g["two_s"]) // 2, g["irrep"])
    ham = c2g.Hamiltonian(0, g["group"], [], filename=str(path))
    prob = c2g.Problem(ham, g["two_s"], g["n"], g["irrep"])
    scheme = c2g.ConvergenceScheme(len(g["schedule"]))
    for i, instr in enumerate(g["schedule"]):
        scheme.set_instruction(i, *instr)
    c2g.srand(1)
    gpu = c2g.DMRG(prob, scheme)
    try:
        e = gpu.Solve()
    finally:
        gpu.close()
    assert abs(e - efci) < g["tolerance"], (e, efci)


def test_n2_sto3g_sectors_against_fci_of_reference_test1():
    """The reference's tests/test1.cpp.in: N2 STO-3G (D2h, N = 14) in six (2S, irrep)
    sectors, singlet to quintet, with its schedule (D = 500, then D = 1000 to a 1e-10
    residual); every GPU energy equals the oracle's FCI energy of its sector to 1e-8."""
    g = GOLDEN["n2_sto3g_sectors"]
    path = GOLDEN_DIR / g["fcidump"]
    m = ol.fcidump_model(path, g["group"])
    for two_s, irrep in zip(g["two_s"], g["irreps"]):
        efci = ol.fci_energy(m, (g["n"] + two_s) // 2, (g["n"] - two_s) // 2, irrep)
        ham = c2g.Hamiltonian(0, g["group"], [], filename=str(path))
        prob = c2g.Problem(ham, two_s, g["n"], irrep)
        scheme = c2g.ConvergenceScheme(len(g["schedule"]))
        for i, instr in enumerate(g["schedule"]):
            scheme.set_instruction(i, *instr)
        c2g.srand(1)
        gpu = c2g.DMRG(prob, scheme)
        try:
            e = gpu.Solve()
        finally:
            gpu.close()
        assert abs(e - efci) < g["tolerance"], (two_s, irrep, e, efci)


def test_hubbard_3x3_site_against_momentum_basis_of_reference_test9():
    """The reference's tests/test9.cpp.in: the 3 x 3 periodic Hubbard model (U = 5, N = 9,
    doublet) in the site basis and, through setMxElement + PreSolve on the same DMRG
    object's problem, in the momentum basis (matrix elements with only fourfold
    symmetry); the two GPU energies agree to 1e-8."""
    site, mom = models.hubbard_3x3_site_and_momentum()
    sched = [(500, 1e-10, 3, 0.05, 1e-5), (1000, 1e-10, 10, 0.0, 1e-5)]
    ham, prob, scheme = gpu_objects(site, 1, 9, 0, sched)
    c2g.srand(1)
    gpu = c2g.DMRG(prob, scheme)
    try:
        e_site = gpu.Solve()
    finally:
        gpu.close()
    c2g.srand(1)
    gpu = c2g.DMRG(prob, scheme)
    try:
        for i in range(9):
            for j in range(9):
                for k in range(9):
                    for l in range(9):
                        prob.setMxElement(i, j, k, l, mom.get((i, j, k, l), 0.0))
        gpu.PreSolve()
        e_mom = gpu.Solve()
    finally:
        gpu.close()
    assert abs(e_mom - e_site) < 1e-8, (e_site, e_mom)


def test_fci_coefficients_equal_fock_space_amplitudes():
    """getFCIcoefficient / getSpecificCoefficient on the GPU's MPS (downloaded, then the
    host routine) equal the Fock-space amplitudes of the same MPS (oracle/fock.py) for every
    determinant of the sector, to 1e-12; C2v doublet."""
    import itertools

    import fock_checks as fc

    m = models.synthetic_ab_initio(5, 5, 3)
    ham, prob, scheme = gpu_objects(m, 1, 5, 2, [(64, 1e-10, 2, 0.0, 1e-10)])
    c2g.srand(2)
    gpu = c2g.DMRG(prob, scheme)
    try:
        gpu.Solve()
        psi = fc.chain_of(gpu, m, (5, 1, 2)).state()
        worst, count = 0.0, 0
        for ups in itertools.combinations(range(5), 3):
            for dns in itertools.combinations(range(5), 2):
                a = np.zeros(5, dtype=np.int32)
                b = np.zeros(5, dtype=np.int32)
                a[list(ups)] = 1
                b[list(dns)] = 1
                conf = sum(int(a[k] + 2 * b[k]) * 4 ** (4 - k) for k in range(5))
                worst = max(worst, abs(gpu.getFCIcoefficient(a, b) - psi[conf]))
                count += 1
        assert worst < 1e-12, worst
        occ = np.array([2, 2, 1, 0, 0])
        assert gpu.getSpecificCoefficient(occ) == gpu.getFCIcoefficient([1, 1, 1, 0, 0], [1, 1, 0, 0, 0])
    finally:
        gpu.close()


def test_kernels_were_launched():
    before = c2g.kernel_launches()
    m = models.hubbard(6, 4.0)
    ham, prob, scheme = gpu_objects(m, 0, 6, 0, [(32, 1e-10, 1, 0.0, 1e-8)])
    gpu = c2g.DMRG(prob, scheme)
    gpu.heff_apply(4)
    gpu.close()
    assert c2g.kernel_launches() > before


def test_fp32_matvec_close_to_fp64():
    """The FP32-arithmetic matvec of the mixed path: relative error at the FP32 level."""
    m = models.synthetic_ab_initio(10, 7, 31)
    ham, prob, scheme = gpu_objects(m, 0, 10, 0, [(64, 1e-10, 1, 0.0, 1e-8)])
    c2g.srand(4)
    gpu = c2g.DMRG(prob, scheme)
    x, y64, _ = gpu.heff_apply(m.L - 2)
    y32 = gpu.heff_apply_fp32(m.L - 2, x)
    gpu.close()
    assert np.linalg.norm(y32 - y64) / np.linalg.norm(y64) < 1e-5


def test_mixed_precision_solve_matches_fp64():
    """Mixed Davidson (FP32 expansion, FP64 finish) reaches the FP64 energies: within
    1e-8 Ha of the FP64 run and of FCI, and it did use FP32 matvecs."""
    m = models.synthetic_ab_initio(10, 7, 21)
    sched = [(300, 1e-10, 4, 0.0, 1e-8)]
    energies = {}
    for mode in ("fp64", "mixed"):
        ham, prob, scheme = gpu_objects(m, 0, 10, 0, sched)
        c2g.srand(2)
        gpu = c2g.DMRG(prob, scheme)
        gpu.set_precision(mode)
        energies[mode] = gpu.Solve()
        st = gpu.stats()
        if mode == "mixed":
            assert st["n_matvec_fp32"] > 0
        else:
            assert st["n_matvec_fp32"] == 0
        gpu.close()
    assert abs(energies["mixed"] - energies["fp64"]) < 1e-8


def test_program_cache_reuses_programs_across_sweeps():
    """Once the dimensions settle, later sweeps reuse compiled programs: the host compile
    time of a repeated sweep is a small fraction of the first one's, with the same energy."""
    m = models.hubbard(10, 2.0)
    sched = [(1000, 1e-12, 1, 0.0, 1e-9)]
    ham, prob, scheme = gpu_objects(m, 0, 10, 0, sched)
    c2g.srand(3)
    gpu = c2g.DMRG(prob, scheme)
    e1 = gpu.Solve()   # dims reach the full space
    gpu.reset_stats()
    e2 = gpu.Solve()
    t2 = gpu.stats()["t_compile"]
    gpu.reset_stats()
    e3 = gpu.Solve()
    t3 = gpu.stats()["t_compile"]
    gpu.close()
    assert abs(e3 - e2) < 1e-9 and abs(e2 - e1) < 1e-7
    assert t3 <= 0.2 * t2 + 0.05


def test_n2_sto3g_excited_states_golden_of_reference_test5():
    """The reference's tests/test5.cpp.in: ground state, then two excited states of the same
    symmetry with newExcitation(20.0) each, energies to 1e-8 of its goldens."""
    g = GOLDEN["n2_sto3g"]
    ham = c2g.Hamiltonian(0, g["group"], [], filename=str(GOLDEN_DIR / g["fcidump"]))
    prob = c2g.Problem(ham, g["two_s"], g["n"], g["irrep"])
    prob.SetupReorderD2h()
    scheme = c2g.ConvergenceScheme(1)
    scheme.set_instruction(0, *g["schedule"][0])
    c2g.srand(1)
    gpu = c2g.DMRG(prob, scheme)
    try:
        e0 = gpu.Solve()
        assert abs(e0 - g["energy"]) < g["tolerance"]
        gpu.activateExcitations(10)
        energies = []
        for _ in g["excited_energies"]:
            gpu.newExcitation(g["excited_eshift"])
            energies.append(gpu.Solve())
    finally:
        gpu.close()
    for e, ref in zip(energies, g["excited_energies"]):
        assert abs(e - ref) < g["tolerance"], (energies, g["excited_energies"])


def test_mps_checkpoint_restart(tmp_path, monkeypatch):
    """makechkpt (CheMPS2/DMRGmpsio.cpp, CheMPS2/DMRG.cpp:106-158,334): a DMRG writes its MPS
    after every sweep; a new DMRG in the same directory starts from that file and, already
    converged, reproduces the energy in its first sweep."""
    monkeypatch.chdir(tmp_path)
    m = models.synthetic_ab_initio(8, 5, 11)
    ham, prob, scheme = gpu_objects(m, 0, 8, 0, [(64, 1e-10, 4, 0.0, 1e-9)])
    c2g.srand(5)
    first = c2g.DMRG(prob, scheme, makechkpt=True)
    assert not first.loadedMPS()
    e1 = first.Solve()
    first.close()
    assert (tmp_path / "CheMPS2_MPS0.c2g").exists()
    scheme2 = c2g.ConvergenceScheme(1)
    scheme2.set_instruction(0, 64, 1e-10, 1, 0.0, 1e-9)
    second = c2g.DMRG(prob, scheme2, makechkpt=True)
    try:
        assert second.loadedMPS()
        second.reset_stats()
        e2 = second.Solve()
        assert abs(e2 - e1) < 1e-8
        second.deleteStoredMPS()
    finally:
        second.close()
    assert not (tmp_path / "CheMPS2_MPS0.c2g").exists()


def test_heff_apply_on_device_buffers_with_a_stream():
    """c2g_dmrg_heff_apply_device: the same matvec on the caller's device buffers, both
    synchronous and ordered on a caller's CUDA stream (FP64 bit-identical to the host-buffer
    call; FP32 within FP32 rounding)."""
    torch = pytest.importorskip("torch")
    m = models.hubbard(8, 4.0)
    sched = [(64, 1e-10, 1, 0.0, 1e-8)]
    ham, prob, scheme = gpu_objects(m, 0, 8, 0, sched)
    c2g.srand(5)
    gpu = c2g.DMRG(prob, scheme)
    idx = m.L - 2
    n = gpu.sobject_size(idx)
    x = np.random.default_rng(2).standard_normal(n)
    _, y_host, _ = gpu.heff_apply(idx, x)
    xd = torch.from_numpy(x).cuda()
    yd = torch.empty_like(xd)
    gpu.heff_apply_device(idx, xd.data_ptr(), yd.data_ptr(), n)
    assert np.array_equal(yd.cpu().numpy(), y_host)
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        x2 = xd * 2.0  # produced on the caller's stream right before the call
        y2 = torch.empty_like(xd)
    gpu.heff_apply_device(idx, x2.data_ptr(), y2.data_ptr(), n, stream=s.cuda_stream)
    with torch.cuda.stream(s):
        y2h = y2.cpu()
    s.synchronize()
    assert np.max(np.abs(y2h.numpy() - 2.0 * y_host)) <= 1e-12 * np.max(np.abs(y_host))
    y32 = torch.empty_like(xd)
    gpu.heff_apply_device(idx, xd.data_ptr(), y32.data_ptr(), n, precision="fp32")
    assert np.linalg.norm(y32.cpu().numpy() - y_host) / np.linalg.norm(y_host) < 1e-5
    gpu.close()
