"""CPU tests of the product library without a GPU: the C-ABI loads and exports every
symbol of include/chemps2_gb300.h, the host bookkeeping is bit-exact against a direct
restatement of the reference's loops, and the drop-in API keeps the reference's argument
checks. No compute kernel is called here."""
from __future__ import annotations

import ctypes as C
import math
import re
from fractions import Fraction
from pathlib import Path

import numpy as np
import pytest

import chemps2_gb300 as c2g
import models

ROOT = Path(__file__).resolve().parents[1]


def header_symbols():
    text = (ROOT / "include" / "chemps2_gb300.h").read_text()
    return sorted(set(re.findall(r"^\s*(?:int|const char\*)\s+(c2g_\w+)\s*\(", text, re.M)))


def test_library_exports_every_declared_symbol():
    lib = c2g.load()
    syms = header_symbols()
    assert len(syms) > 40
    for s in syms:
        assert hasattr(lib, s), s


def test_dmrg_without_device_fails_loudly():
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    ham = c2g.Hamiltonian(4, 0, np.zeros(4, dtype=np.int32))
    prob = c2g.Problem(ham, 0, 4, 0)
    sc = c2g.ConvergenceScheme(1)
    sc.set_instruction(0, 10, 1e-8, 1, 0.0, 1e-6)
    with pytest.raises(c2g.Chemps2Error):
        c2g.DMRG(prob, sc)


# ---------------------------------------------------------------- bookkeeping parity
def ref_bookkeeper(L, irreps, nirr, N, two_s, irrep, D):
    """Restatement of CheMPS2/SyBookkeeper.cpp:29-269 (FCI dims by the left and right
    recurrences, capped at 262144, then the ceil scaling of the current dims)."""
    cap = 262144
    Nmin = [max(0, N - 2 * (L - b)) for b in range(L + 1)]
    Nmax = [min(2 * b, N) for b in range(L + 1)]
    # left: dict (b, n, s, i) -> dim
    left = {(0, 0, 0, 0): 1}
    for b in range(1, L + 1):
        for (bb, n, s, i), d in list(left.items()):
            if bb != b - 1:
                continue
            for (dn, ds_list, di) in ((0, [0], 0), (2, [0], 0), (1, [-1, 1], irreps[b - 1])):
                for ds in ds_list:
                    key = (b, n + dn, s + ds, i ^ di)
                    if key[2] < 0:
                        continue
                    left[key] = min(cap, left.get(key, 0) + d)
    right = {(L, N, two_s, irrep): 1}
    for b in range(L - 1, -1, -1):
        for (bb, n, s, i), d in list(right.items()):
            if bb != b + 1:
                continue
            for (dn, ds_list, di) in ((0, [0], 0), (2, [0], 0), (1, [-1, 1], irreps[b])):
                for ds in ds_list:
                    key = (b, n - dn, s + ds, i ^ di)
                    if key[2] < 0 or key[1] < 0:
                        continue
                    right[key] = min(cap, right.get(key, 0) + d)
    fci = {}
    for b in range(L + 1):
        for n in range(Nmin[b], Nmax[b] + 1):
            for s in range(0, 2 * L + 2):
                for i in range(nirr):
                    v = min(left.get((b, n, s, i), 0), right.get((b, n, s, i), 0))
                    if v > 0:
                        fci[(b, n, s, i)] = v
    cur = {}
    for b in range(L + 1):
        tot = sum(v for (bb, *_), v in fci.items() if bb == b)
        for k, v in fci.items():
            if k[0] != b:
                continue
            cur[k] = v if tot <= D else min(v, math.ceil(D * v / tot))
    return fci, cur


@pytest.mark.parametrize("L,group,N,two_s,irrep,D", [
    (8, 0, 8, 0, 0, 20), (10, 7, 10, 0, 0, 50), (9, 5, 9, 1, 2, 30), (12, 7, 12, 2, 3, 200), (16, 0, 16, 0, 0, 200),
])
def test_bookkeeper_dims_bit_exact(L, group, N, two_s, irrep, D):
    nirr = models.NIRREPS[group]
    irreps = [i % nirr for i in range(L)]
    ham = c2g.Hamiltonian(L, group, np.array(irreps, dtype=np.int32))
    prob = c2g.Problem(ham, two_s, N, irrep)
    fci, cur = ref_bookkeeper(L, irreps, nirr, N, two_s, irrep, D)
    for b in range(L + 1):
        got = prob.bookkeeper_sectors(D, b)
        got_f = {(b, int(r[0]), int(r[1]), int(r[2])): int(r[3]) for r in got if r[3] > 0}
        got_c = {(b, int(r[0]), int(r[1]), int(r[2])): int(r[4]) for r in got if r[3] > 0}
        exp_f = {k: v for k, v in fci.items() if k[0] == b}
        exp_c = {k: v for k, v in cur.items() if k[0] == b}
        assert got_f == exp_f, b
        assert got_c == exp_c, b


def ref_sobject_blocks(prob: c2g.Problem, D, index, L, irreps, nirr):
    """Restatement of the block enumeration of CheMPS2/Sobject.cpp:36-145: loops NL, 2SL,
    IL, N1, N2, 2J, NR, 2SR, IR in that order, then the stable size sort of :115-145."""
    sec = {}
    for b in (index, index + 2):
        for r in prob.bookkeeper_sectors(D, b):
            sec[(b, int(r[0]), int(r[1]), int(r[2]))] = int(r[4])
    blocks = []
    I1, I2 = irreps[index], irreps[index + 1]
    keys_l = sorted(k for k in sec if k[0] == index)
    for (_, NL, TwoSL, IL) in keys_l:
        dimL = sec[(index, NL, TwoSL, IL)]
        if dimL <= 0:
            continue
        for N1 in range(3):
            for N2 in range(3):
                TwoJmin = (N1 + N2) % 2 if False else (1 if (N1 == 1) != (N2 == 1) else 0)
                TwoJmax = (1 if N1 == 1 else 0) + (1 if N2 == 1 else 0)
                for TwoJ in range(TwoJmin, TwoJmax + 1, 2):
                    NR = NL + N1 + N2
                    IR = IL ^ (I1 if N1 == 1 else 0) ^ (I2 if N2 == 1 else 0)
                    for TwoSR in range(TwoSL - TwoJ, TwoSL + TwoJ + 1, 2):
                        if TwoSR < 0:
                            continue
                        dimR = sec.get((index + 2, NR, TwoSR, IR), 0)
                        if dimR > 0:
                            blocks.append(((NL, TwoSL, IL, N1, N2, TwoJ, NR, TwoSR, IR), dimL * dimR))
    return blocks


@pytest.mark.parametrize("L,group,N,two_s,irrep,D,index", [
    (8, 0, 8, 0, 0, 30, 3), (10, 7, 10, 0, 0, 60, 4), (9, 5, 9, 1, 2, 40, 2), (12, 7, 12, 0, 0, 200, 5),
])
def test_sobject_layout_bit_exact(L, group, N, two_s, irrep, D, index):
    nirr = models.NIRREPS[group]
    irreps = [i % nirr for i in range(L)]
    ham = c2g.Hamiltonian(L, group, np.array(irreps, dtype=np.int32))
    prob = c2g.Problem(ham, two_s, N, irrep)
    labels, k2i, order = prob.sobject_layout(D, index)
    exp = ref_sobject_blocks(prob, D, index, L, irreps, nirr)
    assert [tuple(int(v) for v in r) for r in labels] == [b[0] for b in exp]
    sizes = [b[1] for b in exp]
    assert list(k2i) == list(np.concatenate([[0], np.cumsum(sizes)]))
    # visiting order: non-increasing size, stable among equal sizes
    exp_order = sorted(range(len(sizes)), key=lambda k: -sizes[k])
    assert list(order) == exp_order


# The benchmark configurations: Hubbard L=16 C1 D=200, synthetic ab initio L=24 D2h
# D=1000, L=30 D2h D=2000 and L=40 C2v D=4000 (N = L, S = 0, irreps round robin, target
# irrep 0). Every boundary's FCI and scaled dimensions are checked against the restatement
# of CheMPS2/SyBookkeeper.cpp, and the middle two-site object's block list, kappa2index and
# visiting order against the restatement of CheMPS2/Sobject.cpp:36-145. The pinned counts
# (sectors at the middle boundary, blocks and amplitudes of the middle two-site object)
# are those of an independent probe of the reference's bookkeeping.
BENCH_CONFIGS = [
    # L, group, D, middle-boundary sectors, nKappa, two-site vector length
    (16, 0, 200, 45, 466, 38028),
    (24, 7, 1000, 707, 8412, 97786),
    (30, 7, 2000, 1066, 13452, 221852),
    (40, 5, 4000, 915, 12220, 523676),
]


@pytest.mark.parametrize("L,group,D,nsec,nkappa,veclen", BENCH_CONFIGS)
def test_bookkeeper_and_sobject_at_benchmark_configs(L, group, D, nsec, nkappa, veclen):
    nirr = models.NIRREPS[group]
    irreps = [i % nirr for i in range(L)]
    ham = c2g.Hamiltonian(L, group, np.array(irreps, dtype=np.int32))
    prob = c2g.Problem(ham, 0, L, 0)
    fci, cur = ref_bookkeeper(L, irreps, nirr, L, 0, 0, D)
    for b in range(L + 1):
        got = prob.bookkeeper_sectors(D, b)
        got_f = {(b, int(r[0]), int(r[1]), int(r[2])): int(r[3]) for r in got if r[3] > 0}
        got_c = {(b, int(r[0]), int(r[1]), int(r[2])): int(r[4]) for r in got if r[3] > 0}
        assert got_f == {k: v for k, v in fci.items() if k[0] == b}, b
        assert got_c == {k: v for k, v in cur.items() if k[0] == b}, b
    mid = L // 2
    assert sum(1 for r in prob.bookkeeper_sectors(D, mid) if r[4] > 0) == nsec
    index = L // 2 - 1
    labels, k2i, order = prob.sobject_layout(D, index)
    exp = ref_sobject_blocks(prob, D, index, L, irreps, nirr)
    assert len(labels) == nkappa and int(k2i[-1]) == veclen
    assert [tuple(int(v) for v in r) for r in labels] == [b[0] for b in exp]
    sizes = [b[1] for b in exp]
    assert list(k2i) == list(np.concatenate([[0], np.cumsum(sizes)]))
    assert list(order) == sorted(range(len(sizes)), key=lambda k: -sizes[k])


# ---------------------------------------------------------------- Wigner symbols
def racah_6j(a, b, c, d, e, f):
    """Exact 6j symbol in rationals (arguments twice the spins), Racah's formula."""
    def tri(x, y, z):
        return (x + y + z) % 2 == 0 and abs(x - y) <= z <= x + y

    if not (tri(a, b, c) and tri(d, e, c) and tri(a, e, f) and tri(d, b, f)):
        return 0.0
    F = math.factorial

    def delta(x, y, z):
        return Fraction(F((x + y - z) // 2) * F((x - y + z) // 2) * F((-x + y + z) // 2), F((x + y + z) // 2 + 1))

    a1, a2, a3, a4 = (a + b + c) // 2, (d + e + c) // 2, (a + e + f) // 2, (d + b + f) // 2
    b1, b2, b3 = (a + b + d + e) // 2, (a + c + d + f) // 2, (b + c + e + f) // 2
    s = Fraction(0)
    for k in range(max(a1, a2, a3, a4), min(b1, b2, b3) + 1):
        s += Fraction((-1) ** k * F(k + 1), F(k - a1) * F(k - a2) * F(k - a3) * F(k - a4) * F(b1 - k) * F(b2 - k)
                      * F(b3 - k))
    pref2 = delta(a, b, c) * delta(d, e, c) * delta(a, e, f) * delta(d, b, f)
    return float(s) * math.sqrt(float(pref2))


def test_wigner6j_against_exact_racah():
    rng = np.random.default_rng(0)
    n = 0
    for _ in range(3000):
        a, b, d, e = (int(x) for x in rng.integers(0, 12, size=4))
        for c in range(abs(a - b), a + b + 1, 2):
            for f in range(abs(a - e), a + e + 1, 2):
                ref = racah_6j(a, b, c, d, e, f)
                got = c2g.wigner6j(a, b, c, d, e, f)
                assert abs(got - ref) < 1e-13, (a, b, c, d, e, f)
                n += 1
    assert n > 1000
    # large arguments stay accurate (|err| <= 7e-12 at 2j <= 95 in the reference)
    assert abs(c2g.wigner6j(90, 90, 0, 90, 90, 0) - 1.0 / 91) < 1e-12


def test_wigner3j_against_sympy():
    """The 3j symbol of getFCIcoefficient's Clebsch-Gordan couplings against sympy's exact
    values, over all projections of random spins up to 11/2 and a large case."""
    from sympy import Rational
    from sympy.physics.wigner import wigner_3j

    rng = np.random.default_rng(1)
    n = 0
    for _ in range(150):
        a, b = (int(x) for x in rng.integers(0, 12, size=2))
        for c in range(abs(a - b), a + b + 1, 2):
            for ma in range(-a, a + 1, 2):
                for mb in range(-b, b + 1, 2):
                    mc = -ma - mb
                    if abs(mc) > c:
                        continue
                    ref = float(wigner_3j(Rational(a, 2), Rational(b, 2), Rational(c, 2), Rational(ma, 2),
                                          Rational(mb, 2), Rational(mc, 2)))
                    assert abs(c2g.wigner3j(a, b, c, ma, mb, mc) - ref) < 1e-13, (a, b, c, ma, mb, mc)
                    n += 1
    assert n > 1000
    assert c2g.wigner3j(2, 2, 2, 2, 2, -2) == 0.0  # projections that do not add to zero
    assert c2g.wigner3j(2, 2, 6, 0, 0, 0) == 0.0  # triangle rule
    ref = float(wigner_3j(40, 40, 0, 3, -3, 0))
    assert abs(c2g.wigner3j(80, 80, 0, 6, -6, 0) - ref) < 1e-12


def ninej_from_6j(a, b, c, d, e, f, g, h, i):
    """9j symbol {a b c; d e f; g h i} (arguments twice the spins) as the sum over x of
    (-1)^(2x) (2x + 1) {a b c; f i x} {d e f; b x h} {g h i; x a d} (Edmonds 6.4.3), from
    the exact-rational 6j symbols above."""
    tot = 0.0
    for x in range(0, 2 * max(a, b, c, d, e, f, g, h, i) + 2):
        w = racah_6j(a, b, c, f, i, x)
        if w == 0.0:
            continue
        w *= racah_6j(d, e, f, b, x, h)
        if w == 0.0:
            continue
        w *= racah_6j(g, h, i, x, a, d)
        tot += (-1) ** x * (x + 1) * w
    return tot


def test_wigner9j_against_6j_sums():
    rng = np.random.default_rng(5)
    n = 0
    for _ in range(4000):
        a, b, d, e = (int(x) for x in rng.integers(0, 6, size=4))
        for c in range(abs(a - b), a + b + 1, 2):
            for f in range(abs(d - e), d + e + 1, 2):
                g = int(rng.integers(0, 6))
                for h in range(abs(b - e) + ((abs(b - e) + g) % 2 != (b + e + g) % 2), b + e + 1, 2):
                    for i in range(abs(c - f), c + f + 1, 2):
                        if not (abs(a - d) <= g <= a + d and (a + d + g) % 2 == 0):
                            continue
                        if not (abs(g - h) <= i <= g + h and (g + h + i) % 2 == 0):
                            continue
                        ref = ninej_from_6j(a, b, c, d, e, f, g, h, i)
                        got = c2g.wigner9j(a, b, c, d, e, f, g, h, i)
                        assert abs(got - ref) < 1e-12, (a, b, c, d, e, f, g, h, i, got, ref)
                        n += 1
        if n > 400:
            break
    assert n > 400


def test_wigner_argument_errors_are_status_codes():
    with pytest.raises(c2g.Chemps2Error):
        c2g.wigner6j(-1, 1, 0, 1, 1, 0)


def test_hamiltonian_symmetry_and_checks():
    L = 4
    ham = c2g.Hamiltonian(L, 5, np.array([0, 1, 2, 3], dtype=np.int32))  # C2v
    ham.setVmat(0, 1, 0, 1, 0.3)
    for perm in [(0, 1, 0, 1), (1, 0, 1, 0), (0, 1, 0, 1)]:
        assert ham.getVmat(*perm) == 0.3
    ham.setVmat(0, 1, 2, 3, 0.2)  # I0 x I1 = 1 = I2 x I3
    for p in [(0, 1, 2, 3), (2, 1, 0, 3), (0, 3, 2, 1), (2, 3, 0, 1), (1, 0, 3, 2), (3, 0, 1, 2), (1, 2, 3, 0),
              (3, 2, 1, 0)]:
        assert ham.getVmat(*p) == 0.2
    with pytest.raises(c2g.Chemps2Error):
        ham.setTmat(0, 1, 1.0)  # different irreps
    with pytest.raises(c2g.Chemps2Error):
        ham.setVmat(0, 0, 0, 1, 1.0)  # irrep product violated
    with pytest.raises(c2g.Chemps2Error):
        ham.getTmat(0, L)


def test_problem_matrix_elements_and_reorder():
    L = 4
    ham = c2g.Hamiltonian(L, 0, np.zeros(L, dtype=np.int32))
    ham.setTmat(0, 1, -1.0)
    ham.setVmat(2, 2, 2, 2, 4.0)
    prob = c2g.Problem(ham, 0, 4, 0)
    with pytest.raises(c2g.Chemps2Error):
        prob.gMxElement(0, 0, 0, 0)  # not yet constructed
    prob.construct_mxelem()
    # h_abcd = V_abcd + (delta_ac T_bd + delta_bd T_ac) / (N - 1)
    assert prob.gMxElement(0, 0, 0, 1) == pytest.approx(-1.0 / 3)
    assert prob.gMxElement(2, 2, 2, 2) == pytest.approx(4.0)
    prob.setMxElement(0, 1, 2, 3, 0.5)
    assert prob.gMxElement(0, 1, 2, 3) == 0.5
    assert prob.checkConsistency()
    bad = c2g.Problem(ham, 1, 4, 0)  # odd spin with even N
    assert not bad.checkConsistency()


def test_convergence_scheme_checks():
    sc = c2g.ConvergenceScheme(2)
    sc.set_instruction(0, 100, 1e-8, 2, 0.1, 1e-5)
    sc.setInstruction(1, 200, 1e-9, 3, 0.0)
    assert sc.getDavidsonRTOL(1) == 1e-5
    for bad in [(0, 0, 1e-8, 2, 0.0, 1e-5), (0, 10, 0.0, 2, 0.0, 1e-5), (0, 10, 1e-8, 0, 0.0, 1e-5),
                (0, 10, 1e-8, 2, 0.0, 0.0), (5, 10, 1e-8, 2, 0.0, 1e-5)]:
        with pytest.raises(c2g.Chemps2Error):
            sc.set_instruction(*bad)
    with pytest.raises(c2g.Chemps2Error):
        c2g.ConvergenceScheme(0)


def test_private_random_stream_equals_srand_rand():
    """A batch member's private generator gives the C library's srand(seed); rand()
    sequence, so a batch reproduces the random starts of sequential runs."""
    libc = C.CDLL(None)
    if not hasattr(libc, "gnu_get_libc_version"):
        pytest.skip("not the GNU C library")
    libc.rand.restype = C.c_int
    for seed in (0, 1, 7, 12345, 2**31 - 1, 2**31, 4000000000):
        ours = c2g.host_rand_sample(seed, 5000)
        libc.srand(C.c_uint(seed))
        theirs = np.array([libc.rand() for _ in range(5000)], dtype=np.int32)
        assert np.array_equal(ours, theirs), seed


def test_batch_argument_errors_are_status_codes():
    lib = c2g.load()
    with pytest.raises(c2g.Chemps2Error):
        c2g._check(lib.c2g_batch_solve(-1, None, None, None, 1, None, None, None, None, None))
    with pytest.raises(c2g.Chemps2Error):
        c2g._check(lib.c2g_batch_solve(2, None, None, None, 1, None, None, None, None, None))
    assert lib.c2g_batch_solve(0, None, None, None, 4, None, None, None, None, None) == 0
    with pytest.raises(ValueError):
        c2g.solve_batch([], [None], [])


def test_batch_without_device_reports_each_problem():
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    ham = c2g.Hamiltonian(4, 0, np.zeros(4, dtype=np.int32))
    probs = [c2g.Problem(ham, 0, 4, 0) for _ in range(3)]
    sc = c2g.ConvergenceScheme(1)
    sc.set_instruction(0, 10, 1e-8, 1, 0.0, 1e-6)
    with pytest.raises(c2g.NoDeviceError):
        c2g.solve_batch(probs, [sc] * 3, [1, 2, 3], workers=2)
    with pytest.raises(c2g.Chemps2Error):
        c2g.solve_batch([probs[0], probs[0]], [sc, sc], [1, 2])  # a Problem twice


def test_batching_workload_generator():
    """The seeded problem set of the batching form: 64 problems, half Hubbard and half
    synthetic ab initio, L in 8..20, N = L, D from the four bond dimensions, spins that the
    electron count allows, identical on every call."""
    from chemps2_gb300.models import BATCH_BOND_DIMS, batch_members

    a = batch_members(64)
    b = batch_members(64)
    assert len(a) == 64
    assert sum(m["kind"] == "hubbard" for m in a) == 32
    for x, y in zip(a, b):
        assert (x["kind"], x["two_s"], x["n"], x["D"], x["seed"]) == (y["kind"], y["two_s"], y["n"], y["D"], y["seed"])
        assert np.array_equal(x["model"].vmat, y["model"].vmat)
        L = x["model"].L
        assert 8 <= L <= 20 and x["n"] == L
        assert x["D"] in BATCH_BOND_DIMS
        assert x["two_s"] % 2 == L % 2 and x["two_s"] <= 3
        assert x["model"].group == (0 if x["kind"] == "hubbard" else 7)


def test_truncation_eig_argument_errors_are_status_codes():
    lib = c2g.load()
    n = np.array([129], dtype=np.int32)
    buf = np.zeros(129 * 129)
    ev = np.zeros(129)
    with pytest.raises(c2g.Chemps2Error):  # order above 128: refused before any device work
        c2g._check(lib.c2g_truncation_eig(1, n.ctypes.data_as(C.POINTER(C.c_int)), c2g._dp(buf), c2g._dp(ev),
                                          c2g._dp(buf)))
    with pytest.raises(c2g.Chemps2Error):
        c2g._check(lib.c2g_truncation_eig(-1, None, None, None, None))
    assert lib.c2g_truncation_eig(0, None, None, None, None) == 0


def test_write_fcidump_round_trip(tmp_path):
    """Hamiltonian::writeFCIDUMP (CheMPS2/Hamiltonian.cpp:539-582) then the FCIDUMP reader
    give back every integral and the constant exactly (17 significant digits are
    written), for a synthetic D2h Hamiltonian and for the reference's N2 STO-3G file;
    the header carries NELEC, MS2 and the target irrep in Molpro numbering."""
    from pathlib import Path

    m = models.synthetic_ab_initio(6, 7, 5)
    h = c2g.Hamiltonian(m.L, m.group, m.irreps)
    for i in range(m.L):
        for j in range(i, m.L):
            if m.irreps[i] == m.irreps[j]:
                h.setTmat(i, j, float(m.tmat[i, j]))
    for i, j, k, l in np.argwhere(m.vmat != 0.0):
        h.setVmat(int(i), int(j), int(k), int(l), float(m.vmat[i, j, k, l]))
    h.setEconst(1.25)
    golden = Path(__file__).parent / "golden" / "N2.STO3G.FCIDUMP"
    for ham, group, name in ((h, 7, "synthetic"), (c2g.Hamiltonian(0, 7, [], filename=str(golden)), 7, "n2")):
        path = tmp_path / f"{name}.FCIDUMP"
        ham.writeFCIDUMP(str(path), 6, 0, 0)
        back = c2g.Hamiltonian(0, group, [], filename=str(path))
        L = ham.getL()
        assert back.getL() == L and back.getEconst() == ham.getEconst()
        assert all(back.getOrbitalIrrep(i) == ham.getOrbitalIrrep(i) for i in range(L))
        for i in range(L):
            for j in range(L):
                assert back.getTmat(i, j) == ham.getTmat(i, j)
                for k in range(L):
                    for l in range(L):
                        assert back.getVmat(i, j, k, l) == ham.getVmat(i, j, k, l), (name, i, j, k, l)
        head = path.read_text().splitlines()[:3]
        assert "NORB= %d" % L in head[0] and "NELEC= 6" in head[0] and "MS2= 0" in head[0]
        assert head[2].strip() == "ISYM=1,"


def test_check_rohf_occ():
    """Problem::check_rohf_occ (CheMPS2/Problem.cpp:422-451): occupations must be 0, 1, 2
    and give N, 2S (open shells high-spin) and the irrep of the targeted sector."""
    h = c2g.Hamiltonian(4, 5, np.array([0, 1, 2, 3], dtype=np.int32))
    p = c2g.Problem(h, 0, 4, 0)
    assert p.check_rohf_occ([2, 2, 0, 0])
    assert not p.check_rohf_occ([2, 1, 1, 0])  # 2S = 2
    p3 = c2g.Problem(h, 2, 4, 3)
    assert p3.check_rohf_occ([2, 1, 1, 0])  # irreps 1 x 2 = 3
    assert not p3.check_rohf_occ([2, 1, 0, 1])  # irreps 1 x 3 = 2
    assert not p.check_rohf_occ([3, 1, 0, 0])
