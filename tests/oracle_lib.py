"""ctypes wrapper of the CPU oracle (oracle/_build/liboracle.so): CPU DMRG sweep and
determinant FCI. Test infrastructure only."""
from __future__ import annotations

import ctypes as C
import sys
from pathlib import Path

import numpy as np

from models import Model, hubbard  # noqa: F401

ROOT = Path(__file__).resolve().parents[1]
_lib = None


def lib():
    global _lib
    if _lib is None:
        sys.path.insert(0, str(ROOT))
        from oracle import build as ob  # noqa: E402

        path = ob.build()
        _lib = C.CDLL(str(path), mode=C.RTLD_GLOBAL)
        _lib.oracle_last_error.restype = C.c_char_p
        _lib.oracle_fci_last_error.restype = C.c_char_p
    return _lib


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int))


def fci_energy(model: Model, n_up: int, n_down: int, irrep: int, tol=1e-10) -> float:
    e = C.c_double()
    dim = C.c_int64()
    rc = lib().oracle_fci_ground_state(model.L, _ip(model.irreps), _dp(model.tflat()), _dp(model.vflat()),
                                       C.c_double(model.econst), n_up, n_down, irrep, C.c_double(tol), 400,
                                       C.byref(e), C.byref(dim))
    if rc != 0:
        raise RuntimeError(lib().oracle_fci_last_error().decode())
    return e.value


def fci_2rdm(model: Model, n_up: int, n_down: int, irrep: int, tol=1e-11):
    """FCI ground state energy and its spin-summed 2-RDMs A, B as [a, b, c, d] arrays."""
    L = model.L
    e = C.c_double()
    dim = C.c_int64()
    A = np.zeros(L ** 4)
    B = np.zeros(L ** 4)
    rc = lib().oracle_fci_state(L, _ip(model.irreps), _dp(model.tflat()), _dp(model.vflat()), C.c_double(model.econst),
                                n_up, n_down, irrep, C.c_double(tol), 600, C.byref(e), C.byref(dim), _dp(A), _dp(B))
    if rc != 0:
        raise RuntimeError(lib().oracle_fci_last_error().decode())
    return e.value, A.reshape((L, L, L, L), order="F"), B.reshape((L, L, L, L), order="F")


def fci_mutual_information(model: Model, n_up: int, n_down: int, irrep: int, tol=1e-11, jw=False):
    """FCI energy, single-orbital entropies [L] and mutual information [L, L]; jw: with the
    parity string of the orbitals between the pair (fermionic RDM), otherwise the
    tensor-product partial trace of the reference's definition."""
    L = model.L
    e = C.c_double()
    s1 = np.zeros(L)
    mi = np.zeros(L * L)
    rc = lib().oracle_fci_mutual_information(L, _ip(model.irreps), _dp(model.tflat()), _dp(model.vflat()),
                                             C.c_double(model.econst), n_up, n_down, irrep, C.c_double(tol), 600,
                                             int(bool(jw)), C.byref(e), _dp(s1), _dp(mi))
    if rc != 0:
        raise RuntimeError(lib().oracle_fci_last_error().decode())
    return e.value, s1, mi.reshape((L, L), order="F")


class OracleDMRG:
    """CPU DMRG of the oracle. schedule: list of (D, econv, max_sweeps, noise, rtol)."""

    def __init__(self, model: Model | None, two_s, n, irrep, schedule, reorder=0, fcidump=None, group=None,
                 check=True, dims=None, left_upto=-1):
        """dims: rows (boundary, N, 2S, I, dim) replacing the scaled sector dimensions (the
        state then has those dimensions, random tensors); left_upto: build the left operators
        of the first left_upto boundaries only (-1: all)."""
        L = lib()
        if dims is not None:
            rows = np.ascontiguousarray(np.asarray(dims, dtype=np.int32).reshape(-1, 5))
            tf, vf = model.tflat(), model.vflat()
            self._keep = (rows, tf, vf)
            h = C.c_void_p()
            rc = L.oracle_dmrg_create_dims(model.L, model.group, _ip(model.irreps), _dp(tf), _dp(vf),
                                           C.c_double(model.econst), two_s, n, irrep, int(schedule[0][0]),
                                           len(rows), _ip(rows), int(left_upto), C.byref(h))
            if rc != 0:
                raise RuntimeError(L.oracle_last_error().decode())
            self.h = h
            return
        D = np.array([s[0] for s in schedule], dtype=np.int32)
        ec = np.array([s[1] for s in schedule], dtype=np.float64)
        ms = np.array([s[2] for s in schedule], dtype=np.int32)
        nz = np.array([s[3] for s in schedule], dtype=np.float64)
        rt = np.array([s[4] for s in schedule], dtype=np.float64)
        h = C.c_void_p()
        self._keep = (D, ec, ms, nz, rt)
        if fcidump is not None:
            rc = L.oracle_dmrg_create(str(fcidump).encode(), 0, int(group), None, None, None, C.c_double(0.0),
                                      two_s, n, irrep, reorder, len(schedule), _ip(D), _dp(ec), _ip(ms), _dp(nz),
                                      _dp(rt), int(check), C.byref(h))
        else:
            tf, vf = model.tflat(), model.vflat()
            self._keep += (tf, vf)
            rc = L.oracle_dmrg_create(None, model.L, model.group, _ip(model.irreps), _dp(tf), _dp(vf),
                                      C.c_double(model.econst), two_s, n, irrep, reorder, len(schedule), _ip(D),
                                      _dp(ec), _ip(ms), _dp(nz), _dp(rt), int(check), C.byref(h))
        if rc != 0:
            raise RuntimeError(L.oracle_last_error().decode())
        self.h = h

    def _check(self, rc):
        if rc != 0:
            raise RuntimeError(lib().oracle_last_error().decode())

    def solve(self) -> float:
        e = C.c_double()
        self._check(lib().oracle_dmrg_solve(self.h, C.byref(e)))
        return e.value

    def presolve(self):
        self._check(lib().oracle_dmrg_presolve(self.h))

    def set_mx_element(self, a, b, c, d, v):
        self._check(lib().oracle_set_mx_element(self.h, a, b, c, d, C.c_double(v)))

    def step_energies(self):
        n = C.c_int()
        self._check(lib().oracle_dmrg_step_energies(self.h, None, 0, C.byref(n)))
        out = np.zeros(n.value)
        self._check(lib().oracle_dmrg_step_energies(self.h, _dp(out), n.value, C.byref(n)))
        return out

    def sobject_size(self, index):
        n = C.c_int64()
        self._check(lib().oracle_dmrg_sobject_size(self.h, index, C.byref(n)))
        return n.value

    def heff_apply(self, index, x=None, want_diag=False):
        n = self.sobject_size(index)
        join = x is None
        xx = np.zeros(n) if join else np.ascontiguousarray(x, dtype=np.float64).copy()
        y = np.zeros(n)
        d = np.zeros(n) if want_diag else None
        self._check(lib().oracle_dmrg_heff_apply(self.h, index, int(join), _dp(xx), C.c_int64(len(xx)), _dp(y),
                                                 _dp(d) if d is not None else None))
        return xx, y, d

    def solve_site(self, index, rtol, noise, D, moving_right, change):
        e = C.c_double()
        self._check(lib().oracle_dmrg_solve_site(self.h, index, C.c_double(rtol), C.c_double(noise), D,
                                                 int(moving_right), int(change), C.byref(e)))
        return e.value

    def update(self, index, moving_right):
        self._check(lib().oracle_dmrg_update(self.h, index, int(moving_right)))

    def get_mps(self, site):
        n = C.c_int64()
        self._check(lib().oracle_dmrg_get_mps(self.h, int(site), None, C.c_int64(0), C.byref(n)))
        out = np.zeros(n.value)
        self._check(lib().oracle_dmrg_get_mps(self.h, int(site), _dp(out), C.c_int64(n.value), C.byref(n)))
        return out

    def calc_2dm(self):
        """The 2-RDM pass on the CPU executor: (A, B, trace, energy), A and B as L^4 arrays
        indexed [a, b, c, d] in DMRG orbital order."""
        nl = C.c_int()
        self._check(lib().oracle_dmrg_num_orbitals(self.h, C.byref(nl)))
        L = nl.value
        A = np.zeros(L ** 4)
        B = np.zeros(L ** 4)
        tr, en = C.c_double(), C.c_double()
        self._check(lib().oracle_dmrg_calc_2dm(self.h, _dp(A), _dp(B), C.byref(tr), C.byref(en)))
        return A.reshape((L,) * 4, order="F"), B.reshape((L,) * 4, order="F"), tr.value, en.value

    def calc_correlations(self):
        """The correlation pass after calc_2dm: (mutual information L x L, single-orbital
        entropies), DMRG orbital order."""
        nl = C.c_int()
        self._check(lib().oracle_dmrg_num_orbitals(self.h, C.byref(nl)))
        L = nl.value
        mi = np.zeros(L * L)
        s1 = np.zeros(L)
        self._check(lib().oracle_dmrg_calc_correlations(self.h, _dp(mi), _dp(s1)))
        return mi.reshape((L, L), order="F"), s1

    def fci_coefficient(self, alpha, beta):
        """DMRG::getFCIcoefficient of the oracle's MPS (the product's host routine)."""
        a = np.ascontiguousarray(alpha, dtype=np.int32)
        b = np.ascontiguousarray(beta, dtype=np.int32)
        v = C.c_double()
        self._check(lib().oracle_dmrg_fci_coefficient(self.h, _ip(a), _ip(b), C.byref(v)))
        return v.value

    def gauge(self, site, right):
        """Left-normalise `site` (R into site + 1) or, with right, right-normalise it (L into
        site - 1), with the product's host gauge routines."""
        self._check(lib().oracle_dmrg_gauge(self.h, int(site), 1 if right else 0))

    def sectors(self, boundary):
        n = C.c_int()
        self._check(lib().oracle_dmrg_sectors(self.h, int(boundary), None, 0, C.byref(n)))
        out = np.zeros((max(n.value, 1), 5), dtype=np.int32)
        self._check(lib().oracle_dmrg_sectors(self.h, int(boundary), _ip(out), n.value, C.byref(n)))
        return out[:n.value]

    def stats(self):
        out = np.zeros(3)
        self._check(lib().oracle_dmrg_stats(self.h, _dp(out)))
        return {"n_matvec": out[0], "t_matvec": out[1], "flops": out[2]}

    def __del__(self):
        try:
            if getattr(self, "h", None):
                lib().oracle_dmrg_destroy(self.h)
        except Exception:
            pass


def fcidump_model(path, group) -> Model:
    """The Hamiltonian of an FCIDUMP file (read by the product's reader, whose conversions
    the N2 golden pins) as a Model for the determinant FCI."""
    import chemps2_gb300 as c2g

    ham = c2g.Hamiltonian(0, int(group), [], filename=str(path))
    L = ham.getL()
    irreps = np.array([ham.getOrbitalIrrep(i) for i in range(L)], dtype=np.int32)
    T = np.array([[ham.getTmat(i, j) for j in range(L)] for i in range(L)])
    V = np.zeros((L, L, L, L))
    for i in range(L):
        for j in range(L):
            for k in range(L):
                for l in range(L):
                    V[i, j, k, l] = ham.getVmat(i, j, k, l)
    return Model(L, int(group), irreps, T, V, ham.getEconst())


def set_threads(n: int):
    """Host threads of the oracle's task-program executor (results do not depend on it)."""
    lib().oracle_set_threads(int(n))


def srand(seed: int):
    C.CDLL(None).srand(C.c_uint(seed))
