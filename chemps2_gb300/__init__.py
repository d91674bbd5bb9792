"""GB300 implementation of CheMPS2's two-site DMRG sweep.

Python mirror of the reference's Python interface (PyCheMPS2/PyCheMPS2.pyx:47-188):
Hamiltonian, Problem, ConvergenceScheme and DMRG with the same method names, bound with
ctypes to the C-ABI of libchemps2_gb300.so (include/chemps2_gb300.h). The library is built
in-tree by chemps2_gb300.build; the DMRG object runs only on a CUDA device and raises
NoDeviceError when there is none.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

_PKG = Path(__file__).resolve().parent
_LIB = None

C2G_OK = 0
C2G_ERR_INVALID = -1
C2G_ERR_CUDA = -2
C2G_ERR_NO_DEVICE = -3
C2G_ERR_INTERNAL = -4
C2G_ERR_OTHER = -5
NUM_STATS = 13
STAT_NAMES = ("n_matvec", "n_davidson", "t_join", "t_solve", "t_split", "t_update", "t_matvec", "t_compile",
              "matvec_flops", "matvec_bytes", "last_energy", "n_matvec_fp32", "t_upload")


class Chemps2Error(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"[{code}] {msg}")
        self.code = code


class NoDeviceError(Chemps2Error):
    pass


def library_path() -> Path:
    return _PKG / "_lib" / "libchemps2_gb300.so"


def load(build_if_missing: bool = True):
    """Loads the native library (building it first when it is missing)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = library_path()
    if not path.exists():
        if not build_if_missing:
            raise FileNotFoundError(f"{path} is missing; run chemps2_gb300.build.build()")
        from . import build as _build

        _build.build()
    lib = C.CDLL(str(path))
    lib.c2g_last_error.restype = C.c_char_p
    _LIB = lib
    return lib


def _check(rc):
    if rc != C2G_OK:
        msg = load().c2g_last_error().decode(errors="replace")
        if rc == C2G_ERR_NO_DEVICE:
            raise NoDeviceError(rc, msg)
        raise Chemps2Error(rc, msg)


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int))


def srand(seed: int) -> None:
    """Seeds the generator of the random initial MPS, Davidson fallback guess and noise."""
    _check(load().c2g_srand(C.c_uint(seed)))


def kernel_launches() -> int:
    n = C.c_longlong()
    _check(load().c2g_kernel_launches(C.byref(n)))
    return n.value


def wigner3j(ja, jb, jc, ma, mb, mc) -> float:
    """3j symbol (ja jb jc; ma mb mc), arguments twice the spins and projections."""
    v = C.c_double()
    _check(load().c2g_wigner3j(ja, jb, jc, ma, mb, mc, C.byref(v)))
    return v.value


def wigner6j(a, b, c, d, e, f) -> float:
    v = C.c_double()
    _check(load().c2g_wigner6j(a, b, c, d, e, f, C.byref(v)))
    return v.value


def wigner9j(a, b, c, d, e, f, g, h, i) -> float:
    v = C.c_double()
    _check(load().c2g_wigner9j(a, b, c, d, e, f, g, h, i, C.byref(v)))
    return v.value


class Hamiltonian:
    """CheMPS2::Hamiltonian (PyHamiltonian): Hamiltonian(L, group, irreps) or
    Hamiltonian(L, group, irreps, filename=fcidump)."""

    def __init__(self, Norbitals, nGroup, OrbIrreps, filename="none"):
        self._h = C.c_void_p()
        lib = load()
        if filename and filename != "none":
            _check(lib.c2g_hamiltonian_create_fcidump(str(filename).encode(), int(nGroup), C.byref(self._h)))
        else:
            irr = np.ascontiguousarray(OrbIrreps, dtype=np.int32)
            if irr.size != Norbitals:
                raise ValueError("one irrep per orbital is required")
            _check(lib.c2g_hamiltonian_create(int(Norbitals), int(nGroup), irr.ctypes.data_as(C.POINTER(C.c_int)),
                                              C.byref(self._h)))

    def __del__(self):
        if getattr(self, "_h", None) and _LIB is not None:
            _LIB.c2g_hamiltonian_destroy(self._h)
            self._h = None

    def getL(self):
        v = C.c_int()
        _check(load().c2g_hamiltonian_get_L(self._h, C.byref(v)))
        return v.value

    def getNGroup(self):
        v = C.c_int()
        _check(load().c2g_hamiltonian_get_group(self._h, C.byref(v)))
        return v.value

    def getOrbitalIrrep(self, orb):
        v = C.c_int()
        _check(load().c2g_hamiltonian_get_irrep(self._h, int(orb), C.byref(v)))
        return v.value

    def setEconst(self, value):
        _check(load().c2g_hamiltonian_set_econst(self._h, C.c_double(value)))

    def getEconst(self):
        v = C.c_double()
        _check(load().c2g_hamiltonian_get_econst(self._h, C.byref(v)))
        return v.value

    def setTmat(self, i, j, value):
        _check(load().c2g_hamiltonian_set_tmat(self._h, int(i), int(j), C.c_double(value)))

    def getTmat(self, i, j):
        v = C.c_double()
        _check(load().c2g_hamiltonian_get_tmat(self._h, int(i), int(j), C.byref(v)))
        return v.value

    def setVmat(self, i, j, k, l, value):
        _check(load().c2g_hamiltonian_set_vmat(self._h, int(i), int(j), int(k), int(l), C.c_double(value)))

    def getVmat(self, i, j, k, l):
        v = C.c_double()
        _check(load().c2g_hamiltonian_get_vmat(self._h, int(i), int(j), int(k), int(l), C.byref(v)))
        return v.value

    def writeFCIDUMP(self, filename, Nelec, TwoS, TargetIrrep):
        """Hamiltonian::writeFCIDUMP: this Hamiltonian as an FCIDUMP file."""
        _check(load().c2g_hamiltonian_write_fcidump(self._h, str(filename).encode(), int(Nelec), int(TwoS),
                                                    int(TargetIrrep)))


class Problem:
    """CheMPS2::Problem (PyProblem)."""

    def __init__(self, Hami: Hamiltonian, TwoS, N, Irrep):
        self._ham = Hami  # the Hamiltonian must outlive the Problem
        self._p = C.c_void_p()
        _check(load().c2g_problem_create(Hami._h, int(TwoS), int(N), int(Irrep), C.byref(self._p)))
        self._TwoS, self._N, self._Irrep = int(TwoS), int(N), int(Irrep)

    def __del__(self):
        if getattr(self, "_p", None) and _LIB is not None:
            _LIB.c2g_problem_destroy(self._p)
            self._p = None

    def gL(self):
        return self._ham.getL()

    def gSy(self):
        return self._ham.getNGroup()

    def gTwoS(self):
        return self._TwoS

    def gN(self):
        return self._N

    def gIrrep(self, orb=None):
        return self._Irrep if orb is None else self._ham.getOrbitalIrrep(orb)

    def gEconst(self):
        return self._ham.getEconst()

    def construct_mxelem(self):
        _check(load().c2g_problem_construct_mxelem(self._p))

    def gMxElement(self, a, b, c, d):
        v = C.c_double()
        _check(load().c2g_problem_get_mx_element(self._p, a, b, c, d, C.byref(v)))
        return v.value

    def setMxElement(self, a, b, c, d, value):
        _check(load().c2g_problem_set_mx_element(self._p, a, b, c, d, C.c_double(value)))

    def SetupReorderD2h(self):
        _check(load().c2g_problem_setup_reorder_d2h(self._p))

    def SetupReorderC2v(self):
        _check(load().c2g_problem_setup_reorder_c2v(self._p))

    def setup_reorder_custom(self, dmrg2ham):
        a = np.ascontiguousarray(dmrg2ham, dtype=np.int32)
        _check(load().c2g_problem_setup_reorder_custom(self._p, a.ctypes.data_as(C.POINTER(C.c_int))))

    def checkConsistency(self):
        v = C.c_int()
        _check(load().c2g_problem_check_consistency(self._p, C.byref(v)))
        return bool(v.value)

    def check_rohf_occ(self, occupancies):
        """Whether occupations 0, 1, 2 of the DMRG sites give the targeted sector
        (Problem::check_rohf_occ)."""
        occ = np.ascontiguousarray(occupancies, dtype=np.int32)
        if occ.size != self.gL():
            raise ValueError("one occupation per orbital")
        v = C.c_int()
        _check(load().c2g_problem_check_rohf_occ(self._p, occ.ctypes.data_as(C.POINTER(C.c_int)), C.byref(v)))
        return bool(v.value)

    def bookkeeper_sectors(self, D, boundary):
        """(N, 2S, I, FCI dim, current dim) of every sector at `boundary` (no GPU needed)."""
        n = C.c_int()
        _check(load().c2g_bookkeeper_sectors(self._p, int(D), int(boundary), None, 0, C.byref(n)))
        out = np.zeros((max(n.value, 1), 5), dtype=np.int32)
        _check(load().c2g_bookkeeper_sectors(self._p, int(D), int(boundary), out.ctypes.data_as(C.POINTER(C.c_int)),
                                             n.value, C.byref(n)))
        return out[: n.value]

    def sobject_layout(self, D, index):
        """Block labels (nkappa x 9), kappa2index and the visiting order of the two-site
        object at sites (index, index + 1) (no GPU needed)."""
        n = C.c_int()
        _check(load().c2g_sobject_layout(self._p, int(D), int(index), None, None, None, 0, C.byref(n)))
        k = n.value
        labels = np.zeros((max(k, 1), 9), dtype=np.int32)
        k2i = np.zeros(k + 1, dtype=np.int64)
        order = np.zeros(max(k, 1), dtype=np.int32)
        _check(load().c2g_sobject_layout(self._p, int(D), int(index), labels.ctypes.data_as(C.POINTER(C.c_int)),
                                         k2i.ctypes.data_as(C.POINTER(C.c_int64)),
                                         order.ctypes.data_as(C.POINTER(C.c_int)), k, C.byref(n)))
        return labels[:k], k2i, order[:k]


class ConvergenceScheme:
    """CheMPS2::ConvergenceScheme (PyConvergenceScheme)."""

    def __init__(self, nInstructions):
        self._s = C.c_void_p()
        _check(load().c2g_scheme_create(int(nInstructions), C.byref(self._s)))
        self._instr = {}

    def __del__(self):
        if getattr(self, "_s", None) and _LIB is not None:
            _LIB.c2g_scheme_destroy(self._s)
            self._s = None

    def set_instruction(self, instruction, D, Econv, nMax, noisePrefactor, dvdson_rtol):
        _check(load().c2g_scheme_set_instruction(self._s, int(instruction), int(D), C.c_double(Econv), int(nMax),
                                                 C.c_double(noisePrefactor), C.c_double(dvdson_rtol)))
        self._instr[instruction] = (D, Econv, nMax, noisePrefactor, dvdson_rtol)

    def setInstruction(self, instruction, D, Econv, nMax, noisePrefactor):
        self.set_instruction(instruction, D, Econv, nMax, noisePrefactor, 1e-5)

    def getD(self, i):
        return self._instr[i][0]

    def getEconv(self, i):
        return self._instr[i][1]

    def getMaxSweeps(self, i):
        return self._instr[i][2]

    def getNoisePrefactor(self, i):
        return self._instr[i][3]

    def getDavidsonRTOL(self, i):
        return self._instr[i][4]


class TwoDM:
    """CheMPS2::TwoDM: the spin-summed 2-RDMs A[a,b,c,d] and B[a,b,c,d] of a DMRG state
    (CheMPS2/include/chemps2/TwoDM.h), as numpy arrays, with trace() and energy()."""

    def __init__(self, A, B, trace, energy):
        self.A, self.B = A, B
        self._trace, self._energy = trace, energy

    def getTwoDMA(self, a, b, c, d):
        return float(self.A[a, b, c, d])

    def getTwoDMB(self, a, b, c, d):
        return float(self.B[a, b, c, d])

    def get1RDM(self, N):
        """1-RDM: sum_r A[a, r, b, r] / (N - 1)."""
        return np.einsum("arbr->ab", self.A) / (N - 1.0)

    def trace(self):
        return self._trace

    def energy(self):
        return self._energy


class DMRG:
    """CheMPS2::DMRG (PyDMRG): the sweep runs on the GPU."""

    def __init__(self, Probl: Problem, OptScheme: ConvergenceScheme, makechkpt=False, tmpfolder="/tmp",
                 occupancies=None):
        self._prob, self._scheme = Probl, OptScheme
        self._L = Probl.gL()
        self._d = C.c_void_p()
        occ = None
        if occupancies is not None:
            occ = np.ascontiguousarray(occupancies, dtype=np.int32)
        _check(load().c2g_dmrg_create_chkpt(Probl._p, OptScheme._s, int(bool(makechkpt)),
                                            occ.ctypes.data_as(C.POINTER(C.c_int)) if occ is not None else None,
                                            C.byref(self._d)))

    def close(self):
        if getattr(self, "_d", None) and _LIB is not None:
            _check(_LIB.c2g_dmrg_destroy(self._d))
            self._d = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def Solve(self):
        e = C.c_double()
        _check(load().c2g_dmrg_solve(self._d, C.byref(e)))
        return e.value

    def PreSolve(self):
        _check(load().c2g_dmrg_presolve(self._d))

    def set_verbose(self, v=True):
        _check(load().c2g_dmrg_set_verbose(self._d, int(bool(v))))

    def get_num_mps_var(self):
        n = C.c_int()
        _check(load().c2g_dmrg_num_mps_var(self._d, C.byref(n)))
        return n.value

    def get_max_discarded_weight(self):
        w = C.c_double()
        _check(load().c2g_dmrg_max_discarded_weight(self._d, C.byref(w)))
        return w.value

    def solve_site(self, index, dvdson_rtol, noise_level, D, moving_right, change):
        e = C.c_double()
        _check(load().c2g_dmrg_solve_site(self._d, int(index), C.c_double(dvdson_rtol), C.c_double(noise_level),
                                          int(D), int(bool(moving_right)), int(bool(change)), C.byref(e)))
        return e.value

    def update(self, index, moving_right):
        _check(load().c2g_dmrg_update(self._d, int(index), int(bool(moving_right))))

    def stats(self):
        out = np.zeros(NUM_STATS)
        _check(load().c2g_dmrg_stats(self._d, _dp(out), NUM_STATS))
        return dict(zip(STAT_NAMES, out.tolist()))

    def reset_stats(self):
        _check(load().c2g_dmrg_reset_stats(self._d))

    def sobject_size(self, index):
        n = C.c_int64()
        _check(load().c2g_dmrg_sobject_size(self._d, int(index), C.byref(n)))
        return n.value

    def heff_apply(self, index, x=None, want_diag=False):
        """y = Heff x at sites (index, index + 1); x None: the joined current state."""
        n = self.sobject_size(index)
        join = x is None
        xx = np.zeros(n) if join else np.ascontiguousarray(x, dtype=np.float64).copy()
        y = np.zeros(n)
        d = np.zeros(n) if want_diag else None
        _check(load().c2g_dmrg_heff_apply(self._d, int(index), int(join), _dp(xx), _dp(y),
                                          _dp(d) if d is not None else None, C.c_int64(n)))
        return xx, y, d

    def heff_apply_fp32(self, index, x):
        """y = Heff x with FP32 arithmetic (FP64 operands and output)."""
        xx = np.ascontiguousarray(x, dtype=np.float64).copy()
        y = np.zeros_like(xx)
        _check(load().c2g_dmrg_heff_apply_fp32(self._d, int(index), _dp(xx), _dp(y), C.c_int64(xx.size)))
        return y

    def heff_apply_precision(self, index, x, precision="tc"):
        """y = Heff x with the matvec arithmetic 'fp64', 'fp32' or 'tc' (large blocks on the
        tensor cores as split-BF16 products, the rest FP32)."""
        xx = np.ascontiguousarray(x, dtype=np.float64).copy()
        y = np.zeros_like(xx)
        _check(load().c2g_dmrg_heff_apply_precision(self._d, int(index), _dp(xx), _dp(y), C.c_int64(xx.size),
                                                    int(PRECISION_CODES[precision])))
        return y

    def loadedMPS(self):
        """True when the MPS was loaded from a checkpoint file (makechkpt)."""
        v = C.c_int()
        _check(load().c2g_dmrg_loaded_mps(self._d, C.byref(v)))
        return bool(v.value)

    def deleteStoredMPS(self):
        """DMRG::deleteStoredMPS: remove the checkpoint files of this working directory."""
        _check(load().c2g_dmrg_delete_stored_mps(self._d))

    def activateExcitations(self, maxExcIn):
        """DMRG::activateExcitations: allow up to maxExcIn stored lower states."""
        _check(load().c2g_dmrg_activate_excitations(self._d, int(maxExcIn)))

    def newExcitation(self, EshiftIn):
        """DMRG::newExcitation: store the current state; Solve() then targets the next one."""
        _check(load().c2g_dmrg_new_excitation(self._d, C.c_double(EshiftIn)))

    def calc2DMandCorrelations(self):
        """The two-particle density matrices of the current state (DMRG::calc2DMandCorrelations)."""
        _check(load().c2g_dmrg_calc_2dm(self._d))

    def get2DM(self, ham_order=False):
        """(A, B) 2-RDMs as L x L x L x L arrays indexed [a, b, c, d] (DMRG orbital order unless
        ham_order), plus trace and energy: TwoDM.getTwoDMA_DMRG etc."""
        L = self._L
        A = np.zeros(L ** 4)
        B = np.zeros(L ** 4)
        _check(load().c2g_dmrg_get_2dm(self._d, int(bool(ham_order)), _dp(A), _dp(B)))
        tr, en = C.c_double(), C.c_double()
        _check(load().c2g_dmrg_2dm_trace_energy(self._d, C.byref(tr), C.byref(en)))
        # element (a,b,c,d) at a + L*(b + L*(c + L*d)): Fortran order
        return TwoDM(A.reshape((L, L, L, L), order="F"), B.reshape((L, L, L, L), order="F"), tr.value, en.value)

    # PyDMRG's element accessors (PyCheMPS2/PyCheMPS2.pyx:141-178), Hamiltonian orbital
    # order as there; each reads the arrays of the last calc2DMandCorrelations.
    def calc_rdms_and_correlations(self, do_3rdm=False):
        """DMRG::calc_rdms_and_correlations: the 2-RDM and correlations; the 3-RDM is not
        built here, so do_3rdm must be False."""
        if do_3rdm:
            raise NotImplementedError("the 3-RDM is not available in this implementation")
        self.calc2DMandCorrelations()

    def deleteStoredOperators(self):
        """The renormalized operators live in device memory, never on disk: nothing to
        delete (PyDMRG.deleteStoredOperators)."""

    def get2DMA(self, i1, i2, i3, i4):
        return self.get2DM(ham_order=True).getTwoDMA(i1, i2, i3, i4)

    def get2DMB(self, i1, i2, i3, i4):
        return self.get2DM(ham_order=True).getTwoDMB(i1, i2, i3, i4)

    def get2DMenergy(self):
        return self.get2DM().energy()

    def getDoubleTrace2DMA(self):
        return self.get2DM().trace()

    def getCspin(self, row, col):
        return float(self.getCorrelations(ham_order=True)["Cspin"][row, col])

    def getCdens(self, row, col):
        return float(self.getCorrelations(ham_order=True)["Cdens"][row, col])

    def getCspinflip(self, row, col):
        return float(self.getCorrelations(ham_order=True)["Cspinflip"][row, col])

    def getCdirad(self, row, col):
        return float(self.getCorrelations(ham_order=True)["Cdirad"][row, col])

    def getMutInfo(self, row, col):
        return float(self.getCorrelations(ham_order=True)["MutInfo"][row, col])

    def getSingleOrbEntropy(self, index):
        return float(self.getCorrelations(ham_order=True)["SingleOrbitalEntropy"][index])

    def getMutInfoDistance(self, power):
        """sum_{r != c} I(r, c) |r - c|^power over the DMRG chain order
        (CheMPS2/Correlations.cpp:188-201)."""
        mi = self.getCorrelations(ham_order=False)["MutInfo"]
        L = mi.shape[0]
        r, c = np.meshgrid(np.arange(L), np.arange(L), indexing="ij")
        mask = r != c
        return float(np.sum(mi[mask] * np.abs(r - c)[mask].astype(float) ** power))

    def getCorrelations(self, ham_order=False):
        """Correlation tables and mutual information (CheMPS2::Correlations) as a dict of
        L x L arrays [row, col] plus the single-orbital entropies."""
        L = self._L
        arrs = {k: np.zeros(L * L) for k in ("Cspin", "Cdens", "Cspinflip", "Cdirad", "MutInfo")}
        ent = np.zeros(L)
        _check(load().c2g_dmrg_get_correlations(self._d, int(bool(ham_order)), _dp(arrs["Cspin"]), _dp(arrs["Cdens"]),
                                                _dp(arrs["Cspinflip"]), _dp(arrs["Cdirad"]), _dp(arrs["MutInfo"]),
                                                _dp(ent)))
        out = {k: v.reshape((L, L), order="F") for k, v in arrs.items()}
        out["SingleOrbitalEntropy"] = ent
        return out

    def sectors(self, boundary):
        """Rows (N, 2S, I, FCI dim, current dim) of the object's bookkeeper at `boundary`."""
        n = C.c_int()
        _check(load().c2g_dmrg_sectors(self._d, int(boundary), None, 0, C.byref(n)))
        out = np.zeros((max(n.value, 1), 5), dtype=np.int32)
        _check(load().c2g_dmrg_sectors(self._d, int(boundary), out.ctypes.data_as(C.POINTER(C.c_int)), n.value,
                                       C.byref(n)))
        return out[:n.value]

    def get_mps(self, site):
        """The current MPS tensor of `site` (TensorT storage order) as a host array."""
        n = C.c_int64()
        _check(load().c2g_dmrg_get_mps(self._d, int(site), None, C.c_int64(0), C.byref(n)))
        out = np.zeros(n.value)
        _check(load().c2g_dmrg_get_mps(self._d, int(site), _dp(out), C.c_int64(n.value), C.byref(n)))
        return out

    def getFCIcoefficient(self, alpha, beta):
        """The coefficient of the determinant with up occupations alpha[h] and down
        occupations beta[h] (0 or 1) of the Hamiltonian orbitals (PyDMRG.getFCIcoefficient;
        0 outside the targeted sector)."""
        a = np.ascontiguousarray(alpha, dtype=np.int32)
        b = np.ascontiguousarray(beta, dtype=np.int32)
        if a.size != b.size:
            raise ValueError("alpha and beta differ in length")
        v = C.c_double()
        _check(load().c2g_dmrg_fci_coefficient(self._d, _ip(a), _ip(b), C.byref(v)))
        return v.value

    def getSpecificCoefficient(self, coeff):
        """The coefficient of the determinant with occupations coeff[h] in {0, 1, 2} (1: one
        up electron), DMRG::getSpecificCoefficient."""
        c = np.asarray(coeff, dtype=np.int32)
        if np.any((c < 0) | (c > 2)):
            raise ValueError("occupations must be 0, 1 or 2")
        return self.getFCIcoefficient((c >= 1).astype(np.int32), (c == 2).astype(np.int32))

    def step_energies(self):
        """Energies of every two-site step Solve() has run, in order."""
        n = C.c_int()
        _check(load().c2g_dmrg_step_energies(self._d, None, 0, C.byref(n)))
        out = np.zeros(n.value)
        _check(load().c2g_dmrg_step_energies(self._d, _dp(out), n.value, C.byref(n)))
        return out

    def heff_apply_noalloc(self, index, x):
        """y = Heff x (FP64) with no device allocation, for callers that cannot allocate
        device memory while they run: x and y are staged through the library's one
        file-scope device array (two-site objects of at most 1 048 544 doubles). Needs a
        prior heff_apply at this index and state. Calls that overlap on the GPU race for
        the array; calls made one after another are safe."""
        xx = np.ascontiguousarray(x, dtype=np.float64)
        y = np.zeros_like(xx)
        _check(load().c2g_dmrg_heff_apply_noalloc(self._d, int(index), _dp(xx), _dp(y), C.c_int64(xx.size)))
        return y

    def heff_apply_device(self, index, x_ptr, y_ptr, n, precision="fp64", stream=0):
        """y = Heff x on device buffers given as integer addresses (e.g. torch's data_ptr())
        of n doubles; `stream` an integer cudaStream_t (0: synchronous)."""
        p = PRECISION_CODES[precision] if isinstance(precision, str) else int(precision)
        _check(load().c2g_dmrg_heff_apply_device(self._d, int(index), C.c_void_p(int(x_ptr)), C.c_void_p(int(y_ptr)),
                                                 C.c_int64(int(n)), int(p), C.c_void_p(int(stream) or None)))

    def set_precision(self, mode="fp64", mixed_tol=1e-5):
        """'fp64' (the reference's arithmetic), 'mixed' (FP32 Davidson expansion, FP64
        refinement) or 'mixed_tc' (as 'mixed', the large blocks of the reduced-precision
        matvecs on the tensor cores as split-BF16 products)."""
        m = {"fp64": 0, "mixed": 1, "mixed_tc": 2}[mode] if isinstance(mode, str) else int(mode)
        _check(load().c2g_dmrg_set_precision(self._d, m, C.c_double(mixed_tol)))

    def bench_heff(self, index, warmup, steps, flush_bytes=0, precision="fp64"):
        ms, fl, by = C.c_double(), C.c_double(), C.c_double()
        nl = C.c_longlong()
        p = PRECISION_CODES[precision]
        _check(load().c2g_dmrg_bench_heff(self._d, int(index), int(warmup), int(steps), C.c_longlong(flush_bytes),
                                          int(p), C.byref(ms), C.byref(fl), C.byref(by), C.byref(nl)))
        return {"ms_per_matvec": ms.value, "flops": fl.value, "bytes": by.value, "launches": nl.value}


# matvec arithmetic codes of the C-ABI
PRECISION_CODES = {"fp64": 0, "fp32": 1, "mixed": 1, "tc": 2, "mixed_tc": 2}


def solve_batch(problems, schemes, seeds, workers=8, raise_on_error=True):
    """Solves independent problems on one GPU (no counterpart in the reference, whose
    callers loop over problems): problems[i] with schemes[i] and the random start that
    srand(seeds[i]) gives, at most `workers` at a time, each on its own host thread and CUDA
    stream. Returns one dict per problem with its energy, matvec count, seconds and status
    (0 or the C-ABI error code). When a problem failed, all others are still solved; the
    call then raises unless raise_on_error is False."""
    n = len(problems)
    if len(schemes) != n or len(seeds) != n:
        raise ValueError("problems, schemes and seeds differ in length")
    P = (C.c_void_p * max(n, 1))(*[p._p.value for p in problems])
    S = (C.c_void_p * max(n, 1))(*[s._s.value for s in schemes])
    sd = np.ascontiguousarray(seeds, dtype=np.uint32)
    energies = np.zeros(n)
    matvecs = np.zeros(n, dtype=np.int64)
    seconds = np.zeros(n)
    statuses = np.zeros(n, dtype=np.int32)
    stats = np.zeros((max(n, 1), NUM_STATS))
    rc = load().c2g_batch_solve(int(n), P, S, sd.ctypes.data_as(C.POINTER(C.c_uint)), int(workers), _dp(energies),
                                matvecs.ctypes.data_as(C.POINTER(C.c_longlong)), _dp(seconds),
                                statuses.ctypes.data_as(C.POINTER(C.c_int)), _dp(stats))
    if raise_on_error or not statuses.any():
        _check(rc)
    return [{"energy": float(energies[i]), "matvecs": int(matvecs[i]), "seconds": float(seconds[i]),
             "status": int(statuses[i]), "stats": dict(zip(STAT_NAMES, stats[i].tolist()))} for i in range(n)]


def rayleigh_ritz_eig(mat, prev_evecs=None, reps=1):
    """The Davidson solver's device eigensolver on a symmetric matrix of order <= 32:
    (eigenvalues ascending, eigenvectors as columns, microseconds per call). prev_evecs:
    eigenvectors of the leading (n-1) x (n-1) block (warm start)."""
    a = np.asfortranarray(mat, dtype=np.float64)
    n = a.shape[0]
    ev = np.zeros(n)
    vec = np.zeros((n, n), order="F")
    warm = prev_evecs is not None
    if warm:
        vec[: n - 1, : n - 1] = prev_evecs
        buf = np.asfortranarray(np.asarray(prev_evecs, dtype=np.float64)).ravel(order="F").copy()
        flat = np.zeros(n * n)
        flat[: buf.size] = buf
    else:
        flat = np.zeros(n * n)
    us = C.c_double()
    _check(load().c2g_rayleigh_ritz_eig(int(n), _dp(a.ravel(order="F")), int(warm), _dp(ev), _dp(flat), int(reps),
                                        C.byref(us)))
    return ev, flat.reshape((n, n), order="F"), us.value


def device_memory_info(device: int = -1):
    """(free bytes of the device, bytes in use from its default stream-ordered pool)."""
    fr, used = C.c_int64(), C.c_int64()
    _check(load().c2g_device_memory_info(int(device), C.byref(fr), C.byref(used)))
    return fr.value, used.value


def host_rand_sample(seed: int, n: int) -> np.ndarray:
    """The first n draws of a batch member's private generator seeded with `seed`."""
    out = np.zeros(n, dtype=np.int32)
    _check(load().c2g_host_rand_sample(C.c_uint(seed), int(n), out.ctypes.data_as(C.POINTER(C.c_int))))
    return out


# Names of the reference's Cython module.
PyHamiltonian = Hamiltonian
PyProblem = Problem
PyConvergenceScheme = ConvergenceScheme
PyDMRG = DMRG

__all__ = ["Hamiltonian", "Problem", "ConvergenceScheme", "DMRG", "PyHamiltonian", "PyProblem",
           "PyConvergenceScheme", "PyDMRG", "srand", "solve_batch", "host_rand_sample", "wigner3j", "wigner6j", "wigner9j", "kernel_launches", "load",
           "Chemps2Error", "NoDeviceError"]
