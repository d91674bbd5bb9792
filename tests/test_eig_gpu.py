"""The Davidson solver's Rayleigh-Ritz eigensolver on the device (parallel-ordering
Jacobi, vector.cu rr_eig_kernel; the reference calls dsyev, CheMPS2/Davidson.cpp:242-276)
against LAPACK (numpy.linalg.eigh): eigenvalues to 1e-12 relative to the matrix norm,
eigenvectors orthonormal and diagonalising the matrix to the same bar; cold starts and
warm starts from the eigenvectors of the leading block (a Davidson expansion step)."""
from __future__ import annotations

import numpy as np
import pytest

import chemps2_gb300 as c2g

pytestmark = pytest.mark.gpu


def check(M, ev, V):
    n = M.shape[0]
    ref = np.linalg.eigvalsh(M)
    scale = max(1.0, np.linalg.norm(M, 2))
    assert np.max(np.abs(ev - ref)) < 1e-12 * scale
    assert np.all(np.diff(ev) >= 0)
    assert np.max(np.abs(V.T @ V - np.eye(n))) < 1e-12
    assert np.max(np.abs(V.T @ M @ V - np.diag(ev))) < 1e-12 * scale


@pytest.mark.parametrize("n", [1, 2, 3, 7, 16, 31, 32])
def test_rayleigh_ritz_cold(n):
    rng = np.random.default_rng(n)
    A = rng.standard_normal((n, n))
    M = A + A.T
    ev, V, _ = c2g.rayleigh_ritz_eig(M)
    check(M, ev, V)


@pytest.mark.parametrize("n", [2, 5, 17, 32])
def test_rayleigh_ritz_warm(n):
    rng = np.random.default_rng(100 + n)
    # a Davidson-like projected matrix: dominant diagonal, small couplings, a new border
    M = np.diag(np.sort(rng.uniform(-5, 5, n))) + 1e-2 * rng.standard_normal((n, n))
    M = 0.5 * (M + M.T)
    _, prev = np.linalg.eigh(M[: n - 1, : n - 1])
    ev, V, _ = c2g.rayleigh_ritz_eig(M, prev_evecs=prev)
    check(M, ev, V)


def test_rayleigh_ritz_degenerate_and_timing():
    # exactly degenerate eigenvalues and a diagonal matrix; timing printed for the record
    M = np.diag(np.repeat(np.arange(16.0), 2))
    ev, V, _ = c2g.rayleigh_ritz_eig(M)
    check(M, ev, V)
    rng = np.random.default_rng(7)
    A = rng.standard_normal((32, 32))
    M = A + A.T
    _, _, us_cold = c2g.rayleigh_ritz_eig(M, reps=20)
    M2 = np.diag(np.sort(rng.uniform(-5, 5, 32))) + 1e-3 * rng.standard_normal((32, 32))
    M2 = 0.5 * (M2 + M2.T)
    _, prev = np.linalg.eigh(M2[:31, :31])
    _, _, us_warm = c2g.rayleigh_ritz_eig(M2, prev_evecs=prev, reps=20)
    print(f"rayleigh-ritz n=32: cold {us_cold:.1f} us, warm {us_warm:.1f} us per call")
