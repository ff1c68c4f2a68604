"""The oracle's 3x3 DGETRF+DGETRI restatement: accuracy against the exact
rational inverse, no worse than the installed LAPACK (scipy), and identical
results on blocks where the operation order cannot matter."""
from fractions import Fraction

import numpy as np
import pytest

import pyoracle as O


def exact_inverse(A):
    M = [[Fraction(float(A[i, j])) for j in range(3)] for i in range(3)]
    det = (M[0][0] * (M[1][1] * M[2][2] - M[1][2] * M[2][1])
           - M[0][1] * (M[1][0] * M[2][2] - M[1][2] * M[2][0])
           + M[0][2] * (M[1][0] * M[2][1] - M[1][1] * M[2][0]))
    inv = np.empty((3, 3))
    for i in range(3):
        for j in range(3):
            cof = (M[(j + 1) % 3][(i + 1) % 3] * M[(j + 2) % 3][(i + 2) % 3]
                   - M[(j + 1) % 3][(i + 2) % 3] * M[(j + 2) % 3][(i + 1) % 3])
            inv[i, j] = float(cof / det)
    return inv


def test_inverse_accuracy_vs_exact_and_lapack():
    lapack = pytest.importorskip("scipy.linalg.lapack")
    rng = np.random.default_rng(0)
    worst_mine = worst_lapack = 0.0
    for t in range(400):
        A = rng.standard_normal((3, 3))
        if t % 2:
            A = A @ A.T + 0.1 * np.eye(3)
        X = exact_inverse(A)
        mine, info = O.getrf_getri3(A.flatten(order="F"))
        assert info == 0
        mine = mine.reshape(3, 3, order="F")
        lu, piv, _ = lapack.dgetrf(A)
        ref, _ = lapack.dgetri(lu, piv)
        cond = np.linalg.cond(A)
        scale = np.abs(X).max() * np.finfo(float).eps * cond
        worst_mine = max(worst_mine, np.abs(mine - X).max() / scale)
        worst_lapack = max(worst_lapack, np.abs(ref - X).max() / scale)
    assert worst_mine < 10.0
    assert worst_mine <= 2.0 * worst_lapack + 1.0


def test_pivot_free_diagonal_block_is_exact():
    A = np.diag([4.0, 2.0, 0.5])
    inv, info = O.getrf_getri3(A.flatten(order="F"))
    assert info == 0
    assert np.array_equal(inv.reshape(3, 3, order="F"), np.diag([0.25, 0.5, 2.0]))


def test_singular_block_reports_info_and_keeps_lu():
    A = np.array([[1.0, 2.0, 3.0], [2.0, 4.0, 6.0], [1.0, 0.0, 1.0]])
    out, info = O.getrf_getri3(A.flatten(order="F"))
    assert info != 0
    assert np.all(np.isfinite(out))
