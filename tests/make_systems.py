"""Linear systems the reference's unit tests build, restated for the tests.

* helper_system: FdmLinearSystemSolverTestHelper3::buildTestLinearSystem
  (src/tests/unit_tests/fdm_linear_system_solver_test_helper3.h:13-48).
* poisson_system: the multi-level Poisson system of
  src/tests/unit_tests/fdm_mgpcg_solver3_tests.cpp:13-60 and
  fdm_mg_solver3_tests.cpp:13-69 (a matrix on every level, h doubling).

Rows are (nz, ny, nx, 4) float64 arrays {center, right, up, front}.
"""
import numpy as np


def _grid(n):
    return np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")


def helper_system(n: int):
    k, j, i = _grid(n)
    A = np.zeros((n, n, n, 4))
    b = np.zeros((n, n, n))
    one = lambda m: m.astype(np.float64)
    A[..., 0] += one(i > 0) + one(i < n - 1)
    A[..., 1] -= one(i < n - 1)
    A[..., 0] += one(j > 0) + one(j < n - 1)
    b += np.where(j > 0, 0.0, 1.0)
    A[..., 2] -= one(j < n - 1)
    b -= np.where(j < n - 1, 0.0, 1.0)
    A[..., 0] += one(k > 0) + one(k < n - 1)
    A[..., 3] -= one(k < n - 1)
    return A, b


def poisson_system(levels: int = 4, coarsest: int = 4):
    A_levels, b_levels = [], []
    for l in range(levels):
        n = coarsest << (levels - 1 - l)
        invdx = 0.5 ** l
        s = invdx * invdx
        k, j, i = _grid(n)
        A = np.zeros((n, n, n, 4))
        b = np.zeros((n, n, n))
        A[..., 0] += np.where(i > 0, s, 0) + np.where(i < n - 1, s, 0)
        A[..., 1] -= np.where(i < n - 1, s, 0)
        A[..., 0] += np.where(j > 0, s, 0)
        b += np.where(j > 0, 0, invdx)
        A[..., 0] += np.where(j < n - 1, s, 0)
        A[..., 2] -= np.where(j < n - 1, s, 0)
        b -= np.where(j < n - 1, 0, invdx)
        A[..., 0] += np.where(k > 0, s, 0) + np.where(k < n - 1, s, 0)
        A[..., 3] -= np.where(k < n - 1, s, 0)
        A_levels.append(A)
        b_levels.append(b)
    return A_levels, b_levels
