"""FP32 LU of the mixed-form system through the test hooks of the C ABI:
the factors reproduce the FP32 system matrix, and the block triangular
sweeps (forward and transposed) agree with a CPU solve on the same factors."""
import numpy as np
import pytest

from helpers import wigley
from wavebem_gb300.bem_problem import PREC_MIXED, SOLVER_LU, BEMProblem

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def factored():
    m, ptr, idx, b = wigley(2000)
    g = BEMProblem(m.X, m.cells, m.dirichlet, ptr, idx, precision=PREC_MIXED, solver=SOLVER_LU)
    g.assemble_system()
    S, LU, perm = g.lu_factors()
    return g, S, LU, perm, m


def test_lu_factor_residual(factored):
    g, S, LU, perm, m = factored
    N = S.shape[0]
    assert sorted(perm.tolist()) == list(range(N))
    L = np.tril(LU.astype(np.float64), -1) + np.eye(N)
    U = np.triu(LU.astype(np.float64))
    R = S.astype(np.float64) - L @ U
    # FP32 factors with TF32 trailing updates (11 significant bits per
    # operand, one product): measured 3.0e-5 of the largest entry at N = 2,000
    assert np.abs(R).max() <= 1e-4 * np.abs(S).max()
    # no pivoting: the diagonal dominates, no growth
    assert np.abs(U).max() <= 1.5 * np.abs(S).max()


@pytest.mark.parametrize("transpose", [False, True])
def test_lu_sweeps_match_cpu(factored, transpose):
    import scipy.linalg as sla
    g, S, LU, perm, m = factored
    N = S.shape[0]
    L = np.tril(LU.astype(np.float64), -1) + np.eye(N)
    U = np.triu(LU.astype(np.float64))
    v = np.random.default_rng(5).normal(size=N)
    z = g.lu_apply(v, transpose=transpose)
    if transpose:
        zc = sla.solve_triangular(L.T, sla.solve_triangular(U.T, v, lower=True), lower=False,
                                  unit_diagonal=True)
        Sz = S.astype(np.float64).T @ z
    else:
        zc = sla.solve_triangular(U, sla.solve_triangular(L, v, lower=True, unit_diagonal=True))
        Sz = S.astype(np.float64) @ z
    assert np.linalg.norm(z - zc) <= 1e-6 * np.linalg.norm(zc)
    # the factors as a preconditioner of S (TF32 trailing updates: measured
    # 1.0e-4 at N = 2,000; the FP64 GMRES refinement sets the final accuracy)
    assert np.linalg.norm(v - Sz) <= 3e-4 * np.linalg.norm(v)
