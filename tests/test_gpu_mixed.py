"""Mixed-precision form against the FP64 oracle.

Entries: double-float panel base + FP32 point differences; tolerance 2e-8
relative to the largest entry (measured 1e-9 on the Wigley tank, 1.05e-8 on
the coarse 866-node sphere whose strongly curved panels make the point
differences larger). Solution, for each solver of the mixed form (FP64
refinement over inner block-Jacobi GMRES on the FP32 system; FP32 LU with
BF16x3 tensor-core updates preconditioning FP64 GMRES; plain block-Jacobi
GMRES on the mixed storage): tolerance 1e-8 relative 2-norm."""
import numpy as np
import pytest

from helpers import oracle_problem, rel2, relmax
from wavebem_gb300 import meshes as M
from wavebem_gb300.bem_problem import (PREC_MIXED, SOLVER_GMRES, SOLVER_GMRES_IR, SOLVER_LU,
                                       BEMProblem)

SOLVERS = [SOLVER_GMRES_IR, SOLVER_LU, SOLVER_GMRES]

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("kind,n", [("wigley", 2000), ("sphere", 12)])
def test_mixed_matrices_alpha(kind, n):
    P, m, b = oracle_problem(kind, n)
    g = BEMProblem(m.X, m.cells, m.dirichlet, P.dn_ptr, P.dn_idx, precision=PREC_MIXED)
    g.assemble_system()
    Nm, Dm = g.matrices()
    a = g.compute_alpha()
    assert relmax(Nm, P.Nm) <= 2e-8
    assert relmax(Dm, P.Dm) <= 2e-8
    assert relmax(a, P.alpha) <= 2e-8


@pytest.mark.parametrize("solver", SOLVERS)
@pytest.mark.parametrize("kind,n", [("wigley", 2000), ("sphere", 12)])
def test_mixed_solve_within_1e8(kind, n, solver):
    P, m, b = oracle_problem(kind, n)
    phi_o, dphi_o, _ = P.solve_system(b)
    g = BEMProblem(m.X, m.cells, m.dirichlet, P.dn_ptr, P.dn_idx, precision=PREC_MIXED,
                   solver=solver)
    phi, dphi = b.copy(), b.copy()
    g.solve(phi, dphi, b)
    st = g.stats()
    assert rel2(phi, phi_o) <= 1e-8
    assert rel2(dphi, dphi_o) <= 1e-8
    if solver == SOLVER_LU:
        assert st["iterations"] <= 20
    if solver == SOLVER_GMRES_IR:
        assert 1 <= st["outer_iterations"] <= 10


def test_mixed_residual_of_solution():
    P, m, b = oracle_problem("wigley", 2000)
    g = BEMProblem(m.X, m.cells, m.dirichlet, P.dn_ptr, P.dn_idx, precision=PREC_MIXED)
    phi, dphi = b.copy(), b.copy()
    g.solve(phi, dphi, b)
    res = np.zeros(P.N)
    g.residual(res, phi, dphi)
    # the residual of the double-float operator the refinement converged on
    assert np.linalg.norm(res) <= 1e-9 * np.linalg.norm(P.system(b)[1])


def test_mixed_hull_force_within_1e8():
    P, m, b = oracle_problem("wigley", 2000)
    phi_o, dphi_o, _ = P.solve_system(b)
    hull = np.nonzero(m.face == M.HULL)[0].astype(np.int32)
    F_o = P.hull_force(m.cells[hull], phi_o, dphi_o)
    g = BEMProblem(m.X, m.cells, m.dirichlet, P.dn_ptr, P.dn_idx, precision=PREC_MIXED)
    phi, dphi = b.copy(), b.copy()
    g.solve(phi, dphi, b)
    F = g.hull_force(hull, phi, dphi)
    assert abs(F - F_o) <= 1e-8 * abs(F_o)


@pytest.mark.parametrize("solver", [SOLVER_GMRES_IR, SOLVER_LU])
def test_mixed_solve_system_reuses_factors(solver):
    P, m, b = oracle_problem("wigley", 2000)
    g = BEMProblem(m.X, m.cells, m.dirichlet, P.dn_ptr, P.dn_idx, precision=PREC_MIXED,
                   solver=solver)
    g.assemble_system()
    for k, seed in enumerate((1, 2)):
        b2 = M.wigley_bc(m, seed=seed)
        phi_o, dphi_o, _ = P.solve_system(b2)
        phi, dphi = b2.copy(), b2.copy()
        g.solve_system(phi, dphi, b2)
        assert rel2(phi, phi_o) <= 1e-8 and rel2(dphi, dphi_o) <= 1e-8
        if k == 1:  # the second solve prepares nothing
            assert g.stats()["t_factor_ms"] == 0.0


@pytest.mark.parametrize("solver", [SOLVER_LU, SOLVER_GMRES_IR])
def test_mixed_mask_change_after_assembly(solver):
    """set_bc with a new mask after the assembly: the FP32 system is formed
    again from the stored N and D (the copy written during the assembly
    belongs to the old mask); an unchanged mask keeps everything."""
    import oracle as O
    P, m, b = oracle_problem("wigley", 2000)
    single = np.nonzero((np.diff(P.dn_ptr) == 1) & (m.dirichlet == 0))[0]
    mask2 = m.dirichlet.copy()
    mask2[single[::10]] = 1
    P2 = O.Problem(m.X, m.cells, P.dn_ptr, P.dn_idx, mask2)
    P2.Nm, P2.Dm, P2.alpha = P.Nm, P.Dm, P.alpha
    phi_o, dphi_o, _ = P2.solve_system(b)
    g = BEMProblem(m.X, m.cells, m.dirichlet, P.dn_ptr, P.dn_idx, precision=PREC_MIXED,
                   solver=solver)
    g.assemble_system()
    g.set_bc(mask2)
    phi, dphi = b.copy(), b.copy()
    g.solve_system(phi, dphi, b)
    assert rel2(phi, phi_o) <= 1e-8 and rel2(dphi, dphi_o) <= 1e-8
    g.set_bc(mask2)  # unchanged: nothing to prepare again
    phi, dphi = b.copy(), b.copy()
    g.solve_system(phi, dphi, b)
    assert g.stats()["t_factor_ms"] == 0.0
    assert rel2(phi, phi_o) <= 1e-8 and rel2(dphi, dphi_o) <= 1e-8


@pytest.mark.parametrize("prec", [PREC_MIXED, 0])
def test_handle_reused_for_a_mesh_of_another_size(prec):
    """One handle, two meshes of different size (the sphere after the tank):
    every size-dependent device buffer is allocated anew."""
    P1, m1, b1 = oracle_problem("wigley", 2000)
    P2, m2, b2 = oracle_problem("sphere", 12)
    g = BEMProblem(m1.X, m1.cells, m1.dirichlet, P1.dn_ptr, P1.dn_idx, precision=prec)
    phi, dphi = b1.copy(), b1.copy()
    g.solve(phi, dphi, b1)
    g.set_geometry(m2.X, m2.cells, P2.dn_ptr, P2.dn_idx)
    g.set_bc(m2.dirichlet)
    phi_o, dphi_o, _ = P2.solve_system(b2)
    phi, dphi = b2.copy(), b2.copy()
    g.solve(phi, dphi, b2)
    assert rel2(phi, phi_o) <= 1e-8 and rel2(dphi, dphi_o) <= 1e-8
    g.set_geometry(m1.X, m1.cells, P1.dn_ptr, P1.dn_idx)  # and back
    g.set_bc(m1.dirichlet)
    phi_o, dphi_o, _ = P1.solve_system(b1)
    phi, dphi = b1.copy(), b1.copy()
    g.solve(phi, dphi, b1)
    assert rel2(phi, phi_o) <= 1e-8 and rel2(dphi, dphi_o) <= 1e-8
