"""Parity at the benchmark configurations' own sizes, against the CPU oracle
(the reference algorithm restated in FP64) and against exact answers.

* Cube-sphere of the unit sphere at n = 52 (16,226 nodes, the conforming
  cube-sphere nearest to 16,386), all-Dirichlet, data a seeded combination of
  degree-1 and degree-2 harmonic polynomials: the FP64 normal derivative
  against its exact value deg * p (discretisation error, converging as h^2),
  matrix entries of sampled rows against the oracle (1e-10 of the largest
  entry), the solution against the oracle's (FP64 1e-9, mixed 1e-8).
* Wigley tank with 8 seeded shape parameters at N = 8,192: every matrix
  entry, alpha, phi, dphi/dn and the hull force against the oracle (FP64:
  1e-10 on entries, 1e-9 on the solution; mixed: 2e-8 and 1e-8), and the
  gradient with respect to the 8 shape parameters against central
  differences (h = 1e-6) of the GPU forward map and of the oracle.

The oracle's solution is its reference-faithful GMRES(100) with the band-100
preconditioner run to an absolute residual of 1e-14 (the converged answer of
the reference's solver)."""
import os

import numpy as np
import pytest

import oracle as O
from helpers import rel2, relmax
from wavebem_gb300 import meshes as M
from wavebem_gb300.bem_problem import PREC_FP64, PREC_MIXED, BEMProblem

pytestmark = pytest.mark.gpu


def _oracle(m, ptr, idx, b):
    O.set_threads(os.cpu_count() or 1)
    P = O.Problem(m.X, m.cells, ptr, idx, m.dirichlet)
    P.assemble()
    phi, dphi, st, it, res = P.solve_system_gmres(b, restart=100, max_steps=3000, tol=1e-14, band=100)
    assert st == 0, (it, res)
    return P, phi, dphi


@pytest.fixture(scope="module")
def sphere52():
    m, ptr, idx, b = M.config_case("c1")
    return m, ptr, idx, b, m.info["exact_dphi_dn"]


@pytest.fixture(scope="module")
def tank8192():
    m, ptr, idx, b = M.config_case("c3")
    P, phi, dphi = _oracle(m, ptr, idx, b)
    return m, ptr, idx, b, P, phi, dphi


def test_sphere_n52_exact_normal_derivative_and_sampled_rows(sphere52):
    m, ptr, idx, p, dpdn = sphere52
    assert m.n_dofs == 16226
    g = BEMProblem(m.X, m.cells, m.dirichlet, ptr, idx, precision=PREC_FP64)
    phi, dphi = p.copy(), np.zeros_like(p)
    g.solve(phi, dphi, p)
    err52 = rel2(dphi, dpdn)
    # the same on the 866-node sphere: the error falls as h^2 ~ (12 / 52)^2
    m12 = M.cube_sphere_mesh(12)
    p12, d12 = M.sphere_harmonics(m12.X, seed=1)
    g12 = BEMProblem(m12.X, m12.cells, m12.dirichlet, *M.double_nodes(m12.X, m12.cells))
    ph12, dp12 = p12.copy(), np.zeros_like(p12)
    g12.solve(ph12, dp12, p12)
    err12 = rel2(dp12, d12)
    assert err52 < 1e-3 and err52 < 2.0 * (12 / 52) ** 2 * err12, (err52, err12)
    # matrix entries of four 16-row blocks spread over the mesh
    Nm, Dm = g.matrices()
    P = O.Problem(m.X, m.cells, ptr, idx, m.dirichlet)
    O.set_threads(os.cpu_count() or 1)
    scale_n = scale_d = 0.0
    worst_n = worst_d = 0.0
    for r0 in (0, 4000, 9000, m.n_dofs - 16):
        No, Do = P.assemble(rows=(r0, r0 + 16))
        worst_n = max(worst_n, np.abs(Nm[r0:r0 + 16] - No).max())
        worst_d = max(worst_d, np.abs(Dm[r0:r0 + 16] - Do).max())
        scale_n = max(scale_n, np.abs(No).max())
        scale_d = max(scale_d, np.abs(Do).max())
    assert worst_n <= 1e-10 * scale_n and worst_d <= 1e-10 * scale_d, (worst_n / scale_n,
                                                                         worst_d / scale_d)


def test_sphere_n52_solution_against_oracle(sphere52):
    m, ptr, idx, p, dpdn = sphere52
    P, phi_o, dphi_o = _oracle(m, ptr, idx, p)
    for prec, tol in ((PREC_FP64, 1e-9), (PREC_MIXED, 1e-8)):
        g = BEMProblem(m.X, m.cells, m.dirichlet, ptr, idx, precision=prec)
        phi, dphi = p.copy(), np.zeros_like(p)
        g.solve(phi, dphi, p)
        assert rel2(dphi, dphi_o) <= tol, (prec, rel2(dphi, dphi_o))
        g.close()


def test_tank_n8192_fp64_entries_and_solution(tank8192):
    m, ptr, idx, b, P, phi_o, dphi_o = tank8192
    assert m.n_dofs == 8192
    g = BEMProblem(m.X, m.cells, m.dirichlet, ptr, idx, precision=PREC_FP64)
    phi, dphi = b.copy(), b.copy()
    g.solve(phi, dphi, b)
    Nm, Dm = g.matrices()
    assert relmax(Nm, P.Nm) <= 1e-10
    assert relmax(Dm, P.Dm) <= 1e-10
    assert relmax(g.compute_alpha(), P.alpha) <= 1e-10
    assert rel2(phi, phi_o) <= 1e-9 and rel2(dphi, dphi_o) <= 1e-9
    hull = np.nonzero(m.face == M.HULL)[0].astype(np.int32)
    F_o = P.hull_force(m.cells[hull], phi_o, dphi_o)
    assert abs(g.hull_force(hull, phi, dphi) - F_o) <= 1e-9 * abs(F_o)


def test_tank_n8192_mixed_entries_and_solution(tank8192):
    m, ptr, idx, b, P, phi_o, dphi_o = tank8192
    g = BEMProblem(m.X, m.cells, m.dirichlet, ptr, idx, precision=PREC_MIXED)
    phi, dphi = b.copy(), b.copy()
    g.solve(phi, dphi, b)
    Nm, Dm = g.matrices()
    assert relmax(Nm, P.Nm) <= 2e-8
    assert relmax(Dm, P.Dm) <= 2e-8
    assert rel2(phi, phi_o) <= 1e-8 and rel2(dphi, dphi_o) <= 1e-8
    hull = np.nonzero(m.face == M.HULL)[0].astype(np.int32)
    F_o = P.hull_force(m.cells[hull], phi_o, dphi_o)
    assert abs(g.hull_force(hull, phi, dphi) - F_o) <= 1e-8 * abs(F_o)


def _shape_case():
    """The N = 8,192 tank's shape parameters, mesh and data as functions of a."""
    rng = np.random.default_rng(3)
    a0 = rng.normal(0.0, 1e-3, 8)

    def case(a):
        m = M.wigley_mesh(8192, a=a)
        return m, M.wigley_bc(m, seed=3)
    return a0, case


def test_tank_n8192_shape_gradient_against_central_differences(tank8192):
    """dF_x/da_j for the 8 shape parameters: the adjoint chained with dX/da
    and db/da against central differences (h = 1e-6) of the GPU FP64 forward
    map, and against central differences of the oracle along a random
    direction in parameter space."""
    m, ptr, idx, b, P, _, _ = tank8192
    a0, case = _shape_case()
    hull = np.nonzero(m.face == M.HULL)[0].astype(np.int32)
    h = 1e-6

    def force_gpu(a):
        mm, bb = case(a)
        g = BEMProblem(mm.X, mm.cells, mm.dirichlet, ptr, idx, tolerance=1e-14)
        phi, dphi = bb.copy(), bb.copy()
        g.solve(phi, dphi, bb)
        F = g.hull_force(hull, phi, dphi)
        g.close()
        return F

    g = BEMProblem(m.X, m.cells, m.dirichlet, ptr, idx, tolerance=1e-14)
    phi, dphi = b.copy(), b.copy()
    g.solve(phi, dphi, b)
    gX, gb = g.force_adjoint(hull, b)
    grad = np.zeros(8)
    fd = np.zeros(8)
    for j in range(8):
        e = np.zeros(8)
        e[j] = h
        mp, bp = case(a0 + e)
        mm, bm = case(a0 - e)
        # chain rule through the mesh generator (exact up to h^2)
        grad[j] = np.sum(gX * (mp.X - mm.X)) / (2 * h) + gb @ (bp - bm) / (2 * h)
        fd[j] = (force_gpu(a0 + e) - force_gpu(a0 - e)) / (2 * h)
    assert rel2(grad, fd) <= 1e-6, (grad, fd)
    # the oracle (reference algorithm) along one random direction in a
    u = np.random.default_rng(5).normal(size=8)
    O.set_threads(os.cpu_count() or 1)

    def force_oracle(a):
        mm, bb = case(a)
        Po = O.Problem(mm.X, mm.cells, ptr, idx, mm.dirichlet)
        Po.assemble()
        ph, dp, st, _, _ = Po.solve_system_gmres(bb, restart=100, max_steps=3000, tol=1e-14, band=100)
        assert st == 0
        return Po.hull_force(mm.cells[hull], ph, dp)

    fd_o = (force_oracle(a0 + h * u) - force_oracle(a0 - h * u)) / (2 * h)
    assert abs(grad @ u - fd_o) <= 1e-6 * abs(fd_o), (grad @ u, fd_o)
