"""GPU (libwbem.so, sm_103a) against the CPU oracle: the plain FP64 form.

Tolerances: matrix entries and alpha 1e-10 relative to the largest entry;
solved phi / dphi_dn 1e-9 in the relative 2-norm."""
import numpy as np
import pytest

from helpers import oracle_problem, rel2, relmax
from wavebem_gb300 import meshes as M
from wavebem_gb300.bem_problem import BEMProblem

pytestmark = pytest.mark.gpu


def _gpu(m, ptr, idx, **opt):
    return BEMProblem(m.X, m.cells, m.dirichlet, ptr, idx, **opt)


@pytest.mark.parametrize("kind,n", [("wigley", 2000), ("sphere", 12)])
def test_fp64_matrices_alpha(kind, n):
    P, m, b = oracle_problem(kind, n)
    g = _gpu(m, P.dn_ptr, P.dn_idx)
    g.assemble_system()
    Nm, Dm = g.matrices()
    a = g.compute_alpha()
    assert relmax(Nm, P.Nm) <= 1e-10
    assert relmax(Dm, P.Dm) <= 1e-10
    assert relmax(a, P.alpha) <= 1e-10


@pytest.mark.parametrize("kind,n", [("wigley", 2000), ("sphere", 12)])
def test_fp64_solve(kind, n):
    P, m, b = oracle_problem(kind, n)
    phi_o, dphi_o, _ = P.solve_system(b)
    g = _gpu(m, P.dn_ptr, P.dn_idx)
    phi = b.copy()
    dphi = b.copy()
    g.solve(phi, dphi, b)
    assert rel2(phi, phi_o) <= 1e-9
    assert rel2(dphi, dphi_o) <= 1e-9


def test_fp64_operators():
    P, m, b = oracle_problem("wigley", 2000)
    g = _gpu(m, P.dn_ptr, P.dn_idx)
    g.assemble_system()
    v = np.random.default_rng(5).normal(size=P.N)
    assert rel2(g.vmult(v), P.vmult(v)) <= 1e-12
    assert rel2(g.compute_rhs(v), P.compute_rhs(v)) <= 1e-12


def test_fp64_residual():
    """BEMProblem::residual: A_c sol - rhs_c of the constrained system for given
    (phi, dphi_dn), against the oracle's constrained system; and ~0 for the
    solution of a solve."""
    P, m, b = oracle_problem("wigley", 2000)
    g = _gpu(m, P.dn_ptr, P.dn_idx)
    g.assemble_system()
    rng = np.random.default_rng(11)
    phi, dphi = rng.normal(size=P.N), rng.normal(size=P.N)
    mask = m.dirichlet.astype(bool)
    A, rhs = P.system(np.where(mask, phi, dphi))
    ref = A @ np.where(mask, dphi, phi) - rhs
    res = np.zeros(P.N)
    g.residual(res, phi, dphi)
    assert rel2(res, ref) <= 1e-11
    phi, dphi = b.copy(), b.copy()
    g.solve_system(phi, dphi, b)
    g.residual(res, phi, dphi)
    assert np.linalg.norm(res) <= 1e-9 * np.linalg.norm(P.system(b)[1])


def test_fp64_double_nodes_found_by_library():
    P, m, b = oracle_problem("wigley", 2000)
    g = BEMProblem(m.X, m.cells, m.dirichlet)  # library finds the double nodes
    g.assemble_system()
    Nm, Dm = g.matrices()
    assert relmax(Nm, P.Nm) <= 1e-10
    assert relmax(Dm, P.Dm) <= 1e-10


def test_hull_force_matches_oracle():
    P, m, b = oracle_problem("wigley", 2000)
    phi_o, dphi_o, _ = P.solve_system(b)
    hull = np.nonzero(m.face == M.HULL)[0].astype(np.int32)
    g = _gpu(m, P.dn_ptr, P.dn_idx)
    F = g.hull_force(hull, phi_o, dphi_o)
    Fo = P.hull_force(m.cells[hull], phi_o, dphi_o)
    assert abs(F - Fo) <= 1e-12 * max(1.0, abs(Fo))


def test_sphere_exact_normal_derivative():
    P, m, b = oracle_problem("sphere", 12)
    from helpers import sphere
    _, _, _, p, dpdn = sphere(12)
    g = _gpu(m, P.dn_ptr, P.dn_idx)
    phi = p.copy()
    dphi = np.zeros_like(p)
    g.solve(phi, dphi, p)
    # discretisation error of the Q1 collocation BEM on a coarse sphere
    assert rel2(dphi, dpdn) < 0.01


@pytest.mark.parametrize("prec,tol", [(0, 1e-12), (1, 2e-8)])
def test_vmult_all_neumann_norm_shift(prec, tol):
    """vmult with no Dirichlet node subtracts ||dst||_2 from every entry
    (source/bem_problem.cc:667-668), like the oracle's; a solve of that
    singular system is refused with an argument error."""
    import oracle as O
    from wavebem_gb300.bem_problem import WBEMError
    P, m, b = oracle_problem("wigley", 2000)
    g = _gpu(m, P.dn_ptr, P.dn_idx, precision=prec)
    g.assemble_system()
    neu = np.zeros(P.N, np.uint8)
    g.set_bc(neu)
    P0 = O.Problem(m.X, m.cells, P.dn_ptr, P.dn_idx, neu)
    P0.Nm, P0.Dm, P0.alpha = P.Nm, P.Dm, P.alpha
    v = np.random.default_rng(7).normal(size=P.N)
    ref = P0.vmult(v)
    assert rel2(g.vmult(v), ref) <= tol
    # without the shift the two would differ by ||dst|| in every entry
    assert np.abs(ref - (P.Nm @ v + P.alpha * v)).max() > 1e-3 * np.abs(ref).max()
    phi, dphi = b.copy(), b.copy()
    with pytest.raises(WBEMError):
        g.solve_system(phi, dphi, b)
