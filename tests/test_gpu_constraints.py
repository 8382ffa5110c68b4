"""Double-node constraints through the library (BEMProblem<3>::compute_constraints,
source/bem_problem.cc:990-1105), on meshes that have every kind of line:

* the unit cube with all faces Dirichlet: every edge node pair is a sharp
  Dirichlet-Dirichlet pair, whose two normal derivatives are fixed from the
  L2-projected normals and surface gradients;
* the same cube with its top face split in two patches: flat
  Dirichlet-Dirichlet pairs along the split line (equal normal derivatives),
  and triples (two flat copies, one sharp) where the split meets the edges;
* the split cube with only the top Dirichlet: Dirichlet-Neumann and
  Neumann-Neumann pairs beside the flat ones.

Checked against the oracle: the projected normals and surface gradients
(compute_normals, compute_surface_gradients) to 1e-12, the solution (FP64
1e-9, mixed 1e-8), and the adjoint of a linear objective (with the sharp
lines' dependence on X and on the Dirichlet data) against central
differences (h = 1e-6) of the GPU and of the oracle."""
import numpy as np
import pytest

import oracle as O
from helpers import cube_mesh, rel2
from wavebem_gb300 import meshes as M
from wavebem_gb300.bem_problem import PREC_FP64, PREC_MIXED, SOLVER_GMRES_IR, SOLVER_LU, BEMProblem

pytestmark = pytest.mark.gpu


def _potential(X):
    # harmonic: x y + z + 0.3 (x^2 - z^2)
    return X[:, 0] * X[:, 1] + X[:, 2] + 0.3 * (X[:, 0] ** 2 - X[:, 2] ** 2)


def _case(kind):
    X, cells, face = cube_mesh(8, split_top=kind != "sharp")
    ptr, idx = M.double_nodes(X, cells)
    if kind == "top":
        mask = np.zeros(len(X), np.uint8)
        top = np.all(np.isclose(X[cells][:, :, 2], 1.0), axis=1)
        mask[np.unique(cells[top])] = 1
        b = np.where(mask == 1, _potential(X), 0.1 * np.cos(3 * X[:, 0]))
    else:
        mask = np.ones(len(X), np.uint8)
        b = _potential(X)
    return X, cells, ptr, idx, mask, b


KINDS = ["sharp", "split", "top"]


@pytest.mark.parametrize("kind", KINDS)
def test_projections_match_oracle(kind):
    X, cells, ptr, idx, mask, b = _case(kind)
    P = O.Problem(X, cells, ptr, idx, mask)
    g = BEMProblem(X, cells, mask, ptr, idx)
    n, n_o = g.compute_normals(), P.node_normals()
    assert np.abs(n - n_o).max() <= 1e-12
    gr, gr_o = g.compute_surface_gradients(b), P.surface_gradients(b)
    assert np.abs(gr - gr_o).max() <= 1e-12 * np.abs(gr_o).max()


@pytest.mark.parametrize("prec,tol", [(PREC_FP64, 1e-9), (PREC_MIXED, 1e-8)])
@pytest.mark.parametrize("kind", KINDS)
def test_solution_matches_oracle(kind, prec, tol):
    X, cells, ptr, idx, mask, b = _case(kind)
    P = O.Problem(X, cells, ptr, idx, mask)
    P.assemble()
    phi_o, dphi_o, _ = P.solve_system(b)
    g = BEMProblem(X, cells, mask, ptr, idx, precision=prec)
    phi, dphi = b.copy(), b.copy()
    g.solve(phi, dphi, b)
    assert rel2(dphi, dphi_o) <= tol
    assert rel2(phi, phi_o) <= tol
    # the residual of the constrained system vanishes at the solution
    res = np.zeros(len(b))
    g.residual(res, phi, dphi)
    assert np.linalg.norm(res) <= 1e-9 * np.linalg.norm(P.system(b)[1])


@pytest.mark.parametrize("kind", ["sharp", "split"])
def test_sharp_lines_fix_exact_normal_derivatives_for_a_linear_potential(kind):
    """For a linear potential the projected surface gradients are exact, so
    the sharp lines prescribe the exact normal derivatives g . n on the edges."""
    X, cells, ptr, idx, mask, _ = _case(kind)
    grad = np.array([1.0, 2.0, -0.5])
    b = X @ grad
    g = BEMProblem(X, cells, mask, ptr, idx)
    phi, dphi = b.copy(), b.copy()
    g.solve(phi, dphi, b)
    sizes = np.diff(ptr)
    n = g.compute_normals()
    edge = sizes > 1
    # every copy on a sharp edge carries the normal of its own face
    P = O.Problem(X, cells, ptr, idx, mask)
    flags, inh, (er, ec, ev) = P.constraints(b)
    sharp = np.array([i for i in np.nonzero(flags)[0] if not np.any(er == i)])
    assert len(sharp) > 0 and edge[sharp].all()
    assert np.abs(dphi[sharp] - n[sharp] @ grad).max() <= 1e-9


def _fd_case(kind, prec):
    X, cells, ptr, idx, mask, b = _case(kind)
    rng = np.random.default_rng(11)
    c = rng.normal(size=len(X))
    d = rng.normal(size=len(X))

    def J(Xp, bb):
        g = BEMProblem(Xp, cells, mask, ptr, idx, precision=prec, tolerance=1e-14)
        phi, dphi = bb.copy(), bb.copy()
        g.solve(phi, dphi, bb)
        return g, float(c @ phi + d @ dphi)

    # a smooth displacement: coincident copies move together
    A = rng.normal(size=(3, 3))
    disp = 0.1 * np.sin(X @ A + rng.uniform(0, 2 * np.pi, 3))
    db = rng.normal(size=len(X))
    return X, cells, ptr, idx, mask, b, c, d, J, disp, db


@pytest.mark.parametrize("kind", KINDS)
def test_adjoint_through_constraint_lines_fd(kind):
    X, cells, ptr, idx, mask, b, c, d, J, disp, db = _fd_case(kind, PREC_FP64)
    g, _ = J(X, b)
    gX, gb = g.adjoint(c, d)
    h = 1e-6
    fd = (J(X + h * disp, b)[1] - J(X - h * disp, b)[1]) / (2 * h)
    ad = float(np.sum(gX * disp))
    assert abs(ad - fd) <= 1e-6 * abs(fd), (ad, fd)
    fd = (J(X, b + h * db)[1] - J(X, b - h * db)[1]) / (2 * h)
    assert abs(float(gb @ db) - fd) <= 1e-6 * abs(fd), (float(gb @ db), fd)
    # the oracle's forward map along the same displacement
    def J_o(Xp):
        P = O.Problem(Xp, cells, ptr, idx, mask)
        P.assemble()
        phi, dphi, _ = P.solve_system(b)
        return float(c @ phi + d @ dphi)

    fd_o = (J_o(X + h * disp) - J_o(X - h * disp)) / (2 * h)
    assert abs(ad - fd_o) <= 1e-6 * abs(fd_o), (ad, fd_o)


@pytest.mark.parametrize("solver", [SOLVER_LU, SOLVER_GMRES_IR])
def test_adjoint_through_constraint_lines_mixed_matches_fp64(solver):
    X, cells, ptr, idx, mask, b, c, d, J, disp, db = _fd_case("split", PREC_FP64)
    g, _ = J(X, b)
    gX, gb = g.adjoint(c, d)
    gm = BEMProblem(X, cells, mask, ptr, idx, precision=PREC_MIXED, solver=solver, tolerance=1e-14)
    phi, dphi = b.copy(), b.copy()
    gm.solve(phi, dphi, b)
    gXm, gbm = gm.adjoint(c, d)
    assert rel2(gXm, gX) <= 1e-6 and rel2(gbm, gb) <= 1e-6
