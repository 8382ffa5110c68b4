"""Adjoint of assemble + solve + hull force against central finite
differences (h = 1e-6) of the FP64 forward map, and mixed against FP64.

The shape-parameter check: Wigley hull offset perturbed by
sum_j a_j sin(j pi (x + 0.5)) (1 - (z/T)^2); gradient with respect to the a_j
through X(a) and the Neumann data b(a) = -U . n(a), chained in a
torch.autograd.Function wrapper (test harness only)."""
import numpy as np
import pytest

from helpers import rel2
from wavebem_gb300 import meshes as M
from wavebem_gb300.bem_problem import PREC_FP64, PREC_MIXED, SOLVER_GMRES_IR, SOLVER_LU, BEMProblem

pytestmark = pytest.mark.gpu


def _setup(n, a):
    m = M.wigley_mesh(n, a=a)
    ptr, idx = M.double_nodes(m.X, m.cells)
    hull = np.nonzero(m.face == M.HULL)[0].astype(np.int32)
    return m, ptr, idx, hull


def _force(g, m, b, hull):
    phi, dphi = b.copy(), b.copy()
    g.solve(phi, dphi, b)
    return g.hull_force(hull, phi, dphi)


def test_adjoint_fd_hull_nodes_fp64():
    m, ptr, idx, hull = _setup(800, None)
    b = M.wigley_bc(m, seed=3)
    g = BEMProblem(m.X, m.cells, m.dirichlet, ptr, idx, precision=PREC_FP64, tolerance=1e-14)
    F0 = _force(g, m, b, hull)
    gX, gb = g.force_adjoint(hull, b)
    rng = np.random.default_rng(0)
    hull_nodes = np.unique(m.cells[hull])
    # directional derivative along a random direction on the hull nodes
    d = np.zeros_like(m.X)
    d[hull_nodes] = rng.normal(size=(len(hull_nodes), 3))
    h = 1e-6
    fp = _force(g.__class__(m.X + h * d, m.cells, m.dirichlet, ptr, idx, tolerance=1e-14), m, b, hull)
    fm = _force(g.__class__(m.X - h * d, m.cells, m.dirichlet, ptr, idx, tolerance=1e-14), m, b, hull)
    fd = (fp - fm) / (2 * h)
    ad = float(np.sum(gX * d))
    assert abs(ad - fd) <= 1e-6 * abs(fd), (ad, fd)
    # and with respect to the known data
    db = rng.normal(size=len(b))
    fp = _force(g, m, b + h * db, hull)
    fm = _force(g, m, b - h * db, hull)
    fd = (fp - fm) / (2 * h)
    assert abs(float(gb @ db) - fd) <= 1e-6 * abs(fd)


def test_adjoint_componentwise_few_nodes_fp64():
    m, ptr, idx, hull = _setup(800, None)
    b = M.wigley_bc(m, seed=3)
    g = BEMProblem(m.X, m.cells, m.dirichlet, ptr, idx, tolerance=1e-14)
    _force(g, m, b, hull)
    gX, gb = g.force_adjoint(hull, b)
    hull_nodes = np.unique(m.cells[hull])
    h = 1e-6
    for node in hull_nodes[:: max(1, len(hull_nodes) // 4)][:4]:
        for c in range(3):
            Xp = m.X.copy(); Xp[node, c] += h
            Xm = m.X.copy(); Xm[node, c] -= h
            fd = (_force(BEMProblem(Xp, m.cells, m.dirichlet, ptr, idx, tolerance=1e-14), m, b, hull)
                  - _force(BEMProblem(Xm, m.cells, m.dirichlet, ptr, idx, tolerance=1e-14), m, b, hull)) / (2 * h)
            scale = np.abs(gX).max()
            assert abs(gX[node, c] - fd) <= 1e-6 * scale, (node, c, gX[node, c], fd)


@pytest.mark.parametrize("solver", [SOLVER_GMRES_IR, SOLVER_LU])
def test_adjoint_mixed_matches_fp64(solver):
    m, ptr, idx, hull = _setup(2000, None)
    b = M.wigley_bc(m, seed=3)
    g64 = BEMProblem(m.X, m.cells, m.dirichlet, ptr, idx, precision=PREC_FP64, tolerance=1e-14)
    _force(g64, m, b, hull)
    gX64, gb64 = g64.force_adjoint(hull, b)
    gm = BEMProblem(m.X, m.cells, m.dirichlet, ptr, idx, precision=PREC_MIXED, solver=solver)
    _force(gm, m, b, hull)
    gXm, gbm = gm.force_adjoint(hull, b)
    assert rel2(gXm, gX64) <= 1e-6
    assert rel2(gbm, gb64) <= 1e-6


def test_adjoint_shape_parameters_autograd():
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(3)
    a0 = rng.normal(0.0, 1e-3, 8)
    n = 800

    class Force(torch.autograd.Function):
        """Forward: F(X, b) through the C ABI; backward: the library adjoint."""

        @staticmethod
        def forward(ctx, X, b, prob):
            g = BEMProblem(X.detach().numpy(), prob["cells"], prob["mask"], prob["ptr"], prob["idx"],
                           tolerance=1e-14)
            bb = b.detach().numpy()
            F = _force(g, None, bb, prob["hull"])
            gX, gb = g.force_adjoint(prob["hull"], bb)
            ctx.save_for_backward(torch.from_numpy(gX), torch.from_numpy(gb))
            return X.new_tensor(F)

        @staticmethod
        def backward(ctx, gout):
            gX, gb = ctx.saved_tensors
            return gout * gX, gout * gb, None

    def mesh_of(a):
        # X(a) and b(a) in torch so the chain rule runs through autograd
        m = M.wigley_mesh(n, a=a.detach().numpy())
        return m

    a = torch.tensor(a0, dtype=torch.float64, requires_grad=True)
    m = mesh_of(a)
    ptr, idx = M.double_nodes(m.X, m.cells)
    hull = np.nonzero(m.face == M.HULL)[0].astype(np.int32)
    prob = {"cells": m.cells, "mask": m.dirichlet, "ptr": ptr, "idx": idx, "hull": hull}
    # differentiable X(a), b(a): only hull-patch nodes (and the waterline of the
    # free surface, the centre-plane edges) move; use central differences of the
    # numpy generator for the Jacobians dX/da, db/da (exact up to h^2)
    h = 1e-6
    J_X, J_b = [], []
    for j in range(8):
        e = np.zeros(8); e[j] = h
        mp_, mm_ = M.wigley_mesh(n, a=a0 + e), M.wigley_mesh(n, a=a0 - e)
        J_X.append((mp_.X - mm_.X) / (2 * h))
        J_b.append((M.wigley_bc(mp_, seed=3) - M.wigley_bc(mm_, seed=3)) / (2 * h))
    JX = torch.tensor(np.stack(J_X, -1))  # (N,3,8)
    Jb = torch.tensor(np.stack(J_b, -1))  # (N,8)
    X = torch.tensor(m.X) + torch.einsum("nck,k->nc", JX, a - a.detach())
    b = torch.tensor(M.wigley_bc(m, seed=3)) + Jb @ (a - a.detach())
    F = Force.apply(X, b, prob)
    F.backward()
    grad = a.grad.numpy()
    # central differences of the full forward map in each a_j
    fd = np.zeros(8)
    for j in range(8):
        e = np.zeros(8); e[j] = h
        vals = []
        for s in (1, -1):
            mm = M.wigley_mesh(n, a=a0 + s * e)
            g = BEMProblem(mm.X, mm.cells, mm.dirichlet, ptr, idx, tolerance=1e-14)
            vals.append(_force(g, mm, M.wigley_bc(mm, seed=3), hull))
        fd[j] = (vals[0] - vals[1]) / (2 * h)
    assert rel2(grad, fd) <= 1e-6, (grad, fd)


@pytest.mark.parametrize("prec", [PREC_FP64, PREC_MIXED])
def test_adjoint_matches_oracle_directional_differences(prec):
    """The GPU adjoint against FP64 central differences of the CPU oracle
    (the reference algorithm restated: assembly, constrained solve, hull
    force), along a random direction over the hull nodes."""
    import oracle as O
    m, ptr, idx, hull = _setup(800, None)
    b = M.wigley_bc(m, seed=3)
    g = BEMProblem(m.X, m.cells, m.dirichlet, ptr, idx, precision=prec, tolerance=1e-14)
    _force(g, m, b, hull)
    gX, _ = g.force_adjoint(hull, b)
    d = np.zeros_like(m.X)
    hull_nodes = np.unique(m.cells[hull])
    d[hull_nodes] = np.random.default_rng(11).normal(size=(len(hull_nodes), 3))
    # a double node is one point: its copies on the free surface move with
    # the hull copy. (Moving one copy alone tears the vertex-singular panels
    # apart; the discrete map then has third derivatives of order 1/r^4 at the
    # nearest quadrature points, and central differences with h = 1e-6 are off
    # by ~1e-6 relative, shrinking as h^2, while the adjoint stays exact.)
    for i in hull_nodes:
        for j in idx[ptr[i]:ptr[i + 1]]:
            d[j] = d[i]
    h = 1e-6

    def oracle_force(X):
        P = O.Problem(X, m.cells, ptr, idx, m.dirichlet)
        P.assemble()
        phi, dphi, _ = P.solve_system(b)
        return P.hull_force(m.cells[hull], phi, dphi)

    fd = (oracle_force(m.X + h * d) - oracle_force(m.X - h * d)) / (2 * h)
    ad = float(np.sum(gX * d))
    # FP64: the spec bar; mixed: its forward map differs from FP64 by
    # ~1e-9 and its gradient by <= 1e-6 (test_adjoint_mixed_matches_fp64)
    tol = 1e-6 if prec == PREC_FP64 else 2e-6
    assert abs(ad - fd) <= tol * abs(fd), (ad, fd)


def test_adjoint_of_a_linear_objective_fp64_and_mixed():
    """wbem_adjoint for J = c . phi + d . dphi_dn (all entries, known and
    solved) against central differences, along a smooth displacement of every
    node (coincident double-node copies move together) and along the known
    data; the mixed form against the FP64 form."""
    m, ptr, idx, _ = _setup(800, None)
    b = M.wigley_bc(m, seed=3)
    rng = np.random.default_rng(11)
    c = rng.normal(size=m.n_dofs)
    dd = rng.normal(size=m.n_dofs)

    def J(X, bb, prec=PREC_FP64):
        g = BEMProblem(X, m.cells, m.dirichlet, ptr, idx, precision=prec, tolerance=1e-14)
        phi, dphi = bb.copy(), bb.copy()
        g.solve(phi, dphi, bb)
        return g, float(c @ phi + dd @ dphi)

    g, _ = J(m.X, b)
    gX, gb = g.adjoint(c, dd)
    A = rng.normal(size=(3, 3))
    d = 0.1 * np.sin(m.X @ A + rng.uniform(0, 2 * np.pi, 3))
    h = 1e-6
    fd = (J(m.X + h * d, b)[1] - J(m.X - h * d, b)[1]) / (2 * h)
    assert abs(float(np.sum(gX * d)) - fd) <= 1e-6 * abs(fd), (float(np.sum(gX * d)), fd)
    db = rng.normal(size=len(b))
    fd = (J(m.X, b + h * db)[1] - J(m.X, b - h * db)[1]) / (2 * h)
    assert abs(float(gb @ db) - fd) <= 1e-6 * abs(fd), (float(gb @ db), fd)
    gm, _ = J(m.X, b, PREC_MIXED)
    gXm, gbm = gm.adjoint(c, dd)
    assert rel2(gXm, gX) <= 1e-6
    assert rel2(gbm, gb) <= 1e-6
