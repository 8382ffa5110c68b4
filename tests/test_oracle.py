"""CPU oracle pinned against closed-form answers (the reference's own tests
hold no golden vectors for this path, and the reference cannot be built here
without deal.II; these known answers are the pins)."""
import math

import numpy as np
import pytest

import oracle as O
from helpers import oracle_problem, rel2, sphere, wigley
from wavebem_gb300 import meshes as M


def test_gauss_legendre_exactness():
    for n in range(1, 9):
        x, w = O.gauss01(n)
        assert np.all(np.diff(x) > 0) and abs(w.sum() - 1) < 1e-15
        for k in range(2 * n):
            assert abs((w * x ** k).sum() - 1.0 / (k + 1)) < 1e-14


def test_gauss4_closed_form():
    x, w = O.gauss01(4)
    a = math.sqrt(3 / 7 - 2 / 7 * math.sqrt(6 / 5))
    b = math.sqrt(3 / 7 + 2 / 7 * math.sqrt(6 / 5))
    ref = np.sort(0.5 * (1 + np.array([-b, -a, a, b])))
    assert np.abs(x - ref).max() < 1e-15


@pytest.mark.parametrize("v", range(4))
def test_vertex_singular_rule_flat_square(v):
    # int_[0,1]^2 1/|x - vertex| dA = 2 ln(1 + sqrt 2); the polar rule integrates
    # 1/R * R exactly in the radial direction, so the error is the angular one
    exact = 2 * math.log(1 + math.sqrt(2))
    vx, vy = [(0, 0), (1, 0), (0, 1), (1, 1)][v]
    prev = None
    for n in (3, 5, 8):
        px, py, w = O.singular_rule(n, v)
        val = (w / np.hypot(px - vx, py - vy)).sum()
        err = abs(val - exact)
        if prev is not None:
            assert err < prev
        prev = err
    px, py, w = O.singular_rule(5, v)
    assert abs((w / np.hypot(px - vx, py - vy)).sum() - exact) < 1e-7
    assert np.all((px >= 0) & (px <= 1) & (py >= 0) & (py <= 1))


def test_solid_angles_of_the_tank():
    P, m, b = oracle_problem("wigley", 2000)
    X, a = m.X, P.alpha
    x0, x1 = M.BOX_X
    y1 = M.BOX_Y[1]
    zb = M.BOX_Z[0]
    corner = np.isclose(X[:, 0], x0) & np.isclose(X[:, 1], y1) & np.isclose(X[:, 2], zb)
    assert corner.sum() == 3
    assert np.abs(a[corner] - 0.125).max() < 1e-9
    edge = np.isclose(X[:, 0], x1) & np.isclose(X[:, 2], zb) & (X[:, 1] > 0.2) & (X[:, 1] < 1.3)
    assert np.abs(a[edge] - 0.25).max() < 1e-9
    face = np.isclose(X[:, 2], zb) & (X[:, 0] > x0 + 0.5) & (X[:, 0] < x1 - 0.5) & (X[:, 1] > 0.3) & (X[:, 1] < 1.2)
    assert np.abs(a[face] - 0.5).max() < 1e-9


def test_alpha_is_minus_row_sum_of_N():
    P, m, b = oracle_problem("wigley", 2000)
    assert np.abs(P.alpha + P.Nm.sum(1)).max() < 1e-12


def test_greens_identity_converges():
    # alpha u + N u - D du/dn -> 0 for a harmonic u (O(h^2) collocation error)
    errs = []
    for n in (800, 2000):
        P, m, b = oracle_problem("wigley", n)
        X = m.X
        u = X[:, 0] * X[:, 1] + X[:, 2]
        gu = np.stack([X[:, 1], X[:, 0], np.ones(len(X))], 1)
        un = np.einsum("ij,ij->i", gu, m.normal)
        r = P.alpha * u + P.Nm @ u - P.Dm @ un
        errs.append(np.sqrt(np.mean(r ** 2)))
    assert errs[1] < 0.8 * errs[0] and errs[1] < 5e-4


def test_sphere_exact_solution_converges():
    errs = []
    for n in (8, 16):
        P, m, b = oracle_problem("sphere", n)
        _, _, _, p, dpdn = sphere(n)
        phi, dphi, _ = P.solve_system(p)
        errs.append(rel2(dphi, dpdn))
    assert errs[0] < 0.02 and errs[1] < errs[0] / 3


def test_reference_gmres_matches_direct_solve():
    P, m, b = oracle_problem("wigley", 2000)
    phi, dphi, _ = P.solve_system(b)
    phi2, dphi2, st, it, res = P.solve_system_gmres(b, tol=1e-13)
    assert st == 0 and it < 200
    assert rel2(phi2, phi) < 1e-10 and rel2(dphi2, dphi) < 1e-10


def test_constraints_dirichlet_neumann_and_neumann_neumann():
    P, m, b = oracle_problem("wigley", 2000)
    flags, inh, (er, ec, ev) = P.constraints(b)
    d = m.dirichlet.astype(bool)
    ptr, idx = P.dn_ptr, P.dn_idx
    n_dn = n_nn = 0
    for i in np.nonzero(flags)[0]:
        s = idx[ptr[i]:ptr[i + 1]]
        dir_members = [j for j in s if d[j]]
        assert not d[i]  # only Neumann members are constrained here (no D-D pairs)
        if dir_members:
            first = dir_members[0]
            assert inh[i] == b[first] and not np.any(er == i)
            n_dn += 1
        else:
            first = s[0]
            assert i != first
            k = np.nonzero(er == i)[0]
            assert len(k) == 1 and ec[k[0]] == first and ev[k[0]] == 1.0
            n_nn += 1
    assert n_dn > 0 and n_nn > 0


def _cube_dirichlet(n=6):
    # all-Dirichlet unit cube, every face its own patch (sharp D-D edges)
    t = np.linspace(0, 1, n + 1)
    pts, cells = [], []
    off = 0
    for ax in range(3):
        for side, sgn in ((0.0, -1), (1.0, 1)):
            U, V = np.meshgrid(t, t, indexing="xy")
            P = np.zeros(U.shape + (3,))
            a1, a2 = [k for k in range(3) if k != ax]
            P[..., ax] = side
            P[..., a1] = U
            P[..., a2] = V
            P = P.reshape(-1, 3)
            c = []
            for l in range(n):
                for k in range(n):
                    i0 = l * (n + 1) + k
                    c.append([i0, i0 + 1, i0 + n + 1, i0 + n + 2])
            c = np.array(c)
            e1 = np.zeros(3); e1[a1] = 1
            e2 = np.zeros(3); e2[a2] = 1
            nrm = np.cross(e1, e2)
            if nrm[ax] * sgn < 0:
                c = c[:, [0, 2, 1, 3]]
            pts.append(P)
            cells.append(c + off)
            off += len(P)
    return np.concatenate(pts), np.concatenate(cells).astype(np.int32)


def test_constraints_dirichlet_dirichlet_sharp_edges():
    X, cells = _cube_dirichlet(6)
    ptr, idx = M.double_nodes(X, cells)
    mask = np.ones(len(X), np.uint8)
    g = np.array([1.0, 2.0, -0.5])
    phi = X @ g  # linear, harmonic
    P = O.Problem(X, cells, ptr, idx, mask)
    flags, inh, (er, ec, ev) = P.constraints(phi)
    nn = P.node_normals()
    # on sharp edges both normal derivatives are fixed to the exact g . n
    k = np.nonzero(flags)[0]
    assert len(k) > 0 and len(er) == 0
    assert np.abs(inh[k] - nn[k] @ g).max() < 1e-10


def test_constraints_dirichlet_dirichlet_flat_edge():
    # free surface split in two patches along x = 0: flat D-D double nodes
    t = np.linspace(0, 1, 5)
    X1 = np.array([[x, y, 0.0] for y in t for x in t - 1.0])
    X2 = np.array([[x, y, 0.0] for y in t for x in t])
    X = np.concatenate([X1, X2])
    c = []
    for off in (0, 25):
        for l in range(4):
            for k in range(4):
                i0 = off + l * 5 + k
                c.append([i0, i0 + 1, i0 + 5, i0 + 6])
    cells = np.array(c, np.int32)
    ptr, idx = M.double_nodes(X, cells)
    mask = np.ones(len(X), np.uint8)
    P = O.Problem(X, cells, ptr, idx, mask)
    flags, inh, (er, ec, ev) = P.constraints(np.sin(X[:, 0]))
    k = np.nonzero(flags)[0]
    assert len(k) == 5
    for i in k:
        j = np.nonzero(er == i)[0]
        assert len(j) == 1 and ev[j[0]] == 1.0 and ec[j[0]] < i


def test_double_nodes_match_reference_rule():
    m, ptr, idx, b = wigley(800)
    sizes = np.diff(ptr)
    bnd = M.boundary_nodes(m.cells, m.n_dofs)
    assert np.all(sizes[~bnd] == 1)
    for i in np.nonzero(sizes > 1)[0]:
        s = idx[ptr[i]:ptr[i + 1]]
        assert i in s and np.all(np.diff(s) > 0)
        assert np.abs(m.X[s] - m.X[i]).max() < 1e-8
