"""The FMA method ("Solution method = FMA" of the reference,
source/bem_problem.cc:87 and source/bem_fma.cc): the collocation operators
through an octree with an exact near field and Chebyshev-interpolation
expansions for the far field, against the dense FP64 operators of the same
mesh (which the oracle pins).

Tolerances (measured on the N = 8,192 tank, with about a 3x margin): the far
field's error falls about sevenfold per order (the dipoles are expansion
sets of their own, their kernel gradient applied exactly in the M2L). At the
default order 6 the operators agree with the dense ones to 1.4e-5 in the
relative 2-norm, alpha to 5.6e-5 of its largest entry, phi to 1.1e-5 and
dphi/dn to 5.1e-5; at order 8 the operator error is 2.8e-7 and alpha's
2.0e-6."""
import numpy as np
import pytest

from helpers import rel2
from wavebem_gb300 import meshes as M
from wavebem_gb300.bem_problem import METHOD_FMA, PREC_FP64, BEMProblem, WBEMError

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def tank8192():
    m, ptr, idx, b = M.config_case("c3")
    g = BEMProblem(m.X, m.cells, m.dirichlet, ptr, idx, precision=PREC_FP64)
    g.assemble_system()
    phi, dphi = b.copy(), b.copy()
    g.solve_system(phi, dphi, b)
    return m, ptr, idx, b, g, phi, dphi


def _fma(m, ptr, idx, order=6, **kw):
    return BEMProblem(m.X, m.cells, m.dirichlet, ptr, idx, method=METHOD_FMA, fma_order=order,
                      **kw)


def test_fma_operators_and_alpha_against_dense(tank8192):
    m, ptr, idx, b, g, _, _ = tank8192
    v = np.random.default_rng(3).normal(size=m.n_dofs)
    ref_v, ref_r, ref_a = g.vmult(v), g.compute_rhs(v), g.compute_alpha()
    errs = {}
    for order in (4, 6, 8):
        f = _fma(m, ptr, idx, order)
        f.assemble_system()
        ev, er = rel2(f.vmult(v), ref_v), rel2(f.compute_rhs(v), ref_r)
        ea = np.abs(f.compute_alpha() - ref_a).max() / np.abs(ref_a).max()
        errs[order] = (ev, er, ea)
        print(f"order {order}: vmult {ev:.2e} rhs {er:.2e} alpha {ea:.2e}")
        f.close()
    assert max(errs[6][:2]) <= 5e-5 and errs[6][2] <= 2e-4
    assert max(errs[8][:2]) <= 1e-6 and errs[8][2] <= 6e-6
    # convergence in the order
    assert errs[6][0] < errs[4][0] / 10 and errs[8][0] < errs[6][0] / 10


def test_fma_solution_and_force_against_dense(tank8192):
    m, ptr, idx, b, g, phi_d, dphi_d = tank8192
    f = _fma(m, ptr, idx)
    phi, dphi = b.copy(), b.copy()
    f.solve(phi, dphi, b)
    ep, ed = rel2(phi, phi_d), rel2(dphi, dphi_d)
    hull = np.nonzero(m.face == M.HULL)[0].astype(np.int32)
    F, Fd = f.hull_force(hull, phi, dphi), g.hull_force(hull, phi_d, dphi_d)
    print(f"phi {ep:.2e} dphi {ed:.2e} force {abs(F - Fd) / abs(Fd):.2e}")
    assert ep <= 3e-5 and ed <= 1.5e-4
    # F is a near-cancelling integral on this almost symmetric hull (|F| is
    # 5e-5): its relative error is about ten times that of dphi/dn (4.3e-4)
    assert abs(F - Fd) <= 1.5e-3 * abs(Fd)
    # the solve converged on the operator it applies: the residual of the
    # FMA system at the FMA solution is at the round-off of its FP32 far
    # field (the product is linear to that level only; measured 3e-7)
    res = np.zeros(m.n_dofs)
    f.residual(res, phi, dphi)
    st = f.stats()
    assert st["iterations"] > 0
    assert np.linalg.norm(res) <= 2e-6 * np.linalg.norm(b)


def test_fma_has_no_matrices_and_no_adjoint(tank8192):
    m, ptr, idx, b, g, _, _ = tank8192
    f = _fma(m, ptr, idx, 4)
    phi, dphi = b.copy(), b.copy()
    f.solve(phi, dphi, b)
    with pytest.raises(WBEMError):
        f.matrices()
    with pytest.raises(WBEMError):
        f.adjoint(np.ones(m.n_dofs), np.ones(m.n_dofs))


def test_fma_two_handles_of_different_order(tank8192):
    """Handles share no state: two FMA handles of different orders (and
    different meshes) interleave their products and each gives what it gives
    alone."""
    m, ptr, idx, b, g, _, _ = tank8192
    m2, ptr2, idx2, b2 = M.config_case("c0")
    v = np.random.default_rng(5).normal(size=m.n_dofs)
    v2 = np.random.default_rng(6).normal(size=m2.n_dofs)
    f4 = _fma(m, ptr, idx, 4)
    f4.assemble_system()
    alone = f4.vmult(v)
    f7 = _fma(m2, ptr2, idx2, 7)
    f7.assemble_system()
    alone2 = f7.vmult(v2)
    for _ in range(2):
        assert np.array_equal(f4.vmult(v), alone)
        assert np.array_equal(f7.vmult(v2), alone2)


def test_fma_sphere_beyond_dense_size():
    """A cube-sphere of 135,002 nodes (dense N and D would need 290 GB): the
    FMA solve at order 8 against the exact normal derivative of a harmonic
    polynomial."""
    m = M.cube_sphere_mesh(150)
    ptr, idx = M.double_nodes(m.X, m.cells)
    p, dpdn = M.sphere_harmonics(m.X, seed=1)
    f = BEMProblem(m.X, m.cells, m.dirichlet, ptr, idx, method=METHOD_FMA, fma_order=8,
                   max_steps=2000)
    phi, dphi = p.copy(), np.zeros_like(p)
    f.solve(phi, dphi, p)
    e = rel2(dphi, dpdn)
    print(f"sphere N={m.n_dofs}: dphi vs exact {e:.2e}, {f.stats()['iterations']} iterations")
    assert e < 1e-3


def test_fma_refuses_a_mesh_too_coarse_for_two_levels():
    """The 866-node cube-sphere: its panels are too large for the leaf margin
    of a two-level tree, so the FMA assembly reports an argument error."""
    from helpers import sphere
    m, ptr, idx, p, dpdn = sphere(12)
    f = _fma(m, ptr, idx)
    with pytest.raises(WBEMError):
        f.assemble_system()


def test_fma_sphere_and_moved_nodes():
    """A 9,602-node cube-sphere against the dense FP64 operator, and the same
    handle after its nodes move (update_nodes rebuilds the tree and the
    close pairs) against a new handle on the moved mesh."""
    from helpers import sphere
    m, ptr, idx, p, dpdn = sphere(40)
    v = np.random.default_rng(11).normal(size=m.n_dofs)
    g = BEMProblem(m.X, m.cells, m.dirichlet, ptr, idx, precision=PREC_FP64)
    g.assemble_system()
    f = _fma(m, ptr, idx, 8)
    f.assemble_system()
    # the octree and lists are built by the first assembly only
    assert f.stats()["t_assemble_ms"] > 0
    f.assemble_system()
    assert f.stats()["t_assemble_ms"] == 0
    e1 = rel2(f.vmult(v), g.vmult(v))
    # a smooth displacement of every node (double nodes move together)
    X2 = m.X * (1.0 + 0.05 * np.sin(3.0 * m.X[:, :1]))
    f.update_nodes(X2)
    f.assemble_system()
    assert f.stats()["t_assemble_ms"] > 0  # rebuilt for the moved nodes
    fresh = BEMProblem(X2, m.cells, m.dirichlet, ptr, idx, method=METHOD_FMA, fma_order=8)
    fresh.assemble_system()
    assert np.array_equal(f.vmult(v), fresh.vmult(v))
    g2 = BEMProblem(X2, m.cells, m.dirichlet, ptr, idx, precision=PREC_FP64)
    g2.assemble_system()
    e2 = rel2(f.vmult(v), g2.vmult(v))
    print(f"sphere n=40 order 8: vmult {e1:.2e}, moved {e2:.2e}")
    assert e1 <= 2e-5 and e2 <= 2e-5
