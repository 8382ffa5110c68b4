"""wbem_hull_force_noalloc: the hull force for callers that must not allocate
device memory (a time loop evaluating the force every Newton iteration on its
own stream, or device memory owned by another framework's allocator). It must
give the same force as wbem_hull_force, call after call, while keeping its
partial sums in the library's fixed device array. This file is collected last."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _lib():
    from wavebem_gb300.bem_problem import load_library
    L = load_library()
    L.wbem_hull_force_noalloc.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                          np.ctypeslib.ndpointer(np.float64, flags="C"),
                                          ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                          ctypes.c_void_p, ctypes.c_void_p]
    return L


def _setup():
    from wavebem_gb300 import meshes as M
    from wavebem_gb300.bem_problem import BEMProblem
    m = M.wigley_mesh(2000)
    ptr, idx = M.double_nodes(m.X, m.cells)
    hull = np.nonzero(m.face == M.HULL)[0].astype(np.int32)
    bem = BEMProblem(m.X, m.cells, m.dirichlet, ptr, idx)
    return m, hull, bem


def test_noalloc_hull_force_matches_allocating_entry_point_twice():
    torch = pytest.importorskip("torch")
    from wavebem_gb300 import meshes as M
    L = _lib()
    m, hull, bem = _setup()
    U = np.array([1.0, 0.0, 0.0])
    d_hull = torch.from_numpy(hull).cuda()
    d_force = torch.full((1,), -7.0, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream()
    for seed in (0, 5):  # two calls in a row with different fields
        b = M.wigley_bc(m, seed=seed)
        phi, dphi = b.copy(), b.copy()
        bem.solve(phi, dphi, b)
        F_ref = bem.hull_force(hull, phi, dphi, U=U)
        d_phi = torch.from_numpy(phi).cuda()
        d_dphi = torch.from_numpy(dphi).cuda()
        st = L.wbem_hull_force_noalloc(bem.h, d_hull.data_ptr(), hull.size, U, 0, d_phi.data_ptr(),
                                       d_dphi.data_ptr(), d_force.data_ptr(),
                                       ctypes.c_void_p(stream.cuda_stream))
        assert st == 0, L.wbem_last_error(bem.h)
        torch.cuda.synchronize()
        F = float(d_force.item())
        assert abs(F - F_ref) <= 1e-12 * max(1.0, abs(F_ref)), (F, F_ref)


def test_noalloc_rejects_hulls_beyond_the_static_array():
    L = _lib()
    m, hull, bem = _setup()
    st = L.wbem_hull_force_noalloc(bem.h, None, 65537, np.array([1.0, 0.0, 0.0]), 0, None, None,
                                   None, None)
    assert st != 0
    st = L.wbem_hull_force_noalloc(bem.h, ctypes.c_void_p(1), 65537, np.array([1.0, 0.0, 0.0]), 0,
                                   ctypes.c_void_p(1), ctypes.c_void_p(1), ctypes.c_void_p(1), None)
    assert st == 1 and b"65536" in L.wbem_last_error(bem.h)
