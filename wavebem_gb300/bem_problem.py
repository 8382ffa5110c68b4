"""Host-side mirror of WaveBEM's BEMProblem<3> over the C ABI (include/wbem.h).

The member names and argument meanings follow the reference class
(include/bem_problem.h:87-180): `reinit`, `assemble_system`, `compute_alpha`,
`solve_system(phi, dphi_dn, tmp_rhs)`, `solve(phi, dphi_dn, tmp_rhs)`,
`vmult`, `compute_rhs`, with `neumann_matrix` / `dirichlet_matrix` / `alpha`
available after assembly. Errors raise `WBEMError` (the reference throws
deal.II exceptions; GMRES non-convergence is `NoConvergence`, like
SolverControl::NoConvergence).

Everything runs in the CUDA library `libwbem.so`; there is no CPU fallback.
Loading fails loudly if the library has not been built.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libwbem.so")

WBEM_OK = 0
STATUS = {1: "ERR_ARG", 2: "ERR_STATE", 3: "ERR_CUDA", 4: "ERR_NOMEM", 5: "ERR_SINGULAR",
          6: "ERR_NOCONV", 7: "ERR_NONFINITE", 8: "ERR_TIMEOUT"}
PREC_FP64, PREC_MIXED = 0, 1
SOLVER_AUTO, SOLVER_GMRES, SOLVER_LU, SOLVER_GMRES_IR = 0, 1, 2, 3
METHOD_DIRECT, METHOD_FMA = 0, 1

# every entry point declared in include/wbem.h
EXPORTS = ["wbem_default_options", "wbem_create", "wbem_destroy", "wbem_last_error",
           "wbem_set_geometry", "wbem_update_nodes", "wbem_set_bc", "wbem_assemble",
           "wbem_solve_system", "wbem_solve", "wbem_get_alpha", "wbem_get_matrices",
           "wbem_vmult", "wbem_compute_rhs", "wbem_residual", "wbem_node_normals",
           "wbem_surface_gradients", "wbem_hull_force", "wbem_force_adjoint", "wbem_adjoint",
           "wbem_get_stats"]


class WBEMError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{STATUS.get(code, code)}: {msg}")
        self.code = code


class NoConvergence(WBEMError):
    pass


class Options(C.Structure):
    _fields_ = [("precision", C.c_int), ("solver", C.c_int), ("quadrature_order", C.c_int),
                ("singular_quadrature_order", C.c_int), ("gmres_restart", C.c_int),
                ("max_steps", C.c_int), ("tolerance", C.c_double),
                ("near_field_ratio", C.c_double), ("keep_matrices", C.c_int),
                ("inner_digits", C.c_int), ("method", C.c_int), ("fma_order", C.c_int),
                ("reserved", C.c_int * 4)]


class Stats(C.Structure):
    _fields_ = [("t_geometry_ms", C.c_double), ("t_assemble_ms", C.c_double),
                ("t_singular_ms", C.c_double), ("t_alpha_ms", C.c_double),
                ("t_system_ms", C.c_double), ("t_factor_ms", C.c_double),
                ("t_solve_ms", C.c_double), ("t_adjoint_ms", C.c_double),
                ("iterations", C.c_int), ("residual", C.c_double),
                ("kernel_launches", C.c_int), ("n_dofs", C.c_int), ("n_cells", C.c_int),
                ("outer_iterations", C.c_int), ("reserved", C.c_int * 7)]


_lib = None
dp = np.ctypeslib.ndpointer(np.float64, flags="C")
ip = np.ctypeslib.ndpointer(np.int32, flags="C")
up = np.ctypeslib.ndpointer(np.uint8, flags="C")


def load_library(path: str = LIB_PATH):
    """Load libwbem.so; raises if it is missing (no fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise ImportError(f"{path} not found: build it with `python -c 'import __graft_entry__ as g; g.build()'`")
    L = C.CDLL(path)
    H = C.c_void_p
    L.wbem_default_options.argtypes = [C.POINTER(Options)]
    L.wbem_create.argtypes = [C.POINTER(H), C.c_int]
    L.wbem_destroy.argtypes = [H]
    L.wbem_last_error.argtypes = [H]
    L.wbem_last_error.restype = C.c_char_p
    L.wbem_set_geometry.argtypes = [H, dp, C.c_int, ip, C.c_int, C.c_void_p, C.c_void_p]
    L.wbem_update_nodes.argtypes = [H, dp]
    L.wbem_set_bc.argtypes = [H, up]
    L.wbem_assemble.argtypes = [H, C.POINTER(Options)]
    L.wbem_solve_system.argtypes = [H, dp, dp, dp]
    L.wbem_solve.argtypes = [H, C.POINTER(Options), dp, dp, dp]
    L.wbem_get_alpha.argtypes = [H, dp]
    L.wbem_get_matrices.argtypes = [H, C.c_void_p, C.c_void_p]
    L.wbem_vmult.argtypes = [H, dp, dp]
    L.wbem_compute_rhs.argtypes = [H, dp, dp]
    L.wbem_residual.argtypes = [H, dp, dp, dp]
    L.wbem_node_normals.argtypes = [H, dp]
    L.wbem_surface_gradients.argtypes = [H, dp, dp]
    L.wbem_hull_force.argtypes = [H, ip, C.c_int, dp, C.c_int, dp, dp, C.POINTER(C.c_double)]
    L.wbem_force_adjoint.argtypes = [H, ip, C.c_int, dp, C.c_int, dp, dp, dp]
    L.wbem_adjoint.argtypes = [H, dp, dp, dp, dp]
    L.wbem_get_stats.argtypes = [H, C.POINTER(Stats)]
    L.wbem_test_lu_factors.argtypes = [H, C.c_void_p, C.c_void_p, C.c_void_p]
    L.wbem_test_lu_apply.argtypes = [H, dp, dp, C.c_int]
    _lib = L
    return L


def default_options(**kw) -> Options:
    o = Options()
    load_library().wbem_default_options(C.byref(o))
    for k, v in kw.items():
        setattr(o, k, v)
    return o


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


class BEMProblem:
    """GPU drop-in for BEMProblem<3> on one mesh (one handle, one device)."""

    def __init__(self, X, cells, dirichlet=None, dn_ptr=None, dn_idx=None, device=0, **options):
        self.L = load_library()
        self.h = C.c_void_p()
        st = self.L.wbem_create(C.byref(self.h), int(device))
        if st != WBEM_OK:
            raise WBEMError(st, "wbem_create failed (no usable CUDA device?)")
        self.options = default_options(**options)
        self.set_geometry(X, cells, dn_ptr, dn_idx)
        if dirichlet is not None:
            self.set_bc(dirichlet)

    def set_geometry(self, X, cells, dn_ptr=None, dn_idx=None):
        """A new mesh (support points, Q1 cells, double-node sets) for this
        handle; a mesh of another size re-allocates the device buffers."""
        self.X = _f64(X).reshape(-1, 3)
        self.cells = np.ascontiguousarray(cells, dtype=np.int32).reshape(-1, 4)
        self.n_dofs = self.X.shape[0]
        if dn_ptr is not None:
            self._dn = (np.ascontiguousarray(dn_ptr, np.int32), np.ascontiguousarray(dn_idx, np.int32))
            pp, pi = self._dn[0].ctypes.data_as(C.c_void_p), self._dn[1].ctypes.data_as(C.c_void_p)
        else:
            self._dn = None
            pp = pi = None
        self._check(self.L.wbem_set_geometry(self.h, self.X.ravel(), self.n_dofs, self.cells.ravel(),
                                             self.cells.shape[0], pp, pi))

    # -- plumbing
    def _check(self, st):
        if st != WBEM_OK:
            msg = self.L.wbem_last_error(self.h).decode()
            if st == 6:
                raise NoConvergence(st, msg)
            raise WBEMError(st, msg)

    def close(self):
        if self.h:
            self.L.wbem_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- reference interface
    def set_bc(self, dirichlet):
        """comp_dom.surface_nodes (1 = Dirichlet)."""
        self.surface_nodes = np.ascontiguousarray(dirichlet, np.uint8)
        self._check(self.L.wbem_set_bc(self.h, self.surface_nodes))

    def update_nodes(self, X):
        self.X = _f64(X).reshape(-1, 3)
        self._check(self.L.wbem_update_nodes(self.h, self.X.ravel()))

    def reinit(self):
        """Matrices are (re)allocated on the device by assemble_system."""
        return None

    def assemble_system(self, **options):
        o = default_options(**{**self._opt_dict(), **options})
        self.options = o
        self._check(self.L.wbem_assemble(self.h, C.byref(o)))

    def compute_alpha(self):
        a = np.zeros(self.n_dofs)
        self._check(self.L.wbem_get_alpha(self.h, a))
        self.alpha = a
        return a

    def solve_system(self, phi, dphi_dn, tmp_rhs):
        """Writes phi on Neumann nodes and dphi_dn on Dirichlet nodes, in place."""
        phi_a = _f64(phi).copy()
        dphi_a = _f64(dphi_dn).copy()
        self._check(self.L.wbem_solve_system(self.h, _f64(tmp_rhs), phi_a, dphi_a))
        phi[...] = phi_a
        dphi_dn[...] = dphi_a
        return phi, dphi_dn

    def solve(self, phi, dphi_dn, tmp_rhs, **options):
        self.assemble_system(**options)
        return self.solve_system(phi, dphi_dn, tmp_rhs)

    def vmult(self, src):
        dst = np.zeros(self.n_dofs)
        self._check(self.L.wbem_vmult(self.h, _f64(src), dst))
        return dst

    def compute_rhs(self, src):
        dst = np.zeros(self.n_dofs)
        self._check(self.L.wbem_compute_rhs(self.h, _f64(src), dst))
        return dst

    def residual(self, res, phi, dphi_dn):
        """BEMProblem::residual (source/bem_problem.cc:903-961): res = A_c sol -
        rhs_c, with the known data of (phi, dphi_dn) forming the right-hand side
        and the unknown entries the solution vector."""
        out = np.zeros(self.n_dofs)
        self._check(self.L.wbem_residual(self.h, _f64(phi), _f64(dphi_dn), out))
        res[:] = out
        return res

    def compute_normals(self):
        """ComputationalDomain::compute_normals: L2-projected node normals (N, 3)."""
        n = np.zeros(3 * self.n_dofs)
        self._check(self.L.wbem_node_normals(self.h, n))
        return n.reshape(-1, 3)

    def compute_surface_gradients(self, tmp_rhs):
        """BEMProblem::compute_surface_gradients: L2-projected surface gradients
        (N, 3) of tmp_rhs on the Dirichlet nodes (zero elsewhere)."""
        g = np.zeros(3 * self.n_dofs)
        self._check(self.L.wbem_surface_gradients(self.h, _f64(tmp_rhs), g))
        return g.reshape(-1, 3)

    def matrices(self, neumann=True, dirichlet=True):
        N = self.n_dofs
        Nm = np.zeros((N, N)) if neumann else None
        Dm = np.zeros((N, N)) if dirichlet else None
        self._check(self.L.wbem_get_matrices(
            self.h, Nm.ctypes.data_as(C.c_void_p) if neumann else None,
            Dm.ctypes.data_as(C.c_void_p) if dirichlet else None))
        return Nm, Dm

    @property
    def neumann_matrix(self):
        return self.matrices(True, False)[0]

    @property
    def dirichlet_matrix(self):
        return self.matrices(False, True)[1]

    def hull_force(self, hull_cells, phi, dphi_dn, U=(1.0, 0.0, 0.0), direction=0):
        F = C.c_double(0)
        hc = np.ascontiguousarray(hull_cells, np.int32)
        self._check(self.L.wbem_hull_force(self.h, hc, hc.size, _f64(U), int(direction), _f64(phi),
                                           _f64(dphi_dn), C.byref(F)))
        return F.value

    def force_adjoint(self, hull_cells, tmp_rhs, U=(1.0, 0.0, 0.0), direction=0):
        """dF/dX (N,3) with tmp_rhs fixed, and dF/dtmp_rhs (N,), at the last solve."""
        gX = np.zeros(3 * self.n_dofs)
        gb = np.zeros(self.n_dofs)
        hc = np.ascontiguousarray(hull_cells, np.int32)
        self._check(self.L.wbem_force_adjoint(self.h, hc, hc.size, _f64(U), int(direction),
                                              _f64(tmp_rhs), gX, gb))
        return gX.reshape(-1, 3), gb

    def adjoint(self, dJ_dphi, dJ_ddn):
        """dJ/dX (N,3) with tmp_rhs fixed, and dJ/dtmp_rhs (N,), at the last solve,
        for an objective J(phi, dphi_dn) with the given partial derivatives."""
        a, c = _f64(dJ_dphi).ravel(), _f64(dJ_ddn).ravel()
        if a.size != self.n_dofs or c.size != self.n_dofs:
            raise ValueError("dJ_dphi and dJ_ddn need one entry per dof")
        gX = np.zeros(3 * self.n_dofs)
        gb = np.zeros(self.n_dofs)
        self._check(self.L.wbem_adjoint(self.h, a, c, gX, gb))
        return gX.reshape(-1, 3), gb

    def lu_factors(self):
        """(S, LU, perm) of the current mixed assembly: the FP32 system matrix and
        its packed FP32 factors in the internal dof order, perm[k] = caller dof
        of internal dof k (factor tests)."""
        N = self.n_dofs
        S = np.zeros((N, N), np.float32)
        LU = np.zeros((N, N), np.float32)
        perm = np.zeros(N, np.int32)
        self._check(self.L.wbem_test_lu_factors(self.h, S.ctypes.data_as(C.c_void_p),
                                                LU.ctypes.data_as(C.c_void_p),
                                                perm.ctypes.data_as(C.c_void_p)))
        return S, LU, perm

    def lu_apply(self, v, transpose=False):
        """M^{-1} v with the current FP32 LU factors (internal dof order)."""
        z = np.zeros(self.n_dofs)
        self._check(self.L.wbem_test_lu_apply(self.h, _f64(v), z, int(bool(transpose))))
        return z

    def stats(self) -> dict:
        s = Stats()
        self._check(self.L.wbem_get_stats(self.h, C.byref(s)))
        return {k: getattr(s, k) for k, _ in Stats._fields_ if k != "reserved"}

    def _opt_dict(self):
        return {k: getattr(self.options, k) for k, _ in Options._fields_ if k != "reserved"}
