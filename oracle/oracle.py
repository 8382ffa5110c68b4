"""ctypes bindings of the CPU oracle (test infrastructure only)."""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = os.path.join(_HERE, "liboracle.so")
_lib = None

dp = np.ctypeslib.ndpointer(np.float64, flags="C")
ip = np.ctypeslib.ndpointer(np.int32, flags="C")
up = np.ctypeslib.ndpointer(np.uint8, flags="C")


def build(force: bool = False) -> str:
    src = os.path.join(_HERE, "wbem_oracle.cpp")
    if force or not os.path.exists(_LIB) or os.path.getmtime(_LIB) < os.path.getmtime(src):
        subprocess.check_call(["make", "-s", "-C", _HERE, "liboracle.so"])
    return _LIB


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(_LIB)
        L.orc_gauss01.argtypes = [C.c_int, dp, dp]
        L.orc_singular_rule.argtypes = [C.c_int, C.c_int, dp, dp, dp]
        L.orc_assemble.argtypes = [C.c_int, dp, C.c_int, ip, ip, ip, C.c_int, C.c_int, dp, dp]
        L.orc_assemble_rows.argtypes = [C.c_int, dp, C.c_int, ip, ip, ip, C.c_int, C.c_int,
                                        C.c_int, C.c_int, dp, dp]
        L.orc_alpha.argtypes = [C.c_int, dp, dp]
        L.orc_compute_rhs.argtypes = [C.c_int, dp, dp, dp, up, dp, dp]
        L.orc_vmult.argtypes = [C.c_int, dp, dp, dp, up, dp, dp]
        L.orc_constraints.argtypes = [C.c_int, dp, C.c_int, ip, C.c_int, ip, ip, up, dp, up, dp,
                                      C.c_int, ip, ip, dp]
        L.orc_node_normals.argtypes = [C.c_int, dp, C.c_int, ip, C.c_int, dp]
        L.orc_surface_gradients.argtypes = [C.c_int, dp, C.c_int, ip, C.c_int, up, dp, dp]
        L.orc_system.argtypes = [C.c_int, dp, C.c_int, ip, C.c_int, ip, ip, dp, dp, dp, up, dp,
                                 dp, dp]
        L.orc_solve_system.argtypes = [C.c_int, dp, C.c_int, ip, C.c_int, ip, ip, dp, dp, dp, up,
                                       dp, dp, dp, dp]
        L.orc_solve_system_gmres.argtypes = [C.c_int, dp, C.c_int, ip, C.c_int, ip, ip, dp, dp,
                                             dp, up, dp, C.c_int, C.c_int, C.c_double, C.c_int,
                                             dp, dp, C.POINTER(C.c_int), C.POINTER(C.c_double)]
        L.orc_hull_force.argtypes = [C.c_int, dp, C.c_int, ip, C.c_int, dp, dp, dp]
        L.orc_hull_force.restype = C.c_double
        L.orc_num_threads.restype = C.c_int
        L.orc_set_threads.argtypes = [C.c_int]
        _lib = L
    return _lib


def _c(a, dt):
    return np.ascontiguousarray(a, dtype=dt)


def gauss01(n):
    x = np.zeros(n); w = np.zeros(n)
    lib().orc_gauss01(n, x, w)
    return x, w


def singular_rule(n, v):
    px = np.zeros(2 * n * n); py = np.zeros(2 * n * n); w = np.zeros(2 * n * n)
    lib().orc_singular_rule(n, v, px, py, w)
    return px, py, w


class Problem:
    """One mesh + Dirichlet mask, with the oracle's FP64 operators."""

    def __init__(self, X, cells, dn_ptr, dn_idx, dirichlet, qorder=4, sorder=5):
        self.X = _c(X, np.float64).reshape(-1, 3)
        self.cells = _c(cells, np.int32).reshape(-1, 4)
        self.dn_ptr = _c(dn_ptr, np.int32)
        self.dn_idx = _c(dn_idx, np.int32)
        self.mask = _c(dirichlet, np.uint8)
        self.N = self.X.shape[0]
        self.C = self.cells.shape[0]
        self.qorder, self.sorder = qorder, sorder
        self.Nm = self.Dm = self.alpha = None

    def assemble(self, rows=None):
        L = lib()
        N = self.N
        if rows is None:
            Nm = np.zeros((N, N)); Dm = np.zeros((N, N))
            L.orc_assemble_rows(N, self.X.ravel(), self.C, self.cells.ravel(), self.dn_ptr,
                                self.dn_idx, self.qorder, self.sorder, 0, N, Nm.ravel(), Dm.ravel())
            self.Nm, self.Dm = Nm, Dm
            self.alpha = self.compute_alpha()
            return Nm, Dm
        r0, r1 = rows
        Nm = np.zeros((r1 - r0, N)); Dm = np.zeros((r1 - r0, N))
        L.orc_assemble_rows(N, self.X.ravel(), self.C, self.cells.ravel(), self.dn_ptr,
                            self.dn_idx, self.qorder, self.sorder, r0, r1, Nm.ravel(), Dm.ravel())
        return Nm, Dm

    def assemble_serial(self):
        N = self.N
        Nm = np.zeros((N, N)); Dm = np.zeros((N, N))
        lib().orc_assemble(N, self.X.ravel(), self.C, self.cells.ravel(), self.dn_ptr, self.dn_idx,
                           self.qorder, self.sorder, Nm.ravel(), Dm.ravel())
        return Nm, Dm

    def compute_alpha(self):
        a = np.zeros(self.N)
        lib().orc_alpha(self.N, self.Nm.ravel(), a)
        return a

    def compute_rhs(self, src):
        d = np.zeros(self.N)
        lib().orc_compute_rhs(self.N, self.Nm.ravel(), self.Dm.ravel(), self.alpha, self.mask,
                              _c(src, np.float64), d)
        return d

    def vmult(self, src):
        d = np.zeros(self.N)
        lib().orc_vmult(self.N, self.Nm.ravel(), self.Dm.ravel(), self.alpha, self.mask,
                        _c(src, np.float64), d)
        return d

    def constraints(self, tmp_rhs, max_entries=None):
        N = self.N
        me = max_entries or 8 * N + 16
        flags = np.zeros(N, np.uint8); inh = np.zeros(N)
        er = np.zeros(me, np.int32); ec = np.zeros(me, np.int32); ev = np.zeros(me)
        ne = lib().orc_constraints(N, self.X.ravel(), self.C, self.cells.ravel(), self.qorder,
                                   self.dn_ptr, self.dn_idx, self.mask, _c(tmp_rhs, np.float64),
                                   flags, inh, me, er, ec, ev)
        if ne < 0:
            raise RuntimeError("too many constraint entries")
        return flags, inh, (er[:ne], ec[:ne], ev[:ne])

    def node_normals(self):
        nn = np.zeros(3 * self.N)
        lib().orc_node_normals(self.N, self.X.ravel(), self.C, self.cells.ravel(), self.qorder, nn)
        return nn.reshape(-1, 3)

    def surface_gradients(self, tmp_rhs):
        g = np.zeros(3 * self.N)
        lib().orc_surface_gradients(self.N, self.X.ravel(), self.C, self.cells.ravel(),
                                    self.qorder, self.mask, _c(tmp_rhs, np.float64), g)
        return g.reshape(-1, 3)

    def system(self, tmp_rhs):
        N = self.N
        A = np.zeros((N, N)); rhs = np.zeros(N)
        lib().orc_system(N, self.X.ravel(), self.C, self.cells.ravel(), self.qorder, self.dn_ptr,
                         self.dn_idx, self.Nm.ravel(), self.Dm.ravel(), self.alpha, self.mask,
                         _c(tmp_rhs, np.float64), A.ravel(), rhs)
        return A, rhs

    def solve_system(self, tmp_rhs, phi=None, dphi_dn=None):
        N = self.N
        b = _c(tmp_rhs, np.float64)
        phi = b.copy() if phi is None else _c(phi, np.float64).copy()
        dphi = b.copy() if dphi_dn is None else _c(dphi_dn, np.float64).copy()
        sol = np.zeros(N)
        st = lib().orc_solve_system(N, self.X.ravel(), self.C, self.cells.ravel(), self.qorder,
                                    self.dn_ptr, self.dn_idx, self.Nm.ravel(), self.Dm.ravel(),
                                    self.alpha, self.mask, b, phi, dphi, sol)
        if st:
            raise RuntimeError(f"oracle solve failed ({st})")
        return phi, dphi, sol

    def solve_system_gmres(self, tmp_rhs, restart=100, max_steps=1000, tol=1e-10, band=100):
        N = self.N
        b = _c(tmp_rhs, np.float64)
        phi = b.copy(); dphi = b.copy()
        it = C.c_int(0); res = C.c_double(0)
        st = lib().orc_solve_system_gmres(N, self.X.ravel(), self.C, self.cells.ravel(),
                                          self.qorder, self.dn_ptr, self.dn_idx, self.Nm.ravel(),
                                          self.Dm.ravel(), self.alpha, self.mask, b, restart,
                                          max_steps, tol, band, phi, dphi, C.byref(it),
                                          C.byref(res))
        return phi, dphi, st, it.value, res.value

    def hull_force(self, hull_cells, phi, dphi_dn, U=(1.0, 0.0, 0.0)):
        hc = _c(hull_cells, np.int32)
        return lib().orc_hull_force(self.N, self.X.ravel(), hc.shape[0], hc.ravel(), self.qorder,
                                    _c(U, np.float64), _c(phi, np.float64), _c(dphi_dn, np.float64))


def num_threads():
    return lib().orc_num_threads()


def set_threads(n):
    lib().orc_set_threads(int(n))
