"""Stand-in for the reference's time-integrated run (100 BDF steps of the
Wigley tank at N = 12,000).

The reference integrates its free-surface DAE with SUNDIALS IDA (BDF,
`source/dae_time_integrator.cc:212-305`). Each residual evaluation of the
FreeSurface equations calls `bem.solve` on the updated mesh, and each
Jacobian-vector product calls `bem.solve_system` with the matrices of that
assembly (`source/free_surface.cc:4877, 4993, 6103-6108`). Neither SUNDIALS
nor the Sacado FreeSurface residual exists here, so this module keeps the
same calling pattern on a simplified linear free-surface model.

State on the free-surface nodes: elevation eta and potential phi. In the
frame of the hull (forward speed U along x):

    d eta / dt = dphi/dn - U d eta / dx
    d phi / dt = -g eta  - U d phi / dx

dphi/dn comes from the BEM's Dirichlet-to-Neumann map on the current mesh.
The free-surface nodes and their double nodes follow eta vertically. The
integrator is BDF1 on the first step, then BDF2. Newton uses a Jacobian-free
GMRES on the state, and its Jacobian-vector products reuse the assembly of
the residual through solve_system.

This is a stand-in for timing the calling pattern, not a validated wave
model.
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

from . import meshes as M
from .bem_problem import PREC_FP64, PREC_MIXED, BEMProblem


class FreeSurfaceStandIn:
    def __init__(self, n=12000, precision=PREC_MIXED, U=1.0, g=None, Fr=0.316, seed=4,
                 amplitude=1e-3):
        self.m = M.wigley_mesh(n)
        m = self.m
        self.ptr, self.idx = M.double_nodes(m.X, m.cells)
        self.U = U
        self.g = g if g is not None else U * U / (Fr * Fr)  # L = 1
        self.F = np.nonzero(m.dirichlet)[0]                 # free-surface nodes
        # nodes that move with the free surface: F and their double nodes
        mov = set(self.F.tolist())
        for i in self.F:
            mov.update(self.idx[self.ptr[i]:self.ptr[i + 1]].tolist())
        self.moving = np.array(sorted(mov))
        self.owner = {}
        for i in self.F:
            for j in self.idx[self.ptr[i]:self.ptr[i + 1]]:
                self.owner.setdefault(int(j), int(i))
        self.owner_of_moving = np.array([self.owner[int(j)] for j in self.moving])
        self.b0 = amplitude * M.wigley_bc(m, seed=seed)     # Neumann data elsewhere
        self.hull = np.nonzero(m.face == M.HULL)[0].astype(np.int32)
        # free surface patch is the first patch: (nx+1) x (ny+1) nodes, x fastest
        nxl, nxh, nxr, ny, nzh, nzb = m.info["resolution"]
        self.nx1, self.ny1 = nxl + nxh + nxr + 1, ny + 1
        assert self.nx1 * self.ny1 == len(self.F) and np.all(self.F == np.arange(len(self.F)))
        self.xrow = m.X[: self.nx1, 0]
        self.bem = BEMProblem(m.X, m.cells, m.dirichlet, self.ptr, self.idx, precision=precision)
        self.t_bem = 0.0
        self.n_solve = 0
        self.n_assemble = 0

    # ---- BEM calls
    def _mesh(self, eta):
        X = self.m.X.copy()
        X[self.moving, 2] = eta[self.owner_of_moving]
        return X

    def dtn(self, eta, phi, assemble=True):
        """dphi/dn on the free surface for Dirichlet data phi (and the tank's
        Neumann data), on the mesh displaced by eta."""
        b = self.b0.copy()
        b[self.F] = phi
        out_phi, out_dn = b.copy(), b.copy()
        t0 = time.perf_counter()
        if assemble:
            self.bem.update_nodes(self._mesh(eta))
            self.bem.solve(out_phi, out_dn, b)
            self.n_assemble += 1
        else:
            self.bem.solve_system(out_phi, out_dn, b)
        self.t_bem += time.perf_counter() - t0
        self.n_solve += 1
        return out_dn[self.F]

    def dtn_linear(self, v_phi):
        """Frozen-geometry Jacobian of the DtN map (solve_system on the last
        assembly, zero Neumann data)."""
        b = np.zeros_like(self.b0)
        b[self.F] = v_phi
        o1, o2 = b.copy(), b.copy()
        t0 = time.perf_counter()
        self.bem.solve_system(o1, o2, b)
        self.t_bem += time.perf_counter() - t0
        self.n_solve += 1
        return o2[self.F]

    def ddx(self, f):
        return np.gradient(f.reshape(self.ny1, self.nx1), self.xrow, axis=1).ravel()

    def rhs(self, y, assemble=True):
        nF = len(self.F)
        eta, phi = y[:nF], y[nF:]
        dn = self.dtn(eta, phi, assemble)
        return np.concatenate([dn - self.U * self.ddx(eta), -self.g * eta - self.U * self.ddx(phi)])

    def jac_vec(self, v):
        nF = len(self.F)
        ve, vp = v[:nF], v[nF:]
        return np.concatenate([self.dtn_linear(vp) - self.U * self.ddx(ve),
                               -self.g * ve - self.U * self.ddx(vp)])

    def force(self, y):
        nF = len(self.F)
        b = self.b0.copy()
        b[self.F] = y[nF:]
        phi, dn = b.copy(), b.copy()
        self.bem.solve_system(phi, dn, b)
        return self.bem.hull_force(self.hull, phi, dn)

    # ---- BDF with Jacobian-free Newton-GMRES
    def run(self, steps=100, dt=0.01, newton_tol=1e-8, max_newton=4):
        from scipy.sparse.linalg import LinearOperator, gmres
        nF = len(self.F)
        y = np.zeros(2 * nF)
        hist = [y.copy()]
        step_times = []
        newton_res = []
        t_start = time.perf_counter()
        for n in range(steps):
            ts = time.perf_counter()
            if n == 0:
                a0, pred, base = 1.0, y.copy(), y.copy()       # BDF1: y - y0 - h f = 0
            else:
                a0 = 2.0 / 3.0                                   # BDF2
                base = (4.0 * hist[-1] - hist[-2]) / 3.0
                pred = 2.0 * hist[-1] - hist[-2]
            z = pred.copy()
            for it in range(max_newton + 1):
                G = z - base - a0 * dt * self.rhs(z, assemble=True)
                gn = np.linalg.norm(G)
                if gn <= newton_tol * max(1.0, np.linalg.norm(z)) or it == max_newton:
                    newton_res.append(gn / max(1.0, np.linalg.norm(z)))
                    break
                op = LinearOperator((2 * nF, 2 * nF), matvec=lambda v: v - a0 * dt * self.jac_vec(v),
                                    dtype=np.float64)
                try:
                    dz, info = gmres(op, -G, rtol=1e-10, atol=0.0, restart=30, maxiter=3)
                except TypeError:  # scipy < 1.12
                    dz, info = gmres(op, -G, tol=1e-10, atol=0.0, restart=30, maxiter=3)
                z = z + dz
            y = z
            hist.append(y.copy())
            if len(hist) > 3:
                hist.pop(0)
            step_times.append(time.perf_counter() - ts)
        total = time.perf_counter() - t_start
        F = self.force(y)
        return {"steps": steps, "dt": dt, "n_dofs": self.m.n_dofs,
                "per_step_s": total / steps, "step_s_median": float(np.median(step_times)),
                "bem_fraction": self.t_bem / total, "assemblies": self.n_assemble,
                "solves": self.n_solve, "final_Fx": F,
                "max_eta": float(np.abs(y[:nF]).max()),
                "newton_residual_max": float(max(newton_res)), "final_state": y}


def main():
    p = argparse.ArgumentParser()
    p.add_argument("--n", type=int, default=12000)
    p.add_argument("--steps", type=int, default=100)
    p.add_argument("--dt", type=float, default=0.01)
    args = p.parse_args()
    out = {}
    for name, prec in (("mixed", PREC_MIXED), ("fp64", PREC_FP64)):
        out[name] = FreeSurfaceStandIn(args.n, precision=prec).run(args.steps, args.dt)
    ym, y64 = out["mixed"].pop("final_state"), out["fp64"].pop("final_state")
    out["final_state_drift_mixed_vs_fp64"] = float(np.linalg.norm(ym - y64) / np.linalg.norm(y64))
    out["final_Fx_drift_mixed_vs_fp64"] = abs(out["mixed"]["final_Fx"] - out["fp64"]["final_Fx"]) / max(
        abs(out["fp64"]["final_Fx"]), 1e-300)
    print(json.dumps(out))


if __name__ == "__main__":
    main()
