"""Writes the small regression fixtures of tests/golden/ from the CPU oracle.

The reference cannot run here (no deal.II), so these vectors are the
oracle's own outputs on two tiny meshes; they guard the oracle and the GPU
path against regressions (the closed-form pins live in tests/test_oracle.py).

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle as O  # noqa: E402
from wavebem_gb300 import meshes as M  # noqa: E402


def case(name):
    if name == "wigley300":
        m = M.wigley_mesh(300)
        b = M.wigley_bc(m, seed=7)
    else:
        m = M.cube_sphere_mesh(6)
        b, _ = M.sphere_harmonics(m.X, seed=7)
    return m, b


def main():
    for name in ("wigley300", "sphere6"):
        m, b = case(name)
        ptr, idx = M.double_nodes(m.X, m.cells)
        P = O.Problem(m.X, m.cells, ptr, idx, m.dirichlet)
        P.assemble()
        v = np.cos(np.arange(P.N) * 0.37)
        phi, dphi, _ = P.solve_system(b)
        rng = np.random.default_rng(11)
        ii = rng.integers(0, P.N, 64)
        jj = rng.integers(0, P.N, 64)
        np.savez_compressed(
            os.path.join(HERE, f"{name}.npz"), X=m.X, cells=m.cells, dirichlet=m.dirichlet, b=b,
            dn_ptr=ptr, dn_idx=idx, alpha=P.alpha, Nv=P.Nm @ v, Dv=P.Dm @ v, v=v, phi=phi,
            dphi=dphi, ii=ii, jj=jj, Nij=P.Nm[ii, jj], Dij=P.Dm[ii, jj])
        print("wrote", name, P.N)


if __name__ == "__main__":
    main()
