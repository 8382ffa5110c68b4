"""Shared test fixtures: meshes and oracle problems, cached per session."""
import functools

import numpy as np

import oracle as O
from wavebem_gb300 import meshes as M


@functools.lru_cache(maxsize=None)
def wigley(n=2000, seed=0):
    m = M.wigley_mesh(n)
    ptr, idx = M.double_nodes(m.X, m.cells)
    b = M.wigley_bc(m, seed=seed)
    return m, ptr, idx, b


@functools.lru_cache(maxsize=None)
def sphere(n=12, seed=1):
    m = M.cube_sphere_mesh(n)
    ptr, idx = M.double_nodes(m.X, m.cells)
    p, dpdn = M.sphere_harmonics(m.X, seed=seed)
    return m, ptr, idx, p, dpdn


@functools.lru_cache(maxsize=None)
def oracle_problem(kind="wigley", n=2000):
    if kind == "wigley":
        m, ptr, idx, b = wigley(n)
    else:
        m, ptr, idx, b, _ = sphere(n)
    P = O.Problem(m.X, m.cells, ptr, idx, m.dirichlet)
    P.assemble()
    return P, m, b


def relmax(a, b):
    return float(np.abs(a - b).max() / np.abs(b).max())


def rel2(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))
