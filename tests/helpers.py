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


def cube_mesh(n=6, split_top=False):
    """Unit cube [0,1]^3 as six Q1 patches, each face its own nodes (double
    nodes on every edge, sharp Dirichlet-Dirichlet pairs when all faces are
    Dirichlet), normals pointing outwards. With split_top the face z = 1 is
    two patches meeting at x = 1/2, which adds flat double nodes along that
    line, and triples (two flat copies, one sharp) where it meets the cube's
    edges. Returns (X, cells, face id per cell)."""
    t = np.linspace(0, 1, n + 1)
    pts, cells, face = [], [], []
    off = 0
    fid = 0
    for ax in range(3):
        for side, sgn in ((0.0, -1), (1.0, 1)):
            a1, a2 = [k for k in range(3) if k != ax]
            ranges = [(0.0, 1.0)]
            if split_top and ax == 2 and side == 1.0:
                ranges = [(0.0, 0.5), (0.5, 1.0)]
            for lo, hi in ranges:
                m = n if len(ranges) == 1 else n // 2
                tu = np.linspace(lo, hi, m + 1)
                U, V = np.meshgrid(tu, t, indexing="xy")
                P = np.zeros(U.shape + (3,))
                P[..., ax] = side
                P[..., a1] = U
                P[..., a2] = V
                P = P.reshape(-1, 3)
                c = []
                for l in range(n):
                    for k in range(m):
                        i0 = l * (m + 1) + k
                        c.append([i0, i0 + 1, i0 + m + 1, i0 + m + 2])
                c = np.array(c)
                e1 = np.zeros(3); e1[a1] = 1
                e2 = np.zeros(3); e2[a2] = 1
                if np.cross(e1, e2)[ax] * sgn < 0:
                    c = c[:, [0, 2, 1, 3]]
                pts.append(P)
                cells.append(c + off)
                face.append(np.full(len(c), fid))
                off += len(P)
                fid += 1
    return (np.concatenate(pts), np.concatenate(cells).astype(np.int32),
            np.concatenate(face).astype(np.int32))
