"""Synthetic Q1 boundary meshes and boundary data for the collocation BEM.

The reference builds its meshes from IGES hulls through OpenCASCADE
(`source/numerical_towing_tank.cc:582-716`); that pipeline is not part of the
assemble+solve path, so the meshes here are analytic stand-ins with the same
structure:

* every face of the towing-tank box is its own structured Q1 patch with its own
  nodes, so nodes on face edges are duplicated ("double nodes", found by
  coincidence, `source/computational_domain.cc:258-307`);
* cell vertices are listed in deal.II's lexicographic order
  (0:(0,0) 1:(1,0) 2:(0,1) 3:(1,1)) and oriented so that
  d x/d xi  x  d x/d eta  points out of the fluid;
* the Dirichlet mask marks every node of a free-surface cell
  (`source/free_surface.cc:8756-8774`).

All arrays are plain numpy: X (N,3) float64, cells (C,4) int32,
dirichlet (N,) uint8, face (C,) int32.
"""
from __future__ import annotations

import itertools
import math
from dataclasses import dataclass, field

import numpy as np

# face ids of the Wigley towing tank
FREE_SURFACE, HULL, CENTER_PLANE, BOTTOM, WALL_XM, WALL_XP, WALL_YP = range(7)
FACE_NAMES = ["free_surface", "hull", "center_plane", "bottom", "wall_x-", "wall_x+", "wall_y+"]

# Wigley hull and tank dimensions (half domain, y >= 0)
WIGLEY_L, WIGLEY_B, WIGLEY_T = 1.0, 0.1, 0.0625
BOX_X = (-1.5, 2.5)
BOX_Y = (0.0, 1.5)
BOX_Z = (-1.0, 0.0)


@dataclass
class Mesh:
    X: np.ndarray            # (N,3) node positions
    cells: np.ndarray        # (C,4) int32 node indices, lexicographic order
    face: np.ndarray         # (C,) int32 face id per cell
    dirichlet: np.ndarray    # (N,) uint8, 1 on free-surface (Dirichlet) nodes
    normal: np.ndarray       # (N,3) analytic outward (out of the fluid) normal per node
    info: dict = field(default_factory=dict)

    @property
    def n_dofs(self) -> int:
        return int(self.X.shape[0])

    @property
    def n_cells(self) -> int:
        return int(self.cells.shape[0])


def _patch(points_fn, u, v, outward):
    """Structured patch over the parameter grid u (nu+1) x v (nv+1).

    Returns nodes (row-major, u fastest) and cells in lexicographic vertex
    order, flipped (xi <-> eta) when needed so that every cell normal has a
    positive component along `outward(P)`.
    """
    U, V = np.meshgrid(u, v, indexing="xy")
    P = np.stack(points_fn(U, V), axis=-1).reshape(-1, 3)
    nu, nv = len(u) - 1, len(v) - 1
    K, L = np.meshgrid(np.arange(nu), np.arange(nv), indexing="xy")
    i00 = (L * (nu + 1) + K).ravel()
    cells = np.stack([i00, i00 + 1, i00 + nu + 1, i00 + nu + 2], axis=-1)
    a = P[cells[:, 1]] - P[cells[:, 0]] + P[cells[:, 3]] - P[cells[:, 2]]
    b = P[cells[:, 2]] - P[cells[:, 0]] + P[cells[:, 3]] - P[cells[:, 1]]
    n = np.cross(a, b)
    centre = P[cells].mean(axis=1)
    s = np.einsum("ij,ij->i", n, outward(centre))
    if np.all(s < 0):
        cells = cells[:, [0, 2, 1, 3]]
    elif not np.all(s > 0):
        raise ValueError("patch orientation is not consistent")
    return P, cells.astype(np.int64)


def _assemble(patches):
    Xs, Cs, Fs, Ns = [], [], [], []
    off = 0
    for P, cells, fid, nrm in patches:
        Xs.append(P)
        Cs.append(cells + off)
        Fs.append(np.full(len(cells), fid, np.int32))
        Ns.append(nrm)
        off += len(P)
    return np.concatenate(Xs), np.concatenate(Cs).astype(np.int32), np.concatenate(Fs), np.concatenate(Ns)


def wigley_counts(nxl, nxh, nxr, ny, nzh, nzb):
    nx, nz = nxl + nxh + nxr, nzh + nzb
    return ((nx + 1) * (ny + 1) * 2 + (nxh + 1) * (nzh + 1) + (nxl + 1) * (nz + 1)
            + (nxh + 1) * (nzb + 1) + (nxr + 1) * (nz + 1) + 2 * (ny + 1) * (nz + 1)
            + (nx + 1) * (nz + 1))


def wigley_resolution(target_n: int):
    """Integer resolutions (nxl, nxh, nxr, ny, nzh, nzb) whose node count is
    closest to `target_n`, preferring the ideal proportions of one cell size h:
    hull length 1/h cells, 1/h ahead, 2/h behind, 1.5/h across, the hull draft
    in 0.25/h cells and the rest of the depth in 0.9375/h cells."""
    s = math.sqrt(target_n / 25.1)
    ideal = np.array([s, s, 2 * s, 1.5 * s, max(2.0, 0.25 * s), 0.9375 * s])
    best = None
    base = np.maximum(np.round(ideal).astype(int), 1)
    rng = range(-3, 4)
    for d in itertools.product(rng, rng, rng, rng, rng, rng):
        r = base + np.array(d)
        if np.any(r < 1) or r[4] < 2:
            continue
        n = wigley_counts(*r)
        dev = float(np.sum(((r - ideal) / ideal) ** 2))
        key = (abs(n - target_n), dev)
        if best is None or key < best[0]:
            best = (key, tuple(int(v) for v in r), n)
    return best[1], best[2]


def hull_offset(x, z, a=None):
    """Half-breadth y(x,z) of the (optionally perturbed) Wigley hull."""
    L, B, T = WIGLEY_L, WIGLEY_B, WIGLEY_T
    zt = 1.0 - (z / T) ** 2
    y = 0.5 * B * (1.0 - (2.0 * x / L) ** 2) * zt
    if a is not None:
        for j, aj in enumerate(a, start=1):
            y = y + aj * np.sin(j * np.pi * (x + 0.5)) * zt
    return y


def hull_normal(x, z, a=None):
    """Analytic normal of the hull surface pointing out of the fluid (into the
    hull), i.e. along (dy/dx, -1, dy/dz)."""
    L, B, T = WIGLEY_L, WIGLEY_B, WIGLEY_T
    zt = 1.0 - (z / T) ** 2
    dzt = -2.0 * z / T ** 2
    fx = 0.5 * B * (1.0 - (2.0 * x / L) ** 2)
    dfx = 0.5 * B * (-8.0 * x / L ** 2)
    hx = dfx * zt
    g = fx
    if a is not None:
        for j, aj in enumerate(a, start=1):
            hx = hx + aj * j * np.pi * np.cos(j * np.pi * (x + 0.5)) * zt
            g = g + aj * np.sin(j * np.pi * (x + 0.5))
    hz = g * dzt
    n = np.stack([hx, -np.ones_like(hx), hz], axis=-1)
    return n / np.linalg.norm(n, axis=-1, keepdims=True)


def wigley_mesh(target_n: int = 2000, a=None, resolution=None) -> Mesh:
    """Half-domain Wigley towing tank: free surface z=0 outside the waterplane,
    hull, centre plane y=0 outside the hull (3 patches), bottom z=-1 and the
    walls x=-1.5, x=2.5, y=1.5. Every patch has its own nodes."""
    if resolution is None:
        resolution, _ = wigley_resolution(target_n)
    nxl, nxh, nxr, ny, nzh, nzb = resolution
    T = WIGLEY_T
    x0, x1 = BOX_X
    y0, y1 = BOX_Y
    zb, zt = BOX_Z
    xl = np.linspace(x0, -0.5, nxl + 1)
    xh = np.linspace(-0.5, 0.5, nxh + 1)
    xr = np.linspace(0.5, x1, nxr + 1)
    xall = np.concatenate([xl, xh[1:], xr[1:]])
    eta = np.linspace(0.0, 1.0, ny + 1)
    yall = y0 + (y1 - y0) * eta
    zh = np.linspace(-T, zt, nzh + 1)
    zbel = np.linspace(zb, -T, nzb + 1)
    zall = np.concatenate([zbel, zh[1:]])

    def waterline(x):
        inside = np.abs(x) <= 0.5
        yw = np.where(inside, hull_offset(np.clip(x, -0.5, 0.5), np.zeros_like(x), a), 0.0)
        return np.maximum(yw, 0.0)

    def hull_y(x, z):
        y = hull_offset(x, z, a)
        # the bow/stern lines x=+-0.5 and the keel z=-T lie on the centre plane
        y = np.where((np.abs(x) == 0.5) | (z == -T), 0.0, y)
        return np.maximum(y, 0.0)

    const = lambda v: (lambda P: np.broadcast_to(np.asarray(v, float), P.shape))
    patches = []

    def add(fn, u, v, outward, fid, nfn):
        P, c = _patch(fn, u, v, outward)
        patches.append((P, c, fid, nfn(P)))

    # free surface: (x, eta) -> (x, yw(x) + eta (1.5 - yw(x)), 0)
    add(lambda X, E: (X, waterline(X) + E * (y1 - waterline(X)), np.zeros_like(X)),
        xall, eta, const([0, 0, 1]), FREE_SURFACE, const([0, 0, 1]))
    # hull: (x, z) -> (x, h(x,z), z)
    add(lambda X, Z: (X, hull_y(X, Z), Z), xh, zh, const([0, -1, 0]), HULL,
        lambda P: hull_normal(P[:, 0], P[:, 2], a))
    # centre plane pieces y=0
    for xs, zs in ((xl, zall), (xh, zbel), (xr, zall)):
        add(lambda X, Z: (X, np.zeros_like(X), Z), xs, zs, const([0, -1, 0]), CENTER_PLANE,
            const([0, -1, 0]))
    # bottom z=-1
    add(lambda X, Y: (X, Y, np.full_like(X, zb)), xall, yall, const([0, 0, -1]), BOTTOM,
        const([0, 0, -1]))
    # walls
    add(lambda Y, Z: (np.full_like(Y, x0), Y, Z), yall, zall, const([-1, 0, 0]), WALL_XM,
        const([-1, 0, 0]))
    add(lambda Y, Z: (np.full_like(Y, x1), Y, Z), yall, zall, const([1, 0, 0]), WALL_XP,
        const([1, 0, 0]))
    add(lambda X, Z: (X, np.full_like(X, y1), Z), xall, zall, const([0, 1, 0]), WALL_YP,
        const([0, 1, 0]))

    X, cells, face, normal = _assemble(patches)
    dirichlet = np.zeros(len(X), np.uint8)
    dirichlet[np.unique(cells[face == FREE_SURFACE])] = 1
    return Mesh(X=np.ascontiguousarray(X), cells=np.ascontiguousarray(cells), face=face,
                dirichlet=dirichlet, normal=normal,
                info={"kind": "wigley", "resolution": tuple(resolution), "a": None if a is None else list(map(float, a))})


def cube_sphere_mesh(n: int = 52) -> Mesh:
    """Conforming equiangular cube-sphere of the unit sphere: 6 n^2 cells and
    6 n^2 + 2 shared nodes (no double nodes), normals pointing outwards (the
    fluid is the ball)."""
    t = np.tan(np.pi / 4 * np.linspace(-1.0, 1.0, n + 1))
    key_to_id = {}
    Xs, cells = [], []
    faces = [(0, 1, 2, 1.0), (0, 1, 2, -1.0), (1, 2, 0, 1.0), (1, 2, 0, -1.0), (2, 0, 1, 1.0), (2, 0, 1, -1.0)]
    for ax_u, ax_v, ax_n, sgn in faces:
        ids = np.empty((n + 1, n + 1), np.int64)
        for l in range(n + 1):
            for k in range(n + 1):
                p = np.zeros(3)
                p[ax_u], p[ax_v], p[ax_n] = t[k], t[l], sgn
                ik = [0, 0, 0]
                ik[ax_u], ik[ax_v], ik[ax_n] = k, l, (n if sgn > 0 else 0)
                key = tuple(ik)
                if key not in key_to_id:
                    key_to_id[key] = len(Xs)
                    Xs.append(p / np.linalg.norm(p))
                ids[l, k] = key_to_id[key]
        fc = []
        for l in range(n):
            for k in range(n):
                fc.append([ids[l, k], ids[l, k + 1], ids[l + 1, k], ids[l + 1, k + 1]])
        cells.extend(fc)
    X = np.array(Xs)
    cells = np.array(cells, np.int64)
    a = X[cells[:, 1]] - X[cells[:, 0]] + X[cells[:, 3]] - X[cells[:, 2]]
    b = X[cells[:, 2]] - X[cells[:, 0]] + X[cells[:, 3]] - X[cells[:, 1]]
    s = np.einsum("ij,ij->i", np.cross(a, b), X[cells].mean(axis=1))
    flip = s < 0
    cells[flip] = cells[flip][:, [0, 2, 1, 3]]
    cells = cells.astype(np.int32)
    return Mesh(X=X, cells=cells, face=np.zeros(len(cells), np.int32),
                dirichlet=np.ones(len(X), np.uint8), normal=X.copy(),
                info={"kind": "cube_sphere", "n": n})


def boundary_nodes(cells: np.ndarray, n_dofs: int) -> np.ndarray:
    """Nodes on an edge that belongs to exactly one cell (the boundary of the
    surface mesh), as deal.II's extract_boundary_dofs would flag them."""
    e = np.concatenate([cells[:, [0, 1]], cells[:, [1, 3]], cells[:, [3, 2]], cells[:, [2, 0]]])
    e = np.sort(e, axis=1)
    uniq, cnt = np.unique(e, axis=0, return_counts=True)
    b = np.zeros(n_dofs, bool)
    b[uniq[cnt == 1].ravel()] = True
    return b


def double_nodes(X: np.ndarray, cells: np.ndarray, tol: float = 1e-8):
    """Double-node sets in CSR form (dn_ptr, dn_idx): row i lists, in ascending
    order, i itself and, for boundary nodes, every node closer than `tol`
    (`source/computational_domain.cc:258-307`)."""
    N = len(X)
    bnd = boundary_nodes(cells, N)
    # exact grouping through a grid hash of cell size >> tol
    h = 1e-6
    keys = np.floor(X / h).astype(np.int64)
    from collections import defaultdict
    grid = defaultdict(list)
    bidx = np.nonzero(bnd)[0]
    for i in range(N):
        grid[tuple(keys[i])].append(i)
    sets = [[i] for i in range(N)]
    for i in bidx:
        k = keys[i]
        cand = []
        for d in itertools.product((-1, 0, 1), repeat=3):
            cand.extend(grid.get((k[0] + d[0], k[1] + d[1], k[2] + d[2]), ()))
        s = {i}
        for j in cand:
            if np.linalg.norm(X[i] - X[j]) < tol:
                s.add(j)
        sets[i] = sorted(s)
    ptr = np.zeros(N + 1, np.int32)
    ptr[1:] = np.cumsum([len(s) for s in sets])
    idx = np.array([j for s in sets for j in s], np.int32)
    return ptr, idx


# ---------------------------------------------------------------- boundary data

def wigley_bc(mesh: Mesh, seed: int = 0, Fr: float = 0.316, U=(1.0, 0.0, 0.0)):
    """Known data (the reference's `tmp_rhs`): phi = 1e-3 sin(k x + theta) on
    Dirichlet (free-surface) nodes, k = 1/Fr^2, theta = 2 pi U[0,1) from the
    seed; dphi/dn = -U.n on Neumann nodes."""
    rng = np.random.default_rng(seed)
    theta = 2 * np.pi * rng.random()
    k = 1.0 / Fr ** 2
    b = -(mesh.normal @ np.asarray(U, float))
    d = mesh.dirichlet.astype(bool)
    b[d] = 1e-3 * np.sin(k * mesh.X[d, 0] + theta)
    return b


def sphere_harmonics(X: np.ndarray, seed: int = 1):
    """Seeded combination of 9 harmonic polynomials of degree 1 and 2:
    x, y, z, xy, yz, zx, x^2-y^2, y^2-z^2, z^2-x^2 (the last three are
    linearly dependent; they are kept as listed), coefficients U[-1,1].
    Returns (p, exact dp/dn on the unit sphere = degree * p)."""
    rng = np.random.default_rng(seed)
    c = rng.uniform(-1.0, 1.0, 9)
    x, y, z = X[:, 0], X[:, 1], X[:, 2]
    p1 = c[0] * x + c[1] * y + c[2] * z
    p2 = (c[3] * x * y + c[4] * y * z + c[5] * z * x + c[6] * (x * x - y * y)
          + c[7] * (y * y - z * z) + c[8] * (z * z - x * x))
    return p1 + p2, p1 + 2.0 * p2


def config_case(name: str):
    """The five benchmark cases as (mesh, dn_ptr, dn_idx, tmp_rhs, extra)."""
    if name == "c0":
        m = wigley_mesh(2000)
        b = wigley_bc(m, seed=0)
    elif name == "c1":
        m = cube_sphere_mesh(52)
        p, dpdn = sphere_harmonics(m.X, seed=1)
        b = p
        m.info["exact_dphi_dn"] = dpdn
    elif name == "c2":
        m = wigley_mesh(32768)
        b = wigley_bc(m, seed=2)
    elif name == "c3":
        rng = np.random.default_rng(3)
        a = rng.normal(0.0, 1e-3, 8)
        m = wigley_mesh(8192, a=a)
        b = wigley_bc(m, seed=3)
    elif name == "c4":
        m = wigley_mesh(12000)
        b = wigley_bc(m, seed=4)
    else:
        raise KeyError(name)
    ptr, idx = double_nodes(m.X, m.cells)
    return m, ptr, idx, b
