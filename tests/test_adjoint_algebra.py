"""Host-side checks of the algebra the mixed adjoint kernel relies on
(wavebem_gb300/csrc/adjoint.cu, k_adj_tile_mixed), no GPU needed.

1. Moment form of the vertex gradients. For one Q1 panel with vertices
   P0..P3 and regular points (s, u), the adjoint sums
       g_v = sum_q [N4_v aR_q + Ns_v (je_q x ac_q) + Nt_v (ac_q x jx_q)]
   over the points q (and over the rows). With jx = (1-u) F0 + u F1 and
   je = (1-s) E0 + s E1, this equals B_v plus eight cross products of the
   panel edges with the moments D_v = sum N4_v ac. The kernel forms it per
   output component with the index arithmetic replayed here.
2. The warp reduce-scatter of 24 values (warp_sum24): lane l ends with the
   sums of v[3 (l >> 2) + i], i = 0..2.
"""
import numpy as np


def _gauss01(n):
    x, w = np.polynomial.legendre.leggauss(n)
    return (x + 1) / 2, w / 2


def _direct(P, pts, aR, ac):
    g = np.zeros(12)
    for (s, u), a, c in zip(pts, aR, ac):
        N4 = np.array([(1 - s) * (1 - u), s * (1 - u), (1 - s) * u, s * u])
        Ns = np.array([-(1 - u), 1 - u, -u, u])
        Nt = np.array([-(1 - s), -s, 1 - s, s])
        jx, je = Ns @ P, Nt @ P
        gjx, gje = np.cross(je, c), np.cross(c, jx)
        for v in range(4):
            g[3 * v:3 * v + 3] += N4[v] * a + Ns[v] * gjx + Nt[v] * gje
    return g


def _moment_form(P, pts, aR, ac):
    """The kernel's epilogue: B, D moments, then one output component at a time."""
    B = np.zeros(12)
    D = np.zeros(12)
    for (s, u), a, c in zip(pts, aR, ac):
        N4 = [(1 - s) * (1 - u), s * (1 - u), (1 - s) * u, s * u]
        for v in range(4):
            B[3 * v:3 * v + 3] += N4[v] * a
            D[3 * v:3 * v + 3] += N4[v] * c
    G = np.concatenate([P[2] - P[0], P[3] - P[1], P[1] - P[0], P[3] - P[2]])  # E0 E1 F0 F1
    out = np.zeros(12)
    for o in range(12):
        w, e = o // 3, o % 3
        e1 = 0 if e == 2 else e + 1
        e2 = 2 if e == 0 else e - 1
        ix = 0 if w < 2 else 2
        xs = (G[e1] * D[3 * ix + e2] - G[e2] * D[3 * ix + e1]
              + G[3 + e1] * D[3 * ix + 3 + e2] - G[3 + e2] * D[3 * ix + 3 + e1])
        iy = w & 1
        ys = (D[3 * iy + e1] * G[6 + e2] - D[3 * iy + e2] * G[6 + e1]
              + D[3 * iy + 6 + e1] * G[9 + e2] - D[3 * iy + 6 + e2] * G[9 + e1])
        out[o] = B[o] + (xs if w & 1 else -xs) + (ys if w >= 2 else -ys)
    return out


def test_moment_form_matches_direct_vertex_gradients():
    rng = np.random.default_rng(3)
    for q1 in (2, 4, 6):
        x, _ = _gauss01(q1)
        pts = [(x[a], x[b]) for b in range(q1) for a in range(q1)]
        for _ in range(5):
            P = rng.normal(size=(4, 3))
            aR = rng.normal(size=(len(pts), 3))
            ac = rng.normal(size=(len(pts), 3))
            g0 = _direct(P, pts, aR, ac)
            g1 = _moment_form(P, pts, aR, ac)
            assert np.abs(g1 - g0).max() <= 1e-12 * max(1.0, np.abs(g0).max())


def test_row_part_sums_to_minus_vertex_parts():
    """Translation invariance: moving the collocation point and all four
    vertices together leaves every term unchanged, so the row part -sum_q aR
    equals minus the sum of the four vertex parts (the cross-product parts
    cancel because sum_v Ns_v = sum_v Nt_v = 0)."""
    rng = np.random.default_rng(4)
    x, _ = _gauss01(4)
    pts = [(x[a], x[b]) for b in range(4) for a in range(4)]
    P = rng.normal(size=(4, 3))
    aR = rng.normal(size=(16, 3))
    ac = rng.normal(size=(16, 3))
    g = _moment_form(P, pts, aR, ac).reshape(4, 3)
    assert np.allclose(g.sum(0), aR.sum(0), rtol=0, atol=1e-12)


def test_warp_sum24_lane_map():
    rng = np.random.default_rng(5)
    v = rng.normal(size=(32, 24))

    def step(vals, width, bit):
        half = width // 2
        out = np.zeros((32, half))
        for lane in range(32):
            p = lane ^ bit
            for i in range(half):
                keep = vals[lane, half + i] if lane & bit else vals[lane, i]
                send = vals[p, i] if p & bit else vals[p, half + i]
                out[lane, i] = keep + send
        return out

    w = step(v, 24, 16)
    x = step(w, 12, 8)
    y = step(x, 6, 4)
    y = y + y[[lane ^ 2 for lane in range(32)]]
    y = y + y[[lane ^ 1 for lane in range(32)]]
    total = v.sum(0)
    for lane in range(32):
        for i in range(3):
            assert abs(y[lane, i] - total[3 * (lane >> 2) + i]) <= 1e-12
