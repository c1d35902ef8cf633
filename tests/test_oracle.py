"""The CPU oracle, pinned before anything is compared with it.

Pins, in order of strength:
* exact-rational golden fixtures (tests/golden/make_golden.py): pieces, adjacency,
  value, masses, moments and Hessian;
* the invariants the reference's drivers print: total area of the pieces
  (tests/test_voronoi_tri.cpp:67, tests/test_voronoi.cpp:50, tests/test_power.cpp:51),
  conservation of mass (tests/test_quantization.cpp:78-79), and finite-difference
  consistency of the gradient and Hessian (tests/test_opttransport_eval.cpp:20-55);
* the regular-triangulation adjacency recomputed independently from scipy's qhull
  (power diagram = lower convex hull of the lifted sites);
* the exact predicates against rational arithmetic on near-degenerate inputs.
"""
from fractions import Fraction as Fr

import numpy as np
import pytest

from conftest import golden_cases, hessian_dict, load_golden
from mongeampere_gb300 import workloads as W
from mongeampere_gb300.mesh import GridMesh, unit_grid


@pytest.mark.parametrize("name", golden_cases())
@pytest.mark.parametrize("mode", [0, 1])
def test_oracle_matches_exact_golden(oracle, name, mode):
    d = load_golden(name)
    r = oracle.kantorovich(d["mesh_obj"], d["x"], d["y"], d["w"], mode=mode, keep_pieces=True)
    gs = max(1.0, np.abs(d["g"]).max())
    assert abs(r.value - d["value"]) <= 1e-14 * gs
    np.testing.assert_allclose(r.g, d["g"], rtol=0, atol=1e-14 * gs)
    np.testing.assert_allclose(r.moments, d["moments"], rtol=0, atol=1e-14 * gs)
    H = {(i, j): v for i, j, v in d["hessian"]}
    Ho = hessian_dict(r.rows, r.cols, r.vals)
    assert set(H) == set(Ho), "adjacency differs from the exact pieces"
    hs = max([abs(v) for v in H.values()] + [1.0])
    for k, v in H.items():
        assert abs(Ho[k] - v) <= 1e-13 * hs
    got = sorted(zip(r.pieces.face.tolist(), r.pieces.site.tolist(), r.pieces.nvert.tolist()))
    assert got == sorted(tuple(p) for p in d["pieces"])


def test_flood_fill_modes_identical(oracle):
    p = W.make_problem(16, 200, seed=3)
    w = np.random.default_rng(1).uniform(-1e-3, 1e-3, p.n)
    a = oracle.kantorovich(p.mesh, p.x, p.y, w, mode=0)
    b = oracle.kantorovich(p.mesh, p.x, p.y, w, mode=1)
    assert a.value == b.value
    assert np.array_equal(a.g, b.g)
    assert np.array_equal(a.vals, b.vals) and np.array_equal(a.cols, b.cols)


def test_total_area_and_mass(oracle):
    # tests/test_voronoi_tri.cpp:67 (sum of piece areas), test_quantization.cpp:78 (mass)
    p = W.make_problem(32, 500, seed=5)
    r = oracle.kantorovich(p.mesh, p.x, p.y, p.w0)
    assert abs(r.total_area - 1.0) < 1e-12
    assert abs(r.g.sum() - p.mesh.total_mass()) < 1e-12
    # the Hessian is a graph Laplacian: rows sum to zero, symmetric
    H = r.hessian()
    assert np.abs(np.asarray(H.sum(axis=1))).max() < 1e-12
    assert abs(H - H.T).max() < 1e-13


def test_voronoi_of_square_has_area_four(oracle):
    # tests/test_voronoi.cpp:25-51: 10k Voronoi cells of [-1, 1]^2 have total area 4
    g = np.array([-1.0, 0.0, 1.0])
    mesh = GridMesh(g, g, np.ones(9))
    rng = np.random.default_rng(0)
    pts = rng.uniform(-1, 1, (5000, 2))
    r = oracle.kantorovich(mesh, pts[:, 0], pts[:, 1], np.zeros(5000))
    assert abs(r.total_area - 4.0) < 1e-11
    assert abs(r.g.sum() - 4.0) < 1e-11


def test_fd_gradient_and_hessian(oracle):
    # the method of tests/test_opttransport_eval.cpp:20-55 (central differences,
    # eps = 1e-5) on 50 sites
    p = W.make_problem(24, 50, seed=11)
    rng = np.random.default_rng(2)
    w = rng.uniform(-2e-3, 2e-3, p.n)
    r = oracle.kantorovich(p.mesh, p.x, p.y, w)
    H = r.hessian().toarray()
    eps = 1e-5
    gfd = np.zeros(p.n)
    hfd = np.zeros((p.n, p.n))
    for i in range(p.n):
        wp, wm = w.copy(), w.copy()
        wp[i] += eps
        wm[i] -= eps
        rp = oracle.kantorovich(p.mesh, p.x, p.y, wp)
        rm = oracle.kantorovich(p.mesh, p.x, p.y, wm)
        gfd[i] = (rp.value - rm.value) / (2 * eps)
        hfd[i] = (rp.g - rm.g) / (2 * eps)
    assert np.linalg.norm(gfd - r.g) < 1e-5 * np.linalg.norm(r.g)
    assert np.linalg.norm(hfd - H) < 1e-3 * np.linalg.norm(H)


def _lower_hull_edges(x, y, w):
    from scipy.spatial import ConvexHull
    pts = np.c_[x, y, x * x + y * y - w]
    hull = ConvexHull(pts)
    edges = set()
    for simplex, eq in zip(hull.simplices, hull.equations):
        if eq[2] < -1e-12:
            a, b, c = sorted(int(v) for v in simplex)
            edges |= {(a, b), (a, c), (b, c)}
    return edges


def test_adjacency_vs_qhull(oracle):
    # independent cross-check of the (domain-restricted) regular-triangulation
    # adjacency: every Hessian off-diagonal pair is an edge of the lower hull of the
    # lifted sites, and every lower-hull edge whose Laguerre edge crosses the square
    # appears in the Hessian
    p = W.make_problem(16, 400, seed=7)
    rng = np.random.default_rng(3)
    w = rng.uniform(-5e-4, 5e-4, p.n)
    r = oracle.kantorovich(p.mesh, p.x, p.y, w)
    pairs = {(min(i, j), max(i, j)) for i, j in zip(r.rows, r.cols) if i != j}
    rt = _lower_hull_edges(p.x, p.y, w)
    assert pairs <= rt
    # an RT edge whose radical axis meets the cell pair inside the square must appear:
    # sample the midpoint of the Laguerre edge via the two cells' common points
    missing = rt - pairs
    for (i, j) in missing:
        # points on the radical axis of (i, j) that are closer to i, j than to all
        # others and inside the square would contradict the Hessian: check a fine
        # sample of the axis
        d = np.array([p.x[j] - p.x[i], p.y[j] - p.y[i]])
        c = 0.5 * (np.dot(d, d) - (w[j] - w[i]))
        base = np.array([p.x[i], p.y[i]]) + d * (c / np.dot(d, d))
        t = np.array([-d[1], d[0]]) / np.linalg.norm(d)
        s = np.linspace(-1.5, 1.5, 3001)
        q = base[None, :] + s[:, None] * t[None, :]
        inside = (q > 1e-9).all(1) & (q < 1 - 1e-9).all(1)
        q = q[inside]
        if q.size == 0:
            continue
        pw = (q[:, 0, None] - p.x[None]) ** 2 + (q[:, 1, None] - p.y[None]) ** 2 - w[None]
        own = pw[:, i]
        others = np.delete(pw, [i, j], axis=1).min(axis=1)
        assert not np.any(own < others - 1e-9), f"pair {(i, j)} has a Laguerre edge inside the domain"


def _exact_pi(v, w, e):
    v = [Fr(t) for t in v]
    w = [Fr(t) for t in w]
    e = [Fr(t) for t in e]
    return ((e[0] - v[0]) ** 2 + (e[1] - v[1]) ** 2 - v[2]) - ((e[0] - w[0]) ** 2 + (e[1] - w[1]) ** 2 - w[2])


def test_predicates_exact_on_near_degenerate_inputs(oracle):
    rng = np.random.default_rng(4)
    for _ in range(300):
        v = rng.uniform(0, 1, 3)
        w = rng.uniform(0, 1, 3)
        # a point on (or within a few ulps of) the radical axis of v and w
        d = w[:2] - v[:2]
        c = 0.5 * (d @ d - (w[2] - v[2]))
        base = v[:2] + d * (c / (d @ d))
        e = base + rng.uniform(-1, 1) * np.array([-d[1], d[0]])
        e = e + rng.integers(-3, 4, 2) * np.spacing(e)
        assert oracle.side1(v, w, e) == (_exact_pi(v, w, e) < 0)
        # Side3: segment through e
        pq = rng.uniform(-1, 1, 2)
        p_, q_ = e - pq, e + pq * rng.uniform(0.5, 2)
        u = rng.uniform(0, 1, 3)
        A = lambda x: _exact_pi(v, u, x)
        B = lambda x: _exact_pi(v, w, x)
        den = A(p_) - A(q_)
        if den != 0:
            want = (A(p_) * B(q_) - A(q_) * B(p_)) / den < 0
            assert oracle.side3(v, u, p_, q_, w) == want
    # Side2 on co-circular configurations (exact ties must be "outside") and
    # perturbations of them
    for _ in range(200):
        cx, cy, R = rng.uniform(0.3, 0.7), rng.uniform(0.3, 0.7), rng.uniform(0.05, 0.2)
        ang = np.sort(rng.uniform(0, 2 * np.pi, 4))
        P = [np.array([cx + R * np.cos(a), cy + R * np.sin(a), 0.0]) for a in ang]
        P[3][:2] += rng.integers(-2, 3, 2) * np.spacing(P[3][:2])
        v, a, b, w = P
        Fv, Fa, Fb, Fw = ([Fr(t) for t in q] for q in (v, a, b, w))
        d = lambda q: (q[0] - Fv[0], q[1] - Fv[1], (q[0] - Fv[0]) ** 2 + (q[1] - Fv[1]) ** 2 - (q[2] - Fv[2]))
        da, db, dw = d(Fa), d(Fb), d(Fw)
        D = da[0] * db[1] - da[1] * db[0]
        M = dw[0] * (da[2] * db[1] - db[2] * da[1]) + dw[1] * (da[0] * db[2] - db[0] * da[2]) - dw[2] * D
        want = D != 0 and (M / D) < 0
        assert oracle.side2(v, a, b, w) == want


def test_ot_solve_reference_semantics(oracle):
    p = W.make_problem(24, 150, seed=2)
    s = oracle.ot_solve(p.mesh, p.x, p.y, p.nu, tol_rel=1e-10)
    assert s.max_rel_err <= 1e-10
    assert s.w[-1] == 0.0           # gauge of solve_laplacian_matrix: d[N-1] = 0
    assert s.niter <= 10


def test_empty_cell_is_reported(oracle):
    # optimal_transport.hpp:137-148: a non-positive minimum mass stops the solve
    mesh = unit_grid(4, np.ones((4, 4)))
    x = np.array([0.2, 0.8, 0.5])
    y = np.array([0.5, 0.5, 0.5])
    w = np.array([0.0, 0.0, -1.0])
    with pytest.raises(oracle.EmptyCellError):
        oracle.ot_solve(mesh, x, y, np.full(3, 1 / 3), w=w)


def test_double_double_oracle_is_translation_invariant(oracle):
    # the reference's FP64 absolute-coordinate constructions move short-edge
    # Hessian entries under a translation of the input; the double-double mode
    # (the parity anchor) does not, and both modes find the same pieces
    from mongeampere_gb300.mesh import GridMesh
    p = W.make_problem(64, 2000, "gauss", "uniform", "random", seed=3)
    w = np.random.default_rng(6).uniform(-5e-5, 5e-5, p.n)
    a = oracle.kantorovich(p.mesh, p.x, p.y, w)
    f = oracle.kantorovich(p.mesh, p.x, p.y, w, arith="fp64")
    assert np.array_equal(a.rows, f.rows) and np.array_equal(a.cols, f.cols)
    scale = np.abs(a.vals).max()
    assert np.abs(a.vals - f.vals).max() <= 1e-8 * scale
    sh = 0.375
    m2 = GridMesh(p.mesh.gx + sh, p.mesh.gy + sh, p.mesh.values)
    b = oracle.kantorovich(m2, p.x + sh, p.y + sh, w)
    assert np.array_equal(a.rows, b.rows) and np.array_equal(a.cols, b.cols)
    assert np.all(np.abs(a.vals - b.vals) <= 1e-12 * (np.abs(a.vals) + scale))
    assert np.all(np.abs(a.g - b.g) <= 1e-13 * np.abs(a.g).max())


def test_cocircular_quadruples_have_no_exact_ties(oracle):
    # the near-degenerate input of the GPU parity test: co-circular up to rounding,
    # never exactly (so adjacency does not depend on the order of the input)
    from mongeampere_gb300.mesh import unit_grid
    rng = np.random.default_rng(3)
    nq = 150
    c = rng.uniform(0.08, 0.92, (nq, 2))
    r = rng.uniform(0.01, 0.04, nq)
    ang = rng.uniform(0, 2 * np.pi, (nq, 4))
    x = (c[:, 0, None] + r[:, None] * np.cos(ang)).ravel()
    y = (c[:, 1, None] + r[:, None] * np.sin(ang)).ravel()
    for q in range(nq):
        P = [(Fr(x[4 * q + t]), Fr(y[4 * q + t])) for t in range(4)]
        a = P[0]
        rows = [(p[0] - a[0], p[1] - a[1], (p[0] - a[0]) ** 2 + (p[1] - a[1]) ** 2) for p in P[1:]]
        det = (rows[0][0] * (rows[1][1] * rows[2][2] - rows[1][2] * rows[2][1])
               - rows[0][1] * (rows[1][0] * rows[2][2] - rows[1][2] * rows[2][0])
               + rows[0][2] * (rows[1][0] * rows[2][1] - rows[1][1] * rows[2][0]))
        assert det != 0
    mesh = unit_grid(16, np.random.default_rng(2).uniform(0.5, 1.5, (16, 16)))
    a = oracle.kantorovich(mesh, x, y, np.zeros(x.size))
    assert a.exact_calls > 100
    perm = np.random.default_rng(0).permutation(x.size)
    b = oracle.kantorovich(mesh, x[perm], y[perm], np.zeros(x.size))
    A = {(int(i), int(j)) for i, j in zip(a.rows, a.cols)}
    B = {(int(perm[i]), int(perm[j])) for i, j in zip(b.rows, b.cols)}
    assert A == B


def _shoelace(xy):
    if xy.shape[0] == 0:
        return 0.0
    x, y = xy[:, 0], xy[:, 1]
    return 0.5 * np.sum(x * np.roll(y, -1) - np.roll(x, -1) * y)


def test_polygon_cells_area_invariants(oracle):
    # voronoi_polygon_intersection over every site: [-1, 1]^2 gives 4
    # (tests/test_voronoi.cpp:39-50), the 12-corner cross of
    # tests/test_voronoi_ad.cpp:30-57 gives 12
    rng = np.random.default_rng(1)
    X = rng.uniform(-1, 1, (800, 2))
    sq = np.array([[-1, -1], [1, -1], [1, 1], [-1, 1]], dtype=np.float64)
    off, xy, _ = oracle.polygon_cells(X[:, 0], X[:, 1], np.zeros(800), sq[:, 0], sq[:, 1])
    a = np.array([_shoelace(xy[off[i]:off[i + 1]]) for i in range(800)])
    assert a.min() > 0 and abs(a.sum() - 4.0) < 1e-12
    cross = np.array([[1, -1], [2, -1], [2, 1], [1, 1], [1, 2], [-1, 2], [-1, 1], [-2, 1], [-2, -1], [-1, -1],
                      [-1, -2], [1, -2]], dtype=np.float64)
    off, xy, _ = oracle.polygon_cells(X[:, 0], X[:, 1], np.zeros(800), cross[:, 0], cross[:, 1])
    a = np.array([_shoelace(xy[off[i]:off[i + 1]]) for i in range(800)])
    assert abs(a.sum() - 12.0) < 1e-11


def test_polygon_cells_agree_with_pieces(oracle):
    # clipped to the mesh's box, each site's polygon has the area of its pieces, and
    # its neighbour labels are the site's regular-triangulation neighbours
    rng = np.random.default_rng(2)
    n = 300
    X = rng.uniform(0, 1, (n, 2))
    w = rng.uniform(-1, 1, n) * 3e-3
    mesh = unit_grid(9, np.ones(81))
    r = oracle.kantorovich(mesh, X[:, 0], X[:, 1], w, keep_pieces=True)
    P = r.pieces
    piece_area = np.zeros(n)
    for k in range(P.site.shape[0]):
        piece_area[P.site[k]] += _shoelace(P.xy[P.offsets[k]:P.offsets[k + 1]])
    box = np.array([[0, 0], [1, 0], [1, 1], [0, 1]], dtype=np.float64)
    off, xy, lab = oracle.polygon_cells(X[:, 0], X[:, 1], w, box[:, 0], box[:, 1])
    a = np.array([_shoelace(xy[off[i]:off[i + 1]]) for i in range(n)])
    np.testing.assert_allclose(a, piece_area, rtol=0, atol=1e-14)
    for i in range(n):
        nb = set(int(v) for v in lab[off[i]:off[i + 1]] if v >= 0)
        assert nb == set(int(v) for v in r.neighbors[i])


def test_polygon_cells_candidates_change_nothing(oracle):
    # clipping by every other site gives the same polygons as the triangulation's
    # neighbours: the candidate lists hide no cut
    rng = np.random.default_rng(3)
    n = 90
    X = rng.uniform(-1, 1, (n, 2))
    w = rng.uniform(-1, 1, n) * 1e-2
    q = np.array([[-0.8, -0.9], [0.9, -0.7], [0.6, 0.8], [-0.7, 0.5]])
    off, xy, lab = oracle.polygon_cells(X[:, 0], X[:, 1], w, q[:, 0], q[:, 1])
    L = oracle.lib()
    import ctypes
    dp = ctypes.POINTER(ctypes.c_double)
    ip = ctypes.POINTER(ctypes.c_int)
    xs, ys, ws = (np.ascontiguousarray(v) for v in (X[:, 0], X[:, 1], w))
    qx, qy = np.ascontiguousarray(q[:, 0]), np.ascontiguousarray(q[:, 1])
    allc = np.arange(n, dtype=np.int32)
    out = np.zeros((512, 2))
    ol = np.zeros(512, np.int32)
    for i in range(n):
        m = L.ora_polygon_cell(n, xs.ctypes.data_as(dp), ys.ctypes.data_as(dp), ws.ctypes.data_as(dp), i,
                               allc.ctypes.data_as(ip), n, 4, qx.ctypes.data_as(dp), qy.ctypes.data_as(dp), 512,
                               out.ctypes.data_as(dp), ol.ctypes.data_as(ip))
        assert m == off[i + 1] - off[i]
        if m:
            a = xy[off[i]:off[i + 1]]
            s = int(np.argmin(np.abs(out[:m] - a[0]).max(1)))
            np.testing.assert_array_equal(np.roll(out[:m], -s, axis=0), a)


def _exact_triangle_integrals(lin, site, tri):
    """Exact integrals over a triangle with rational corners of rho |x - s|^2, rho,
    rho x, rho y, rho x^2, rho y^2, rho x y (rho = a x + b y + c): the integrand as a
    polynomial in the reference coordinates (u, v), x = A + u (B - A) + v (C - A), and
    int_ref u^i v^j = i! j! / (i + j + 2)!."""
    from fractions import Fraction as Fr
    from math import factorial

    def mul(p, q):
        r = {}
        for (i, j), a in p.items():
            for (k, l), b in q.items():
                r[(i + k, j + l)] = r.get((i + k, j + l), 0) + a * b
        return r

    def add(*ps):
        r = {}
        for p in ps:
            for k, a in p.items():
                r[k] = r.get(k, 0) + a
        return r

    def const(c):
        return {(0, 0): Fr(c)}

    (ax, ay), (bx, by), (cx, cy) = [(Fr(p[0]), Fr(p[1])) for p in tri]
    X = {(0, 0): ax, (1, 0): bx - ax, (0, 1): cx - ax}
    Y = {(0, 0): ay, (1, 0): by - ay, (0, 1): cy - ay}
    a, b, c = (Fr(t) for t in lin)
    rho = add(mul(const(a), X), mul(const(b), Y), const(c))
    dx, dy = add(X, const(-Fr(site[0]))), add(Y, const(-Fr(site[1])))
    polys = [mul(rho, add(mul(dx, dx), mul(dy, dy))), rho, mul(rho, X), mul(rho, Y), mul(rho, mul(X, X)),
             mul(rho, mul(Y, Y)), mul(rho, mul(X, Y))]
    jac = abs((bx - ax) * (cy - ay) - (cx - ax) * (by - ay))
    return [float(jac * sum(v * Fr(factorial(i) * factorial(j), factorial(i + j + 2)) for (i, j), v in p.items()))
            for p in polys]


def test_albrecht_collatz_is_exact_for_cubics(oracle):
    # tests/test_quadrature_triangle.cpp:10-21: the 6-point rule integrates x y^2 (and
    # every integrand of degree <= 3) exactly; here on random triangles with dyadic
    # corners (exact in binary) against rational arithmetic
    from fractions import Fraction as Fr
    rng = np.random.default_rng(12)
    for _ in range(50):
        tri = rng.integers(-64, 64, size=(3, 2)) / 32.0
        cr = (tri[1, 0] - tri[0, 0]) * (tri[2, 1] - tri[0, 1]) - (tri[2, 0] - tri[0, 0]) * (tri[1, 1] - tri[0, 1])
        if abs(cr) < 1e-3:
            continue
        if cr < 0:  # the rule weighs by CGAL's signed area: counter-clockwise corners
            tri = tri[[0, 2, 1]]
        lin = rng.integers(-16, 16, size=3) / 8.0
        site = rng.integers(-32, 32, size=2) / 16.0
        got = oracle.albrecht_collatz(lin, site, tri)
        want = _exact_triangle_integrals([Fr(t) for t in lin], [Fr(t) for t in site], tri.tolist())
        scale = max(1e-300, max(abs(v) for v in want))
        np.testing.assert_allclose(got, want, rtol=0, atol=1e-14 * scale)
        # clockwise corners give the negated integrals (signed area)
        np.testing.assert_allclose(oracle.albrecht_collatz(lin, site, tri[[0, 2, 1]]), -got, rtol=0,
                                   atol=1e-14 * scale)
    # the reference test's own integrand: x y^2 is rho = x times the y^2 moment
    got = oracle.albrecht_collatz((1.0, 0.0, 0.0), (0.0, 0.0), [[0, 0], [1, 0], [0, 1]])
    assert got[5] == pytest.approx(1.0 / 60.0, rel=1e-15)
