"""Materialised pieces (ma_pieces / ma_pieces_copy) against the oracle's restatement of
MA::voronoi_triangulation_intersection (voronoi_triangulation_intersection.hpp:219-343):
the same (site, triangle) pairs, the same polygons (vertices and edge labels), and the
area invariant of tests/test_voronoi_tri.cpp:67 at scale."""
import numpy as np
import pytest

from mongeampere_gb300 import workloads as W

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    from mongeampere_gb300 import api
    return api.Context(0)


def _area(xy):
    x, y = xy[:, 0], xy[:, 1]
    return 0.5 * np.sum(x * np.roll(y, -1) - np.roll(x, -1) * y)


@pytest.mark.parametrize("seed,density", [(1, "uniform"), (2, "gauss")])
def test_pieces_match_oracle(ctx, oracle, seed, density):
    from mongeampere_gb300 import api
    p = W.make_problem(24, 300, density, "uniform", "equal", seed=seed)
    w = np.random.default_rng(seed).uniform(-1, 1, p.n) * 3e-4
    P = api.pieces(p.mesh, np.c_[p.x, p.y], w, ctx=ctx)
    r = oracle.kantorovich(p.mesh, p.x, p.y, w, keep_pieces=True, arith="dd")
    R = r.pieces
    gpu = {(int(s), int(t)): k for k, (s, t) in enumerate(zip(P.site, P.tri))}
    ora = {(int(s), int(t)): k for k, (s, t) in enumerate(zip(R.site, R.face))}
    assert set(gpu) == set(ora)
    assert len(gpu) == len(P.site)  # each pair once
    for key, kg in gpu.items():
        ko = ora[key]
        xg, eg = P.polygon(kg)
        xo = R.xy[R.offsets[ko]:R.offsets[ko + 1]]
        eo = R.label[R.offsets[ko]:R.offsets[ko + 1]]
        assert xg.shape == xo.shape, key
        # the same polygon up to the starting vertex
        d = np.abs(xo[:, None, :] - xg[None, 0, :]).max(-1)
        s = int(np.argmin(d))
        xo = np.roll(xo, -s, axis=0)
        eo = np.roll(eo, -s)
        np.testing.assert_allclose(xg, xo, rtol=0, atol=1e-12)
        np.testing.assert_array_equal(np.where(eg < 0, -1, eg), eo)
        assert _area(xg) > 0  # counter-clockwise


def test_pieces_tile_the_domain_at_scale(ctx):
    # the pieces partition the unit square: total area 1, and every triangle's
    # pieces add up to its area
    from mongeampere_gb300 import api
    p = W.make_problem(128, 20000, "gauss", "uniform", "random", seed=3)
    P = api.pieces(p.mesh, np.c_[p.x, p.y], np.zeros(p.n), ctx=ctx)
    x, y = P.xy[:, 0], P.xy[:, 1]
    nxt = np.arange(len(x)) + 1
    last = P.off[1:] - 1
    nxt[last] = P.off[:-1]
    cr = x * y[nxt] - x[nxt] * y
    area = 0.5 * np.add.reduceat(cr, P.off[:-1])
    assert area.min() > 0
    assert abs(area.sum() - 1.0) < 1e-12
    tri_area = np.bincount(P.tri, weights=area, minlength=2 * 127 * 127)
    np.testing.assert_allclose(tri_area, 0.5 / 127 ** 2, rtol=1e-10)
    assert np.unique(P.site).shape[0] == p.n


def _lattice(k):
    g = (np.arange(k) + 0.5) / k
    X, Y = np.meshgrid(g, g)
    return X.ravel().copy(), Y.ravel().copy()


def test_pieces_of_an_exactly_degenerate_lattice(ctx, oracle):
    # Lattice sites: every vertex of every cell is co-circular with four sites and the
    # bisectors run through mesh vertices, so the clips meet exact ties, which send the
    # cells to the one-thread exact pass (the reference lists these pieces too,
    # voronoi_triangulation_intersection.hpp:315-343).  The pieces tile the square, each
    # cell is its 1/256 square, and the pieces of positive area are the oracle's.
    from mongeampere_gb300 import api
    from mongeampere_gb300.mesh import unit_grid
    x, y = _lattice(16)
    mesh = unit_grid(9, np.ones((9, 9)))
    w = np.zeros(x.size)
    P = api.pieces(mesh, np.c_[x, y], w, ctx=ctx)
    area = np.array([_area(P.polygon(k)[0]) for k in range(len(P.site))])
    assert area.min() >= -1e-15
    assert abs(area.sum() - 1.0) < 1e-12
    np.testing.assert_allclose(np.bincount(P.site, weights=area, minlength=x.size), 1.0 / x.size, rtol=1e-12)
    np.testing.assert_allclose(np.bincount(P.tri, weights=area, minlength=2 * 64), 0.5 / 64, rtol=1e-12)
    r = oracle.kantorovich(mesh, x, y, w, keep_pieces=True, arith="dd")
    R = r.pieces
    oarea = np.array([_area(R.xy[R.offsets[k]:R.offsets[k + 1]]) for k in range(len(R.site))])
    gpu = {(int(s), int(t)) for s, t, a in zip(P.site, P.tri, area) if a > 1e-14}
    ora = {(int(s), int(t)) for s, t, a in zip(R.site, R.face, oarea) if a > 1e-14}
    assert gpu == ora
    # the drawing goes through the same listing: colour 1 and a constant density give
    # each pixel's covered area
    img = api.draw_laguerre_diagram(mesh, np.c_[x, y], w, np.ones(x.size), (0, 0, 1, 1), 64, 64, ctx=ctx)
    np.testing.assert_allclose(img, 1.0, rtol=0, atol=1e-12)
