"""Every cell clipped to a polygon (ma_polygon_cells) against the oracle's restatement of
MA::voronoi_polygon_intersection (voronoi_polygon_intersection.hpp:27-188), and the area
invariants of the reference's drivers: Voronoi cells of random points in [-1, 1]^2
clipped to that square add up to 4 (tests/test_voronoi.cpp:39-50,
tests/test_power.cpp:42-51), and clipped to the non-convex cross of
tests/test_voronoi_ad.cpp:30-57 to the cross's area 12."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SQUARE = np.array([[-1, -1], [1, -1], [1, 1], [-1, 1]], dtype=np.float64)
CROSS = np.array([[1, -1], [2, -1], [2, 1], [1, 1], [1, 2], [-1, 2], [-1, 1], [-2, 1], [-2, -1], [-1, -1],
                  [-1, -2], [1, -2]], dtype=np.float64)


@pytest.fixture(scope="module")
def ctx():
    from mongeampere_gb300 import api
    return api.Context(0)


def _area(xy):
    if xy.shape[0] == 0:
        return 0.0
    x, y = xy[:, 0], xy[:, 1]
    return 0.5 * np.sum(x * np.roll(y, -1) - np.roll(x, -1) * y)


def _same_polygons(R, off, xy, lab, n):
    for i in range(n):
        xg, eg = R.polygon(i)
        xo, eo = xy[off[i]:off[i + 1]], lab[off[i]:off[i + 1]]
        assert xg.shape == xo.shape, i
        if xg.shape[0] == 0:
            continue
        # the same polygon up to the starting vertex
        s = int(np.argmin(np.abs(xo - xg[0]).max(1)))
        np.testing.assert_allclose(xg, np.roll(xo, -s, axis=0), rtol=0, atol=1e-12)
        np.testing.assert_array_equal(eg, np.roll(eo, -s))


def _sites(n, seed, lo=-1.0, hi=1.0):
    rng = np.random.default_rng(seed)
    return rng.uniform(lo, hi, (n, 2))


@pytest.mark.parametrize("seed,weighted", [(1, False), (2, True)])
def test_square_matches_oracle(ctx, oracle, seed, weighted):
    from mongeampere_gb300 import api
    X = _sites(300, seed)
    w = np.random.default_rng(seed + 50).uniform(-1, 1, 300) * 4e-3 if weighted else None
    R = api.voronoi_polygon_intersection(SQUARE, X, w, ctx=ctx)
    off, xy, lab = oracle.polygon_cells(X[:, 0], X[:, 1], np.zeros(300) if w is None else w, SQUARE[:, 0],
                                        SQUARE[:, 1])
    _same_polygons(R, off, xy, lab, 300)
    assert abs(R.areas().sum() - 4.0) < 1e-12
    assert np.all(R.areas() >= 0)


def test_voronoi_area_invariant_at_scale(ctx):
    # tests/test_power.cpp:42-51: 100,000 sites, total area of the clipped cells = 4
    from mongeampere_gb300 import api
    X = _sites(100000, 3)
    R = api.voronoi_polygon_intersection(SQUARE, X, ctx=ctx)
    a = R.areas()
    assert a.min() > 0
    assert abs(a.sum() - 4.0) < 1e-11
    # every site's cell contains the site: each polygon is the site's Voronoi cell
    assert np.all(R.off[1:] - R.off[:-1] >= 3)


def test_cross_non_convex(ctx, oracle):
    # tests/test_voronoi_ad.cpp:30-57: a 12-corner cross around [-1, 1]^2, sites inside
    # the square: the clipped areas add up to the cross's area 12
    from mongeampere_gb300 import api
    X = _sites(400, 4)
    R = api.voronoi_polygon_intersection(CROSS, X, ctx=ctx)
    off, xy, lab = oracle.polygon_cells(X[:, 0], X[:, 1], np.zeros(400), CROSS[:, 0], CROSS[:, 1])
    ref = np.array([_area(xy[off[i]:off[i + 1]]) for i in range(400)])
    np.testing.assert_allclose(R.areas(), ref, rtol=0, atol=1e-12)
    assert abs(R.areas().sum() - 12.0) < 1e-11
    X = _sites(20000, 5)
    assert abs(api.voronoi_polygon_intersection(CROSS, X, ctx=ctx).areas().sum() - 12.0) < 1e-10


def test_many_corners_second_pass(ctx, oracle):
    # a 40-gon holds more corners than the first pass: every site goes to the second
    from mongeampere_gb300 import api
    t = np.linspace(0, 2 * np.pi, 41)[:-1]
    P = np.c_[0.9 * np.cos(t), 0.9 * np.sin(t)]
    X = _sites(250, 6)
    w = np.random.default_rng(7).uniform(-1, 1, 250) * 2e-3
    R = api.voronoi_polygon_intersection(P, X, w, ctx=ctx)
    off, xy, lab = oracle.polygon_cells(X[:, 0], X[:, 1], w, P[:, 0], P[:, 1])
    _same_polygons(R, off, xy, lab, 250)
    assert abs(R.areas().sum() - _area(P)) < 1e-12


def test_small_polygon_and_empty_cells(ctx, oracle):
    # a small triangle: most cells miss it (empty polygons), sites outside it keep
    # the parts of their cells that reach in, and hidden sites (weights) are empty
    from mongeampere_gb300 import api
    P = np.array([[0.1, 0.1], [0.35, 0.15], [0.2, 0.4]])
    X = _sites(500, 8)
    w = np.random.default_rng(9).uniform(-1, 1, 500) * 2e-2
    R = api.voronoi_polygon_intersection(P, X, w, ctx=ctx)
    off, xy, lab = oracle.polygon_cells(X[:, 0], X[:, 1], w, P[:, 0], P[:, 1])
    _same_polygons(R, off, xy, lab, 500)
    cnt = R.off[1:] - R.off[:-1]
    assert (cnt == 0).sum() > 400
    assert abs(R.areas().sum() - _area(P)) < 1e-14


def test_clockwise_polygon_and_corner_copies(ctx, oracle):
    # the polygon's orientation is kept; its corners come out bit for bit
    from mongeampere_gb300 import api
    P = SQUARE[::-1].copy()
    X = _sites(60, 10)
    R = api.voronoi_polygon_intersection(P, X, ctx=ctx)
    off, xy, lab = oracle.polygon_cells(X[:, 0], X[:, 1], np.zeros(60), P[:, 0], P[:, 1])
    _same_polygons(R, off, xy, lab, 60)
    assert abs(R.areas().sum() + 4.0) < 1e-12
    corners = {tuple(c) for c in P}
    got = {tuple(v) for v in R.xy} & corners
    assert got == corners


def test_device_inputs_and_errors(ctx):
    torch = pytest.importorskip("torch")
    from mongeampere_gb300 import api
    from mongeampere_gb300 import _lib as L
    X = _sites(1000, 11)
    Xd = torch.tensor(X, device="cuda")
    a = api.voronoi_polygon_intersection(SQUARE, X, ctx=ctx)
    b = api.voronoi_polygon_intersection(SQUARE, Xd, ctx=ctx)
    np.testing.assert_array_equal(a.off, b.off)
    np.testing.assert_array_equal(a.xy, b.xy)
    with pytest.raises(RuntimeError):
        api.voronoi_polygon_intersection(SQUARE[:2], X, ctx=ctx)
    with pytest.raises(RuntimeError):
        api.voronoi_polygon_intersection(np.zeros((65, 2)), X, ctx=ctx)
    with pytest.raises(RuntimeError):
        api.voronoi_polygon_intersection(np.array([[0, 0], [1, 0], [np.nan, 1]]), X, ctx=ctx)
    # copy before any computation on a fresh context
    fresh = api.Context(0)
    st = fresh.lib.ma_polygon_cells_copy(fresh.h, None, None, None, L.MA_MEM_HOST)
    assert st == L.MA_ERR_INVALID_ARGUMENT
