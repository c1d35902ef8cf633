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
