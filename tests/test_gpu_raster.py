"""Laguerre-cell rasterisation (ma_draw_laguerre) against the oracle's restatement of
MA::draw_laguerre_diagram (include/MA/rasterization.hpp:403-547)."""
import numpy as np
import pytest

from mongeampere_gb300 import workloads as W

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    from mongeampere_gb300 import api
    return api.Context(0)


@pytest.mark.parametrize("seed,bbox,size", [(1, (0.0, 0.0, 1.0, 1.0), (64, 48)),
                                            (2, (-0.1, 0.2, 0.9, 1.1), (37, 53))])
def test_raster_matches_oracle(ctx, oracle, seed, bbox, size):
    from mongeampere_gb300 import api
    p = W.make_problem(16, 60, "uniform", "uniform", "equal", seed=seed)
    rng = np.random.default_rng(seed)
    w = rng.uniform(-1, 1, p.n) * 1e-3
    colors = rng.uniform(0, 1, (p.n, 3))
    width, height = size
    img = api.draw_laguerre_diagram(p.mesh, np.c_[p.x, p.y], w, colors, bbox, width, height, ctx=ctx)
    ref = oracle.draw_laguerre_diagram(p.mesh, p.x, p.y, w, colors, bbox, width, height)
    assert img.shape == ref.shape
    # exact coverage on both sides (clipped relative to each pixel's corner); the
    # order of the atomic sums leaves a few units of 1e-16
    np.testing.assert_allclose(img, ref, rtol=0, atol=1e-12 * max(1.0, np.abs(ref).max()))


def test_raster_coverage_sums_to_mass(ctx):
    # colour 1 and a constant density: the image holds each pixel's covered area, so
    # the image integrates to the mesh area in pixel units
    from mongeampere_gb300 import api
    from mongeampere_gb300.mesh import unit_grid
    mesh = unit_grid(40, np.ones((40, 40)))
    rng = np.random.default_rng(3)
    x, y = rng.uniform(0, 1, 3000), rng.uniform(0, 1, 3000)
    img = api.draw_laguerre_diagram(mesh, np.c_[x, y], np.zeros(3000), np.ones(3000), (0, 0, 1, 1), 300, 200,
                                    ctx=ctx)
    np.testing.assert_allclose(img, 1.0, rtol=0, atol=1e-12)
