"""MA::first_moment, MA::second_moment and MA::lloyd (include/MA/lloyd.hpp:30-144)
against the oracle's moments: mass, int rho x, int rho y, int rho x^2, int rho y^2,
int rho x y per cell, and the centroids (first moments over mass).  The bar is the
FP64 one: 1e-12 relative, with a floor of 1e-12 of the largest entry for moments that
are themselves sums of cancelling parts."""
import numpy as np
import pytest

from mongeampere_gb300 import workloads as W

pytestmark = pytest.mark.gpu

RTOL = 1e-12


@pytest.fixture(scope="module")
def ctx():
    from mongeampere_gb300 import api
    return api.Context(0)


def _close(a, b, what):
    a, b = np.asarray(a, float), np.asarray(b, float)
    err = np.abs(a - b)
    bad = err > RTOL * np.abs(b) + RTOL * np.abs(b).max()
    assert not bad.any(), f"{what}: max err {err.max():.3e}, {bad.sum()} entries off"


CASES = [
    ("c1 grid, random weights", lambda: (W.c1(1), 3e-4)),
    ("gauss density", lambda: (W.make_problem(128, 5000, "gauss", "uniform", "random", seed=3), 5e-5)),
    ("clustered sites", lambda: (W.make_problem(128, 8000, "uniform", "blobs", "equal", seed=4), 0.0)),
]


@pytest.mark.parametrize("name,make", CASES, ids=[c[0] for c in CASES])
def test_moments_match_oracle(ctx, oracle, name, make):
    from mongeampere_gb300 import api
    p, amp = make()
    w = np.random.default_rng(11).uniform(-amp, amp, p.n) if amp else np.zeros(p.n)
    X = np.c_[p.x, p.y]
    r = oracle.kantorovich(p.mesh, p.x, p.y, w)
    m1, first = api.first_moment(p.mesh, X, w, ctx=ctx)
    m2, first2, inertia = api.second_moment(p.mesh, X, w, ctx=ctx)
    ml, cen = api.lloyd(p.mesh, X, w, ctx=ctx)
    for m in (m1, m2, ml):
        _close(m, r.moments[:, 0], "mass")
    _close(first, r.moments[:, 1:3], "first moments")
    _close(first2, r.moments[:, 1:3], "first moments (second_moment call)")
    _close(inertia, r.moments[:, 3:6], "second moments")
    # lloyd.hpp:126-144: the centroid is the first moment over the mass
    _, cref = oracle.lloyd(p.mesh, p.x, p.y, w)
    live = r.moments[:, 0] > 0
    _close(np.asarray(cen)[live], cref[live], "centroids")
    # the inertia tensor is positive semidefinite about the centroid
    m = r.moments[live, 0]
    cx, cy = cref[live, 0], cref[live, 1]
    ixx = np.asarray(inertia)[live, 0] / m - cx * cx
    iyy = np.asarray(inertia)[live, 1] / m - cy * cy
    ixy = np.asarray(inertia)[live, 2] / m - cx * cy
    assert (ixx > -1e-15).all() and (iyy > -1e-15).all()
    assert (ixx * iyy - ixy * ixy > -1e-15).all()


def test_moments_on_explicit_mesh(ctx, oracle):
    from scipy.spatial import Delaunay

    from mongeampere_gb300 import api
    from mongeampere_gb300.mesh import TriMesh
    rng = np.random.default_rng(12)
    g = np.linspace(0, 1, 20)
    X, Y = np.meshgrid(g, g)
    pts = np.c_[X.ravel(), Y.ravel()]
    inner = (pts > 0).all(1) & (pts < 1).all(1)
    pts[inner] += rng.uniform(-0.01, 0.01, (inner.sum(), 2))
    mesh = TriMesh(pts[:, 0], pts[:, 1], rng.uniform(0.5, 1.5, len(pts)), Delaunay(pts).simplices)
    x, y = rng.uniform(0, 1, 600), rng.uniform(0, 1, 600)
    w = rng.uniform(-2e-4, 2e-4, 600)
    r = oracle.kantorovich(mesh, x, y, w)
    m, first, inertia = api.second_moment(mesh, np.c_[x, y], w, ctx=ctx)
    _close(m, r.moments[:, 0], "mass")
    _close(first, r.moments[:, 1:3], "first moments")
    _close(inertia, r.moments[:, 3:6], "second moments")
