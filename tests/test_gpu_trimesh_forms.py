"""The later forms on an explicit triangulation (binned triangles, one linear function
per face -- the path of include/CGAL/Triangulation_incremental_builder_2.h meshes):
listed pieces against the oracle, the adjoint against central differences of the
oracle (including the per-vertex density gradient through the mesh's own vertex
indices), and the mixed-precision evaluation's error."""
import numpy as np
import pytest

from mongeampere_gb300.mesh import TriMesh

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    from mongeampere_gb300 import api
    return api.Context(0)


def _mesh(seed=7, side=20):
    from scipy.spatial import Delaunay
    rng = np.random.default_rng(seed)
    g = np.linspace(0, 1, side)
    X, Y = np.meshgrid(g, g)
    pts = np.c_[X.ravel(), Y.ravel()]
    inner = (pts > 0).all(1) & (pts < 1).all(1)
    pts[inner] += rng.uniform(-0.01, 0.01, (inner.sum(), 2))
    tri = Delaunay(pts).simplices
    return TriMesh(pts[:, 0], pts[:, 1], rng.uniform(0.5, 1.5, len(pts)), tri), rng


def test_trimesh_pieces_match_oracle(ctx, oracle):
    from mongeampere_gb300 import api
    mesh, rng = _mesh()
    x, y = rng.uniform(0, 1, 400), rng.uniform(0, 1, 400)
    w = rng.uniform(-2e-4, 2e-4, 400)
    P = api.pieces(mesh, np.c_[x, y], w, ctx=ctx)
    R = oracle.kantorovich(mesh, x, y, w, keep_pieces=True, arith="dd").pieces
    gpu = {(int(s), int(t)): k for k, (s, t) in enumerate(zip(P.site, P.tri))}
    ora = {(int(s), int(t)): k for k, (s, t) in enumerate(zip(R.site, R.face))}
    assert set(gpu) == set(ora)
    for key, kg in gpu.items():
        ko = ora[key]
        xg, eg = P.polygon(kg)
        xo = R.xy[R.offsets[ko]:R.offsets[ko + 1]]
        eo = R.label[R.offsets[ko]:R.offsets[ko + 1]]
        s = int(np.argmin(np.abs(xo - xg[0]).max(1)))
        np.testing.assert_allclose(xg, np.roll(xo, -s, axis=0), rtol=0, atol=1e-12)
        np.testing.assert_array_equal(np.where(eg < 0, -1, eg), np.roll(eo, -s))


def test_trimesh_adjoint_matches_oracle_differences(ctx, oracle):
    from mongeampere_gb300 import api
    mesh, rng = _mesh(seed=9)
    n = 300
    x, y = rng.uniform(0, 1, n), rng.uniform(0, 1, n)
    w = np.zeros(n)
    a, b, e = float(rng.normal()), rng.normal(size=n), rng.normal(size=(n, 2))
    gX, gw, gr = api.kantorovich_vjp(mesh, np.c_[x, y], w, a, b, e, ctx=ctx)

    def f(xx, yy, ww, vals=None):
        m = mesh if vals is None else TriMesh(mesh.vx, mesh.vy, vals, mesh.tri)
        r = oracle.kantorovich(m, xx, yy, ww, arith="dd")
        return a * r.value + b @ r.g + np.sum(e * r.moments[:, 1:3])

    def central(fun, h=1e-6):
        d1 = (fun(h) - fun(-h)) / (2 * h)
        d2 = (fun(h / 2) - fun(-h / 2)) / h
        return (4 * d2 - d1) / 3

    checks = []
    for i in rng.choice(n, 4, replace=False):
        def fx(t, i=i):
            xx = x.copy()
            xx[i] += t
            return f(xx, y, w)
        checks.append((central(fx), gX[i, 0]))

        def fw(t, i=i):
            ww = w.copy()
            ww[i] += t
            return f(x, y, ww)
        checks.append((central(fw), gw[i]))
    for k in rng.choice(len(mesh.vx), 6, replace=False):
        def fr(t, k=k):
            vv = mesh.values.copy()
            vv[k] += t
            return f(x, y, w, vv)
        checks.append((central(fr), gr[k]))
    fd = np.array([c[0] for c in checks])
    ad = np.array([c[1] for c in checks])
    scale = np.maximum(np.abs(fd), 1e-3 * np.abs(fd).max())
    assert np.all(np.abs(ad - fd) <= 1e-5 * scale), np.c_[fd, ad]


def test_trimesh_mixed_precision_error(ctx):
    from mongeampere_gb300 import api
    mesh, rng = _mesh(seed=11, side=40)
    x, y = rng.uniform(0, 1, 3000), rng.uniform(0, 1, 3000)
    w = np.zeros(3000)
    v64, g64, h64 = api.kantorovich(mesh, np.c_[x, y], w, ctx=ctx)
    v32, g32, h32 = api.kantorovich(mesh, np.c_[x, y], w, precision="mixed", ctx=ctx)
    rel = np.abs(np.asarray(g32) - np.asarray(g64)) / np.asarray(g64)
    assert rel.max() < 2e-5
    np.testing.assert_array_equal(h32.col, h64.col)
