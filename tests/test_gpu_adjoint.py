"""The adjoint (ma_kantorovich_vjp): vector-Jacobian products of the Kantorovich value,
the cell masses and the first moments with respect to the sites, the weights and the
density's vertex values.  The reference has no adjoint; its finite-difference harness
(tests/test_opttransport_eval.cpp:20-55, method only) is the model: central differences
of the oracle, which restates the reference's evaluation, and of the GPU forward pass."""
import numpy as np
import pytest

from mongeampere_gb300 import workloads as W
from mongeampere_gb300.mesh import GridMesh

pytestmark = pytest.mark.gpu

FD_H = 1e-6
FD_RTOL = 1e-5  # relative agreement of adjoint and central differences


@pytest.fixture(scope="module")
def ctx():
    from mongeampere_gb300 import api
    return api.Context(0)


def _problem(seed=3, n=300, grid=24):
    p = W.make_problem(grid, n, "uniform", "uniform", "equal", seed=seed)
    rng = np.random.default_rng(seed + 100)
    w = rng.uniform(-1.0, 1.0, n) * 2e-4  # small weights: every cell stays non-empty
    return p, w


def _cotangents(n, seed):
    rng = np.random.default_rng(seed)
    return float(rng.normal()), rng.normal(size=n), rng.normal(size=(n, 2))


def _objective_oracle(oracle, mesh, x, y, w, a, b, e):
    r = oracle.kantorovich(mesh, x, y, w, arith="dd")
    return a * r.value + b @ r.g + np.sum(e * r.moments[:, 1:3])


def test_weight_gradient_is_hessian_transpose_times_cotangent(ctx):
    # d m_i / d w_j = H_ij: the masses' part of grad_w is H^T b (H symmetric)
    from mongeampere_gb300 import api
    p, w = _problem()
    X = np.c_[p.x, p.y]
    _, b, _ = _cotangents(p.n, 1)
    _, g, h = api.kantorovich(p.mesh, X, w, ctx=ctx)
    _, gw, _ = api.kantorovich_vjp(p.mesh, X, w, 0.0, b, None, ctx=ctx)
    ref = h.to_scipy() @ b
    np.testing.assert_allclose(gw, ref, rtol=0, atol=1e-12 * np.abs(ref).max())


def test_value_gradients_are_masses_and_moments(ctx):
    # d Phi / d w_i = m_i and d Phi / d x_i = 2 (int rho x - x_i m_i)
    from mongeampere_gb300 import api
    p, w = _problem(seed=5)
    X = np.c_[p.x, p.y]
    m, first = api.first_moment(p.mesh, X, w, ctx=ctx)
    gX, gw, _ = api.kantorovich_vjp(p.mesh, X, w, 1.0, None, None, grad_rho=False, ctx=ctx)
    np.testing.assert_allclose(gw, m, rtol=0, atol=1e-13 * m.max())
    ref = 2.0 * (first - X * m[:, None])
    np.testing.assert_allclose(gX, ref, rtol=0, atol=1e-12 * np.abs(ref).max())


def _central(fun, h):
    # central difference at steps h and h/2, Richardson-extrapolated (O(h^4)): the
    # outputs are smooth but strongly curved in w at nearly vanishing cells
    d1 = (fun(h) - fun(-h)) / (2 * h)
    d2 = (fun(h / 2) - fun(-h / 2)) / h
    return (4 * d2 - d1) / 3


@pytest.mark.parametrize("seed", [11, 12])
def test_adjoint_matches_oracle_central_differences(ctx, oracle, seed):
    from mongeampere_gb300 import api
    p, w = _problem(seed=seed)
    x, y = p.x.copy(), p.y.copy()
    a, b, e = _cotangents(p.n, seed)
    gX, gw, gr = api.kantorovich_vjp(p.mesh, np.c_[x, y], w, a, b, e, ctx=ctx)
    rng = np.random.default_rng(seed + 7)
    f = lambda xx, yy, ww, mesh=p.mesh: _objective_oracle(oracle, mesh, xx, yy, ww, a, b, e)
    checks = []
    for i in rng.choice(p.n, 6, replace=False):
        for comp in (0, 1):
            def fx(t, i=i, comp=comp):
                xx, yy = x.copy(), y.copy()
                (xx if comp == 0 else yy)[i] += t
                return f(xx, yy, w)
            checks.append((_central(fx, FD_H), gX[i, comp]))
    for i in rng.choice(p.n, 6, replace=False):
        def fw(t, i=i):
            ww = w.copy()
            ww[i] += t
            return f(x, y, ww)
        checks.append((_central(fw, FD_H), gw[i]))
    vals = p.mesh.values.ravel()
    for k in rng.choice(vals.size, 6, replace=False):
        def fr(t, k=k):
            vv = vals.copy()
            vv[k] += t
            return f(x, y, w, GridMesh(p.mesh.gx, p.mesh.gy, vv.reshape(p.mesh.values.shape)))
        checks.append((_central(fr, FD_H), gr[k]))
    fd = np.array([c[0] for c in checks])
    ad = np.array([c[1] for c in checks])
    scale = np.maximum(np.abs(fd), 1e-3 * np.abs(fd).max())
    assert np.all(np.abs(ad - fd) <= FD_RTOL * scale), np.c_[fd, ad]


def test_directional_derivative_of_gpu_forward(ctx):
    # all coordinates at once: <grad, v> against central differences of the GPU's
    # own FP64 forward along a random direction
    from mongeampere_gb300 import api
    p, w = _problem(seed=21, n=2000, grid=64)
    X = np.c_[p.x, p.y]
    a, b, e = _cotangents(p.n, 21)
    gX, gw, gr = api.kantorovich_vjp(p.mesh, X, w, a, b, e, ctx=ctx)
    rng = np.random.default_rng(22)
    vX = rng.normal(size=X.shape) * 1e-3
    vw = rng.normal(size=w.shape) * 1e-5

    def f(t):
        v, g, _ = api.kantorovich(p.mesh, X + t * vX, w + t * vw, hessian=False, ctx=ctx)
        _, first = api.first_moment(p.mesh, X + t * vX, w + t * vw, ctx=ctx)
        return a * v + b @ np.asarray(g) + np.sum(e * np.asarray(first))

    h = 1e-4
    fd = (f(h) - f(-h)) / (2 * h)
    ad = np.sum(gX * vX) + gw @ vw
    assert abs(ad - fd) <= FD_RTOL * abs(fd)


def test_density_gradient_is_linear_functional(ctx):
    # the cells do not depend on rho and every output is linear in it, so Euler's
    # relation holds: grad_rho . rho = a value + b . m + e . first
    from mongeampere_gb300 import api
    p, w = _problem(seed=31)
    X = np.c_[p.x, p.y]
    a, b, e = _cotangents(p.n, 31)
    _, _, gr = api.kantorovich_vjp(p.mesh, X, w, a, b, e, ctx=ctx)
    v, g, _ = api.kantorovich(p.mesh, X, w, hessian=False, ctx=ctx)
    m, first = api.first_moment(p.mesh, X, w, ctx=ctx)
    ref = a * v + b @ m + np.sum(e * first)
    assert abs(gr @ p.mesh.values.ravel() - ref) <= 1e-10 * max(1.0, abs(ref))


def test_torch_autograd_binding(ctx):
    torch = pytest.importorskip("torch")
    from mongeampere_gb300 import api
    from mongeampere_gb300.autograd import centroids, laguerre
    p, _ = _problem(seed=41)
    w = np.zeros(p.n)  # Voronoi cells: every mass positive, every centroid defined
    dev = torch.device("cuda", 0)
    dm = ctx.mesh(p.mesh)
    X = torch.tensor(np.c_[p.x, p.y], device=dev, requires_grad=True)
    wt = torch.tensor(w, device=dev, requires_grad=True)
    rho = torch.tensor(p.mesh.values.ravel(), device=dev, requires_grad=True)
    value, m, first = laguerre(X, wt, rho, dm, ctx)
    c, _ = centroids(X, wt, rho, dm, ctx)
    loss = value + (m * m).sum() + (c * c).sum()
    loss.backward()
    gX, gw, gr = X.grad.cpu().numpy(), wt.grad.cpu().numpy(), rho.grad.cpu().numpy()
    assert np.isfinite(loss.item()) and np.isfinite(gX).all() and np.isfinite(gw).all() and np.isfinite(gr).all()
    # against the ABI call with the chain rule written out
    mm, ff = api.first_moment(p.mesh, np.c_[p.x, p.y], w, ctx=ctx)
    assert mm.min() > 0
    cc = ff / mm[:, None]
    e = 2 * cc / mm[:, None]
    b = 2 * mm - np.sum(2 * cc * cc, 1) / mm
    rX, rw, rr = api.kantorovich_vjp(p.mesh, np.c_[p.x, p.y], w, 1.0, b, e, ctx=ctx)
    np.testing.assert_allclose(gX, rX, rtol=1e-10, atol=1e-12 * np.abs(rX).max())
    np.testing.assert_allclose(gw, rw, rtol=1e-10, atol=1e-12 * np.abs(rw).max())
    np.testing.assert_allclose(gr, rr, rtol=1e-9, atol=1e-12 * np.abs(rr).max())


def _gpu_objective(api, ctx, mesh, X, w, a, b, e):
    v, g, _ = api.kantorovich(mesh, X, w, hessian=False, ctx=ctx)
    _, first = api.first_moment(mesh, X, w, ctx=ctx)
    return a * v + float(np.dot(b, np.asarray(g))) + float(np.sum(e * np.asarray(first)))


@pytest.mark.parametrize("solved", [False, True])
def test_fp32_adjoint_against_fp64_adjoint_and_central_differences(ctx, solved):
    # The FP32 adjoint (precision="mixed": the pieces' integrals in FP32 about a point of
    # each cell) against the FP64 adjoint, at w = 0 and at the solution of a Gaussian
    # density (cells far from their sites); and both against central differences
    # of the GPU's FP64 forward pass on 100 random coordinates of the sites, the weights
    # and the density's vertex values, with h = 1e-6 in each coordinate's own scale: the
    # mean cell size 1/sqrt(n) for the sites, the mean cell area 1/n for the weights, 1 for
    # the vertex values.  (A weight step of 1e-6 is several percent of a cell's weight
    # scale here, and near a short edge the objective bends within it: the central
    # difference converges to the adjoint only for smaller steps.)
    from mongeampere_gb300 import api
    p = W.make_problem(128, 20000, "gauss", "uniform", "random", seed=21)
    X = np.c_[p.x, p.y]
    w = np.zeros(p.n)
    if solved:
        w = np.asarray(api.ot_solve(p.mesh, X, p.nu, eps_g=1e-6, stop="rel", ctx=ctx))
    a, b, e = _cotangents(p.n, 8)
    g64 = api.kantorovich_vjp(p.mesh, X, w, a, b, e, ctx=ctx)
    g32 = api.kantorovich_vjp(p.mesh, X, w, a, b, e, precision="mixed", ctx=ctx)
    for q64, q32 in zip(g64, g32):
        q64, q32 = np.asarray(q64), np.asarray(q32)
        assert np.linalg.norm(q32 - q64) <= 1e-4 * np.linalg.norm(q64)
    rng = np.random.default_rng(9)
    vals = p.mesh.values.copy()
    dm = ctx.mesh(p.mesh)
    kinds = rng.integers(0, 4, 100)
    fd, ad64, ad32 = [], [], []
    for kind in kinds:
        if kind < 2:  # a site coordinate
            i = int(rng.integers(p.n))
            def f(t):
                Xp = X.copy()
                Xp[i, kind] += t
                return _gpu_objective(api, ctx, dm, Xp, w, a, b, e)
            ad64.append(g64[0][i, kind])
            ad32.append(g32[0][i, kind])
        elif kind == 2:  # a weight
            i = int(rng.integers(p.n))
            def f(t):
                wp = w.copy()
                wp[i] += t
                return _gpu_objective(api, ctx, dm, X, wp, a, b, e)
            ad64.append(g64[1][i])
            ad32.append(g32[1][i])
        else:  # a density vertex value
            j = int(rng.integers(vals.size))
            def f(t):
                vp = vals.copy().reshape(-1)
                vp[j] += t
                dm.set_values(vp)
                r = _gpu_objective(api, ctx, dm, X, w, a, b, e)
                dm.set_values(vals.reshape(-1))
                return r
            ad64.append(g64[2][j])
            ad32.append(g32[2][j])
        hk = FD_H * (1.0 / p.n if kind == 2 else (p.n ** -0.5 if kind < 2 else 1.0))
        fd.append((f(hk) - f(-hk)) / (2 * hk))
    fd, ad64, ad32 = np.array(fd), np.array(ad64), np.array(ad32)
    scale = np.abs(fd).max()
    assert np.max(np.abs(ad64 - fd)) <= FD_RTOL * scale, f"FP64 adjoint vs FD: {np.max(np.abs(ad64 - fd)) / scale:.2e}"
    assert np.max(np.abs(ad32 - fd)) <= 1e-4 * scale, f"FP32 adjoint vs FD: {np.max(np.abs(ad32 - fd)) / scale:.2e}"
