"""The W2-flow / Lloyd driver (ma_w2_flow) against the same iteration restated with the
oracle (tests/test_zeldovich.cpp:99-119: solve, centroids, x <- x + tau (x - c))."""
import numpy as np
import pytest

from mongeampere_gb300 import workloads as W

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("tau", [0.03, -1.0])
def test_w2_flow_matches_oracle_iteration(oracle, tau):
    from mongeampere_gb300 import api
    ctx = api.Context(0)
    p = W.make_problem(24, 300, "uniform", "uniform", "equal", seed=4)
    X, w, st = api.w2_flow(p.mesh, np.c_[p.x, p.y], p.nu, steps=3, tau=tau, eps_g=1e-11, ctx=ctx)
    x, y, wo = p.x.copy(), p.y.copy(), np.zeros(p.n)
    for _ in range(3):
        try:
            r = oracle.ot_solve(p.mesh, x, y, p.nu, w=wo, tol_rel=1e-11)
        except oracle.EmptyCellError:  # restart from zero weights, as the driver does
            r = oracle.ot_solve(p.mesh, x, y, p.nu, w=np.zeros(p.n), tol_rel=1e-11)
        wo = r.w
        m, c = oracle.lloyd(p.mesh, x, y, wo)
        x = x + tau * (x - c[:, 0])
        y = y + tau * (y - c[:, 1])
    np.testing.assert_allclose(X[:, 0], x, rtol=0, atol=1e-9)
    np.testing.assert_allclose(X[:, 1], y, rtol=0, atol=1e-9)
    assert st.max_rel_err <= 1e-11


def test_lloyd_steps_reduce_the_quantization_energy():
    # tau = -1 moves every site to its cell's centroid: the Laguerre energy at the
    # solved weights decreases step after step
    from mongeampere_gb300 import api
    ctx = api.Context(0)
    p = W.make_problem(32, 500, "gauss", "uniform", "equal", seed=5)
    X = np.c_[p.x, p.y]
    w = None
    energies = []
    for _ in range(4):
        X, w, _ = api.w2_flow(p.mesh, X, p.nu, steps=1, tau=-1.0, w=w, ctx=ctx)
        v, g, _ = api.kantorovich(p.mesh, X, w, hessian=False, ctx=ctx)
        energies.append(float(np.sum(np.asarray(w) * np.asarray(g)) - v))  # int rho |x - x_i|^2
    assert all(b < a for a, b in zip(energies, energies[1:]))
