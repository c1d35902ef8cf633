"""Failure statuses of the solver, each made by the inputs on the host (no GPU fault):
the iteration cap, a target the masses cannot reach, a cell beyond every capacity, and a
conjugate-gradient solve stopped by its cap.  The reference reports the first with
Statistics::niter, loops forever on the second (optimal_transport.hpp:163-176), and has
no capacity or CG limit (CGAL and Eigen allocate as they go)."""
import numpy as np
import pytest

from mongeampere_gb300 import workloads as W

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    from mongeampere_gb300 import api
    return api.Context(0)


def test_maxiter_status_and_count(ctx):
    # maxiter = 1: the reference's loop `niter++ <= maxiter` runs two Newton steps and
    # leaves niter = 3 (optimal_transport.hpp:150-151)
    from mongeampere_gb300 import _lib, api
    p = W.make_problem(48, 1500, "gauss", "uniform", "random", seed=5)
    st = api.Statistics()
    w = api.ot_solve(p.mesh, np.c_[p.x, p.y], p.nu, eps_g=1e-12, stop="rel", maxiter=1, stats=st, ctx=ctx,
                     raise_on_error=False)
    assert st.status == _lib.MA_MAXITER
    assert st.niter == 3
    assert np.isfinite(w).all() and st.max_rel_err > 1e-12


def test_unreachable_target_fails_the_line_search(ctx, oracle):
    # target masses summing to 1.1x the density's mass: no weights reach them; the
    # reference's backtracking halves alpha forever, here it stops below 2^-40
    from mongeampere_gb300 import _lib, api
    p = W.make_problem(24, 200, seed=3)
    with pytest.raises(RuntimeError, match="line search"):
        oracle.ot_solve(p.mesh, p.x, p.y, p.nu * 1.1, tol_rel=1e-9, arith="fp64", ring=1)
    st = api.Statistics()
    w = api.ot_solve(p.mesh, np.c_[p.x, p.y], p.nu * 1.1, eps_g=1e-9, stop="rel", stats=st, ctx=ctx,
                     raise_on_error=False)
    assert st.status == _lib.MA_LINESEARCH_FAIL
    assert np.isfinite(w).all()
    assert st.linesearch_halvings >= 40


def _ring_of_sites(k):
    t = np.linspace(0.0, 2.0 * np.pi, k, endpoint=False)
    x = np.r_[0.5, 0.5 + 0.3 * np.cos(t)]
    y = np.r_[0.5, 0.5 + 0.3 * np.sin(t)]
    return x, y


def test_cell_beyond_every_capacity(ctx, oracle):
    # the centre site of a ring of 300 sites has 300 neighbours, more than the 256 slots
    # of the large-capacity pass: the evaluation says so instead of truncating the cell
    from mongeampere_gb300 import _lib, api
    from mongeampere_gb300.mesh import unit_grid
    mesh = unit_grid(8, np.ones((8, 8)))
    x, y = _ring_of_sites(300)
    r = oracle.kantorovich(mesh, x, y, np.zeros(x.size))
    assert len(r.neighbors[0]) == 300
    with pytest.raises(_lib.MaError) as ei:
        api.kantorovich(mesh, np.c_[x, y], np.zeros(x.size), ctx=ctx)
    assert ei.value.status == _lib.MA_ERR_CAPACITY
    # 200 neighbours fit the large-capacity pass and match the oracle
    x, y = _ring_of_sites(200)
    v, g, h = api.kantorovich(mesh, np.c_[x, y], np.zeros(x.size), ctx=ctx)
    r = oracle.kantorovich(mesh, x, y, np.zeros(x.size))
    np.testing.assert_allclose(np.asarray(g), r.g, rtol=0, atol=1e-12 * r.g.max())
    assert h.col.shape[0] == r.cols.shape[0]


def test_cg_cap_is_reported(ctx):
    # a Newton direction whose CG is capped at one iteration: ma_laplacian_solve
    # returns MA_CG_NOCONV; in a solve the step is counted in cg_noconv and the
    # line search still decides whether to take it
    from mongeampere_gb300 import _lib, api
    p = W.make_problem(48, 2000, seed=2)
    v, g, h = api.kantorovich(p.mesh, np.c_[p.x, p.y], np.zeros(p.n), ctx=ctx)
    rhs = np.asarray(g) - p.nu
    with pytest.raises(_lib.MaError) as ei:
        api.solve_laplacian_matrix(rhs, rtol=1e-13, maxiter=1, ctx=ctx)
    assert ei.value.status == _lib.MA_CG_NOCONV
    st = api.Statistics()
    api.ot_solve(p.mesh, np.c_[p.x, p.y], p.nu, eps_g=1e-9, stop="rel", cg_maxiter=1, precond="jacobi",
                 maxiter=200, stats=st, ctx=ctx, raise_on_error=False)
    assert st.cg_noconv >= 1 and st.cg_noconv <= st.niter
    st2 = api.Statistics()
    api.ot_solve(p.mesh, np.c_[p.x, p.y], p.nu, eps_g=1e-9, stop="rel", stats=st2, ctx=ctx)
    assert st2.cg_noconv == 0
