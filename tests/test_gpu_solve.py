"""The damped Newton OT solve (ma_ot_solve, ma_laplacian_solve) against the oracle's
restatement of MA::ot_solve (direct sparse solves)."""
import numpy as np
import pytest

from mongeampere_gb300 import workloads as W

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    from mongeampere_gb300 import api
    return api.Context(0)


def test_laplacian_solve_matches_direct(ctx, oracle):
    from mongeampere_gb300 import api
    p = W.make_problem(48, 2000, seed=2)
    w = np.zeros(p.n)
    v, g, h = api.kantorovich(p.mesh, np.c_[p.x, p.y], w, ctx=ctx)
    assert np.asarray(g).min() > 0
    rhs = np.asarray(g) - p.nu
    d, it = api.solve_laplacian_matrix(rhs, rtol=1e-13, ctx=ctx)
    d_ref = oracle.solve_laplacian_matrix(h.to_scipy(), rhs)
    assert d[-1] == 0.0
    np.testing.assert_allclose(d, d_ref, rtol=0, atol=1e-9 * np.abs(d_ref).max())
    assert it > 0


def test_ot_solve_matches_oracle(ctx, oracle):
    from mongeampere_gb300 import api
    p = W.make_problem(48, 1500, "gauss", "uniform", "random", seed=5)
    st = api.Statistics()
    w = api.ot_solve(p.mesh, np.c_[p.x, p.y], p.nu, eps_g=1e-10, stop="rel", stats=st, ctx=ctx)
    ref = oracle.ot_solve(p.mesh, p.x, p.y, p.nu, tol_rel=1e-10)
    assert st.max_rel_err <= 1e-10
    assert w[-1] == 0.0
    # the solution is unique once w[n-1] is fixed
    np.testing.assert_allclose(w, ref.w, rtol=0, atol=1e-9 * np.abs(ref.w).max())
    # masses of the GPU weights, checked by the oracle
    r = oracle.kantorovich(p.mesh, p.x, p.y, np.asarray(w))
    assert np.max(np.abs(r.g - p.nu) / p.nu) <= 2e-10
    assert st.niter <= ref.niter + 3


def test_c1_reference_stop_rule(ctx, oracle):
    # the reference's rule |m - nu|_2 < 1e-7 and the 1e-9 relative rule of the
    # 64^2 / 1000-site workload
    from mongeampere_gb300 import api
    p = W.c1(0)
    st = api.Statistics()
    w = api.ot_solve(p.mesh, np.c_[p.x, p.y], p.nu, eps_g=1e-9, stop="rel", stats=st, ctx=ctx)
    assert st.max_rel_err <= 1e-9
    ref = oracle.ot_solve(p.mesh, p.x, p.y, p.nu, tol_rel=1e-9)
    np.testing.assert_allclose(w, ref.w, rtol=0, atol=1e-8 * np.abs(ref.w).max())
    st2 = api.Statistics()
    api.ot_solve(p.mesh, np.c_[p.x, p.y], p.nu, eps_g=1e-7, stats=st2, ctx=ctx)
    assert st2.grad_norm < 1e-7


def test_empty_cell_status(ctx):
    from mongeampere_gb300 import _lib, api
    from mongeampere_gb300.mesh import unit_grid
    mesh = unit_grid(4, np.ones((4, 4)))
    X = np.array([[0.2, 0.5], [0.8, 0.5], [0.5, 0.5]])
    st = api.Statistics()
    api.ot_solve(mesh, X, np.full(3, 1 / 3), x=np.array([0.0, 0.0, -1.0]), stats=st, ctx=ctx,
                 raise_on_error=False)
    assert st.status == _lib.MA_EMPTY_CELL


def test_solve_reports_the_value_at_its_weights(ctx):
    # the value of the last evaluation, Kantorovich value minus <nu, w> at the returned
    # weights (Statistics::value): at 1e-6 the last Newton steps' evaluations carry the
    # value's integrals; at 1e-11 the last step starts farther than 1e3 x the tolerance
    # from it, and the solve ends with one more FP64 evaluation of its weights
    from mongeampere_gb300 import api
    p = W.make_problem(64, 3000, "gauss", "uniform", "random", seed=12)
    X = np.c_[p.x, p.y]
    for tol in (1e-6, 1e-11):
        st = api.Statistics()
        w = np.asarray(api.ot_solve(p.mesh, X, p.nu, eps_g=tol, stop="rel", stats=st, ctx=ctx))
        assert st.max_rel_err <= tol
        v, g, h = api.kantorovich(p.mesh, X, w, ctx=ctx)
        ref = v - float(p.nu @ w)
        assert abs(st.value - ref) <= 1e-12 * (abs(v) + abs(float(p.nu @ w))), (tol, st.value, ref)


def test_warm_start(ctx):
    # the weights vector is both initial guess and result (optimal_transport.hpp:95)
    from mongeampere_gb300 import api
    p = W.make_problem(32, 800, seed=9)
    st1 = api.Statistics()
    w = api.ot_solve(p.mesh, np.c_[p.x, p.y], p.nu, eps_g=1e-9, stop="rel", stats=st1, ctx=ctx)
    st2 = api.Statistics()
    api.ot_solve(p.mesh, np.c_[p.x, p.y], p.nu, x=w, eps_g=1e-9, stop="rel", stats=st2, ctx=ctx)
    assert st2.niter == 0 and st2.neval == 1


def test_multigrid_and_jacobi_solves_agree(ctx):
    # the aggregation-multigrid preconditioner changes the CG iterations, not the
    # Newton iterates' limit: both reach the same weights
    from mongeampere_gb300 import api
    p = W.make_problem(128, 20000, "gauss", "uniform", "random", seed=7)
    X = np.c_[p.x, p.y]
    st_mg, st_j = api.Statistics(), api.Statistics()
    w_mg = api.ot_solve(p.mesh, X, p.nu, eps_g=1e-10, stop="rel", stats=st_mg, precond="multigrid", ctx=ctx)
    w_j = api.ot_solve(p.mesh, X, p.nu, eps_g=1e-10, stop="rel", stats=st_j, precond="jacobi", ctx=ctx)
    assert st_mg.max_rel_err <= 1e-10 and st_j.max_rel_err <= 1e-10
    np.testing.assert_allclose(w_mg, w_j, rtol=0, atol=1e-9 * np.abs(w_j).max())
    # five multigrid levels here; far fewer CG iterations per Newton step
    assert st_mg.cg_iters * 4 < st_j.cg_iters


def test_multigrid_laplacian_solve_with_empty_cells(ctx, oracle):
    # empty cells give zero rows; they stay at zero on every level and the
    # remaining system is solved as the direct solve of its active part
    from mongeampere_gb300 import api
    p = W.make_problem(40, 3000, seed=4)
    x, y = p.x.copy(), p.y.copy()
    w = np.zeros(p.n)
    w[:3000:97] = -0.05  # sites that lose their cells entirely
    v, g, h = api.kantorovich(p.mesh, np.c_[x, y], w, ctx=ctx)
    g = np.asarray(g)
    empty = g == 0
    assert empty.sum() >= 10 and not empty[-1]
    rhs = g - p.nu
    d, it = api.solve_laplacian_matrix(rhs, rtol=1e-13, ctx=ctx)
    H = h.to_scipy().tocsr()
    act = np.flatnonzero(~empty[:-1])
    import scipy.sparse.linalg as spla
    d_ref = np.zeros(p.n)
    d_ref[act] = spla.spsolve(H[act][:, act].tocsc(), rhs[act])
    assert np.all(d[empty] == 0.0) and d[-1] == 0.0
    np.testing.assert_allclose(d, d_ref, rtol=0, atol=1e-9 * np.abs(d_ref).max())


def test_mixed_precision_evaluation_error(ctx):
    # FP32 piece integrals, FP64 cell sums: the error against the FP64 evaluation
    from mongeampere_gb300 import api
    p = W.make_problem(128, 20000, "gauss", "uniform", "random", seed=9)
    X = np.c_[p.x, p.y]
    w = np.zeros(p.n)
    v64, g64, h64 = api.kantorovich(p.mesh, X, w, ctx=ctx)
    v32, g32, h32 = api.kantorovich(p.mesh, X, w, precision="mixed", ctx=ctx)
    rel = np.abs(np.asarray(g32) - np.asarray(g64)) / np.asarray(g64)
    assert rel.max() < 2e-5 and np.median(rel) < 1e-6
    assert abs(v32 - v64) <= 1e-6 * abs(v64)
    np.testing.assert_array_equal(h32.col, h64.col)  # same combinatorics
    # every Hessian entry within 2.5e-4 of the FP64 one, relative to the entry itself (no
    # absolute floor): an FP32 edge integral is kept only when its certified error is
    # below 2^-12 of the edge, shorter edges are integrated in FP64
    hrel = np.abs(np.asarray(h32.val) - np.asarray(h64.val)) / np.abs(np.asarray(h64.val))
    assert hrel.max() <= 2.5e-4, f"mixed Hessian entry off by {hrel.max():.3e}"


def test_mixed_precision_error_against_the_oracle(ctx, oracle):
    # the clustered-site shape of the 1M-site workload, scaled down: the mixed form's
    # masses, value and every Hessian entry against the double-double oracle
    from mongeampere_gb300 import api
    p = W.make_problem(256, 20000, "uniform", "blobs", "equal", seed=3)
    X = np.c_[p.x, p.y]
    w = np.zeros(p.n)
    v32, g32, h32 = api.kantorovich(p.mesh, X, w, precision="mixed", ctx=ctx)
    r = oracle.kantorovich(p.mesh, p.x, p.y, w, arith="dd", ring=1)
    g32 = np.asarray(g32)
    assert np.max(np.abs(g32 - r.g) / r.g) < 5e-5
    assert abs(v32 - r.value) <= 1e-6 * abs(r.value)
    rows = np.repeat(np.arange(h32.n), np.diff(h32.rowptr)).astype(np.int64)
    kg, ko = rows * p.n + h32.col, r.rows.astype(np.int64) * p.n + r.cols
    og, oo = np.argsort(kg), np.argsort(ko)
    np.testing.assert_array_equal(kg[og], ko[oo])
    hrel = np.abs(np.asarray(h32.val)[og] - r.vals[oo]) / np.abs(r.vals[oo])
    assert hrel.max() <= 2.5e-4, f"mixed Hessian entry off by {hrel.max():.3e}"


def test_mixed_precision_solve_meets_fp64_tolerance(ctx, oracle):
    # the mixed solve stops on FP64 masses: same tolerance, few FP64 evaluations
    from mongeampere_gb300 import api
    p = W.make_problem(96, 8000, "gauss", "uniform", "random", seed=10)
    X = np.c_[p.x, p.y]
    st_m, st_d = api.Statistics(), api.Statistics()
    w_m = api.ot_solve(p.mesh, X, p.nu, eps_g=1e-6, stop="rel", precision="mixed", stats=st_m, ctx=ctx)
    w_d = api.ot_solve(p.mesh, X, p.nu, eps_g=1e-6, stop="rel", stats=st_d, ctx=ctx)
    assert st_m.max_rel_err <= 1e-6 and st_d.max_rel_err <= 1e-6
    # the FP64 check and finish, plus at most one FP64 evaluation for the value at the
    # final weights (when the last evaluation left out the value's integrals)
    assert 1 <= st_m.neval_fp64 <= 7 and st_m.neval_fp64 < st_m.neval
    assert st_d.neval_fp64 == st_d.neval
    # the oracle's masses at the mixed solution
    r = oracle.kantorovich(p.mesh, p.x, p.y, np.asarray(w_m), arith="fp64", ring=1)
    assert np.max(np.abs(r.g - p.nu) / p.nu) <= 1.5e-6
    del w_d


def test_multigrid_at_one_million_sites(ctx):
    # levels wider than the launched grid: coarse rows get teams of fewer than four
    # lanes (every member of an aggregate must still be restricted)
    import torch
    from mongeampere_gb300 import api
    p = W.make_problem(1024, 1_000_000, "uniform", "uniform", "equal", seed=0)
    dev = torch.device("cuda", 0)
    X = torch.stack([torch.tensor(p.x, device=dev), torch.tensor(p.y, device=dev)], 1)
    _, g, h = api.kantorovich(p.mesh, X, torch.zeros(p.n, dtype=torch.float64, device=dev), ctx=ctx)
    rhs = g - torch.tensor(p.nu, device=dev)
    d, it = api.solve_laplacian_matrix(rhs, rtol=1e-8, maxiter=1000, ctx=ctx)
    H = h.to_scipy().tocsr()
    r = rhs.cpu().numpy().copy()
    r[-1] = 0
    res = (H @ d.cpu().numpy() - r)[:-1]
    assert np.linalg.norm(res) <= 1e-7 * np.linalg.norm(r)
    assert it < 400


def test_multiscale_initial_guess(ctx):
    # clustered sites on a uniform density: the coarse-to-fine start reaches the same
    # solution (unique up to the additive constant of the gauge) as the plain start
    from mongeampere_gb300 import api
    p = W.make_problem(128, 20000, "uniform", "blobs", "equal", seed=6)
    X = np.c_[p.x, p.y]
    st_m, st_p = api.Statistics(), api.Statistics()
    w_m = api.ot_solve(p.mesh, X, p.nu, eps_g=1e-8, stop="rel", init="multiscale", stats=st_m, ctx=ctx,
                       maxiter=400)
    w_p = api.ot_solve(p.mesh, X, p.nu, eps_g=1e-8, stop="rel", stats=st_p, ctx=ctx, maxiter=400)
    assert st_m.max_rel_err <= 1e-8 and st_p.max_rel_err <= 1e-8
    a, b = np.asarray(w_m) - w_m[-1], np.asarray(w_p) - w_p[-1]
    np.testing.assert_allclose(a, b, rtol=0, atol=1e-7 * np.abs(b).max())


def test_batch_matches_sequential_solves(ctx):
    # the batch solves every problem with the same ma_ot_solve, on concurrent worker
    # contexts whose CG grids take a share of the GPU (another summation order): the
    # results agree with a sequential loop to the solver's tolerance
    from mongeampere_gb300 import api
    probs = [p for p in W.c5(seed=3, count=40) if p.n <= 8000][:16]
    assert len(probs) >= 8
    items = [(p.mesh, np.c_[p.x, p.y], p.nu) for p in probs]
    ws, stats, used = api.ot_solve_batch(items, eps_g=1e-6, stop="rel", workers=4, ctx=ctx)
    assert used == 4
    for p, w, st in zip(probs, ws, stats):
        assert st.status == 0 and st.max_rel_err <= 1e-6
        s1 = api.Statistics()
        w1 = api.ot_solve(p.mesh, np.c_[p.x, p.y], p.nu, eps_g=1e-6, stop="rel", stats=s1, ctx=ctx)
        assert s1.max_rel_err <= 1e-6
        np.testing.assert_allclose(w, w1, rtol=0, atol=1e-6 * max(1e-30, np.abs(w1).max()))
        assert abs(int(st.niter) - int(s1.niter)) <= 2
    # autotuned worker count
    ws2, stats2, used2 = api.ot_solve_batch(items, eps_g=1e-6, stop="rel", workers=0, ctx=ctx)
    assert used2 in (4, 8, 16, 32, 64)
    assert all(s.status == 0 for s in stats2)


def test_solve_is_reproducible(ctx):
    # the same problem solved again -- after other solves, in a fresh context -- gives the
    # same weights bit for bit and the same Newton path: line-search trials stopped at an
    # empty cell leave seeds that vary with timing, and the neighbour lists are kept in
    # site order so that nothing downstream depends on them
    from mongeampere_gb300 import api
    p = W.make_problem(256, 30000, "gauss", "uniform", "random", seed=5)
    X = np.c_[p.x, p.y]
    runs = []
    for c in (ctx, ctx, api.Context(0)):
        st = api.Statistics()
        w = api.ot_solve(p.mesh, X, p.nu, eps_g=1e-6, stop="rel", stats=st, ctx=c)
        runs.append((w, st.niter, st.neval, st.cg_iters))
    for w, ni, ne, cg in runs[1:]:
        np.testing.assert_array_equal(w, runs[0][0])
        assert (ni, ne, cg) == runs[0][1:]


def test_continuation_solves_clustered_sites(ctx, oracle):
    # the clustered shape of the 1M-site workload, scaled down: the continuation in the
    # target masses reaches 1e-6 (checked by the oracle) in stages of the reference's
    # damped Newton; the plain solve from w = 0 reaches the same weights
    from mongeampere_gb300 import api
    p = W.make_problem(128, 20000, "uniform", "blobs", "equal", seed=0)
    X = np.c_[p.x, p.y]
    st = api.Statistics()
    w = np.asarray(api.ot_solve(p.mesh, X, p.nu, eps_g=1e-6, stop="rel", init="continuation", maxiter=200,
                                stats=st, ctx=ctx))
    assert st.status == 0 and st.max_rel_err <= 1e-6
    r = oracle.kantorovich(p.mesh, p.x, p.y, w, arith="fp64", ring=1)
    assert np.max(np.abs(r.g - p.nu) / p.nu) <= 1.5e-6
    st0 = api.Statistics()
    w0 = np.asarray(api.ot_solve(p.mesh, X, p.nu, eps_g=1e-6, stop="rel", maxiter=200, stats=st0, ctx=ctx))
    assert st0.status == 0
    np.testing.assert_allclose(w, w0, rtol=0, atol=1e-5 * np.abs(w0).max())
    # mixed precision: the stages run on FP32 integrals, the last one finishes in FP64
    stm = api.Statistics()
    api.ot_solve(p.mesh, X, p.nu, eps_g=1e-6, stop="rel", init="continuation", precision="mixed", maxiter=200,
                 stats=stm, ctx=ctx)
    assert stm.status == 0 and stm.max_rel_err <= 1e-6 and stm.neval_fp64 < stm.neval


def test_mixed_precision_with_cells_far_from_their_sites(ctx):
    # at the solution of a 20-fold density contrast the cells lie many cell sizes from
    # their sites; the mixed integrals are taken about a point of the cell, so their
    # error stays that of the FP32 certified bounds: masses within 2^-12, every Hessian
    # entry within 2.5e-4 of the FP64 evaluation
    from mongeampere_gb300 import api
    p = W.make_problem(256, 20000, "gauss", "uniform", "random", seed=11)
    X = np.c_[p.x, p.y]
    w = np.asarray(api.ot_solve(p.mesh, X, p.nu, eps_g=1e-6, stop="rel", ctx=ctx))
    v64, g64, h64 = api.kantorovich(p.mesh, X, w, ctx=ctx)
    v32, g32, h32 = api.kantorovich(p.mesh, X, w, precision="mixed", ctx=ctx)
    g64, g32 = np.asarray(g64), np.asarray(g32)
    rel = np.abs(g32 - g64) / g64
    assert rel.max() <= 2.0 ** -12, f"mixed mass off by {rel.max():.3e}"
    assert abs(v32 - v64) <= 1e-6 * abs(v64)
    np.testing.assert_array_equal(h32.col, h64.col)
    hrel = np.abs(np.asarray(h32.val) - np.asarray(h64.val)) / np.abs(np.asarray(h64.val))
    assert hrel.max() <= 2.5e-4, f"mixed Hessian entry off by {hrel.max():.3e}"
