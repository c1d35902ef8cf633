#!/usr/bin/env python
"""Benchmark of the semi-discrete OT hot path on one GB300.

Workload (the plain-FP64-at-scale configuration): a 512 x 512-vertex grid
triangulation of [0,1]^2 carrying 0.1 + a mixture of 5 Gaussian bumps, 100,000
uniform sites, target masses proportional to U[0.5, 1.5]; damped Newton from
w = 0 until the maximum relative cell-mass error is <= 1e-6.  All inputs are
seeded synthetic data (mongeampere_gb300.workloads.c2).

One step = one complete OT solve (every Laguerre evaluation, every CG solve and
line search of ma_ot_solve).  ``value`` = OT solves/s with the inputs resident in
device memory; ``e2e`` = the same through the C ABI with host buffers (host->device
copy of sites, masses and initial weights, device->host copy of the weights inside
the timed region).  L2 is flushed (a 512 MB write) before every timed step.
Beside the C2 line, rank 0 reports the clustered 1M-site workload (workloads.c3):
complete evaluations at w = 0 in FP64 and in the mixed form (``c3_evaluations``) and
one complete solve of each form from w = 0, each with its own clock record
(``c3_solves``, about 3 minutes; ``--no-c3-solves`` leaves it out).

``--impl reference`` times the reference algorithm's CPU restatement (oracle/) on
the host cores instead.  It first solves the workload once with it (FP64 evaluations,
sparse LU Newton directions, the reference's backtracking), timed as a whole, which
gives the Newton iterations and evaluations the algorithm takes; each step is then a
bounded sample -- one Laguerre evaluation at one of that solve's Newton iterates plus
one sparse LU Newton direction -- and ``value`` scales the samples to a full solve by
those counts (the line says ``"extrapolated": true`` and carries the measured full
solve beside it).
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Laguerre evals/s & OT solves/s at mass err≤1e-6, mixed vs FP64, 1 GB300"
UNIT = "OT solves/s"
WORKLOAD = "plain FP64 OT: 512x512 grid, 0.1 + 5 Gaussians, N=100,000 uniform sites, masses ~U[0.5,1.5], stop max rel mass err 1e-6"
WORKLOAD_C1 = "plain FP64 OT: 64x64 grid U[0.5,1.5], N=1,000 uniform sites, equal masses, stop max rel mass err 1e-9"

# algorithmic bytes of one Laguerre evaluation on an implicit grid mesh:
# X 16N + w 8N + g 8N + CSR Hessian (12 nnz + 4 (N+1)) + value 8 + vertex values 8V
def eval_bytes(n, nnz, nv):
    return 16 * n + 8 * n + 8 * n + 12 * nnz + 4 * (n + 1) + 8 + 8 * nv


# algorithmic bytes of one conjugate-gradient iteration of a Newton step: the sparse
# product reads the CSR matrix (12 nnz + 4N), the vector updates read and write six
# vectors of N doubles (48N)
def cg_iter_bytes(n, nnz):
    return 12 * nnz + 4 * n + 48 * n


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [t.strip() for t in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if f[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        sm.sort()
        med = sm[len(sm) // 2] if sm else None
        return {"sm_mhz": med, "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def max_over_ranks(t, dist, device="cpu"):
    """The slowest rank's time: every rank solves its own problem (weak scaling, no
    exchange between ranks), so the job takes as long as its slowest rank."""
    if dist is None:
        return t
    import torch
    tt = torch.tensor([t], dtype=torch.float64, device=device)
    dist.all_reduce(tt, op=dist.ReduceOp.MAX)
    return float(tt.item())


def job_rate(steps, world, t):
    """Whole-job throughput: each of the `world` ranks completed `steps` solves in t."""
    return steps * world / t


def _oracle():
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    return oracle


def cpu_sample(problem, w):
    """One Laguerre evaluation at weights w in the reference's FP64 arithmetic + one
    sparse LU Newton direction of its Hessian, on all host threads (the oracle)."""
    import numpy as np
    oracle = _oracle()
    t0 = time.perf_counter()
    r = oracle.kantorovich(problem.mesh, problem.x, problem.y, w, arith="fp64", ring=1)
    t1 = time.perf_counter()
    d = oracle.solve_laplacian_matrix(r.hessian(), r.g - problem.nu)
    t2 = time.perf_counter()
    assert np.isfinite(d).all()
    return t1 - t0, t2 - t1, oracle.max_threads()


def reference_full_solve(problem):
    """The reference algorithm's complete solve of the workload (oracle.ot_solve: FP64
    evaluations, sparse LU directions, KMT backtracking from w = 0 to the stopping
    rule), timed as a whole: (result with its Newton iterates, seconds)."""
    oracle = _oracle()
    t0 = time.perf_counter()
    r = oracle.ot_solve(problem.mesh, problem.x, problem.y, problem.nu, tol_rel=problem.tol_rel, arith="fp64",
                        ring=1, keep_iterates=True)
    return r, time.perf_counter() - t0


def run_reference(args, rank):
    import numpy as np

    from mongeampere_gb300 import workloads as W
    if rank != 0:
        return
    problem = W.c1(0) if args.workload == "c1" else W.c2(0)
    ref, full_s = reference_full_solve(problem)
    iterates = [np.zeros(problem.n)] + [h[5] for h in ref.history]
    for k in range(args.warmup):
        cpu_sample(problem, iterates[k % len(iterates)])
    te, tl = [], []
    t0 = time.perf_counter()
    for k in range(args.steps):
        a, b, cores = cpu_sample(problem, iterates[k % len(iterates)])
        te.append(a)
        tl.append(b)
    t_steps = time.perf_counter() - t0
    te_m, tl_m = float(np.mean(te)), float(np.mean(tl))
    solve_s = ref.neval * te_m + ref.niter * tl_m
    value = 1.0 / solve_s
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t_steps / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD_C1 if args.workload == "c1" else WORKLOAD, "seed": 0},
        "extrapolated": True,
        "laguerre_evals_per_s": 1.0 / te_m,
        "full_solve_measured": {"seconds": full_s, "solves_per_s": 1.0 / full_s, "newton_iters": ref.niter,
                                "evals": ref.neval, "max_rel_err": ref.max_rel_err},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "extrapolated": True,
                         "sample": f"per step: 1 Laguerre evaluation at one of the Newton iterates ({te_m:.2f} s "
                                   f"mean) + 1 sparse LU Newton direction ({tl_m:.2f} s mean) of the CPU "
                                   f"restatement on all {cores} threads; a full solve = {ref.neval} evaluations + "
                                   f"{ref.niter} Newton directions, the counts of the complete reference-algorithm "
                                   f"solve run first in this process ({full_s:.1f} s measured)"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def c3_evaluations(ctx, dev, steps, warmup):
    """Complete Laguerre evaluations (masses, value, CSR Hessian) of the clustered 1M-site
    workload (workloads.c3) at w = 0, in FP64 and in the mixed form: evaluations/s of
    each, and the mixed form's errors against FP64."""
    import numpy as np
    import torch

    from mongeampere_gb300 import api
    from mongeampere_gb300 import workloads as W
    p = W.c3(0)
    dm = ctx.mesh(p.mesh)
    X = torch.stack([torch.tensor(p.x, device=dev), torch.tensor(p.y, device=dev)], 1)
    out = {"config": "1,000,000 sites (70% in 20 Gaussian blobs), 2048^2 grid U[0.5,1.5]; masses, value and "
                     "CSR Hessian per evaluation"}
    w = torch.zeros(p.n, dtype=torch.float64, device=dev)
    for name in ("w0",):
        res = {}
        for prec in ("fp64", "mixed"):
            for _ in range(warmup):
                api.kantorovich(dm, X, w, precision=prec, ctx=ctx)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            e0.record()
            for _ in range(steps):
                v, g, h = api.kantorovich(dm, X, w, precision=prec, ctx=ctx)
            e1.record()
            torch.cuda.synchronize()
            res[prec] = (steps / (e0.elapsed_time(e1) * 1e-3), v, g.cpu().numpy(), h)
        g64, g32 = res["fp64"][2], res["mixed"][2]
        same = bool(np.array_equal(res["fp64"][3].col, res["mixed"][3].col))
        hrel = (float(np.max(np.abs(res["mixed"][3].val - res["fp64"][3].val) / np.abs(res["fp64"][3].val)))
                if same else None)
        out[name] = {"fp64_evals_per_s": res["fp64"][0], "mixed_evals_per_s": res["mixed"][0],
                     "mixed_mass_rel_err_max": float(np.max(np.abs(g32 - g64) / g64)),
                     "mixed_value_rel_err": float(abs(res["mixed"][1] - res["fp64"][1]) / abs(res["fp64"][1])),
                     "mixed_hessian_entry_rel_err_max": hrel, "same_sparsity": same}
    return out


def c3_solves(ctx, dev, p=None):
    """One complete OT solve of the clustered 1M-site workload (workloads.c3) in each
    form, FP64 and mixed, from w = 0 to max relative mass error 1e-6 by the continuation
    in the target masses (MA_INIT_CONTINUATION), each timed with CUDA events and its own
    clock record; then the mixed solution's errors against the FP64 evaluation (which
    the tests pin to the oracle at this size): weights, masses and every Hessian entry."""
    import numpy as np
    import torch

    from mongeampere_gb300 import api
    from mongeampere_gb300 import workloads as W
    p = p if p is not None else W.c3(0)
    dm = ctx.mesh(p.mesh)
    X = torch.stack([torch.tensor(p.x, device=dev), torch.tensor(p.y, device=dev)], 1)
    nu = torch.tensor(p.nu, device=dev)
    solves, wsol = {}, {}
    for prec in ("fp64", "mixed"):
        w = torch.zeros(p.n, dtype=torch.float64, device=dev)
        st = api.Statistics()
        clocks = ClockSampler(0)
        clocks.start()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e0.record()
        api.ot_solve(dm, X, nu, x=w, eps_g=1e-6, stop="rel", precision=prec, init="continuation", maxiter=300,
                     stats=st, ctx=ctx)
        e1.record()
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
        clk = clocks.stop()
        secs = e0.elapsed_time(e1) * 1e-3
        wsol[prec] = w
        solves[prec] = {"seconds": secs, "solves_per_s": 1.0 / secs, "wall_s": wall, "newton_iters": st.niter,
                        "evals": st.neval, "fp64_evals": st.neval_fp64, "cg_iters": st.cg_iters,
                        "linesearch_halvings": st.linesearch_halvings, "max_rel_err": st.max_rel_err,
                        "eval_ms": st.t_eval_ms, "linsolve_ms": st.t_linsolve_ms, "clocks": clk}
    # the mixed solution, evaluated in FP64
    v64, g64, h64 = api.kantorovich(dm, X, wsol["mixed"], ctx=ctx)
    v32, g32, h32 = api.kantorovich(dm, X, wsol["mixed"], precision="mixed", ctx=ctx)
    g64n, g32n = g64.cpu().numpy(), g32.cpu().numpy()
    wm, wd = wsol["mixed"].cpu().numpy(), wsol["fp64"].cpu().numpy()
    same = bool(np.array_equal(h32.col, h64.col))
    hrel = float(np.max(np.abs(h32.val - h64.val) / np.abs(h64.val))) if same else None
    return {"config": "1,000,000 sites (70% in 20 Gaussian blobs), 2048^2 grid U[0.5,1.5], equal masses, "
                      "from w = 0 to max rel mass err 1e-6, inputs in device memory",
            "fp64": solves["fp64"], "mixed": solves["mixed"],
            "mixed_speedup": solves["fp64"]["seconds"] / solves["mixed"]["seconds"],
            "mixed_solution_fp64_mass_rel_err_max": float(np.max(np.abs(g64n - p.nu) / p.nu)),
            "mixed_vs_fp64_weights_max_abs_diff": float(np.max(np.abs(wm - wd))),
            "weights_scale": float(np.max(np.abs(wd))),
            "mixed_eval_mass_rel_err_max": float(np.max(np.abs(g32n - g64n) / g64n)),
            "mixed_eval_value_rel_err": float(abs(v32 - v64) / abs(v64)),
            "mixed_eval_hessian_entry_rel_err_max": hrel, "same_sparsity": same}


def run_c3(args, ctx, dev, rank):
    """Mixed precision against FP64 on the clustered 1M-site workload (workloads.c3:
    2048^2 grid U[0.5,1.5], 1,000,000 sites, 70% in 20 Gaussian blobs, equal masses):
    (a) complete Laguerre evaluations at w = 0, evaluations/s of each form; (b) one
    complete OT solve of each form from w = 0 to max relative mass error 1e-6, by the
    continuation in the target masses (MA_INIT_CONTINUATION: the reference's damped
    Newton from w = 0 cuts every step to a few 2^-11 on these sites), each timed with its
    own clock record; (c) the mixed solution's errors against the FP64 evaluation (which
    the tests pin to the oracle at this size): weights, masses and every Hessian entry."""
    import torch

    from mongeampere_gb300 import api
    from mongeampere_gb300 import workloads as W
    out = {"metric": METRIC, "workload": "c3", "n_gpus": 1,
           "config": "1,000,000 sites (70% in 20 Gaussian blobs), 2048^2 grid U[0.5,1.5], equal masses, "
                     "inputs in device memory"}
    p = W.c3(0)
    dm = ctx.mesh(p.mesh)
    X = torch.stack([torch.tensor(p.x, device=dev), torch.tensor(p.y, device=dev)], 1)
    w0 = torch.zeros(p.n, dtype=torch.float64, device=dev)
    ev = {}
    for prec in ("fp64", "mixed"):
        for _ in range(max(args.warmup, 1)):
            api.kantorovich(dm, X, w0, precision=prec, ctx=ctx)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record()
        for _ in range(args.steps):
            api.kantorovich(dm, X, w0, precision=prec, ctx=ctx)
        e1.record()
        torch.cuda.synchronize()
        ev[prec] = args.steps / (e0.elapsed_time(e1) * 1e-3)
    out["evaluations_at_w0"] = {"fp64_evals_per_s": ev["fp64"], "mixed_evals_per_s": ev["mixed"],
                                "mixed_speedup": ev["mixed"] / ev["fp64"]}
    out["solve"] = c3_solves(ctx, dev, p)
    if rank == 0:
        print(json.dumps(out))


def run_c4(args, ctx, dev, rank):
    """The adjoint at 200,000 sites on a 256^2 density (workloads.c4), at the OT solution
    (cells away from their sites): (a) vector-Jacobian products of (value, masses, first
    moments), FP64 and FP32, per second, against forward evaluations, with cotangents
    N(0, 1); (b) central differences of the FP64 forward pass on 1,000 random coordinates
    of the sites, the weights and the density's vertex values, against both adjoints, with
    h = 1e-6 in each coordinate's own scale (the mean cell size 1/sqrt(N) for sites, the
    mean cell area 1/N for weights, 1 for vertex values: a weight step of 1e-6 would be a
    fifth of a cell's weight scale at 200,000 sites, far from the difference's asymptotic
    regime); (c) 50 steps of the W2 gradient flow whose direction is the backward pass:
    after a warm-started solve to max relative mass error 1e-6, x <- x + tau dPhi/dx / (2 m)
    = x + tau (c - x), with dPhi/dx = 2 (int rho x - m x) from the VJP of the value and c
    the cell's centroid (tau = 0.5: half a Lloyd step, the W2 cost's gradient step)."""
    import numpy as np
    import torch

    from mongeampere_gb300 import _lib
    from mongeampere_gb300 import api
    from mongeampere_gb300 import workloads as W
    out = {"metric": METRIC, "workload": "c4", "n_gpus": 1,
           "config": "200,000 uniform sites, 256^2 grid U[0.5,1.5], equal masses, at the OT solution"}
    p = W.c4(0)
    dm = ctx.mesh(p.mesh)
    X = torch.stack([torch.tensor(p.x, device=dev), torch.tensor(p.y, device=dev)], 1)
    nu = torch.tensor(p.nu, device=dev)
    w = torch.zeros(p.n, dtype=torch.float64, device=dev)
    api.ot_solve(dm, X, nu, x=w, eps_g=1e-6, stop="rel", ctx=ctx)
    rng = np.random.default_rng(4)
    a = float(rng.normal())
    b = torch.tensor(rng.normal(size=p.n), device=dev)
    e = torch.tensor(rng.normal(size=(p.n, 2)), device=dev)

    def rate(fn):
        for _ in range(args.warmup):
            fn()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record()
        for _ in range(args.steps):
            fn()
        e1.record()
        torch.cuda.synchronize()
        return args.steps / (e0.elapsed_time(e1) * 1e-3)

    fwd = rate(lambda: api.kantorovich(dm, X, w, hessian=False, ctx=ctx))
    vjp64 = rate(lambda: api.kantorovich_vjp(dm, X, w, a, b, e, ctx=ctx))
    vjp32 = rate(lambda: api.kantorovich_vjp(dm, X, w, a, b, e, precision="mixed", ctx=ctx))
    g64 = [q.cpu().numpy() for q in api.kantorovich_vjp(dm, X, w, a, b, e, ctx=ctx)]
    g32 = [q.cpu().numpy() for q in api.kantorovich_vjp(dm, X, w, a, b, e, precision="mixed", ctx=ctx)]
    vals = np.asarray(p.mesh.values, dtype=np.float64).reshape(-1)
    vals_dev = torch.tensor(vals, device=dev)

    def objective(Xp, wp):
        v, g, _ = api.kantorovich(dm, Xp, wp, hessian=False, ctx=ctx)
        _, first = api.first_moment(dm, Xp, wp, ctx=ctx)
        return a * v + float((b * g).sum()) + float((e * first).sum())

    h = 1e-6
    ncoord = 1000
    fd, ad64, ad32 = np.zeros(ncoord), np.zeros(ncoord), np.zeros(ncoord)
    kinds = rng.integers(0, 4, ncoord)
    t0 = time.perf_counter()
    for q in range(ncoord):
        kind = int(kinds[q])
        if kind < 2:
            i = int(rng.integers(p.n))
            f = []
            hs = h * p.n ** -0.5
            for t in (hs, -hs):
                Xp = X.clone()
                Xp[i, kind] += t
                f.append(objective(Xp, w))
            ad64[q], ad32[q] = g64[0][i, kind], g32[0][i, kind]
            f = [f[0] * p.n ** 0.5, f[1] * p.n ** 0.5]  # divided by 2h below: the step was h / sqrt(N)
        elif kind == 2:
            i = int(rng.integers(p.n))
            f = []
            for t in (h / p.n, -h / p.n):
                wp = w.clone()
                wp[i] += t
                f.append(objective(X, wp))
            ad64[q], ad32[q] = g64[1][i], g32[1][i]
            f = [f[0] * p.n, f[1] * p.n]  # divided by 2h below: the step was h / N
        else:
            j = int(rng.integers(vals.size))
            f = []
            for t in (h, -h):
                vp = vals_dev.clone()
                vp[j] += t
                dm.set_values(vp)
                f.append(objective(X, w))
            dm.set_values(vals_dev)
            ad64[q], ad32[q] = g64[2][j], g32[2][j]
        fd[q] = (f[0] - f[1]) / (2 * h)
    fd_s = time.perf_counter() - t0
    scale = float(np.abs(fd).max())
    big = np.abs(fd) >= 1e-3 * scale

    def agree(ad):
        d = np.abs(ad - fd)
        return {"max_abs_over_max_fd": float(d.max() / scale),
                "max_rel_where_fd_above_1e-3_of_max": float(np.max(d[big] / np.abs(fd[big]))),
                "median_rel": float(np.median(d[big] / np.abs(fd[big])))}

    out["adjoint"] = {"forward_evals_per_s": fwd, "vjp_fp64_per_s": vjp64, "vjp_fp32_per_s": vjp32,
                      "fd": {"h_sites": h * p.n ** -0.5, "h_weights": h / p.n, "h_vertex_values": h,
                             "coordinates": ncoord,
                             "kinds": {"site x": int((kinds == 0).sum()), "site y": int((kinds == 1).sum()),
                                       "weight": int((kinds == 2).sum()), "vertex value": int((kinds == 3).sum())},
                             "seconds": fd_s, "fp64_adjoint": agree(ad64), "fp32_adjoint": agree(ad32)},
                      "fp32_vs_fp64_adjoint_rel_norm": [float(np.linalg.norm(q32 - q64) / np.linalg.norm(q64))
                                                        for q64, q32 in zip(g64, g32)]}
    # the W2 flow driven by the backward pass
    Xf, wf = X.clone(), w.clone()
    tau = 0.5
    st_tot = [0, 0]
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(50):
        st = api.Statistics()
        api.ot_solve(dm, Xf, nu, x=wf, eps_g=1e-6, stop="rel", stats=st, ctx=ctx, raise_on_error=False)
        if st.status == _lib.MA_EMPTY_CELL:
            # a moved site's cell is empty at the previous weights: restart from zero (as ma_w2_flow)
            wf.zero_()
            api.ot_solve(dm, Xf, nu, x=wf, eps_g=1e-6, stop="rel", stats=st, ctx=ctx)
        assert st.status == 0, st.status
        st_tot[0] += st.niter
        st_tot[1] += st.neval
        gX, _, _ = api.kantorovich_vjp(dm, Xf, wf, 1.0, None, None, grad_rho=False, ctx=ctx)
        Xf = Xf + tau * gX / (2.0 * nu[:, None])
    e1.record()
    torch.cuda.synchronize()
    secs = e0.elapsed_time(e1) * 1e-3
    out["w2_flow"] = {"config": "50 steps, x <- x + tau dPhi/dx / (2 m), tau = 0.5, dPhi/dx from the VJP, each "
                                "solve warm-started (from zero where a moved site's cell is empty at the previous "
                                "weights) to max rel mass err 1e-6",
                      "seconds": secs, "steps_per_s": 50 / secs, "newton_iters": st_tot[0], "evals": st_tot[1]}
    if rank == 0:
        print(json.dumps(out))


def run_c5(args, ctx, dev, rank):
    """512 independent problems (workloads.c5: grid side log-uniform in [32, 512], values
    U[0.5, 1.5], 500 .. 50,000 uniform sites, equal masses) solved to max relative mass
    error 1e-6 in the mixed form, device-resident: one ma_ot_solve per problem in a loop
    against one ma_ot_solve_batch (autotuned number of concurrent workers)."""
    import numpy as np
    import torch

    from mongeampere_gb300 import api
    from mongeampere_gb300 import workloads as W
    probs = W.c5(0)
    items = []
    for p in probs:
        dm = ctx.mesh(p.mesh)
        X = torch.stack([torch.tensor(p.x, device=dev), torch.tensor(p.y, device=dev)], 1)
        items.append((dm, X, torch.tensor(p.nu, device=dev)))
    prec = "mixed"
    clocks = ClockSampler(0)
    clocks.start()
    # sequential
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    seq_ok = 0
    for dm, X, nu in items:
        st = api.Statistics()
        api.ot_solve(dm, X, nu, eps_g=1e-6, stop="rel", precision=prec, stats=st, ctx=ctx, raise_on_error=False)
        seq_ok += int(st.status == 0 and st.max_rel_err <= 1e-6)
    torch.cuda.synchronize()
    t_seq = time.perf_counter() - t0
    # batched (the first call autotunes and is timed too)
    runs = []
    for _ in range(2):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ws, stats, used = api.ot_solve_batch(items, eps_g=1e-6, stop="rel", precision=prec, workers=0, ctx=ctx)
        torch.cuda.synchronize()
        runs.append((time.perf_counter() - t0, used, stats))
    t_b, used, stats = runs[-1]
    clk = clocks.stop()
    ok = sum(int(s.status == 0 and s.max_rel_err <= 1e-6) for s in stats)
    sites = int(sum(p.n for p in probs))
    out = {"metric": METRIC, "workload": "c5", "n_gpus": 1,
           "config": "512 problems: grid side log-U[32,512], values U[0.5,1.5], N log-U[500,50000] uniform "
                     "sites, equal masses, mixed form, stop max rel mass err 1e-6, inputs in device memory",
           "total_sites": sites, "sequential_problems_per_s": len(probs) / t_seq,
           "batched_problems_per_s": len(probs) / t_b, "batched_speedup": t_seq / t_b,
           "workers": used, "first_batch_s_with_autotune": runs[0][0], "batched_s": t_b, "sequential_s": t_seq,
           "converged_sequential": seq_ok, "converged_batched": ok, "clocks": clk}
    if rank == 0:
        print(json.dumps(out))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="fp64", choices=["fp64", "mixed"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-c3", action="store_true", help="leave out the 1M-site FP64 / mixed evaluations")
    ap.add_argument("--no-c3-solves", action="store_true",
                    help="leave out the 1M-site FP64 and mixed complete solves (about 3 minutes)")
    ap.add_argument("--profile-evals", type=int, default=0,
                    help="profiling driver: solve once, then run this many Laguerre evaluations at the "
                         "solution weights and print per-kernel device times (no benchmark line)")
    ap.add_argument("--profile-solve", action="store_true",
                    help="profiling driver: one solve with per-kernel device times (no benchmark line)")
    ap.add_argument("--workload", default="c2", choices=["c1", "c2", "c3", "c4", "c5"],
                    help="c3: the 1M-site mixed-precision comparison on the clustered 1M-site / 2048^2 "
                         "workload (evaluations, and complete solves of each form); c5: 512 independent "
                         "problems, batched against sequential solves; one JSON line each; c1 (the "
                         "reference's own 64^2 / 1,000-site case): the reference arm only")
    args = ap.parse_args()
    if args.workload == "c1" and args.impl != "reference":
        ap.error("--workload c1 (the reference's own CPU case) is for --impl reference")
    if args.workload == "c5":
        # the batch's 64 worker streams get 32 hardware queues instead of the default
        # 8 (read when the process creates its CUDA context, so set before any CUDA call)
        os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        backend = "gloo" if args.impl == "reference" else "nccl"
        dist.init_process_group(backend)
    if args.impl == "reference":
        run_reference(args, rank)
        if dist:
            dist.destroy_process_group()
        return

    import numpy as np
    import torch

    from mongeampere_gb300 import api
    from mongeampere_gb300 import workloads as W

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    ctx = api.Context(local)
    ctx.use_torch_stream()
    if args.workload == "c3":
        run_c3(args, ctx, dev, rank)
        return
    if args.workload == "c4":
        run_c4(args, ctx, dev, rank)
        return
    if args.workload == "c5":
        run_c5(args, ctx, dev, rank)
        return
    # weak scaling: every rank solves its own problem (replicas; the solve has no
    # data-path exchange)
    p = W.c2(rank)
    dmesh = ctx.mesh(p.mesh)
    x = torch.tensor(p.x, device=dev)
    y = torch.tensor(p.y, device=dev)
    nu = torch.tensor(p.nu, device=dev)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    def solve_device(stats=None):
        w = torch.zeros(p.n, dtype=torch.float64, device=dev)
        st = stats if stats is not None else api.Statistics()
        api.ot_solve(dmesh, x, nu, x=w, y=y, eps_g=p.tol_rel, stop="rel", precision=args.precision,
                     stats=st, ctx=ctx)
        return w, st

    if args.profile_evals:
        wsol, _ = solve_device()
        X = torch.stack([x, y], 1)
        ctx.profile(True)
        for _ in range(args.profile_evals):
            api.kantorovich(dmesh, X, wsol, ctx=ctx)
        torch.cuda.synchronize()
        print(json.dumps({"profile_evals": args.profile_evals, **ctx.profile_read()}))
        return

    if args.profile_solve:
        solve_device()
        ctx.profile(True)
        _, st = solve_device()
        torch.cuda.synchronize()
        print(json.dumps({"profile_solve": 1, "cg_iters": st.cg_iters, "newton_iters": st.niter, "evals": st.neval,
                          "eval_ms": st.t_eval_ms, "linsolve_ms": st.t_linsolve_ms, **ctx.profile_read()}))
        return

    for _ in range(args.warmup):
        solve_device()
    torch.cuda.synchronize()

    # ---- timed region: device-resident inputs ----
    clocks = ClockSampler(local)
    clocks.start()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    launches0 = ctx.launch_count
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    stats = []
    t_wall0 = time.perf_counter()
    for k in range(args.steps):
        flush.fill_(float(k))
        ev[k][0].record()
        w, st = solve_device()
        ev[k][1].record()
        stats.append(st)
    torch.cuda.synchronize()
    t_wall = time.perf_counter() - t_wall0
    if dist:
        dist.barrier()
    clk = clocks.stop()
    launches = ctx.launch_count - launches0
    step_ms = [a.elapsed_time(b) for a, b in ev]
    t_dev = sum(step_ms) / 1e3
    t_dev = max_over_ranks(t_dev, dist, dev)
    value = job_rate(args.steps, world, t_dev)
    ms_per_step = 1e3 * t_dev / args.steps
    for s in stats:
        assert s.max_rel_err <= p.tol_rel, "solve did not converge"

    # ---- full Laguerre evaluations and the dominant kernel ----------------------
    # evaluations/s: complete evaluations (masses, value, Hessian in CSR) at the
    # solution weights through the public call (which also rebuilds the site index);
    # the solve's own count includes line-search trials that stop at an empty cell
    wsol, _ = solve_device()
    X = torch.stack([x, y], 1)
    api.kantorovich(dmesh, X, wsol, ctx=ctx)
    n_full = 10
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record()
    for _ in range(n_full):
        _, _, h = api.kantorovich(dmesh, X, wsol, ctx=ctx)
    e1.record()
    torch.cuda.synchronize()
    evals_per_s = n_full / (e0.elapsed_time(e1) * 1e-3)
    nnz = int(h.col.shape[0])
    # live per-launch durations of the evaluation kernels (CUDA events on the
    # context's stream, profiled run, untimed)
    ctx.profile(True)
    for _ in range(n_full):
        api.kantorovich(dmesh, X, wsol, ctx=ctx)
    torch.cuda.synchronize()
    prof = ctx.profile_read()
    ctx.profile(False)
    pieces_ms = prof["pieces_ms"] / max(prof["pieces_launches"], 1)
    stage1_ms = prof["cells_ms"] / max(prof["cells_launches"], 1)
    bounds_ms = prof["bounds_ms"] / max(prof["bounds_launches"], 1)
    # and of the CG kernel over one complete solve
    ctx.profile(True)
    _, st_prof = solve_device()
    torch.cuda.synchronize()
    sprof = ctx.profile_read()
    ctx.profile(False)
    bytes_eval = eval_bytes(p.n, nnz, p.mesh.nv)
    bytes_cg = cg_iter_bytes(p.n, nnz)
    peak, peak_kind = measured_peaks()
    cg_iter_ms = sprof["pcg_ms"] / max(sprof["pcg_iters"], 1)

    def leg(ms, nbytes):
        a = nbytes / (ms * 1e-3) / 1e9
        return {"avg_ms": ms, "algorithmic_bytes": nbytes, "achieved_gbs": a, "frac": a / peak}

    kernels = {"k_cells_stage1": leg(stage1_ms, bytes_eval), "k_pieces": leg(pieces_ms, bytes_eval),
               "k_pcg_amg (per CG iteration)": leg(cg_iter_ms, bytes_cg)}
    # the dominant evaluation kernel: the larger share of one evaluation
    dom = "k_cells_stage1" if stage1_ms >= pieces_ms else "k_pieces"
    what = {"k_cells_stage1": "k_cells_stage1 (site-tree search and clipping of every Laguerre cell)",
            "k_pieces": "k_pieces (cell-triangle clipping, integrals and Hessian rows)"}[dom]
    roofline = {"bound": "hbm", "achieved": kernels[dom]["achieved_gbs"], "peak": peak, "unit": "GB/s",
                "frac": kernels[dom]["frac"],
                # DRAM bytes need an ncu capture, which the benchmark does not run: the
                # capture of this kernel is kept with the profiles as evidence
                "traffic": None,
                "kernel": what, "peak_source": peak_kind, "algorithmic_bytes_per_launch": bytes_eval,
                "avg_launch_ms": kernels[dom]["avg_ms"],
                "per_kernel": kernels, "k_tree_bounds_ms": bounds_ms}
    # the whole solve: every evaluation and every CG iteration over the solve's time
    solve_bytes = st_prof.neval * bytes_eval + st_prof.cg_iters * bytes_cg
    solve_gbs = solve_bytes / (ms_per_step * 1e-3) / 1e9
    solve_roofline = {"algorithmic_bytes": solve_bytes, "evals": st_prof.neval, "cg_iters": st_prof.cg_iters,
                      "achieved_gbs": solve_gbs, "frac": solve_gbs / peak}

    # ---- the 1M-site clustered workload: FP64 against mixed evaluations ----------
    c3 = None
    if rank == 0 and not args.no_c3:
        c3 = c3_evaluations(ctx, dev, max(args.steps, 3), 2)
    c3s = None
    if rank == 0 and not args.no_c3_solves:
        try:
            c3s = c3_solves(ctx, dev)
        except Exception as exc:  # the C2 line stands without it
            c3s = {"error": f"{type(exc).__name__}: {exc}"}

    # ---- e2e through the C ABI with host buffers ----
    xh = torch.tensor(p.x).pin_memory().numpy()
    yh = torch.tensor(p.y).pin_memory().numpy()
    nuh = torch.tensor(p.nu).pin_memory().numpy()
    w0h = torch.zeros(p.n, dtype=torch.float64).pin_memory().numpy()
    ctx2 = api.Context(local)
    dmesh2 = ctx2.mesh(p.mesh)
    api.ot_solve(dmesh2, xh, nuh, x=w0h, y=yh, eps_g=p.tol_rel, stop="rel", precision=args.precision, ctx=ctx2)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    e2e_t = 0.0
    for k in range(args.steps):
        flush.fill_(float(k))
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        wres = api.ot_solve(dmesh2, xh, nuh, x=w0h, y=yh, eps_g=p.tol_rel, stop="rel",
                            precision=args.precision, ctx=ctx2)
        e2e_t += time.perf_counter() - t1
    assert np.isfinite(wres).all()
    e2e_t = max_over_ranks(e2e_t, dist, dev)
    e2e = {"value": job_rate(args.steps, world, e2e_t), "unit": UNIT, "h2d_bytes_per_step": 4 * 8 * p.n,
           "d2h_bytes_per_step": 8 * p.n}

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64" if args.precision == "fp64" else "f32+f64",
        "data": "synthetic",
        "config": {"workload": WORKLOAD, "sites": p.n, "grid": 512, "precision": args.precision,
                   "l2": "flushed (512 MB write) before every step", "seed_per_rank": "rank"},
        "laguerre_evals_per_s": evals_per_s,
        "solve_stats": {"newton_iters": stats[0].niter, "evals": stats[0].neval, "cg_iters": stats[0].cg_iters,
                        "eval_ms": stats[0].t_eval_ms, "linsolve_ms": stats[0].t_linsolve_ms,
                        "max_rel_err": stats[0].max_rel_err, "wall_s_per_step": t_wall / args.steps},
        "e2e": e2e,
        "roofline": roofline,
        "solve_roofline": solve_roofline,
        "c3_evaluations": c3,
        "c3_solves": c3s,
        "clocks": clk,
        "gpu_launches": launches,
    }
    if rank == 0 and not args.no_cpu_baseline:
        # the oracle at w = 0 and at the solution (the two ends of the Newton path), one
        # sparse LU direction each, scaled by this run's own solve counts
        pc = W.c2(0)
        te0, tl0, cores = cpu_sample(pc, pc.w0)
        te1, tl1, _ = cpu_sample(pc, wsol.cpu().numpy())
        te, tl = 0.5 * (te0 + te1), 0.5 * (tl0 + tl1)
        neval, niter = stats[0].neval, stats[0].niter
        cpu_solve = neval * te + niter * tl
        line["cpu_baseline"] = {
            "value": 1.0 / cpu_solve, "unit": UNIT, "cores": cores, "kind": "port", "extrapolated": True,
            "sample": f"2 Laguerre evaluations (w = 0 and the solution; {te:.2f} s mean) + 2 sparse LU Newton "
                      f"directions ({tl:.2f} s mean) of the CPU restatement (reference FP64 arithmetic) on "
                      f"{cores} threads, scaled to this run's solve: {neval} evaluations + {niter} Newton "
                      f"directions"}
    if rank == 0:
        print(json.dumps(line))
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
