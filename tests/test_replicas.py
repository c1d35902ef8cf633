"""The multi-GPU form of the benchmark on the CPU: replicas with no data-path exchange.

Every rank solves its own problem; the only collectives are the barriers around the
timed region and the maximum of the ranks' times (bench.max_over_ranks), from which
the whole-job rate is steps x ranks / slowest time.  Run as two gloo ranks on
127.0.0.1.
"""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, times, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        t = bench.max_over_ranks(times[rank], dist)
        out.put((rank, t, bench.job_rate(5, world, t)))
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_two_gloo_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    times = [0.75, 1.25]
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, times, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    # every rank sees the slowest rank's time, and the job rate counts both ranks' work
    for _, t, rate in res:
        assert t == 1.25
        assert rate == pytest.approx(5 * 2 / 1.25)


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(0.5, None) == 0.5
    assert bench.job_rate(3, 1, 0.5) == 6.0


def test_reference_arm_under_torchrun_prints_one_line():
    # two CPU ranks of the reference arm: rank 0 times the oracle sample and prints the
    # one JSON line, rank 1 exits without work
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), os.path.join(ROOT, "bench.py"),
           "--impl", "reference", "--gpus", "2", "--steps", "2", "--warmup", "0", "--workload", "c1"]
    env = dict(os.environ, OMP_NUM_THREADS="2")
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["cpu_baseline"]["kind"] == "port" and d["e2e"]["h2d_bytes_per_step"] == 0
    # the counts come from the complete solve run in the same process, and the line
    # says that its value is scaled from samples
    assert d["extrapolated"] is True and d["full_solve_measured"]["newton_iters"] > 0
    assert d["full_solve_measured"]["max_rel_err"] <= 1e-9
