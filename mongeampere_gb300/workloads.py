"""Seeded synthetic workloads.

The reference ships no input data: its drivers read images from the command line
(tests/bench_opttransport.cpp:34, tests/test_opttransport.cpp:48) and draw sites
with ``rand()`` (bench_opttransport.cpp:20-23).  These generators stand in for
them with the five workload shapes this engine is measured on:

=======  ============================  ===============================  ===========
name     density mesh                  sites                            masses
=======  ============================  ===============================  ===========
c1       64 x 64 grid, U[0.5, 1.5]     1,000 uniform                    equal
c2       512 x 512 grid, 0.1 + 5 bumps 100,000 uniform                  U[0.5, 1.5]
c3       2048 x 2048, U[0.5, 1.5]      1,000,000: 70% in 20 blobs       equal
c4       256 x 256, U[0.5, 1.5]        200,000 uniform                  equal
c5       512 problems, side log-U[32, 512], N log-U[500, 50,000]        equal
=======  ============================  ===============================  ===========

All draws come from ``numpy.random.Generator(PCG64(seed))`` in a fixed order, so
the same seed gives the same doubles on every machine.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from .mesh import GridMesh, unit_grid


@dataclass
class Problem:
    mesh: GridMesh
    x: np.ndarray
    y: np.ndarray
    nu: np.ndarray
    w0: np.ndarray
    tol_rel: float
    name: str = ""
    meta: dict = field(default_factory=dict)

    @property
    def n(self) -> int:
        return int(self.x.shape[0])


def _rng(seed: int) -> np.random.Generator:
    return np.random.Generator(np.random.PCG64(seed))


def density_values(kind: str, n: int, rng: np.random.Generator) -> np.ndarray:
    """Vertex values of an ``n x n`` grid on [0, 1]^2."""
    if kind == "uniform":
        return rng.uniform(0.5, 1.5, size=(n, n))
    if kind == "gauss":
        # 0.1 + sum_k A_k exp(-|x - c_k|^2 / (2 sigma_k^2)), five bumps
        c = rng.uniform(0.0, 1.0, size=(5, 2))
        s = rng.uniform(0.03, 0.15, size=5)
        a = rng.uniform(0.5, 2.0, size=5)
        g = np.linspace(0.0, 1.0, n)
        X, Y = np.meshgrid(g, g)
        v = np.full((n, n), 0.1)
        for k in range(5):
            v += a[k] * np.exp(-((X - c[k, 0]) ** 2 + (Y - c[k, 1]) ** 2) / (2.0 * s[k] ** 2))
        return v
    raise ValueError(kind)


def sites(kind: str, n: int, rng: np.random.Generator):
    if kind == "uniform":
        p = rng.uniform(0.0, 1.0, size=(n, 2))
        return p[:, 0].copy(), p[:, 1].copy()
    if kind == "blobs":
        # 70% from 20 isotropic Gaussian blobs (sigma ~ U[0.005, 0.05]) rejection-
        # clipped to the open unit square, 30% uniform
        nb = int(round(0.7 * n))
        cen = rng.uniform(0.0, 1.0, size=(20, 2))
        sig = rng.uniform(0.005, 0.05, size=20)
        which = rng.integers(0, 20, size=nb)
        out = np.empty((nb, 2))
        todo = np.arange(nb)
        while todo.size:
            p = cen[which[todo]] + sig[which[todo], None] * rng.standard_normal(size=(todo.size, 2))
            ok = (p > 0.0).all(axis=1) & (p < 1.0).all(axis=1)
            out[todo[ok]] = p[ok]
            todo = todo[~ok]
        u = rng.uniform(0.0, 1.0, size=(n - nb, 2))
        p = np.concatenate([out, u])
        p = p[rng.permutation(n)]
        return p[:, 0].copy(), p[:, 1].copy()
    raise ValueError(kind)


def make_problem(grid_n: int, n_sites: int, density: str = "uniform", site_kind: str = "uniform",
                 masses: str = "equal", seed: int = 0, tol_rel: float = 1e-6, name: str = "") -> Problem:
    rng = _rng(seed)
    mesh = unit_grid(grid_n, density_values(density, grid_n, rng))
    x, y = sites(site_kind, n_sites, rng)
    total = mesh.total_mass()
    if masses == "equal":
        nu = np.full(n_sites, total / n_sites)
    elif masses == "random":
        r = rng.uniform(0.5, 1.5, size=n_sites)
        nu = r * (total / r.sum())
    else:
        raise ValueError(masses)
    return Problem(mesh, x, y, nu, np.zeros(n_sites), tol_rel, name or f"grid{grid_n}_n{n_sites}")


def c1(seed: int = 0) -> Problem:
    """Plain FP64 Newton OT at the reference's own CPU scale (stop at 1e-9)."""
    return make_problem(64, 1000, "uniform", "uniform", "equal", seed, 1e-9, "c1")


def c2(seed: int = 0) -> Problem:
    """Plain FP64 at scale: 512^2 Gaussian-mixture density, 1e5 uniform sites."""
    return make_problem(512, 100_000, "gauss", "uniform", "random", seed, 1e-6, "c2")


def c3(seed: int = 0) -> Problem:
    """Mixed precision: 2048^2 density, 1e6 clustered sites, equal masses."""
    return make_problem(2048, 1_000_000, "uniform", "blobs", "equal", seed, 1e-6, "c3")


def c4(seed: int = 0) -> Problem:
    """Differentiation: 256^2 density, 2e5 uniform sites."""
    return make_problem(256, 200_000, "uniform", "uniform", "equal", seed, 1e-6, "c4")


def c5(seed: int = 0, count: int = 512):
    """Batching: ``count`` independent problems with log-uniform sizes."""
    rng = _rng(seed)
    sides = np.exp(rng.uniform(np.log(32), np.log(512), size=count)).astype(int)
    ns = np.exp(rng.uniform(np.log(500), np.log(50_000), size=count)).astype(int)
    seeds = rng.integers(0, 2**31 - 1, size=count)
    return [make_problem(int(s), int(n), "uniform", "uniform", "equal", int(sd), 1e-6, f"c5_{k}")
            for k, (s, n, sd) in enumerate(zip(sides, ns, seeds))]


CONFIGS = {"c1": c1, "c2": c2, "c3": c3, "c4": c4}
