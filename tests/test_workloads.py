"""The seeded synthetic workloads hold the shapes, sizes and value ranges they stand for.

The reference measures on images it does not ship, so the benchmark and the parity
tests run on generated inputs; these checks pin the generators to the configurations
(grid sizes and triangle counts, density ranges, site counts, target masses, stop
tolerances) and to their determinism per seed.
"""
import numpy as np
import pytest

from mongeampere_gb300 import workloads as W


def _check_masses(p, equal):
    total = p.mesh.total_mass()
    assert p.nu.shape == (p.n,) and np.all(p.nu > 0)
    assert p.nu.sum() == pytest.approx(total, rel=1e-12)
    if equal:
        assert np.ptp(p.nu) <= 1e-15 * total
    else:
        # U[0.5, 1.5] normalised: the ratio of two targets is below 3
        assert p.nu.max() / p.nu.min() < 3.0


def _check_sites(p):
    assert p.x.shape == p.y.shape == (p.n,)
    assert np.all((p.x > 0) & (p.x < 1) & (p.y > 0) & (p.y < 1))
    assert np.all(p.w0 == 0.0)


def test_c1_shape():
    p = W.c1(0)
    assert (p.mesh.nx, p.mesh.ny) == (64, 64) and p.mesh.nt == 7938
    assert p.mesh.values.min() >= 0.5 and p.mesh.values.max() <= 1.5
    assert p.n == 1000 and p.tol_rel == 1e-9
    _check_sites(p)
    _check_masses(p, equal=True)


def test_c2_shape():
    p = W.c2(0)
    assert (p.mesh.nx, p.mesh.ny) == (512, 512) and p.mesh.nt == 522242
    v = p.mesh.values
    # 0.1 plus five bumps of amplitude 0.5 .. 2
    assert v.min() >= 0.1 and v.max() >= 0.5 and v.max() <= 0.1 + 5 * 2.0
    assert p.n == 100_000 and p.tol_rel == 1e-6
    _check_sites(p)
    _check_masses(p, equal=False)


def test_c4_shape():
    p = W.c4(0)
    assert (p.mesh.nx, p.mesh.ny) == (256, 256) and p.mesh.nt == 130050
    assert p.n == 200_000
    _check_sites(p)
    _check_masses(p, equal=True)


def test_clustered_sites():
    # the C3 site distribution at a smaller size: 70% of the sites in 20 blobs of
    # sigma <= 0.05 put most sites in a small part of the square
    p = W.make_problem(64, 50_000, "uniform", "blobs", "equal", seed=0)
    _check_sites(p)
    h, _, _ = np.histogram2d(p.x, p.y, bins=20, range=[[0, 1], [0, 1]])
    dense = np.sort(h.ravel())[::-1]
    # uniform sites would put 10% of the sites in the 40 densest bins (10% of the
    # square); the blobs put more than a third there (48% with seed 0)
    assert dense[:40].sum() > 0.35 * p.n


def test_c5_sizes_and_determinism():
    a = W.c5(0, count=64)
    b = W.c5(0, count=64)
    assert len(a) == 64
    sides = np.array([p.mesh.nx for p in a])
    ns = np.array([p.n for p in a])
    assert sides.min() >= 32 and sides.max() <= 512
    assert ns.min() >= 500 and ns.max() <= 50_000
    # log-uniform: both ends of the ranges are used
    assert sides.min() < 64 and sides.max() > 256 and ns.min() < 1500 and ns.max() > 15_000
    for p, q in zip(a, b):
        assert np.array_equal(p.x, q.x) and np.array_equal(p.mesh.values, q.mesh.values)
        _check_masses(p, equal=True)


def test_same_seed_same_doubles_other_seed_other_doubles():
    p, q, r = W.c1(0), W.c1(0), W.c1(1)
    assert np.array_equal(p.x, q.x) and np.array_equal(p.mesh.values, q.mesh.values)
    assert not np.array_equal(p.x, r.x)
