"""The seeded synthetic workloads have the shapes and distributions stated."""
import math

import numpy as np

from steps_gb300 import workloads as W


def test_r3_compactified():
    ps = W.r3_compactified(4096, 480.0, seed=0)
    assert ps.x.shape == (4096, 3)
    r = np.linalg.norm(ps.x, axis=1)
    assert r.max() <= 480.0 * (1 + 1e-12)
    D = ps.meta["D"]
    np.testing.assert_allclose(ps.m / ps.m.sum(), (1 + (r / D) ** 2) ** 3 / ((1 + (r / D) ** 2) ** 3).sum())
    assert abs(ps.m.sum() - 1e5) < 1e-6
    np.testing.assert_allclose(ps.eps, 0.05 * np.cbrt(ps.m / ps.m.min()))
    assert abs(ps.eps.min() - 0.05) < 1e-15
    again = W.r3_compactified(4096, 480.0, seed=0)
    np.testing.assert_array_equal(ps.x, again.x)


def test_r3_displaced_differs_only_by_displacement():
    a = W.r3_compactified(2048, 1000.0, seed=1)
    b = W.r3_compactified(2048, 1000.0, seed=1, displace=True)
    np.testing.assert_array_equal(a.m, b.m)
    d = np.linalg.norm(a.x - b.x, axis=1)
    spacing = np.cbrt(a.m / (1e5 / (4 / 3 * math.pi * 1000.0 ** 3)))
    assert np.median(d / spacing) < 1.5


def test_s1r2():
    ps = W.s1r2_cylindrical(4096, 200.0, 600.0, seed=2)
    assert (ps.x[:, 2] >= 0).all() and (ps.x[:, 2] < 200.0).all()
    rho = np.hypot(ps.x[:, 0], ps.x[:, 1])
    assert rho.max() <= 600.0 * (1 + 1e-12)


def test_t3():
    ps = W.t3_clumpy(4096, 100.0, seed=3)
    assert (ps.x >= 0).all() and (ps.x < 100.0).all()
    assert np.all(ps.m == ps.m[0]) and np.all(ps.eps == 0.02)


def test_ensemble_sizes():
    nk, rmax = W.ensemble_sizes()
    assert nk.size == 64 and (nk % 128 == 0).all()
    assert nk.min() >= 8192 - 64 and nk.max() <= 262144
    assert (rmax >= 200).all() and (rmax <= 800).all()
