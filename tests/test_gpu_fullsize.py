"""Parity at every benchmark workload's real size.

Each case runs the full-range mixed evaluation at the workload's size and
compares it with the FP64 kernel on an i sample (p99 <= 1e-5; the maximum is
recorded in the message), and the FP64 kernel with the oracle on a smaller
sample (<= 1e-12): the force cost is linear in the i range, so samples keep
the checkers fast while the kernels see the full density, extent, image cuts,
half-box wraps and table cells of the workload.

* S1xR2, N = 2^21, L_z = 200, R = 600, 7 images (IS_PERIODIC = 2;
  StePS/src/forces.cc:1221-1305);
* S1xR2 with the (rho, z) table 864 x 128 at orders 0 / 2 / 4, N = 2^20
  (StePS/src/forces.cc:1307-1350, ewald_space.cc:803-1048);
* T^3, N = 2^19 clumpy, on the Ng = 63 table built on the GPU, orders 2 and
  4 (StePS/src/forces.cc:776-876);
* the 64-realisation ensemble, 1 force + 10 KDK steps in the CUDA graph:
  realisation 0, the largest and the smallest against FP64 KDK runs of the
  same realisations (the FP64 KDK is pinned to the reference's step(),
  StePS/src/step.cc:100-312), the smallest also against the oracle's KDK.
"""
import math

import numpy as np
import pyoracle as O
import pytest

import steps_gb300 as S
from helpers import err_stats, port_params, rel_err
from steps_gb300 import workloads as W

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12
MIXED_P99 = 1e-5
SAMPLE = 2048  # i particles of the mixed-vs-FP64 comparison
ORACLE_SAMPLE = 64  # i particles of the FP64-vs-oracle comparison


def _check(engine, port_sys, port, x, p, sample_lo):
    Fm = engine.forces(x, p, S.MIXED)
    assert np.isfinite(Fm).all()
    lo, hi = sample_lo, sample_lo + SAMPLE - 1
    F64 = engine.forces(x, p, S.FP64, lo, hi)
    st = err_stats(Fm[lo:hi + 1], F64)
    assert st["p99"] < MIXED_P99, st
    Fo = port.forces(port_sys, x, lo, lo + ORACLE_SAMPLE - 1)
    e = rel_err(F64[:ORACLE_SAMPLE], Fo).max()
    assert e < FP64_TOL, e
    return st


def test_s1r2_images_full_size(engine, port):
    ps = W.workload("cfg2")
    assert ps.n == 1 << 21
    engine.set_particles(ps.m, ps.eps)
    p = S.params(S.S1R2, is_periodic=2, L=200.0, rsim=600.0, s1r2_images=1)
    s = port.system(3, ps.m, ps.eps, port_params(O, is_periodic=2, L=200.0, rsim=600.0))
    _check(engine, s, port, ps.x, p, 1_000_000)


@pytest.mark.parametrize("order", [0, 2, 4])
def test_s1r2_table_full_size(engine, port, order):
    ps = W.s1r2_cylindrical(1 << 20, 200.0, 600.0, seed=2)
    nz = 128
    nrho = int(math.floor(nz * 2.25 * 600.0 / 200.0))  # StePS/src/main.cc:577-581 at IS_PERIODIC = 2
    engine.set_particles(ps.m, ps.eps)
    engine.build_table_s1r2(nrho, nz, 2.25 * 600.0, 200.0, 0.787875 / 200.0, 4, 10)
    table = engine.get_table_s1r2(nrho, nz)
    p = S.params(S.S1R2, is_periodic=2, L=200.0, rsim=600.0, s1r2_images=0, ewald_order=order)
    s = port.system(2, ps.m, ps.eps, port_params(O, is_periodic=2, L=200.0, rsim=600.0), table=table, nrho=nrho,
                    nz=nz, order=order)
    _check(engine, s, port, ps.x, p, 500_000)


@pytest.mark.parametrize("order", [2, 4])
def test_t3_full_size(engine, port, order):
    ps = W.workload("cfg3")
    assert ps.n == 1 << 19
    ng = 63
    engine.set_particles(ps.m, ps.eps)
    engine.build_table_t3(ng, 100.0, 2.0 / 100.0, 2.0, 5.0 * 2.0 * math.pi / 100.0, 3.0, 6.0)
    table = engine.get_table_t3(ng)
    p = S.params(S.T3, is_periodic=2, L=100.0, rsim=50.0, ewald_order=order)
    s = port.system(1, ps.m, ps.eps, port_params(O, is_periodic=2, L=100.0, rsim=50.0), table=table, ngrid=ng,
                    order=order)
    _check(engine, s, port, ps.x, p, 250_000)


def test_ensemble_full_scale(engine, port):
    sets = W.r3_ensemble(64)
    nsteps, h = 10, 1e-3
    p = S.params(S.R3)
    sizes = [s.n for s in sets]
    check = sorted({0, int(np.argmax(sizes)), int(np.argmin(sizes))})
    engine.set_variant(1)
    try:
        engine.batch_set([s.x for s in sets], [s.m for s in sets], [s.eps for s in sets])
        engine.batch_run(p, S.MIXED, nsteps, h, graph=True)
        got = {k: engine.batch_get(k) for k in check}
    finally:
        engine.set_variant(0)
    for k in check:
        ps = sets[k]
        x, v, F = got[k]
        assert np.isfinite(F).all() and np.isfinite(x).all(), k
        # the last forces, against the FP64 kernel at the same positions
        engine.set_particles(ps.m, ps.eps)
        lo = max(0, ps.n // 2 - SAMPLE // 2)
        hi = min(ps.n, lo + SAMPLE) - 1
        st = err_stats(F[lo:hi + 1], engine.forces(x, p, S.FP64, lo, hi))
        assert st["p99"] < MIXED_P99, (k, st)
        # the trajectory, against an FP64 KDK run of the same realisation
        engine.upload_positions(ps.x)
        engine.upload_velocities(np.zeros_like(ps.x))
        engine.kdk(p, S.FP64, nsteps, h)
        x64, v64, F64 = engine.state()
        assert np.abs(x - x64).max() < 1e-9 * (1 + np.abs(x64).max()), k
        assert err_stats(v, v64)["p99"] < MIXED_P99, (k, err_stats(v, v64))
        assert err_stats(F, F64)["p99"] < MIXED_P99, (k, err_stats(F, F64))
        if k == int(np.argmin(sizes)):
            s = port.system(0, ps.m, ps.eps, port_params(O))
            F0 = port.forces(s, ps.x)
            xo, vo, Fo, _ = port.kdk(s, nsteps, h, ps.x, np.zeros_like(ps.x), F0)
            assert np.abs(x64 - xo).max() < 1e-12 * (1 + np.abs(xo).max()), k
            assert rel_err(F64, Fo).max() < 1e-10, k
            assert err_stats(F, Fo)["p99"] < MIXED_P99, k
