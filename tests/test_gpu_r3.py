"""R^3 (compactified, non-periodic) forces on the GPU through the C-ABI,
against the reference's golden vectors and the plain-C oracle.

Tolerances: the plain FP64 kernel must match the reference FP64 CPU path to
1e-12 relative per particle; the mixed kernel (FP32 pairs, FP64
accumulation) must have p99 relative error <= 1e-5 against FP64."""
import ctypes as C

import numpy as np
import pyoracle as O
import pytest

import steps_gb300 as S
from helpers import err_stats, golden, port_params, rel_err
from steps_gb300 import workloads as W

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12
MIXED_P99 = 1e-5


def test_fp64_golden(engine):
    g = golden("r3_n2048")
    engine.set_particles(g["m"], g["eps"])
    F = engine.forces(g["x"], S.params(S.R3), S.FP64)
    assert rel_err(F, g["F"]).max() < FP64_TOL
    lo, hi = (int(v) for v in g["sub"])
    assert rel_err(engine.forces(g["x"], S.params(S.R3), S.FP64, lo, hi), g["F_sub"]).max() < FP64_TOL
    p = S.params(S.R3, cosmology=1, comoving=1, mius=float(g["mius"]))
    assert rel_err(engine.forces(g["x"], p, S.FP64), g["F_comoving"]).max() < FP64_TOL
    p = S.params(S.R3, cosmology=1, comoving=0, h0=float(g["h0"]), oml=float(g["oml"]))
    assert rel_err(engine.forces(g["x"], p, S.FP64), g["F_de"]).max() < FP64_TOL


def test_mixed_golden(engine):
    g = golden("r3_n2048")
    engine.set_particles(g["m"], g["eps"])
    st = err_stats(engine.forces(g["x"], S.params(S.R3), S.MIXED), g["F"])
    assert st["p99"] < MIXED_P99, st
    lo, hi = (int(v) for v in g["sub"])
    st = err_stats(engine.forces(g["x"], S.params(S.R3), S.MIXED, lo, hi), g["F_sub"])
    assert st["p99"] < MIXED_P99, st
    p = S.params(S.R3, cosmology=1, comoving=1, mius=float(g["mius"]))
    assert err_stats(engine.forces(g["x"], p, S.MIXED), g["F_comoving"])["p99"] < MIXED_P99


@pytest.mark.parametrize("n", [1, 2, 3, 127, 129, 257, 1000])
def test_edge_sizes(engine, port, n):
    ps = W.r3_compactified(n, 300.0, seed=100 + n, displace=True)
    engine.set_particles(ps.m, ps.eps)
    s = port.system(0, ps.m, ps.eps, port_params(O))
    Fo = port.forces(s, ps.x)
    F64 = engine.forces(ps.x, S.params(S.R3), S.FP64)
    if n == 1:
        assert np.all(F64 == 0) and np.all(Fo == 0)
    else:
        assert rel_err(F64, Fo).max() < FP64_TOL
    Fm = engine.forces(ps.x, S.params(S.R3), S.MIXED)
    if n > 1:
        assert err_stats(Fm, Fo)["p99"] < MIXED_P99
    # single-particle i ranges at both ends
    for lo in (0, n - 1):
        Fl = engine.forces(ps.x, S.params(S.R3), S.FP64, lo, lo)
        np.testing.assert_allclose(Fl[0], Fo[lo], rtol=1e-12, atol=1e-300)
        Fl = engine.forces(ps.x, S.params(S.R3), S.MIXED, lo, lo)
        if n > 1:
            assert rel_err(Fl, Fo[lo:lo + 1]).max() < 1e-4


def test_coincident_and_softened_pairs(engine, port):
    # Pairs inside the spline core, a coincident pair (r = 0) and a pair exactly at beta.
    rng = np.random.default_rng(5)
    x = rng.normal(0, 0.05, (300, 3))
    x[1] = x[0]
    x[3] = x[2] + np.array([0.2, 0, 0])
    m = rng.uniform(0.5, 2.0, 300)
    eps = np.full(300, 0.1)
    engine.set_particles(m, eps)
    s = port.system(0, m, eps, port_params(O))
    Fo = port.forces(s, x)
    F64 = engine.forces(x, S.params(S.R3), S.FP64)
    assert np.isfinite(F64).all()
    assert rel_err(F64, Fo).max() < 1e-11
    Fm = engine.forces(x, S.params(S.R3), S.MIXED)
    assert np.isfinite(Fm).all()
    assert err_stats(Fm, Fo)["p99"] < MIXED_P99


def test_two_body(engine):
    x = np.array([[0.0, 0.0, 0.0], [3.0, 4.0, 0.0]])
    m = np.array([2.0, 5.0])
    engine.set_particles(m, np.array([0.1, 0.2]))
    for prec, tol in ((S.FP64, 1e-15), (S.MIXED, 1e-6)):
        F = engine.forces(x, S.params(S.R3), prec)
        np.testing.assert_allclose(F[0], 0.2 * np.array([0.6, 0.8, 0.0]), rtol=tol, atol=1e-12)
        np.testing.assert_allclose(F[1], -0.08 * np.array([0.6, 0.8, 0.0]), rtol=tol, atol=1e-12)


def test_momentum(engine):
    ps = W.r3_compactified(20000, 480.0, seed=7, displace=True)
    engine.set_particles(ps.m, ps.eps)
    for prec, tol in ((S.FP64, 1e-12), (S.MIXED, 1e-6)):
        F = engine.forces(ps.x, S.params(S.R3), prec)
        p = (ps.m[:, None] * F).sum(0)
        assert np.abs(p).max() < tol * (ps.m[:, None] * np.abs(F)).sum()


def test_shapes_agree(engine, port):
    ps = W.r3_compactified(6000, 480.0, seed=8, displace=True)
    engine.set_particles(ps.m, ps.eps)
    Fo = port.forces(port.system(0, ps.m, ps.eps, port_params(O)), ps.x)
    for threads, ipt in ((64, 1), (64, 2), (64, 4), (128, 1), (128, 2), (128, 4), (256, 1), (256, 2)):
        for js in (0, 1, 3):
            engine.set_tuning(threads, ipt, js)
            st = err_stats(engine.forces(ps.x, S.params(S.R3), S.MIXED), Fo)
            assert st["p99"] < MIXED_P99, (threads, ipt, js, st)
    engine.set_tuning(128, 2, 0)


def test_packed_fp32x2_variant(engine, port):
    """The packed FP32x2 pair loop agrees with the reference like the scalar one,
    at each register budget (variants 1-3) and with the bulk-copy pipeline (4)."""
    g = golden("r3_n2048")
    engine.set_particles(g["m"], g["eps"])
    try:
        for variant in (1, 2, 3, 4):
            engine.set_variant(variant)
            for threads, ipt in ((64, 1), (64, 2), (64, 4), (128, 1), (128, 2), (128, 4), (256, 1), (256, 2)):
                engine.set_tuning(threads, ipt, 0)
                st = err_stats(engine.forces(g["x"], S.params(S.R3), S.MIXED), g["F"])
                assert st["p99"] < MIXED_P99, (variant, threads, ipt, st)
        engine.set_variant(1)
        engine.set_tuning(128, 2, 0)
        lo, hi = (int(v) for v in g["sub"])
        assert err_stats(engine.forces(g["x"], S.params(S.R3), S.MIXED, lo, hi), g["F_sub"])["p99"] < MIXED_P99
        for n in (3, 129, 1000):
            ps = W.r3_compactified(n, 300.0, seed=100 + n, displace=True)
            engine.set_particles(ps.m, ps.eps)
            Fo = port.forces(port.system(0, ps.m, ps.eps, port_params(O)), ps.x)
            assert err_stats(engine.forces(ps.x, S.params(S.R3), S.MIXED), Fo)["p99"] < MIXED_P99
        ps = W.r3_compactified(60000, 1000.0, seed=9, displace=True)
        engine.set_particles(ps.m, ps.eps)
        F64 = engine.forces(ps.x, S.params(S.R3), S.FP64, 0, 4095)
        st = err_stats(engine.forces(ps.x, S.params(S.R3), S.MIXED)[:4096], F64)
        assert st["p99"] < MIXED_P99, st
    finally:
        engine.set_variant(0)
        engine.set_tuning(128, 2, 0)


def test_full_size_subset(engine, port):
    """The cfg1 workload at its full size (N = 2^20): mixed against the FP64
    kernel on an i subset, and the FP64 kernel against the oracle on a
    smaller subset (cost is linear in the i range)."""
    ps = W.workload("cfg1")
    engine.set_particles(ps.m, ps.eps)
    lo, hi = 400000, 402047
    F64 = engine.forces(ps.x, S.params(S.R3), S.FP64, lo, hi)
    Fm = engine.forces(ps.x, S.params(S.R3), S.MIXED, lo, hi)
    st = err_stats(Fm, F64)
    assert st["p99"] < MIXED_P99, st
    s = port.system(0, ps.m, ps.eps, port_params(O))
    Fo = port.forces(s, ps.x, lo, lo + 63)
    assert rel_err(F64[:64], Fo).max() < FP64_TOL
    # The full-range mixed evaluation agrees with the subset one on the subset.
    Ff = engine.forces(ps.x, S.params(S.R3), S.MIXED)
    assert err_stats(Ff[lo:hi + 1], F64)["p99"] < MIXED_P99
    assert np.isfinite(Ff).all()


def test_errors(engine):
    g = golden("r3_n2048")
    engine.set_particles(g["m"], g["eps"])
    with pytest.raises(S.StepsError) as e:
        engine.forces(g["x"], S.params(S.R3), S.FP64, 5, 3)
    assert e.value.code == S.STEPS_E_ARG
    with pytest.raises(S.StepsError) as e:
        engine.forces(g["x"], S.params(S.R3), S.FP64, g["m"].size + 1, g["m"].size)
    assert e.value.code == S.STEPS_E_ARG
    with pytest.raises(S.StepsError) as e:
        engine.forces(g["x"], S.params(S.R3), S.FP64, 0, g["m"].size)
    assert e.value.code == S.STEPS_E_ARG
    with pytest.raises(S.StepsError) as e:
        engine.forces(g["x"], S.params(S.R3), 7)
    assert e.value.code == S.STEPS_E_ARG
    with pytest.raises(S.StepsError) as e:
        engine.set_tuning(96, 3)
    assert e.value.code == S.STEPS_E_ARG
    # the context stays usable after errors
    assert rel_err(engine.forces(g["x"], S.params(S.R3), S.FP64), g["F"]).max() < FP64_TOL


@pytest.mark.parametrize("lo", [0, 5, 2048])
def test_empty_range(engine, lo):
    """id_max = id_min - 1 is an empty range: no work and no error, as the
    reference's loop over [ID_min, ID_max] does nothing; the next call is
    unaffected."""
    g = golden("r3_n2048")
    engine.set_particles(g["m"], g["eps"])
    for prec in (S.FP64, S.MIXED):
        F = engine.forces(g["x"], S.params(S.R3), prec, lo, lo - 1)
        assert F.shape == (0, 3)
        assert engine.forces_range() == (lo, 0)
    rc = engine.lib.steps_gpu_forces(C.byref(S.params(S.R3)), S.FP64, g["x"].ctypes.data_as(C.POINTER(C.c_double)),
                                     None, lo, lo - 1)
    assert rc == S.STEPS_OK
    assert rel_err(engine.forces(g["x"], S.params(S.R3), S.FP64), g["F"]).max() < FP64_TOL


def test_resident_forces_range(engine):
    """steps_gpu_download_forces copies the range of the last successful force
    call. New masses leave none, so a caller that shrinks n cannot be handed the
    old, longer range; a call refused by argument checks keeps the range (a
    call that fails while running clears it: tests/test_gpu_timeout.py)."""
    g = golden("r3_n2048")
    p = S.params(S.R3)
    engine.set_particles(g["m"], g["eps"])
    engine.upload_positions(g["x"])
    engine.forces_resident(p, S.FP64, 100, 611)
    assert engine.forces_range() == (100, 512)
    assert rel_err(engine.download_forces(512), g["F"][100:612]).max() < FP64_TOL
    engine.set_particles(g["m"][:16], g["eps"][:16])
    assert engine.forces_range() == (0, 0)
    with pytest.raises(S.StepsError) as e:
        engine.download_forces()
    assert e.value.code == S.STEPS_E_STATE
    engine.set_particles(g["m"], g["eps"])
    engine.upload_positions(g["x"])
    engine.forces_resident(p, S.FP64)
    assert engine.forces_range() == (0, 2048)
    with pytest.raises(S.StepsError):
        engine.forces_resident(p, 7)
    assert engine.forces_range() == (0, 2048)  # refused before any work: the range stands
    with pytest.raises(S.StepsError):
        engine.forces_resident(p, S.FP64, 0, 4096)
    assert engine.forces_range() == (0, 2048)


def test_page_locked_host_buffers(engine):
    """steps_gpu_host_alloc memory works as the host buffers of the drop-in
    call and gives bit-identical results to ordinary host memory."""
    g = golden("r3_n2048")
    engine.set_particles(g["m"], g["eps"])
    x = engine.host_array(g["x"].shape)
    x[...] = g["x"]
    F = engine.host_array((2048, 3))
    try:
        engine.forces(x, S.params(S.R3), S.MIXED, out=F)
        assert np.array_equal(F, engine.forces(g["x"], S.params(S.R3), S.MIXED))
        engine.forces(x, S.params(S.R3), S.FP64, out=F)
        assert rel_err(F, g["F"]).max() < 1e-12
    finally:
        del x, F
        engine.free_host_arrays()
