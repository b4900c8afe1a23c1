"""Failure detection without a GPU fault: the bulk-copy pipeline's waits are
bounded. A test hook withholds one copy, the waits on it run out (about a
second), the kernel records STEPS_E_TIMEOUT and leaves, the call reports it,
and the context keeps working."""
import time

import numpy as np
import pytest

import steps_gb300 as S
from helpers import err_stats, golden

pytestmark = pytest.mark.gpu


def test_pipeline_wait_runs_out_and_reports(engine):
    g = golden("r3_n2048")
    engine.set_particles(g["m"], g["eps"])
    p = S.params(S.R3)
    try:
        engine.set_variant(4)
        engine.set_tuning(128, 1, 0)
        engine.test_stall_copy(0)
        t0 = time.time()
        with pytest.raises(S.StepsError) as e:
            engine.forces(g["x"], p, S.MIXED)
        assert e.value.code == S.STEPS_E_TIMEOUT
        assert time.time() - t0 < 30
        assert engine.forces_range() == (0, 0)  # no forces left from the failed call
        # the hook is one shot and the context is intact
        F = engine.forces(g["x"], p, S.MIXED)
        assert err_stats(F, g["F"])["p99"] < 1e-5
    finally:
        engine.test_stall_copy(-1)
        engine.set_variant(0)
        engine.set_tuning(128, 2, 0)


def test_ensemble_wait_runs_out_and_reports(engine):
    """The persistent ensemble kernel's stage waits are bounded: a test hook
    keeps one realisation from reporting its first stage done, the waits of
    its next stage run out, the call reports STEPS_E_TIMEOUT, and the next run
    is complete and identical to one before the failure."""
    from steps_gb300 import workloads as W

    sets = [W.r3_compactified(n, 300.0 + 50 * k, seed=90 + k, displace=True) for k, n in enumerate((2048, 640, 1280))]
    p = S.params(S.R3)
    args = ([s.x for s in sets], [s.m for s in sets], [s.eps for s in sets])
    engine.batch_set(*args)
    engine.batch_run(p, S.MIXED, 2, 1e-3, graph=1)
    before = [engine.batch_get(k) for k in range(len(sets))]
    engine.batch_set(*args)
    engine.test_stall_ensemble(1)
    t0 = time.time()
    with pytest.raises(S.StepsError) as e:
        engine.batch_run(p, S.MIXED, 2, 1e-3, graph=1)
    assert e.value.code == S.STEPS_E_TIMEOUT
    assert time.time() - t0 < 30
    engine.batch_set(*args)
    engine.batch_run(p, S.MIXED, 2, 1e-3, graph=1)
    for k in range(len(sets)):
        for a, b in zip(engine.batch_get(k), before[k]):
            assert np.array_equal(a, b), k
