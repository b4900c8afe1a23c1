"""Failure detection without a GPU fault: the bulk-copy pipeline's waits are
bounded. A test hook withholds one copy, the waits on it run out (about a
second), the kernel records STEPS_E_TIMEOUT and leaves, the call reports it,
and the context keeps working."""
import time

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
