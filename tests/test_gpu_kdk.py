"""Device-resident KDK leapfrog (StePS/src/step.cc:100-312) against the
reference's own step() (golden vectors: one force then 4 fixed-dt steps)."""
import numpy as np
import pytest

import steps_gb300 as S
from helpers import err_stats, golden, rel_err

pytestmark = pytest.mark.gpu


def test_kdk_fp64(engine):
    g = golden("r3_kdk4")
    engine.set_particles(g["m"], g["eps"])
    engine.upload_positions(g["x"])
    engine.upload_velocities(np.zeros_like(g["x"]))
    e = engine.kdk(S.params(S.R3), S.FP64, 4, float(g["dt"]), rho_part=float(g["rho_part"]))
    x, v, F = engine.state()
    np.testing.assert_allclose(x, g["x4"], rtol=0, atol=1e-12)
    assert rel_err(v, g["v4"]).max() < 1e-10
    assert rel_err(F, g["F4"]).max() < 1e-10
    assert abs(e - float(g["errmax"])) <= 1e-10 * float(g["errmax"])


def test_kdk_mixed(engine):
    g = golden("r3_kdk4")
    engine.set_particles(g["m"], g["eps"])
    engine.upload_positions(g["x"])
    engine.upload_velocities(np.zeros_like(g["x"]))
    e = engine.kdk(S.params(S.R3), S.MIXED, 4, float(g["dt"]), rho_part=float(g["rho_part"]))
    x, v, F = engine.state()
    assert np.abs(x - g["x4"]).max() < 1e-6
    assert err_stats(F, g["F4"])["p99"] < 1e-5
    assert abs(e - float(g["errmax"])) <= 1e-4 * float(g["errmax"])


def test_kdk_needs_state(engine):
    g = golden("r3_kdk4")
    engine.set_particles(g["m"][:100], g["eps"][:100])
    with pytest.raises(S.StepsError) as e:
        engine.kdk(S.params(S.R3), S.FP64, 1, 1e-3)
    assert e.value.code == S.STEPS_E_STATE
