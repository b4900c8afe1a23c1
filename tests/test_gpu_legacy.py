"""The drop-in shim (steps_gb300/legacy/forces_gb300.cc) driven the way the
StePS driver drives it: the StePS globals are filled (tests/legacy_globals.cc
plays main.cc's role) and forces / forces_periodic / forces_periodic_z are
called with the driver's arguments; results against the reference's golden
vectors."""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

import steps_gb300 as S
from helpers import err_stats, golden, rel_err

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
FLAGS = {"r3": [], "t3": ["-DPERIODIC", "-DEWALD_INTERPOLATION_ORDER=4"],
         "s1nl": ["-DPERIODIC_Z", "-DPERIODIC_Z_NOLOOKUP"], "s1tab": ["-DPERIODIC_Z", "-DEWALD_INTERPOLATION_ORDER=2"]}
_dp = C.POINTER(C.c_double)


@pytest.fixture(autouse=True)
def default_shape(engine):
    """The shim autotunes the library's kernel shape after its first mixed
    call; later tests expect the defaults back."""
    yield
    engine.set_tuning(128, 2, 0)
    engine.set_variant(0)
    engine.set_t3_window(0)


def harness(tmp_path_factory, variant):
    d = tmp_path_factory.mktemp("legacy_" + variant)
    out = str(d / f"libharness_{variant}.so")
    lib_dir = os.path.join(ROOT, "steps_gb300", "_build")
    subprocess.run(["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-o", out, "-I", os.path.join(ROOT, "include")] +
                   FLAGS[variant] + [os.path.join(ROOT, "steps_gb300", "legacy", "forces_gb300.cc"),
                                     os.path.join(ROOT, "tests", "legacy_globals.cc"), "-L", lib_dir, "-lsteps_gb300",
                                     "-Wl,-rpath," + lib_dir], check=True)
    h = C.CDLL(out, mode=os.RTLD_LOCAL)
    h.h_set.argtypes = [C.c_int, _dp, _dp, C.c_int, C.c_double, C.c_double, C.c_int, C.c_int, C.c_double]
    h.h_table.argtypes = [_dp, C.c_int, C.c_int]
    h.h_forces.argtypes = [_dp, _dp, C.c_int, C.c_int]
    return h


def run(h, x, ni, lo=0, hi=None):
    x = np.ascontiguousarray(x, dtype=np.float64)
    hi = x.shape[0] - 1 if hi is None else hi
    F = np.zeros((hi - lo + 1, 3))
    rc = h.h_forces(x.ctypes.data_as(_dp), F.ctypes.data_as(_dp), lo, hi)
    return rc, F


def set_particles(h, g, isp=0, L=0.0, rsim=0.0):
    m = np.ascontiguousarray(g["m"]); e = np.ascontiguousarray(g["eps"])
    h.h_set(m.size, m.ctypes.data_as(_dp), e.ctypes.data_as(_dp), isp, L, rsim, 0, 0, 0.0)


def test_forces_r3(tmp_path_factory, engine):
    h = harness(tmp_path_factory, "r3")
    g = golden("r3_n2048")
    set_particles(h, g)
    h.h_precision(S.FP64)
    rc, F = run(h, g["x"], 2048)
    assert rc == 0 and rel_err(F, g["F"]).max() < 1e-12
    lo, hi = (int(v) for v in g["sub"])
    rc, F = run(h, g["x"], 0, lo, hi)
    assert rc == 0 and rel_err(F, g["F_sub"]).max() < 1e-12
    h.h_precision(S.MIXED)
    rc, F = run(h, g["x"], 2048)  # default shape, then the shim autotunes once
    assert rc == 0 and err_stats(F, g["F"])["p99"] < 1e-5
    rc, F = run(h, g["x"], 2048)  # the tuned shape
    assert rc == 0 and err_stats(F, g["F"])["p99"] < 1e-5
    # a bad i range sets ForceError instead of aborting
    rc, F = run(h, g["x"], 0, 10, 5000)
    assert rc == 1
    # an empty range (an MPI rank with no particles) is no work and no error
    x = np.ascontiguousarray(g["x"])
    F = np.zeros((1, 3))
    for lo, hi in ((10, 9), (10, 3)):
        assert h.h_forces(x.ctypes.data_as(_dp), F.ctypes.data_as(_dp), lo, hi) == 0
    assert not F.any()


def test_forces_periodic_t3(tmp_path_factory, engine):
    h = harness(tmp_path_factory, "t3")
    g = golden("t3_o4")
    ng, L = int(g["ngrid"]), float(g["L"])
    set_particles(h, g, 2, L, L / 2)
    t = np.ascontiguousarray(g["table"])
    h.h_table(t.ctypes.data_as(_dp), ng, 0)
    h.h_precision(S.FP64)
    rc, F = run(h, g["x"], 2048)
    assert rc == 0 and rel_err(F, g["F"]).max() < 1e-12
    h.h_precision(S.MIXED)
    rc, F = run(h, g["x"], 2048)
    assert rc == 0 and err_stats(F, g["F"])["p99"] < 1e-5


def test_forces_periodic_z(tmp_path_factory, engine):
    g = golden("s1r2_images")
    h = harness(tmp_path_factory, "s1nl")
    set_particles(h, g, 2, float(g["L"]), float(g["rsim"]))
    h.h_precision(S.FP64)
    rc, F = run(h, g["x"], 2048)
    assert rc == 0 and rel_err(F, g["F_is2"]).max() < 1e-12
    g = golden("s1r2_table_o2")
    h = harness(tmp_path_factory, "s1tab")
    set_particles(h, g, 2, float(g["L"]), float(g["rsim"]))
    t = np.ascontiguousarray(g["table"])
    nrho, nz = (int(v) for v in g["shape"])
    h.h_table(t.ctypes.data_as(_dp), nrho, nz)
    h.h_precision(S.FP64)
    rc, F = run(h, g["x"], 2048)
    assert rc == 0 and rel_err(F, g["F"]).max() < 1e-12
