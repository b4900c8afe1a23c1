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

import pyoracle as O
import steps_gb300 as S
from helpers import err_stats, golden, port_params, rel_err
from steps_gb300 import workloads as W

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
FLAGS = {"r3": [], "t3": ["-DPERIODIC", "-DEWALD_INTERPOLATION_ORDER=4"],
         "s1nl": ["-DPERIODIC_Z", "-DPERIODIC_Z_NOLOOKUP"], "s1tab": ["-DPERIODIC_Z", "-DEWALD_INTERPOLATION_ORDER=2"],
         # REAL = float builds (USE_SINGLE_PRECISION, StePS/src/global_variables.h:26-32)
         "r3sp": ["-DUSE_SINGLE_PRECISION"],
         "t3o2sp": ["-DPERIODIC", "-DEWALD_INTERPOLATION_ORDER=2", "-DUSE_SINGLE_PRECISION"],
         "s1nlsp": ["-DPERIODIC_Z", "-DPERIODIC_Z_NOLOOKUP", "-DUSE_SINGLE_PRECISION"]}
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


def f32(a):
    """What a REAL = float driver holds of a double array."""
    return np.asarray(a, dtype=np.float32).astype(np.float64)


def _single_precision_case(h, engine, port_sys, port, x, m, eps, p, F32_ref, lo, hi):
    """The shim in a REAL = float build. The driver hands it float positions,
    masses and softening, so its results are checked against this library's
    kernels on those float inputs (the shim converts them to double exactly):
    FP64 mode equals the FP64 kernel, and mixed mode the mixed kernel of the
    same shape (the shim's autotuning is off), each to one FP32 rounding of
    the output; the FP64 kernel on them equals the oracle (1e-12); and mixed
    mode keeps p99 <= 1e-5 against that FP64 answer. The reference's own FP32
    build, on the same float inputs, is at the same error level (its
    statistics are in the assertion message); against the FP64 answer on the
    unrounded inputs the mixed kernel is compared with it in
    test_gpu_fp32_floor.py."""
    n = x.shape[0]
    engine.set_particles(f32(m), f32(eps))
    truth = engine.forces(f32(x), p, S.FP64)
    port_truth = port.forces(port_sys, f32(x), lo, hi)
    assert rel_err(truth[lo:hi + 1], port_truth).max() < 1e-12
    engine.set_tuning(128, 2, 0)
    engine.set_variant(0)
    mixed = engine.forces(f32(x), p, S.MIXED)
    h.h_precision(S.FP64)
    rc, F = run(h, x, 0)
    assert rc == 0 and F.shape[0] == n
    assert rel_err(F, truth).max() < 2e-7  # one FP32 rounding of each component
    h.h_precision(S.MIXED)
    rc, F = run(h, x, 0)
    assert rc == 0
    assert rel_err(F, mixed).max() < 2e-7
    ours, theirs = err_stats(F[lo:hi + 1], truth[lo:hi + 1]), err_stats(F32_ref, port_truth)
    assert ours["p99"] < 1e-5, ("mixed", ours, "reference FP32 build", theirs)


@pytest.fixture
def no_shim_autotune(monkeypatch):
    monkeypatch.setenv("STEPS_GB300_AUTOTUNE", "0")


def test_single_precision_build_r3(tmp_path_factory, engine, port, no_shim_autotune):
    f = golden("ref_fp32")
    ps = W.r3_compactified(int(f["r3_n"]), float(f["r3_rmax"]), seed=int(f["r3_seed"]))
    lo, hi = (int(v) for v in f["r3_sub"])
    h = harness(tmp_path_factory, "r3sp")
    h.h_set(ps.n, np.ascontiguousarray(ps.m).ctypes.data_as(_dp), np.ascontiguousarray(ps.eps).ctypes.data_as(_dp),
            0, 0.0, 0.0, 0, 0, 0.0)
    s = port.system(0, f32(ps.m), f32(ps.eps), port_params(O))
    _single_precision_case(h, engine, s, port, ps.x, ps.m, ps.eps, S.params(S.R3), f["r3_F32"], lo, hi)


def test_single_precision_build_t3(tmp_path_factory, engine, port, no_shim_autotune):
    g, f = golden("t3_o2"), golden("ref_fp32")
    ng, L = int(g["ngrid"]), float(g["L"])
    Lf, rf = float(np.float32(L)), float(np.float32(L / 2))
    h = harness(tmp_path_factory, "t3o2sp")
    set_particles(h, g, 2, L, L / 2)
    t = np.ascontiguousarray(g["table"])
    h.h_table(t.ctypes.data_as(_dp), ng, 0)
    engine.set_table_t3(f32(g["table"]), ng)  # what the float build uploads
    p = S.params(S.T3, is_periodic=2, L=Lf, rsim=rf, ewald_order=2)
    s = port.system(1, f32(g["m"]), f32(g["eps"]), port_params(O, is_periodic=2, L=Lf, rsim=rf),
                    table=f32(g["table"]), ngrid=ng, order=2)
    n = g["x"].shape[0]
    _single_precision_case(h, engine, s, port, g["x"], g["m"], g["eps"], p, f["t3o2_F32"], 0, n - 1)


def test_single_precision_build_s1r2(tmp_path_factory, engine, port, no_shim_autotune):
    g, f = golden("s1r2_images"), golden("ref_fp32")
    Lf, rf = float(np.float32(float(g["L"]))), float(np.float32(float(g["rsim"])))
    h = harness(tmp_path_factory, "s1nlsp")
    set_particles(h, g, 2, float(g["L"]), float(g["rsim"]))
    p = S.params(S.S1R2, is_periodic=2, L=Lf, rsim=rf, s1r2_images=1)
    s = port.system(3, f32(g["m"]), f32(g["eps"]), port_params(O, is_periodic=2, L=Lf, rsim=rf))
    n = g["x"].shape[0]
    _single_precision_case(h, engine, s, port, g["x"], g["m"], g["eps"], p, f["s1r2_is2_F32"], 0, n - 1)
