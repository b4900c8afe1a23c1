"""Host-side behaviour of the drop-in shim (steps_gb300/legacy/forces_gb300.cc),
no GPU involved:

* recalculate_softening against the reference's own (StePS/src/forces.cc:43-50,
  compiled unmodified into the oracle's reference build): beta and rho_part
  bit-identical, since step.cc's adaptive step size reads rho_part;
* an empty i range is no work and no error, and every call prints the
  reference CUDA build's wall-clock line (StePS/src/forces_cuda.cu:1115,
  :1702) unless STEPS_GB300_QUIET=1."""
import ctypes as C
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_DIR = os.path.join(ROOT, "steps_gb300", "_build")
REF_LIB = os.path.join(ROOT, "oracle", "_ref", "libref_r3.so")
CASES = [(0.05, 0.7, 1), (0.05, 0.7, 0), (0.0173, 3.1e-4, 1), (1.234567, 12.5, 1), (2.0 ** -7, 1e-9, 1)]


def _build(tmp_path_factory, flags=()):
    if not os.path.exists(os.path.join(LIB_DIR, "libsteps_gb300.so")):
        from steps_gb300 import build
        build.build()
    out = str(tmp_path_factory.mktemp("shim") / "libshim_host.so")
    subprocess.run(["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-o", out, "-I", os.path.join(ROOT, "include")] +
                   list(flags) + [os.path.join(ROOT, "steps_gb300", "legacy", "forces_gb300.cc"),
                                  os.path.join(ROOT, "tests", "legacy_globals.cc"), "-L", LIB_DIR, "-lsteps_gb300",
                                  "-Wl,-rpath," + LIB_DIR], check=True)
    h = C.CDLL(out, mode=os.RTLD_LOCAL)
    h.h_softening.argtypes = [C.c_double, C.c_double, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double)]
    h.h_forces.argtypes = [C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_int, C.c_int]
    return h


@pytest.fixture(scope="module")
def shim(tmp_path_factory):
    return _build(tmp_path_factory)


def _shim(h, radius, m_min, cosmology):
    b, r = C.c_double(0), C.c_double(0)
    h.h_softening(radius, m_min, cosmology, C.byref(b), C.byref(r))
    return b.value, r.value


@pytest.mark.skipif(not os.path.exists(REF_LIB), reason="reference build (oracle/_ref) not present")
@pytest.mark.parametrize("radius,m_min,cosmology", CASES)
def test_matches_reference(shim, radius, m_min, cosmology):
    ref = C.CDLL(REF_LIB, mode=os.RTLD_LOCAL)
    C.c_double.in_dll(ref, "ParticleRadi").value = radius
    C.c_double.in_dll(ref, "M_min").value = m_min
    C.c_int.in_dll(ref, "COSMOLOGY").value = cosmology
    C.c_double.in_dll(ref, "rho_part").value = 0.0
    ref._Z21recalculate_softeningv()
    want = (C.c_double.in_dll(ref, "beta").value, C.c_double.in_dll(ref, "rho_part").value)
    assert _shim(shim, radius, m_min, cosmology) == want


@pytest.mark.parametrize("radius,m_min,cosmology", CASES)
def test_formula(shim, radius, m_min, cosmology):
    import math
    beta, rho = _shim(shim, radius, m_min, cosmology)
    assert beta == radius
    assert rho == (m_min / (4.0 * math.pi * math.pow(radius, 3.0) / 3.0) if cosmology == 1 else 0.0)


@pytest.mark.parametrize("flags,prefix", [((), "Force"), (("-DPERIODIC",), "Force"),
                                          (("-DPERIODIC_Z", "-DPERIODIC_Z_NOLOOKUP"), "Z-periodic force")])
def test_empty_range_and_timing_line(tmp_path_factory, capfd, monkeypatch, flags, prefix):
    h = _build(tmp_path_factory, flags)
    libc = C.CDLL(None)
    x = (C.c_double * 6)()
    F = (C.c_double * 3)(7.0, 7.0, 7.0)
    assert h.h_forces(x, F, 10, 9) == 0  # ID_max < ID_min: no work, no ForceError
    assert list(F) == [7.0, 7.0, 7.0]
    libc.fflush(None)
    out = capfd.readouterr().out
    assert f"{prefix} calculation finished on MPI task 0. Force calculation wall-clock time = " in out
