"""steps_gpu_forces_fp64_noalloc: the FP64 R^3 force entry point for callers
that cannot allocate device memory (their device memory belongs to their own
pool allocator, or they cannot afford cudaMalloc's implicit synchronisation).
The caller passes device buffers; the library uses only its static scratch.

Checked through the C-ABI against the existing host-buffer entry point
(steps_gpu_forces, FP64) on two calls in a row, at the FP64 tolerance.
This file is collected last so a stop-at-first-failure run has already run
every other test."""
import ctypes as C

import numpy as np
import pytest

import steps_gb300 as S
from helpers import golden, rel_err
from steps_gb300 import workloads as W

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12


def _call(lib, p, x_d, m_d, e_d, n, F_d, lo, hi, stream):
    fn = lib.steps_gpu_forces_fp64_noalloc
    fn.argtypes = [C.POINTER(S.Params), C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_int,
                   C.c_void_p]
    return fn(C.byref(p), x_d, m_d, e_d, n, F_d, lo, hi, stream)


@pytest.mark.parametrize("case", ["golden", "clustered"])
def test_noalloc_matches_forces(engine, case):
    torch = pytest.importorskip("torch")
    if case == "golden":
        g = golden("r3_n2048")
        x, m, eps = g["x"], g["m"], g["eps"]
        ranges = [(0, x.shape[0] - 1), (100, 611)]
    else:
        ps = W.r3_compactified(30000, 480.0, seed=77, displace=True)
        x, m, eps = ps.x, ps.m, ps.eps
        ranges = [(0, x.shape[0] - 1), (29990, 29999)]
    n = x.shape[0]
    p = S.params(S.R3)
    engine.set_particles(m, eps)
    dev = torch.device("cuda", 0)
    x_d = torch.from_numpy(np.ascontiguousarray(x)).to(dev)
    m_d = torch.from_numpy(np.ascontiguousarray(m)).to(dev)
    e_d = torch.from_numpy(np.ascontiguousarray(eps)).to(dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    for lo, hi in ranges:
        F_ref = engine.forces(x, p, S.FP64, lo, hi)
        for _ in range(2):  # two calls in a row share the static scratch
            F_d = torch.full((hi - lo + 1, 3), float("nan"), dtype=torch.float64, device=dev)
            rc = _call(engine.lib, p, x_d.data_ptr(), m_d.data_ptr(), e_d.data_ptr(), n, F_d.data_ptr(), lo, hi,
                       stream)
            assert rc == S.STEPS_OK, engine.lib.steps_gpu_error_string()
            torch.cuda.synchronize(dev)
            F = F_d.cpu().numpy()
            assert np.isfinite(F).all()
            assert rel_err(F, F_ref).max() < FP64_TOL


def test_noalloc_rejects_oversized_range(engine):
    torch = pytest.importorskip("torch")
    n = 1_500_000  # above the 1,398,101-particle i range the 32 MiB scratch holds
    dev = torch.device("cuda", 0)
    x_d = torch.zeros((n, 3), dtype=torch.float64, device=dev)
    m_d = torch.ones(n, dtype=torch.float64, device=dev)
    F_d = torch.zeros((n, 3), dtype=torch.float64, device=dev)
    rc = _call(engine.lib, S.params(S.R3), x_d.data_ptr(), m_d.data_ptr(), m_d.data_ptr(), n, F_d.data_ptr(), 0,
               n - 1, None)
    assert rc == S.STEPS_E_ARG
    assert b"exceeds" in engine.lib.steps_gpu_error_string()
