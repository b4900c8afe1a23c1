"""steps_gpu_forces_fp64_noalloc: the FP64 R^3 force entry point for callers
that cannot allocate device memory (their device memory belongs to their own
pool allocator, or they cannot afford cudaMalloc's implicit synchronisation).
The caller passes device buffers; the library uses only its static scratch.

Checked through the C-ABI against the existing host-buffer entry point
(steps_gpu_forces, FP64) on two calls in a row, at the FP64 tolerance, and
against the reference's own golden forces. This file is collected last so a
stop-at-first-failure run has already run every other test."""
import ctypes as C

import numpy as np
import pytest

import steps_gb300 as S
from helpers import golden, rel_err
from steps_gb300 import workloads as W

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12
SCRATCH_ROWS = (32 << 20) // 24  # i rows of FP64 partial forces the 32 MiB scratch holds


def _call(lib, p, x_d, m_d, e_d, n, F_d, lo, hi, stream):
    fn = lib.steps_gpu_forces_fp64_noalloc
    fn.argtypes = [C.POINTER(S.Params), C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_int,
                   C.c_void_p]
    return fn(C.byref(p), x_d, m_d, e_d, n, F_d, lo, hi, stream)


def _device(torch, *arrays):
    dev = torch.device("cuda", 0)
    return [torch.from_numpy(np.ascontiguousarray(a)).to(dev) for a in arrays]


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
    x_d, m_d, e_d = _device(torch, x, m, eps)
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
            if case == "golden":  # the reference's own FP64 CPU build
                assert rel_err(F, g["F"][lo:hi + 1]).max() < FP64_TOL


def test_noalloc_streams(engine):
    """A side stream and the legacy NULL stream order the two kernels and the
    caller's buffers correctly."""
    torch = pytest.importorskip("torch")
    g = golden("r3_n2048")
    x, m, eps = g["x"], g["m"], g["eps"]
    n = x.shape[0]
    p = S.params(S.R3)
    dev = torch.device("cuda", 0)
    x_d, m_d, e_d = _device(torch, x, m, eps)
    side = torch.cuda.Stream(dev)
    torch.cuda.synchronize(dev)  # inputs were written on torch's current stream
    for st in (side, None):
        F_d = torch.full((n, 3), float("nan"), dtype=torch.float64, device=dev)
        torch.cuda.synchronize(dev)
        handle = st.cuda_stream if st is not None else None
        rc = _call(engine.lib, p, x_d.data_ptr(), m_d.data_ptr(), e_d.data_ptr(), n, F_d.data_ptr(), 0, n - 1, handle)
        assert rc == S.STEPS_OK, engine.lib.steps_gpu_error_string()
        if st is not None:
            st.synchronize()
        else:
            torch.cuda.synchronize(dev)
        assert rel_err(F_d.cpu().numpy(), g["F"]).max() < FP64_TOL


def test_noalloc_single_chunk(engine):
    """An i range above half the scratch capacity leaves room for one j chunk
    only (no j split): rows of that result against the existing entry point."""
    torch = pytest.importorskip("torch")
    n = SCRATCH_ROWS // 2 + 64
    ps = W.r3_compactified(n, 1000.0, seed=5, displace=True)
    p = S.params(S.R3)
    engine.set_particles(ps.m, ps.eps)
    dev = torch.device("cuda", 0)
    x_d, m_d, e_d = _device(torch, ps.x, ps.m, ps.eps)
    F_d = torch.full((n, 3), float("nan"), dtype=torch.float64, device=dev)
    torch.cuda.synchronize(dev)
    rc = _call(engine.lib, p, x_d.data_ptr(), m_d.data_ptr(), e_d.data_ptr(), n, F_d.data_ptr(), 0, n - 1, None)
    assert rc == S.STEPS_OK, engine.lib.steps_gpu_error_string()
    torch.cuda.synchronize(dev)
    F = F_d.cpu().numpy()
    assert np.isfinite(F).all()
    for lo in (0, n // 2, n - 1024):
        F_ref = engine.forces(ps.x, p, S.FP64, lo, lo + 1023)
        assert rel_err(F[lo:lo + 1024], F_ref).max() < FP64_TOL


def test_noalloc_empty_range(engine):
    """id_max = id_min - 1 is the empty range: STEPS_OK, nothing written, F may
    be NULL -- as steps_gpu_forces and the reference's loop over an empty range."""
    torch = pytest.importorskip("torch")
    n = 64
    dev = torch.device("cuda", 0)
    x_d = torch.zeros((n, 3), dtype=torch.float64, device=dev)
    m_d = torch.ones(n, dtype=torch.float64, device=dev)
    for lo in (0, 17, n):
        rc = _call(engine.lib, S.params(S.R3), x_d.data_ptr(), m_d.data_ptr(), m_d.data_ptr(), n, None, lo, lo - 1,
                   None)
        assert rc == S.STEPS_OK, engine.lib.steps_gpu_error_string()
    rc = _call(engine.lib, S.params(S.R3), x_d.data_ptr(), m_d.data_ptr(), m_d.data_ptr(), n, None, 5, 3, None)
    assert rc == S.STEPS_E_ARG


def test_noalloc_rejects_oversized_range(engine):
    torch = pytest.importorskip("torch")
    n = SCRATCH_ROWS + 1  # one above the i range the 32 MiB scratch holds
    dev = torch.device("cuda", 0)
    x_d = torch.zeros((n, 3), dtype=torch.float64, device=dev)
    m_d = torch.ones(n, dtype=torch.float64, device=dev)
    F_d = torch.zeros((n, 3), dtype=torch.float64, device=dev)
    rc = _call(engine.lib, S.params(S.R3), x_d.data_ptr(), m_d.data_ptr(), m_d.data_ptr(), n, F_d.data_ptr(), 0,
               n - 1, None)
    assert rc == S.STEPS_E_ARG
    assert b"exceeds" in engine.lib.steps_gpu_error_string()
