"""steps_gb300: GB300-native (sm_103a) StePS direct-summation force evaluation.

The product is the C-ABI shared library ``libsteps_gb300.so`` (declared in
include/steps_gb300.h). This package is a thin ctypes front end used by the
tests and the benchmark; it loads the in-tree library and fails loudly when
it is missing -- there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import workloads  # noqa: F401

PKG = os.path.dirname(os.path.abspath(__file__))
# STEPS_GB300_LIB selects another in-tree build of the library, e.g. the
# bounds-checked _build/check/libsteps_gb300_check.so.
LIB_PATH = os.environ.get("STEPS_GB300_LIB") or os.path.join(PKG, "_build", "libsteps_gb300.so")
CHECK_LIB_PATH = os.path.join(PKG, "_build", "check", "libsteps_gb300_check.so")

(STEPS_OK, STEPS_E_ARG, STEPS_E_STATE, STEPS_E_CUDA, STEPS_E_NOMEM, STEPS_E_TABLE, STEPS_E_TIMEOUT,
 STEPS_E_BOUNDS) = range(8)
R3, T3, S1R2 = 0, 1, 2
FP64, MIXED = 0, 1

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


class StepsError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"steps_gb300 error {code}: {msg}")
        self.code = code


class Params(C.Structure):
    """Mirror of ``steps_params`` (include/steps_gb300.h)."""

    _fields_ = [("topology", C.c_int), ("is_periodic", C.c_int), ("L", C.c_double), ("rsim", C.c_double),
                ("cosmology", C.c_int), ("comoving", C.c_int), ("mass_in_unit_sphere", C.c_double),
                ("h0", C.c_double), ("omega_lambda", C.c_double), ("ewald_order", C.c_int),
                ("s1r2_images", C.c_int)]


def params(topology=R3, is_periodic=0, L=0.0, rsim=0.0, cosmology=0, comoving=0, mius=0.0, h0=0.0, oml=0.0,
           ewald_order=4, s1r2_images=1) -> Params:
    return Params(topology, is_periodic, L, rsim, cosmology, comoving, mius, h0, oml, ewald_order, s1r2_images)


_LIB = None


def load_library(path: str = LIB_PATH) -> C.CDLL:
    """Loads libsteps_gb300.so; raises if it has not been built."""
    global _LIB
    if _LIB is not None:
        return _LIB
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`")
    lib = C.CDLL(path)
    lib.steps_gpu_error_string.restype = C.c_char_p
    lib.steps_gpu_launch_count.restype = C.c_longlong
    lib.steps_gpu_last_phase_ms.restype = C.c_double
    lib.steps_gpu_last_pairs.restype = C.c_double
    lib.steps_gpu_timer_elapsed_ms.restype = C.c_double
    lib.steps_gpu_flush_l2.argtypes = [C.c_longlong]
    for name in ("steps_gpu_build_table_t3",):
        getattr(lib, name).argtypes = [C.c_int] + [C.c_double] * 6
    lib.steps_gpu_build_table_s1r2.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, C.c_int,
                                               C.c_int]
    lib.steps_gpu_kdk.argtypes = [C.POINTER(Params), C.c_int, C.c_int, C.c_double, C.c_double, C.c_double,
                                  C.c_double, C.c_double, _dp]
    lib.steps_gpu_forces.argtypes = [C.POINTER(Params), C.c_int, _dp, _dp, C.c_int, C.c_int]
    lib.steps_gpu_forces_resident.argtypes = [C.POINTER(Params), C.c_int, C.c_int, C.c_int]
    lib.steps_gpu_batch_run.argtypes = [C.POINTER(Params), C.c_int, C.c_int, C.c_double, C.c_int]
    _LIB = lib
    return lib


def h5_read(path, dataset):
    """A dataset of an HDF5 file in the layout the HDF5 library writes by
    default (the reference's table files), as float64, with its shape;
    through steps_h5_read_f64 (no GPU needed)."""
    lib = load_library()
    fn = lib.steps_h5_read_f64
    fn.argtypes = [C.c_char_p, C.c_char_p, C.c_void_p, C.c_longlong, C.POINTER(C.c_longlong), C.POINTER(C.c_int),
                   C.POINTER(C.c_longlong)]
    cnt, rank, dims = C.c_longlong(0), C.c_int(0), (C.c_longlong * 32)()
    args = (os.fsencode(path), dataset.encode())
    rc = fn(*args, None, 0, C.byref(cnt), C.byref(rank), dims)
    if rc != STEPS_OK:
        raise StepsError(rc, lib.steps_gpu_error_string().decode())
    out = np.empty(cnt.value)
    rc = fn(*args, out.ctypes.data, cnt.value, None, None, None)
    if rc != STEPS_OK:
        raise StepsError(rc, lib.steps_gpu_error_string().decode())
    return out.reshape([dims[k] for k in range(rank.value)])


def _d(a: np.ndarray):
    return a.ctypes.data_as(_dp)


class Engine:
    """Host-side handle on the library's single-GPU context.

    Mirrors the reference force interface: positions x (N,3) float64 in,
    accelerations of particles id_min..id_max out (overwritten)."""

    def __init__(self, device: int = 0):
        self.lib = load_library()
        self._check(self.lib.steps_gpu_init(int(device)))
        self.n = 0

    def _check(self, rc: int):
        if rc != STEPS_OK:
            raise StepsError(rc, self.lib.steps_gpu_error_string().decode())

    def shutdown(self):
        self._check(self.lib.steps_gpu_shutdown())

    def set_particles(self, m, eps):
        m = np.ascontiguousarray(m, dtype=np.float64)
        eps = np.ascontiguousarray(eps, dtype=np.float64)
        self._check(self.lib.steps_gpu_set_particles(int(m.size), _d(m), _d(eps)))
        self.n = int(m.size)

    def forces(self, x, p: Params, precision=MIXED, id_min=0, id_max=None, out=None) -> np.ndarray:
        x = np.ascontiguousarray(x, dtype=np.float64)
        if id_max is None:
            id_max = self.n - 1
        ni = max(id_max - id_min + 1, 0)  # the library checks the range itself
        F = np.empty((ni, 3)) if out is None else out
        assert F.shape == (ni, 3) and F.dtype == np.float64 and F.flags.c_contiguous
        self._check(self.lib.steps_gpu_forces(C.byref(p), int(precision), _d(x), _d(F), int(id_min), int(id_max)))
        return F

    def upload_positions(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        self._check(self.lib.steps_gpu_upload_positions(_d(x)))

    def upload_velocities(self, v):
        v = np.ascontiguousarray(v, dtype=np.float64)
        self._check(self.lib.steps_gpu_upload_velocities(_d(v)))

    def forces_resident(self, p: Params, precision=MIXED, id_min=0, id_max=None):
        if id_max is None:
            id_max = self.n - 1
        self._check(self.lib.steps_gpu_forces_resident(C.byref(p), int(precision), int(id_min), int(id_max)))

    def forces_range(self):
        """(id_min, count) of the resident forces; count 0 when there are none."""
        lo, cnt = C.c_int(0), C.c_int(0)
        self._check(self.lib.steps_gpu_forces_range(C.byref(lo), C.byref(cnt)))
        return lo.value, cnt.value

    def download_forces(self, ni=None) -> np.ndarray:
        # The library copies the whole range of the last force call.
        _, cnt = self.forces_range()
        if ni is not None and ni != cnt:
            raise ValueError(f"the resident forces cover {cnt} particles, not {ni}")
        F = np.empty((max(cnt, 1), 3))
        self._check(self.lib.steps_gpu_download_forces(_d(F)))
        return F

    def kdk(self, p: Params, precision, nsteps, h, g=1.0, a=1.0, hubble=0.0, rho_part=1.0) -> float:
        e = C.c_double(0)
        self._check(self.lib.steps_gpu_kdk(C.byref(p), int(precision), int(nsteps), float(h), float(g), float(a),
                                           float(hubble), float(rho_part), C.byref(e)))
        return e.value

    def state(self):
        x = np.empty((self.n, 3)); v = np.empty((self.n, 3)); F = np.empty((self.n, 3))
        self._check(self.lib.steps_gpu_download_state(_d(x), _d(v), _d(F)))
        return x, v, F

    # tables
    def set_table_t3(self, table, ngrid):
        table = np.ascontiguousarray(table, dtype=np.float64)
        self._check(self.lib.steps_gpu_set_table_t3(int(ngrid), _d(table)))

    def build_table_t3(self, ngrid, L, alpha, rel_cut, rec_cut, real_radius, rec_radius):
        self._check(self.lib.steps_gpu_build_table_t3(int(ngrid), L, alpha, rel_cut, rec_cut, real_radius,
                                                      rec_radius))
        self.t3_ng = int(ngrid)

    def get_table_t3(self, ngrid=None):
        ngrid = ngrid or self.t3_ng
        out = np.empty(3 * ngrid ** 3)
        self._check(self.lib.steps_gpu_get_table_t3(_d(out)))
        return out

    def set_table_s1r2(self, table, nrho, nz):
        table = np.ascontiguousarray(table, dtype=np.float64)
        self._check(self.lib.steps_gpu_set_table_s1r2(int(nrho), int(nz), _d(table)))

    def build_table_s1r2(self, nrho, nz, rho_max, lz, alpha, nmax, mmax):
        self._check(self.lib.steps_gpu_build_table_s1r2(int(nrho), int(nz), rho_max, lz, alpha, int(nmax),
                                                        int(mmax)))
        self.s1r2_shape = (int(nrho), int(nz))

    def get_table_s1r2(self, nrho=None, nz=None):
        nrho, nz = (nrho, nz) if nrho else self.s1r2_shape
        out = np.empty(2 * nrho * nz)
        self._check(self.lib.steps_gpu_get_table_s1r2(_d(out)))
        return out

    def load_table_t3_hdf5(self, path):
        ng = C.c_int(0)
        self.lib.steps_gpu_load_table_t3_hdf5.argtypes = [C.c_char_p, C.POINTER(C.c_int)]
        self._check(self.lib.steps_gpu_load_table_t3_hdf5(os.fsencode(path), C.byref(ng)))
        self.t3_ng = ng.value
        return ng.value

    def load_table_s1r2_hdf5(self, path):
        nrho, nz = C.c_int(0), C.c_int(0)
        self.lib.steps_gpu_load_table_s1r2_hdf5.argtypes = [C.c_char_p, C.POINTER(C.c_int), C.POINTER(C.c_int)]
        self._check(self.lib.steps_gpu_load_table_s1r2_hdf5(os.fsencode(path), C.byref(nrho), C.byref(nz)))
        self.s1r2_shape = (nrho.value, nz.value)
        return nrho.value, nz.value

    def set_radial_table(self, tab):
        tab = np.ascontiguousarray(tab, dtype=np.float64)
        self._check(self.lib.steps_gpu_set_radial_table(int(tab.size), _d(tab)))

    def build_radial_table(self, size, rsim, lz, accuracy):
        self.lib.steps_gpu_build_radial_table.argtypes = [C.c_int, C.c_double, C.c_double, C.c_int]
        self._check(self.lib.steps_gpu_build_radial_table(int(size), float(rsim), float(lz), int(accuracy)))
        self.radial_size = int(size)

    def get_radial_table(self, size=None):
        out = np.empty(size or self.radial_size)
        self._check(self.lib.steps_gpu_get_radial_table(_d(out)))
        return out

    # batched ensembles
    def batch_set(self, xs, ms, epss):
        """Registers independent realisations (lists of x[n_k,3], m[n_k], eps[n_k])."""
        self._batch = [(np.ascontiguousarray(x, dtype=np.float64), np.ascontiguousarray(m, dtype=np.float64),
                        np.ascontiguousarray(e, dtype=np.float64)) for x, m, e in zip(xs, ms, epss)]
        k = len(self._batch)
        n = (C.c_int * k)(*[int(m.size) for _, m, _ in self._batch])
        px = (_dp * k)(*[_d(x) for x, _, _ in self._batch])
        pm = (_dp * k)(*[_d(m) for _, m, _ in self._batch])
        pe = (_dp * k)(*[_d(e) for _, _, e in self._batch])
        self._check(self.lib.steps_gpu_batch_set(k, n, px, pm, pe))

    def batch_run(self, p: Params, precision, nsteps, h, graph=1):
        """graph: 1 (or True) one persistent kernel in a CUDA graph, 2 a graph of
        per-phase kernels, 0 (or False) plain per-realisation launches."""
        self._check(self.lib.steps_gpu_batch_run(C.byref(p), int(precision), int(nsteps), float(h), int(graph)))

    def test_stall_ensemble(self, realisation: int):
        self._check(self.lib.steps_gpu_test_stall_ensemble(int(realisation)))

    def checks_compiled(self) -> bool:
        return bool(self.lib.steps_gpu_checks_compiled())

    def test_bounds_check(self, index: int) -> tuple[int, str]:
        """Status and message of one self-test index against the bound 16."""
        rc = self.lib.steps_gpu_test_bounds_check(int(index))
        return rc, self.lib.steps_gpu_error_string().decode() if rc else ""

    def batch_get(self, k):
        n = self._batch[k][1].size
        x = np.empty((n, 3)); v = np.empty((n, 3)); F = np.empty((n, 3))
        self._check(self.lib.steps_gpu_batch_get(int(k), _d(x), _d(v), _d(F)))
        return x, v, F

    # tuning / instrumentation
    def set_tuning(self, threads, ipt, jsplit=0):
        self._check(self.lib.steps_gpu_set_tuning(int(threads), int(ipt), int(jsplit)))

    def autotune(self, p: Params, id_min=0, id_max=None):
        """Returns (threads, ipt, variant) of the fastest mixed-precision kernel."""
        out = (C.c_int * 3)()
        if id_max is None:
            id_max = self.n - 1
        self._check(self.lib.steps_gpu_autotune(C.byref(p), int(id_min), int(id_max), out))
        return int(out[0]), int(out[1]), int(out[2])

    def set_guard(self, ratio: float):
        self.lib.steps_gpu_set_precision_guard.argtypes = [C.c_double]
        self._check(self.lib.steps_gpu_set_precision_guard(float(ratio)))

    def set_t3_window(self, cells: int):
        self._check(self.lib.steps_gpu_set_t3_window(int(cells)))

    def test_stall_copy(self, tile_seq: int):
        self.lib.steps_gpu_test_stall_copy.argtypes = [C.c_longlong]
        self._check(self.lib.steps_gpu_test_stall_copy(int(tile_seq)))

    def set_variant(self, variant: int):
        self._check(self.lib.steps_gpu_set_kernel_variant(int(variant)))

    def launch_count(self) -> int:
        return int(self.lib.steps_gpu_launch_count())

    def phase_ms(self, phase: int) -> float:
        return float(self.lib.steps_gpu_last_phase_ms(int(phase)))

    def mark(self, slot: int):
        self._check(self.lib.steps_gpu_timer_mark(int(slot)))

    def elapsed_ms(self, a: int, b: int) -> float:
        return float(self.lib.steps_gpu_timer_elapsed_ms(int(a), int(b)))

    def flush_l2(self, nbytes: int = 512 << 20):
        self._check(self.lib.steps_gpu_flush_l2(int(nbytes)))

    def host_array(self, shape):
        """A float64 numpy array in page-locked host memory (freed with the
        array's owner, this engine, at shutdown or via free_host_arrays)."""
        n = int(np.prod(shape))
        p = C.c_void_p()
        self.lib.steps_gpu_host_alloc.argtypes = [C.c_longlong, C.POINTER(C.c_void_p)]
        self._check(self.lib.steps_gpu_host_alloc(8 * max(n, 1), C.byref(p)))
        self._pinned = getattr(self, "_pinned", []) + [p.value]
        buf = (C.c_double * max(n, 1)).from_address(p.value)
        return np.frombuffer(buf, dtype=np.float64, count=n).reshape(shape)

    def free_host_arrays(self):
        self.lib.steps_gpu_host_free.argtypes = [C.c_void_p]
        for p in getattr(self, "_pinned", []):
            self._check(self.lib.steps_gpu_host_free(C.c_void_p(p)))
        self._pinned = []

    def synchronize(self):
        self._check(self.lib.steps_gpu_synchronize())

    def measure_peaks(self):
        f32 = C.c_double(0); f64 = C.c_double(0)
        self._check(self.lib.steps_gpu_measure_peaks(C.byref(f32), C.byref(f64)))
        return f32.value, f64.value
