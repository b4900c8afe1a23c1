"""ctypes front end of the TEST ORACLE (never imported by the product).

* ``Port``: oracle/_build/liboracle_steps.so, the plain-C restatement of the
  reference force path (oracle/steps_oracle.c).
* ``Ref``: oracle/_ref/libref_<variant>.so, the UNMODIFIED reference CPU
  sources compiled from the reference tree (oracle/Makefile ``ref``); only
  present where the reference tree is.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this module.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_SO = os.path.join(HERE, "_build", "liboracle_steps.so")
# -O3 -ffast-math build, the reference's release flags: CPU-baseline timing only
PORT_RELEASE_SO = os.path.join(HERE, "_build", "liboracle_steps_release.so")
REF_DIR = os.path.join(HERE, "_ref")

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


def _d(a):
    return a.ctypes.data_as(_dp)


def _i(a):
    return a.ctypes.data_as(_ip)


def build_port():
    subprocess.run(["make", "-s", "-C", HERE, "port"], check=True)


class OracleParams(C.Structure):
    _fields_ = [("is_periodic", C.c_int), ("L", C.c_double), ("rsim", C.c_double),
                ("cosmology", C.c_int), ("comoving", C.c_int),
                ("mass_in_unit_sphere", C.c_double), ("h0", C.c_double),
                ("omega_lambda", C.c_double)]


class OracleSystem(C.Structure):
    _fields_ = [("topology", C.c_int), ("n", C.c_int), ("m", _dp), ("eps", _dp),
                ("p", OracleParams), ("table", _dp), ("ngrid", C.c_int), ("nrho", C.c_int),
                ("nz", C.c_int), ("order", C.c_int), ("radial_table", _dp),
                ("radial_size", C.c_int)]


def make_params(is_periodic=0, L=0.0, rsim=0.0, cosmology=0, comoving=0, mius=0.0, h0=0.0, oml=0.0):
    return OracleParams(is_periodic, L, rsim, cosmology, comoving, mius, h0, oml)


class Port:
    """The plain-C oracle. Arrays are float64 numpy; x is (N,3) C-contiguous."""

    def __init__(self, threads: int | None = None, release: bool = False):
        so = PORT_RELEASE_SO if release else PORT_SO
        if not os.path.exists(so):
            build_port()
        self.lib = C.CDLL(so)
        L = self.lib
        L.oracle_force_softening.restype = C.c_double
        L.oracle_force_softening.argtypes = [C.c_double, C.c_double]
        L.oracle_cyl_correction.restype = C.c_double
        L.oracle_lattice.restype = C.c_int
        L.oracle_kdk.restype = C.c_double
        L.oracle_kdk.argtypes = [C.POINTER(OracleSystem), C.c_int, C.c_double, C.c_double, C.c_double,
                                 C.c_double, C.c_double, _dp, _dp, _dp]
        L.oracle_forces.argtypes = [C.POINTER(OracleSystem), _dp, C.c_int, C.c_int, _dp]
        self.set_threads(threads or os.cpu_count() or 1)

    def set_threads(self, n: int):
        self.lib.oracle_set_threads(C.c_int(int(n)))

    def softening(self, r, b):
        return self.lib.oracle_force_softening(float(r), float(b))

    def system(self, topology: int, m, eps, params: OracleParams, table=None, ngrid=0, nrho=0, nz=0,
               order=0, radial=None):
        m = np.ascontiguousarray(m, dtype=np.float64)
        eps = np.ascontiguousarray(eps, dtype=np.float64)
        keep = [m, eps]
        tp = None
        if table is not None:
            table = np.ascontiguousarray(table, dtype=np.float64)
            keep.append(table)
            tp = _d(table)
        rp, rs = None, 0
        if radial is not None:
            radial = np.ascontiguousarray(radial, dtype=np.float64)
            keep.append(radial)
            rp, rs = _d(radial), int(radial.size)
        s = OracleSystem(topology, int(m.size), _d(m), _d(eps), params, tp, ngrid, nrho, nz, order, rp, rs)
        s._keep = keep
        return s

    def forces(self, sysobj: OracleSystem, x, id_min=0, id_max=None):
        x = np.ascontiguousarray(x, dtype=np.float64)
        if id_max is None:
            id_max = sysobj.n - 1
        F = np.zeros((id_max - id_min + 1, 3))
        self.lib.oracle_forces(C.byref(sysobj), _d(x), int(id_min), int(id_max), _d(F))
        return F

    def kdk(self, sysobj, nsteps, h, x, v, F, g=1.0, a=1.0, hubble=0.0, rho_part=1.0):
        x = np.array(x, dtype=np.float64, order="C")
        v = np.array(v, dtype=np.float64, order="C")
        F = np.array(F, dtype=np.float64, order="C")
        e = self.lib.oracle_kdk(C.byref(sysobj), int(nsteps), float(h), float(g), float(a), float(hubble),
                                float(rho_part), _d(x), _d(v), _d(F))
        return x, v, F, e

    def lattice(self, radius):
        cap = 80000
        out = np.zeros(4 * cap, dtype=np.int32)
        n = self.lib.oracle_lattice(C.c_double(radius), _i(out), C.c_int(cap))
        return out[: 4 * n].reshape(n, 4)

    def t3_table(self, ngrid, L, alpha, rel_cut, rec_cut, real_radius, rec_radius):
        out = np.zeros(3 * ngrid ** 3)
        self.lib.oracle_t3_table(C.c_int(ngrid), C.c_double(L), C.c_double(alpha), C.c_double(rel_cut),
                                 C.c_double(rec_cut), C.c_double(real_radius), C.c_double(rec_radius), _d(out))
        return out

    def t3_interp(self, ngrid, L, table, d, order):
        D = np.zeros(3)
        self.lib.oracle_t3_interp(C.c_int(ngrid), C.c_double(L), _d(table), C.c_double(d[0]),
                                  C.c_double(d[1]), C.c_double(d[2]), C.c_int(order), _d(D))
        return D

    def s1r2_table(self, nrho, nz, rho_max, lz, alpha, nmax, mmax):
        out = np.zeros(2 * nrho * nz)
        self.lib.oracle_s1r2_table(C.c_int(nrho), C.c_int(nz), C.c_double(rho_max), C.c_double(lz),
                                   C.c_double(alpha), C.c_int(nmax), C.c_int(mmax), _d(out))
        return out

    def s1r2_pair(self, d, lz, alpha, nmax, mmax):
        F = np.zeros(3)
        self.lib.oracle_s1r2_pair(C.c_double(d[0]), C.c_double(d[1]), C.c_double(d[2]), C.c_double(lz),
                                  C.c_double(alpha), C.c_int(nmax), C.c_int(mmax), _d(F))
        return F

    def s1r2_interp(self, table, nrho, nz, rho_max, lz, d, order):
        D = np.zeros(3)
        self.lib.oracle_s1r2_interp(_d(table), C.c_int(nrho), C.c_int(nz), C.c_double(rho_max),
                                    C.c_double(lz), C.c_double(d[0]), C.c_double(d[1]), C.c_double(d[2]),
                                    C.c_int(order), _d(D))
        return D

    def cyl_table(self, R, lz, size, accuracy):
        out = np.zeros(size)
        self.lib.oracle_cyl_table(C.c_double(R), C.c_double(lz), C.c_int(size), C.c_int(accuracy), _d(out))
        return out


REF_VARIANTS = ("r3", "t3o2", "t3o4", "s1nl", "s1o0", "s1o2", "s1o4", "s1rs", "r3sp", "t3o2sp", "s1nlsp")


def ref_available(variant: str = "r3") -> bool:
    return os.path.exists(os.path.join(REF_DIR, f"libref_{variant}.so"))


class Ref:
    """The reference StePS CPU force path compiled from source (oracle/_ref)."""

    def __init__(self, variant: str, threads: int | None = None):
        so = os.path.join(REF_DIR, f"libref_{variant}.so")
        # RTLD_LOCAL keeps each variant's globals separate.
        self.lib = C.CDLL(so, mode=os.RTLD_LOCAL)
        self.variant = variant
        L = self.lib
        L.ref_errmax.restype = C.c_double
        L.ref_force_softening.restype = C.c_double
        L.ref_force_softening.argtypes = [C.c_double, C.c_double]
        self.lib.ref_set_threads(C.c_int(int(threads or os.cpu_count() or 1)))

    def set_particles(self, x, m, eps):
        x = np.ascontiguousarray(x, dtype=np.float64)
        m = np.ascontiguousarray(m, dtype=np.float64)
        eps = np.ascontiguousarray(eps, dtype=np.float64)
        self.n = m.size
        self.lib.ref_set_particles(C.c_int(m.size), _d(x), _d(m), _d(eps))

    def softening(self, radius):
        out = np.zeros(self.n)
        self.lib.ref_softening(C.c_double(radius), _d(out))
        return out

    def set_velocities(self, v):
        v = np.ascontiguousarray(v, dtype=np.float64)
        assert v.shape == (self.n, 3)
        self.lib.ref_set_velocities(_d(v))

    def set_params(self, is_periodic=0, L=0.0, rsim=0.0, cosmology=0, comoving=0, mius=0.0, h0=0.0, oml=0.0):
        self.lib.ref_set_params(C.c_int(is_periodic), C.c_double(L), C.c_double(rsim), C.c_int(cosmology),
                                C.c_int(comoving), C.c_double(mius), C.c_double(h0), C.c_double(oml))

    def forces(self, id_min=0, id_max=None):
        if id_max is None:
            id_max = self.n - 1
        F = np.zeros((id_max - id_min + 1, 3))
        self.lib.ref_forces(_d(F), C.c_int(id_min), C.c_int(id_max))
        return F

    def forces_full(self):
        self.lib.ref_forces_full()

    def step(self, h):
        self.lib.ref_step(C.c_double(h))

    def errmax(self):
        return self.lib.ref_errmax()

    def state(self):
        x = np.zeros((self.n, 3)); v = np.zeros((self.n, 3)); F = np.zeros((self.n, 3))
        self.lib.ref_get_state(_d(x), _d(v), _d(F))
        return x, v, F

    def force_softening(self, r, b):
        return self.lib.ref_force_softening(float(r), float(b))

    # T^3
    def build_t3_table(self, ngrid, L, alpha, rel_cut, rec_cut, real_radius, rec_radius):
        out = np.zeros(3 * ngrid ** 3)
        self.lib.ref_build_t3_table(C.c_int(ngrid), C.c_double(L), C.c_double(alpha), C.c_double(rel_cut),
                                    C.c_double(rec_cut), C.c_double(real_radius), C.c_double(rec_radius), _d(out))
        return out

    def ewald_space(self, radius):
        cap = 80000
        out = np.zeros(4 * cap, dtype=np.int32)
        last = self.lib.ref_ewald_space(C.c_double(radius), _i(out), C.c_int(cap))
        return out[: 4 * (last + 1)].reshape(last + 1, 4)

    def set_t3_table(self, table, ngrid):
        table = np.ascontiguousarray(table, dtype=np.float64)
        self.lib.ref_set_t3_table(_d(table), C.c_int(ngrid))

    def t3_interp(self, d):
        D = np.zeros(3)
        self.lib.ref_t3_interp(C.c_double(d[0]), C.c_double(d[1]), C.c_double(d[2]), _d(D))
        return D

    # S1xR2
    def cyl_table(self, R, lz, size, accuracy):
        out = np.zeros(size)
        self.lib.ref_cyl_table(C.c_double(R), C.c_double(lz), C.c_int(size), C.c_int(accuracy), _d(out))
        return out

    def set_radial_table(self, tab):
        tab = np.ascontiguousarray(tab, dtype=np.float64)
        self.lib.ref_set_radial_table(_d(tab), C.c_int(tab.size))

    def build_s1r2_table(self, nrho, nz, rho_max, lz, alpha, nmax, mmax):
        out = np.zeros(2 * nrho * nz)
        self.lib.ref_build_s1r2_table(C.c_int(nrho), C.c_int(nz), C.c_double(rho_max), C.c_double(lz),
                                      C.c_double(alpha), C.c_int(nmax), C.c_int(mmax), _d(out))
        return out

    def s1r2_pair(self, d, lz, alpha, nmax, mmax):
        F = np.zeros(3)
        self.lib.ref_s1r2_pair(C.c_double(d[0]), C.c_double(d[1]), C.c_double(d[2]), C.c_double(lz),
                               C.c_double(alpha), C.c_int(nmax), C.c_int(mmax), _d(F))
        return F

    def set_s1r2_table(self, table, nrho, nz):
        table = np.ascontiguousarray(table, dtype=np.float64)
        self.lib.ref_set_s1r2_table(_d(table), C.c_int(nrho), C.c_int(nz))

    def s1r2_interp(self, d):
        D = np.zeros(3)
        self.lib.ref_s1r2_interp(C.c_double(d[0]), C.c_double(d[1]), C.c_double(d[2]), _d(D))
        return D
