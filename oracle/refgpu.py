"""The reference's own CUDA force kernels, launched the way the reference
launches them. TEST AND BENCHMARK INFRASTRUCTURE: never imported by the
product; only tests/ and the reference arm of bench.py use it.

`make -C oracle refgpu` compiles StePS/src/forces_cuda.cu unmodified (device
code only, sm_103a) into oracle/_ref/forces_cuda_<variant>.cubin, one cubin
per topology flag set and REAL type (oracle/Makefile). This module loads a
cubin through the CUDA driver API into the primary context that PyTorch
uses, and launches its kernel with the reference's shape: 32 x (SM count)
blocks of 256 threads and a grid-stride i loop of stride
n = 32 x SMs x 256 (StePS/src/forces_cuda.cu:1053, :1620-1625).

Kernels, with the signatures StePS/src/forces_cuda.cu declares:
  ForceKernel             forces_cuda.cu:522  R^3
  ForceKernel_periodic    forces_cuda.cu:567  T^3: nearest image; with
                          IS_PERIODIC >= 2 the tricubic Ewald correction
                          (forces_cuda.cu:113-167) whatever the CPU order
  ForceKernel_periodic_z  forces_cuda.cu:652  S1xR2 z-image sum
                          (PERIODIC_Z_NOLOOKUP)
  ForceKernel_periodic_z  forces_cuda.cu:764  S1xR2 nearest z image and the
                          (rho, z) correction table, NGP / CIC / TSC by
                          EWALD_INTERPOLATION_ORDER 0 / 2 / 4
                          (forces_cuda.cu:180-442), rho_max = 2.25 Rsim
Each reads x, M and SOFT_LENGTH as separate REAL arrays, computes the i in
[ID_min, ID_max] against the j in [0, N) and ADDS into F[3 (i - ID_min) + k]
(the reference's host wrapper uploads a zeroed F first, forces_cuda.cu:1045).
Passing N smaller than the particle count restricts j to the first N
particles: a smaller system, which the timing uses as a bounded sample.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")
BLOCKSIZE = 256  # StePS/src/forces_cuda.cu:25
BLOCKS_PER_SM = 32  # the grid is 32 x SMs blocks, forces_cuda.cu:1053

# variant -> (topology, REAL type code of the Itanium C++ ABI)
VARIANTS = {"r3": ("R3", "d"), "r3sp": ("R3", "f"), "t3": ("T3", "d"), "t3sp": ("T3", "f"),
            "s1nl": ("S1", "d"), "s1nlsp": ("S1", "f"),
            "s1o0": ("S1T", "d"), "s1o2": ("S1T", "d"), "s1o4": ("S1T", "d"),
            "s1o0sp": ("S1T", "f"), "s1o2sp": ("S1T", "f"), "s1o4sp": ("S1T", "f")}
# EWALD_LOOKUP_TABLE_RADIAL_EXTENT_FACTOR (StePS/src/global_variables.h:39)
S1_RHO_EXTENT = 2.25


def cubin_path(variant: str) -> str:
    return os.path.join(REF_DIR, f"forces_cuda_{variant}.cubin")


def available(variant: str = "r3") -> bool:
    return os.path.isfile(cubin_path(variant))


def kernel_name(topology: str, t: str) -> str:
    """Mangled (Itanium C++ ABI) name of the reference kernel with REAL = t:
    the parameter lists of forces_cuda.cu:522, :567, :652 and :764 (size_t
    is unsigned long, m)."""
    if topology == "R3":
        return f"_Z11ForceKerneliiPK{t}S0_S0_P{t}S0_S0_{t}{t}iiii"
    if topology == "T3":
        return f"_Z20ForceKernel_periodiciiPK{t}S0_S0_P{t}iS0_S0_{t}S0_iii"
    if topology == "S1T":
        return f"_Z22ForceKernel_periodic_ziiPK{t}S0_S0_P{t}iS0_S0_{t}{t}{t}S0_iS0_mm{t}iiii"
    return f"_Z22ForceKernel_periodic_ziiPK{t}S0_S0_P{t}iS0_S0_{t}{t}{t}S0_{t}{t}iiii"


_cu = None


def _driver():
    global _cu
    if _cu is None:
        cu = C.CDLL("libcuda.so.1")
        cu.cuLaunchKernel.argtypes = [C.c_void_p, C.c_uint, C.c_uint, C.c_uint, C.c_uint, C.c_uint, C.c_uint,
                                      C.c_uint, C.c_void_p, C.POINTER(C.c_void_p), C.POINTER(C.c_void_p)]
        cu.cuModuleGetFunction.argtypes = [C.POINTER(C.c_void_p), C.c_void_p, C.c_char_p]
        cu.cuModuleLoad.argtypes = [C.POINTER(C.c_void_p), C.c_char_p]
        cu.cuOccupancyMaxActiveBlocksPerMultiprocessor.argtypes = [C.POINTER(C.c_int), C.c_void_p, C.c_int,
                                                                   C.c_size_t]
        cu.cuFuncGetAttribute.argtypes = [C.POINTER(C.c_int), C.c_int, C.c_void_p]
        cu.cuGetErrorString.argtypes = [C.c_int, C.POINTER(C.c_char_p)]
        _cu = cu
    return _cu


def _check(rc: int, what: str):
    if rc != 0:
        s = C.c_char_p()
        _driver().cuGetErrorString(rc, C.byref(s))
        raise RuntimeError(f"{what}: CUDA driver error {rc} ({s.value.decode() if s.value else 'unknown'})")


class RefKernel:
    """One reference kernel (variant of VARIANTS) on one device, with the
    particle arrays resident as the reference keeps them (SoA REAL)."""

    def __init__(self, variant: str, device: int = 0):
        import torch

        if variant not in VARIANTS:
            raise ValueError(f"unknown reference kernel variant {variant!r}")
        path = cubin_path(variant)
        if not os.path.isfile(path):
            raise FileNotFoundError(f"{path} is not built (make -C oracle refgpu, where the reference tree is)")
        self.variant = variant
        self.topology, t = VARIANTS[variant]
        self.torch = torch
        self.device = torch.device("cuda", device)
        torch.cuda.set_device(self.device)
        torch.zeros(1, device=self.device)  # creates the primary context
        cu = _driver()
        _check(cu.cuInit(0), "cuInit")
        dev = C.c_int()
        _check(cu.cuDeviceGet(C.byref(dev), device), "cuDeviceGet")
        self._ctx = C.c_void_p()
        _check(cu.cuDevicePrimaryCtxRetain(C.byref(self._ctx), dev), "cuDevicePrimaryCtxRetain")
        _check(cu.cuCtxSetCurrent(self._ctx), "cuCtxSetCurrent")
        self._mod = C.c_void_p()
        _check(cu.cuModuleLoad(C.byref(self._mod), path.encode()), f"cuModuleLoad {path}")
        self._fn = C.c_void_p()
        name = kernel_name(self.topology, t)
        _check(cu.cuModuleGetFunction(C.byref(self._fn), self._mod, name.encode()), f"cuModuleGetFunction {name}")
        self.real = C.c_double if t == "d" else C.c_float
        self.dtype = torch.float64 if t == "d" else torch.float32
        self.sms = torch.cuda.get_device_properties(self.device).multi_processor_count
        self.grid = BLOCKS_PER_SM * self.sms
        self.stride = self.grid * BLOCKSIZE
        nb = C.c_int()
        _check(cu.cuOccupancyMaxActiveBlocksPerMultiprocessor(C.byref(nb), self._fn, BLOCKSIZE, 0), "occupancy")
        self.blocks_per_sm = nb.value
        regs = C.c_int()
        _check(cu.cuFuncGetAttribute(C.byref(regs), 4, self._fn), "cuFuncGetAttribute")  # NUM_REGS
        self.registers = regs.value
        self.n = 0
        self._table = torch.zeros(1, dtype=self.dtype, device=self.device)
        self._ngrid = 0

    def wave(self) -> int:
        """i particles of one full wave of resident blocks."""
        return self.sms * max(self.blocks_per_sm, 1) * BLOCKSIZE

    def set_particles(self, x, m, eps):
        x = np.ascontiguousarray(x, dtype=np.float64).reshape(-1, 3)
        n = x.shape[0]
        if np.shape(m) != (n,) or np.shape(eps) != (n,):
            raise ValueError("x, m and eps disagree on N")
        to = lambda a: self.torch.as_tensor(np.ascontiguousarray(a), device=self.device).to(self.dtype).contiguous()
        self.xx, self.xy, self.xz = to(x[:, 0]), to(x[:, 1]), to(x[:, 2])
        self.m, self.eps = to(m), to(eps)
        self.n = n

    def set_table_t3(self, table, ngrid: int):
        table = np.asarray(table, dtype=np.float64).ravel()
        if table.size != ngrid ** 3 * 3:
            raise ValueError("T^3 table must hold ngrid^3 x 3 values")
        self._table = self.torch.as_tensor(table, device=self.device).to(self.dtype).contiguous()
        self._ngrid = ngrid

    def set_table_s1r2(self, table, nrho: int, nz: int):
        """The (rho, z) table as the reference stores it, nrho x nz x 2, over
        rho in [0, 2.25 Rsim] (the Rsim passed at launch)."""
        table = np.asarray(table, dtype=np.float64).ravel()
        if nrho < 2 or nz < 1 or table.size != nrho * nz * 2:
            raise ValueError("S1xR2 table must hold nrho x nz x 2 values, nrho >= 2")
        self._table = self.torch.as_tensor(table, device=self.device).to(self.dtype).contiguous()
        self._nrho, self._nz = nrho, nz

    def _args(self, F, id_min, id_max, nj, is_periodic, L, rsim, mius, de, cosmology, comoving):
        R, I, P = self.real, C.c_int, C.c_void_p
        head = [I(self.stride), I(nj), P(self.xx.data_ptr()), P(self.xy.data_ptr()), P(self.xz.data_ptr()),
                P(F.data_ptr())]
        if self.topology == "R3":
            vals = head + [P(self.m.data_ptr()), P(self.eps.data_ptr()), R(mius), R(de), I(cosmology), I(comoving),
                           I(id_min), I(id_max)]
        elif self.topology == "T3":
            if is_periodic >= 2 and self._ngrid <= 0:
                raise ValueError("the T^3 kernel with IS_PERIODIC >= 2 needs an Ewald table")
            vals = head + [I(is_periodic), P(self.m.data_ptr()), P(self.eps.data_ptr()), R(L),
                           P(self._table.data_ptr()), I(self._ngrid), I(id_min), I(id_max)]
        elif self.topology == "S1T":
            if is_periodic >= 2 and getattr(self, "_nrho", 0) <= 0:
                raise ValueError("the S1xR2 table kernel with IS_PERIODIC >= 2 needs a (rho, z) table")
            if cosmology:
                raise ValueError("the cylindrical background table is not wired for the reference S1xR2 kernel")
            vals = head + [I(is_periodic), P(self.m.data_ptr()), P(self.eps.data_ptr()), R(L), R(rsim), R(mius),
                           P(self._table.data_ptr()), I(1), P(self._table.data_ptr()),
                           C.c_size_t(getattr(self, "_nrho", 0)), C.c_size_t(getattr(self, "_nz", 0)), R(de),
                           I(cosmology), I(comoving), I(id_min), I(id_max)]
        else:
            if cosmology:
                raise ValueError("the cylindrical background table is not wired for the reference S1xR2 kernel")
            # RADIAL_FORCE_TABLE is read only with COSMOLOGY = 1; a valid one-entry array is passed.
            vals = head + [I(is_periodic), P(self.m.data_ptr()), P(self.eps.data_ptr()), R(L), R(rsim), R(mius),
                           P(self._table.data_ptr()), R(1.0), R(de), I(cosmology), I(comoving), I(id_min),
                           I(id_max)]
        ptrs = (C.c_void_p * len(vals))(*[C.cast(C.pointer(v), C.c_void_p) for v in vals])
        return vals, ptrs

    def launch(self, F, id_min: int, id_max: int, nj: int | None = None, *, is_periodic=0, L=0.0, rsim=0.0,
               mius=0.0, de=0.0, cosmology=0, comoving=0):
        """Adds the forces of i in [id_min, id_max] from j in [0, nj) into the
        device array F (3 (id_max - id_min + 1) REAL), on torch's current stream."""
        nj = self.n if nj is None else nj
        if not (0 <= id_min <= id_max < self.n) or not (1 <= nj <= self.n):
            raise ValueError(f"i range [{id_min}, {id_max}] / j count {nj} outside N = {self.n}")
        if F.dtype != self.dtype or F.device != self.device or F.numel() < 3 * (id_max - id_min + 1):
            raise ValueError("F must be a device REAL array of 3 (id_max - id_min + 1) values")
        keep, ptrs = self._args(F, id_min, id_max, nj, is_periodic, L, rsim, mius, de, cosmology, comoving)
        stream = self.torch.cuda.current_stream(self.device).cuda_stream
        _check(_driver().cuLaunchKernel(self._fn, self.grid, 1, 1, BLOCKSIZE, 1, 1, 0, C.c_void_p(stream), ptrs,
                                        None), "cuLaunchKernel")
        del keep

    def forces(self, id_min: int = 0, id_max: int | None = None, nj: int | None = None, **params) -> np.ndarray:
        """F (ni, 3) float64 of i in [id_min, id_max], as the reference's
        wrapper returns it: zeroed, added into, copied back."""
        id_max = self.n - 1 if id_max is None else id_max
        F = self.torch.zeros(3 * (id_max - id_min + 1), dtype=self.dtype, device=self.device)
        self.launch(F, id_min, id_max, nj, **params)
        self.torch.cuda.synchronize(self.device)
        return F.double().cpu().numpy().reshape(-1, 3)

    def time(self, id_min: int, id_max: int, nj: int, steps: int = 3, warmup: int = 1, **params):
        """Median kernel time in ms over `steps` launches (CUDA events on the
        launching stream, F zeroed before each launch outside the events)."""
        torch = self.torch
        F = torch.zeros(3 * (id_max - id_min + 1), dtype=self.dtype, device=self.device)
        for _ in range(warmup):
            F.zero_()
            self.launch(F, id_min, id_max, nj, **params)
        torch.cuda.synchronize(self.device)
        ms = []
        for _ in range(steps):
            F.zero_()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            self.launch(F, id_min, id_max, nj, **params)
            b.record()
            b.synchronize()
            ms.append(a.elapsed_time(b))
        return float(np.median(ms)), F.double().cpu().numpy().reshape(-1, 3)
