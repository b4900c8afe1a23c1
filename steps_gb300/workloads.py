"""Seeded synthetic particle sets for the five benchmark workloads.

There is no public dataset for this path: the inputs are built from seeds
with the shapes, sizes and value distributions of the benchmark workloads.

* compactified R^3 (``r3_compactified``): points uniform on S^3 inside a polar
  cap omega < omega_max, stereographically projected to r = D tan(omega/2);
  masses m ~ (1 + (r/D)^2)^3 (uniform physical density), normalised to a
  total of 1e5 mass units; softening eps_i = 0.05 (m_i/m_min)^(1/3) Mpc, the
  StePS law with PARTICLE_RADII = 0.05 (StePS/src/utils.cc:59-82).
  omega_max follows the StePS_IC example ratio R/D = 930.03/105
  (StePS_IC/examples/LCDM_SP_1860Mpc_Nr224_Nhp32_ds105.yaml,
  omega_max = 2 atan(R/D) as StePS_IC/src/StePS_IC.py:58), so D = R_max/8.857.
  Optional clustering: a Gaussian displacement with sigma = 0.5 x the local
  mean spacing (m_i / rho_mean)^(1/3).
* S^1 x R^2 (``s1r2_cylindrical``): z uniform in [0, L_z); the transverse
  plane is S^2 compactified onto R^2 the same way, masses ~ (1+(rho/D)^2)^2.
* T^3 (``t3_clumpy``): half uniform in the box, half in Gaussian clumps,
  equal masses, constant softening.
* the batched ensemble (``r3_ensemble``): 64 independent compactified R^3
  realisations of uneven N.

All generators use numpy's PCG64 with an explicit seed, so a (workload,
seed) pair always produces the same particles.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

OMEGA_RATIO = 930.03 / 105.0
TOTAL_MASS = 1.0e5
PARTICLE_RADII = 0.05


@dataclass
class ParticleSet:
    """AoS positions x[N,3] (float64), masses m[N], softening eps[N]."""

    x: np.ndarray
    m: np.ndarray
    eps: np.ndarray
    topology: str  # "r3", "t3", "s1r2"
    L: float = 0.0  # box size (t3) or periodic length L_z (s1r2)
    rsim: float = 0.0  # radius of the simulation volume
    meta: dict = field(default_factory=dict)

    @property
    def n(self) -> int:
        return int(self.x.shape[0])


def _softening(m: np.ndarray, radius: float = PARTICLE_RADII) -> np.ndarray:
    return radius * np.cbrt(m / m.min())


def _cap_points(rng: np.random.Generator, n: int, dim: int, omega_max: float) -> np.ndarray:
    """n points uniform on S^(dim-1) with polar angle (from the last axis) < omega_max."""
    out = []
    have = 0
    while have < n:
        g = rng.standard_normal((max(2 * (n - have), 1024), dim))
        u = g / np.linalg.norm(g, axis=1, keepdims=True)
        keep = u[np.arccos(np.clip(u[:, -1], -1.0, 1.0)) < omega_max]
        out.append(keep)
        have += keep.shape[0]
    return np.concatenate(out)[:n]


def r3_compactified(n: int, r_max: float, seed: int, displace: bool = False) -> ParticleSet:
    rng = np.random.default_rng(seed)
    omega_max = 2.0 * math.atan(OMEGA_RATIO)
    D = r_max / OMEGA_RATIO
    u = _cap_points(rng, n, 4, omega_max)
    omega = np.arccos(np.clip(u[:, 3], -1.0, 1.0))
    r = D * np.tan(omega / 2.0)
    d3 = u[:, :3]
    d3 = d3 / np.linalg.norm(d3, axis=1, keepdims=True)
    x = d3 * r[:, None]
    m = (1.0 + (r / D) ** 2) ** 3
    m *= TOTAL_MASS / m.sum()
    if displace:
        rho_mean = TOTAL_MASS / (4.0 / 3.0 * math.pi * r_max ** 3)
        sigma = 0.5 * np.cbrt(m / rho_mean)
        x = x + rng.standard_normal(x.shape) * sigma[:, None]
    eps = _softening(m)
    return ParticleSet(np.ascontiguousarray(x), m, eps, "r3", 0.0, r_max,
                       {"D": D, "omega_max": omega_max, "seed": seed, "displaced": displace})


def s1r2_cylindrical(n: int, lz: float, r_max: float, seed: int) -> ParticleSet:
    rng = np.random.default_rng(seed)
    omega_max = 2.0 * math.atan(OMEGA_RATIO)
    D = r_max / OMEGA_RATIO
    u = _cap_points(rng, n, 3, omega_max)
    omega = np.arccos(np.clip(u[:, 2], -1.0, 1.0))
    rho = D * np.tan(omega / 2.0)
    phi = np.arctan2(u[:, 1], u[:, 0])
    z = rng.uniform(0.0, lz, n)
    x = np.stack([rho * np.cos(phi), rho * np.sin(phi), z], axis=1)
    m = (1.0 + (rho / D) ** 2) ** 2
    m *= TOTAL_MASS / m.sum()
    eps = _softening(m)
    return ParticleSet(np.ascontiguousarray(x), m, eps, "s1r2", lz, r_max,
                       {"D": D, "omega_max": omega_max, "seed": seed})


def t3_clumpy(n: int, box: float, seed: int, n_clumps: int = 512, sigma: float = 0.5,
              eps_const: float = 0.02) -> ParticleSet:
    rng = np.random.default_rng(seed)
    n_uni = n // 2
    n_cl = n - n_uni
    xu = rng.uniform(0.0, box, (n_uni, 3))
    centres = rng.uniform(0.0, box, (n_clumps, 3))
    which = rng.integers(0, n_clumps, n_cl)
    xc = centres[which] + rng.standard_normal((n_cl, 3)) * sigma
    x = np.mod(np.concatenate([xu, xc]), box)
    x[x >= box] -= box
    m = np.full(n, TOTAL_MASS / n)
    eps = np.full(n, eps_const)
    return ParticleSet(np.ascontiguousarray(x), m, eps, "t3", box, 0.5 * box,
                       {"seed": seed, "n_clumps": n_clumps, "sigma": sigma})


def ensemble_sizes(count: int = 64, lo: int = 8192, hi: int = 262144, seed: int = 4):
    """Log-uniform N_k in [lo, hi] rounded to a multiple of 128, R_max ~ U[200, 800]."""
    rng = np.random.default_rng(seed)
    nk = np.exp(rng.uniform(math.log(lo), math.log(hi), count))
    nk = np.clip(np.round(nk / 128.0).astype(np.int64) * 128, 128, None)
    rmax = rng.uniform(200.0, 800.0, count)
    return nk, rmax


def r3_ensemble(count: int = 64, scale: float = 1.0):
    """The batched ensemble: realisation k uses seed k. ``scale`` shrinks every
    N_k (for small parity cases) while keeping the multiple-of-128 rounding."""
    nk, rmax = ensemble_sizes(count)
    sets = []
    for k in range(count):
        n = int(max(128, round(nk[k] * scale / 128.0) * 128))
        sets.append(r3_compactified(n, float(rmax[k]), seed=k, displace=True))
    return sets


# The five benchmark workloads, by name.
def workload(name: str, scale: float = 1.0) -> ParticleSet:
    if name == "cfg0":
        return r3_compactified(int(32768 * scale), 480.0, seed=0)
    if name == "cfg1":
        return r3_compactified(int(1048576 * scale), 1000.0, seed=1, displace=True)
    if name == "cfg2":
        return s1r2_cylindrical(int(2097152 * scale), 200.0, 600.0, seed=2)
    if name == "cfg3":
        return t3_clumpy(int(524288 * scale), 100.0, seed=3)
    raise ValueError(f"unknown workload {name}")
