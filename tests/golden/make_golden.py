"""Generates the golden vectors in tests/golden/ by running the UNMODIFIED
reference StePS CPU force path, compiled from the reference tree into
oracle/_ref (``make -C oracle ref``), on small seeded inputs.

The reference has no tests or fixtures of its own, so these vectors are the
pin: tests/test_oracle_golden.py checks the plain-C oracle against them on any
machine, and the GPU tests check the CUDA kernels against them.

Run from the repository root:  python tests/golden/make_golden.py
(``... make_golden.py fp32`` regenerates only the single-precision floor,
``... make_golden.py background`` only the S1xR2 background-term vectors,
``... make_golden.py rspace`` only the direct-sum S1xR2 table).
"""
from __future__ import annotations

import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import pyoracle as O  # noqa: E402
from steps_gb300 import workloads as W  # noqa: E402

# Small-case Ewald settings (the workload's T3 settings at a coarse grid).
T3_NG = 17  # the reference builder schedules OpenMP chunks of Ngrid/16, so Ngrid >= 16
T3_L = 100.0
T3_ALPHA = 2.0 / T3_L
T3_REL_CUT = 2.0
T3_REC_CUT = 5.0 * 2.0 * math.pi / T3_L
T3_REAL_R = T3_REL_CUT + 1.0
T3_REC_R = 6.0
S1_LZ = 200.0
S1_RSIM = 600.0
S1_NZ = 32
S1_NRHO = int(math.floor(S1_NZ * 2.25 * S1_RSIM / S1_LZ))
S1_ALPHA = 0.787875 / S1_LZ
S1_NMAX, S1_MMAX = 4, 10


def save(name, **arrs):
    path = os.path.join(HERE, name + ".npz")
    np.savez_compressed(path, **arrs)
    print(f"wrote {path} ({os.path.getsize(path)} bytes)")


def main():
    for v in O.REF_VARIANTS:
        if not O.ref_available(v):
            raise SystemExit(f"oracle/_ref/libref_{v}.so missing: run `make -C oracle ref` first")

    # ---- R^3: compactified, two i ranges, three background modes ----
    ps = W.r3_compactified(2048, 480.0, seed=0)
    ref = O.Ref("r3")
    ref.set_particles(ps.x, ps.m, ps.eps)
    eps_ref = ref.softening(W.PARTICLE_RADII)
    ref.set_params()
    F_full = ref.forces()
    F_sub = ref.forces(100, 611)
    ref.set_params(cosmology=1, comoving=1, mius=0.37)
    F_com = ref.forces()
    ref.set_params(cosmology=1, comoving=0, h0=0.07, oml=0.69)
    F_de = ref.forces()
    save("r3_n2048", x=ps.x, m=ps.m, eps=ps.eps, eps_ref=eps_ref, F=F_full, F_sub=F_sub, sub=np.array([100, 611]),
         F_comoving=F_com, mius=np.array(0.37), F_de=F_de, h0=np.array(0.07), oml=np.array(0.69))

    # ---- R^3 KDK: one force then 4 fixed-dt steps from rest (step.cc:100) ----
    ps = W.r3_compactified(1024, 480.0, seed=10)
    ref = O.Ref("r3")
    ref.set_particles(ps.x, ps.m, ps.eps)
    ref.softening(W.PARTICLE_RADII)  # sets M_min and rho_part used by errmax
    ref.set_params()
    ref.forces_full()
    x0, v0, F0 = ref.state()
    for _ in range(4):
        ref.step(1e-3)
    x4, v4, F4 = ref.state()
    m_min = ps.m.min()
    rho_part = m_min / (4.0 * math.pi * W.PARTICLE_RADII ** 3 / 3.0)
    save("r3_kdk4", x=ps.x, m=ps.m, eps=ps.eps, F0=F0, x4=x4, v4=v4, F4=F4, errmax=np.array(ref.errmax()),
         rho_part=np.array(rho_part), dt=np.array(1e-3))

    # ---- T^3: table (reference builder), orders 2 and 4, plus nearest image ----
    ps = W.t3_clumpy(2048, T3_L, seed=3, n_clumps=16)
    for order, var in ((2, "t3o2"), (4, "t3o4")):
        ref = O.Ref(var)
        ref.set_particles(ps.x, ps.m, ps.eps)
        table = ref.build_t3_table(T3_NG, T3_L, T3_ALPHA, T3_REL_CUT, T3_REC_CUT, T3_REAL_R, T3_REC_R)
        ref.set_t3_table(table, T3_NG)
        ref.set_params(is_periodic=2, L=T3_L, rsim=0.5 * T3_L)
        F = ref.forces()
        ref.set_params(is_periodic=1, L=T3_L, rsim=0.5 * T3_L)
        F_near = ref.forces()
        rng = np.random.default_rng(7)
        probes = rng.uniform(-0.5 * T3_L, 0.5 * T3_L, (64, 3))
        ref.set_params(is_periodic=2, L=T3_L, rsim=0.5 * T3_L)
        D = np.array([ref.t3_interp(p) for p in probes])
        save(f"t3_o{order}", x=ps.x, m=ps.m, eps=ps.eps, table=table, ngrid=np.array(T3_NG), L=np.array(T3_L),
             F=F, F_nearest=F_near, probes=probes, D=D,
             ewald=np.array([T3_ALPHA, T3_REL_CUT, T3_REC_CUT, T3_REAL_R, T3_REC_R]))
    # Lattice enumeration of ewald_space() for the index radii used above.
    ref = O.Ref("t3o4")
    save("t3_lattice", real=ref.ewald_space(T3_REAL_R), rec=ref.ewald_space(T3_REC_R),
         radii=np.array([T3_REAL_R, T3_REC_R]))
    # Full-size table of the T^3 workload (Ng = 63): a sample of entries.
    big = ref.build_t3_table(63, T3_L, T3_ALPHA, T3_REL_CUT, T3_REC_CUT, T3_REAL_R, T3_REC_R)
    idx = np.random.default_rng(11).choice(big.size, 4096, replace=False)
    save("t3_table63_sample", idx=idx, val=big[idx], absum=np.array(np.abs(big).sum()), ngrid=np.array(63),
         ewald=np.array([T3_ALPHA, T3_REL_CUT, T3_REC_CUT, T3_REAL_R, T3_REC_R]))

    # ---- S1 x R2: explicit images (IS_PERIODIC 2 and 1), comoving background ----
    ps = W.s1r2_cylindrical(2048, S1_LZ, S1_RSIM, seed=2)
    ref = O.Ref("s1nl")
    ref.set_particles(ps.x, ps.m, ps.eps)
    ref.set_params(is_periodic=2, L=S1_LZ, rsim=S1_RSIM)
    F2 = ref.forces()
    ref.set_params(is_periodic=1, L=S1_LZ, rsim=S1_RSIM)
    F1 = ref.forces()
    ewald_cut = (2 + 1) - 0.4
    radial = ref.cyl_table(S1_RSIM, S1_LZ * ewald_cut, 200, 400)
    ref.set_radial_table(radial)
    ref.set_params(is_periodic=2, L=S1_LZ, rsim=S1_RSIM, cosmology=1, comoving=1, mius=0.011)
    Fc = ref.forces()
    ref.set_params(is_periodic=4, L=S1_LZ, rsim=S1_RSIM)
    F4 = ref.forces(0, 255)
    save("s1r2_images", x=ps.x, m=ps.m, eps=ps.eps, L=np.array(S1_LZ), rsim=np.array(S1_RSIM), F_is2=F2, F_is1=F1,
         radial=radial, mius=np.array(0.011), F_comoving=Fc, F_is4_head=F4)

    # ---- S1 x R2: (rho, z) table (reference builder), orders 0/2/4 ----
    for order, var in ((0, "s1o0"), (2, "s1o2"), (4, "s1o4")):
        ref = O.Ref(var)
        ref.set_particles(ps.x, ps.m, ps.eps)
        table = ref.build_s1r2_table(S1_NRHO, S1_NZ, 2.25 * S1_RSIM, S1_LZ, S1_ALPHA, S1_NMAX, S1_MMAX)
        ref.set_s1r2_table(table, S1_NRHO, S1_NZ)
        ref.set_params(is_periodic=2, L=S1_LZ, rsim=S1_RSIM)
        F = ref.forces()
        rng = np.random.default_rng(8)
        probes = np.stack([rng.uniform(-700, 700, 64), rng.uniform(-700, 700, 64), rng.uniform(-100, 100, 64)], 1)
        D = np.array([ref.s1r2_interp(p) for p in probes])
        pair = np.array([ref.s1r2_pair(p, S1_LZ, S1_ALPHA, S1_NMAX, S1_MMAX) for p in probes[:16]])
        save(f"s1r2_table_o{order}", x=ps.x, m=ps.m, eps=ps.eps, table=table, shape=np.array([S1_NRHO, S1_NZ]),
             L=np.array(S1_LZ), rsim=np.array(S1_RSIM), F=F, probes=probes, D=D, pair=pair,
             ewald=np.array([S1_ALPHA, S1_NMAX, S1_MMAX]))

    # ---- spline softening kernel on a grid of r/beta ----
    ref = O.Ref("r3")
    rs = np.concatenate([np.linspace(0.0, 2.0, 401), [0.5, 1.0, 0.5 - 1e-12, 1.0 - 1e-12]])
    w = np.array([ref.force_softening(r, 1.0) for r in rs])
    w2 = np.array([ref.force_softening(r * 0.37, 0.37) for r in rs])
    save("softening", r=rs, w_beta1=w, w_beta037=w2)


def s1_background():
    """The S1xR2 background terms the other vectors leave out, on the inputs of
    s1r2_images.npz: the comoving term with the radial correction at
    IS_PERIODIC = 1 (StePS/src/forces.cc:1383-1390), the non-comoving H0^2
    Omega_L x term (forces.cc:1298-1303), and the table mode's plain
    mass_in_unit_sphere x (forces.cc:1340-1344) with its H0^2 Omega_L twin."""
    g = np.load(os.path.join(HERE, "s1r2_images.npz"))
    t = np.load(os.path.join(HERE, "s1r2_table_o2.npz"))
    mius, h0, oml = 0.011, 0.07, 0.69
    ref = O.Ref("s1nl")
    ref.set_particles(g["x"], g["m"], g["eps"])
    ref.set_radial_table(g["radial"])
    ref.set_params(is_periodic=1, L=S1_LZ, rsim=S1_RSIM, cosmology=1, comoving=1, mius=mius)
    F_is1_comoving = ref.forces()
    ref.set_params(is_periodic=2, L=S1_LZ, rsim=S1_RSIM, cosmology=1, comoving=0, h0=h0, oml=oml)
    F_is2_de = ref.forces()
    ref = O.Ref("s1o2")
    ref.set_particles(t["x"], t["m"], t["eps"])
    ref.set_s1r2_table(t["table"], S1_NRHO, S1_NZ)
    ref.set_radial_table(g["radial"])
    ref.set_params(is_periodic=2, L=S1_LZ, rsim=S1_RSIM, cosmology=1, comoving=1, mius=mius)
    F_table_comoving = ref.forces()
    ref.set_params(is_periodic=2, L=S1_LZ, rsim=S1_RSIM, cosmology=1, comoving=0, h0=h0, oml=oml)
    F_table_de = ref.forces()
    save("s1r2_background", mius=np.array(mius), h0=np.array(h0), oml=np.array(oml), F_is1_comoving=F_is1_comoving,
         F_is2_de=F_is2_de, F_table_comoving=F_table_comoving, F_table_de=F_table_de)


def fp32_floor():
    """The reference's own single-precision build (USE_SINGLE_PRECISION) on the
    same inputs as its FP64 build: the error floor of the reference's FP32 path
    that the mixed kernels are compared with."""
    # R^3: the N = 32,768 compactified workload (regenerated from its seed on
    # any machine), i range [16128, 16640) against all j.
    ps = W.r3_compactified(32768, 480.0, seed=0)
    lo, hi = 16128, 16639
    out = {}
    for var in ("r3", "r3sp"):
        ref = O.Ref(var)
        ref.set_particles(ps.x, ps.m, ps.eps)
        ref.set_params()
        out[var] = ref.forces(lo, hi)
    # T^3 trilinear and the S1xR2 image sum on the golden inputs.
    g = np.load(os.path.join(HERE, "t3_o2.npz"))
    ref = O.Ref("t3o2sp")
    ref.set_particles(g["x"], g["m"], g["eps"])
    ref.set_t3_table(g["table"], int(g["ngrid"]))
    ref.set_params(is_periodic=2, L=float(g["L"]), rsim=float(g["L"]) / 2)
    t3sp = ref.forces()
    g = np.load(os.path.join(HERE, "s1r2_images.npz"))
    ref = O.Ref("s1nlsp")
    ref.set_particles(g["x"], g["m"], g["eps"])
    ref.set_params(is_periodic=2, L=float(g["L"]), rsim=float(g["rsim"]))
    s1sp = ref.forces()
    save("ref_fp32", r3_n=np.array(32768), r3_rmax=np.array(480.0), r3_seed=np.array(0), r3_sub=np.array([lo, hi]),
         r3_F64=out["r3"], r3_F32=out["r3sp"], t3o2_F32=t3sp, s1r2_is2_F32=s1sp)


def s1_rspace():
    """The (rho, z) table of the reference's PERIODIC_Z_RSPACELOOKUP build:
    direct real-space image sums, no k-space part (StePS/src/ewald_space.cc:
    710-750), with the arguments that build passes (alpha = 0, mmax = 0,
    StePS/src/main.cc:650) at a small grid and 1000 images per side (the
    IS_PERIODIC = 2 setting, main.cc:608)."""
    nz = 16
    nrho = int(math.floor(nz * 2.25 * S1_RSIM / S1_LZ))
    table = O.Ref("s1rs").build_s1r2_table(nrho, nz, 2.25 * S1_RSIM, S1_LZ, 0.0, 1000, 0)
    save("s1r2_table_rspace", table=table, shape=np.array([nrho, nz]), L=np.array(S1_LZ), rsim=np.array(S1_RSIM),
         nmax=np.array(1000))


if __name__ == "__main__":
    if sys.argv[1:] == ["fp32"]:
        fp32_floor()
    elif sys.argv[1:] == ["background"]:
        s1_background()
    elif sys.argv[1:] == ["rspace"]:
        s1_rspace()
    else:
        main()
        fp32_floor()
        s1_background()
        s1_rspace()
