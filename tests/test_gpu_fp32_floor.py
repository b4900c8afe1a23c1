"""The mixed kernels against the reference's own single-precision build
(USE_SINGLE_PRECISION, REAL = float): on the same inputs, both against the
reference FP64 build, the mixed result must be at least as accurate in p99
and max. Fixture: tests/golden/ref_fp32.npz."""
import pytest

import steps_gb300 as S
from helpers import err_stats, golden
from steps_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def check(ours, theirs, what):
    print(what, "mixed", ours, "reference FP32 build", theirs)
    assert ours["p99"] <= theirs["p99"] and ours["max"] <= theirs["max"], (what, ours, theirs)


def test_r3_n32768(engine):
    g = golden("ref_fp32")
    ps = W.r3_compactified(int(g["r3_n"]), float(g["r3_rmax"]), seed=int(g["r3_seed"]))
    lo, hi = (int(v) for v in g["r3_sub"])
    engine.set_particles(ps.m, ps.eps)
    F = engine.forces(ps.x, S.params(S.R3), S.MIXED)[lo:hi + 1]
    check(err_stats(F, g["r3_F64"]), err_stats(g["r3_F32"], g["r3_F64"]), "R3 N=32768")


def test_t3_trilinear(engine):
    g, f = golden("t3_o2"), golden("ref_fp32")
    L = float(g["L"])
    engine.set_particles(g["m"], g["eps"])
    engine.set_table_t3(g["table"], int(g["ngrid"]))
    F = engine.forces(g["x"], S.params(S.T3, is_periodic=2, L=L, rsim=L / 2, ewald_order=2), S.MIXED)
    check(err_stats(F, g["F"]), err_stats(f["t3o2_F32"], g["F"]), "T3 trilinear")


def test_s1r2_images(engine):
    g, f = golden("s1r2_images"), golden("ref_fp32")
    engine.set_particles(g["m"], g["eps"])
    p = S.params(S.S1R2, is_periodic=2, L=float(g["L"]), rsim=float(g["rsim"]), s1r2_images=1)
    F = engine.forces(g["x"], p, S.MIXED)
    check(err_stats(F, g["F_is2"]), err_stats(f["s1r2_is2_F32"], g["F_is2"]), "S1xR2 images")
