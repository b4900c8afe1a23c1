"""The Ewald tables of the reference's higher precision levels, built on the
GPU and used by the force kernels.

The reference picks the table from IS_PERIODIC (StePS/src/main.cc:416-448 for
T^3, :569-602 for S1xR2):

* T^3 level 3: Ng = 127, rel_cut 3.6, rec_cut 10, over ewald_space(4.6) and
  ewald_space(12); level 4: Ng = 255, rel_cut 4.6, rec_cut 12, over
  ewald_space(5.6) and ewald_space(14); alpha = 2/L in both;
* S1xR2 level 3: Nz = 256, alpha L = 0.71805, cuts 5 / 12; level 4: Nz = 512,
  alpha L = 0.6642, cuts 6 / 13; Nrho = floor(Nz * 2.25 * Rsim / L).

Each case checks the GPU-built table against the oracle's builder, the FP64
kernel against the oracle on that table (<= 1e-12), and the mixed kernel
against the FP64 kernel (p99 <= 1e-5). At Ng = 255 the T^3 kernel's haloed
FP32 copy and stencil records hold (255 + 62)^3 cells, about 2 GB.
"""
import math

import numpy as np
import pyoracle as O
import pytest

import steps_gb300 as S
from helpers import err_stats, port_params, rel_err
from steps_gb300 import workloads as W

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12
# The correction is the difference of lattice sums ~10^3 times larger than
# it; CUDA's and the C library's erfc/exp differ by an ulp or two, which at
# Ng = 127 and 255 moves a few entries by ~1e-12 of max|D|.
TABLE_TOL = 1e-11
MIXED_P99 = 1e-5

T3_LEVELS = {3: (127, 3.6, 10.0), 4: (255, 4.6, 12.0)}
S1_LEVELS = {3: (256, 0.71805, 5, 12), 4: (512, 0.6642, 6, 13)}


@pytest.mark.parametrize("level", [3, 4])
def test_t3_table_levels(engine, port, level):
    ng, rel_cut, rec_cut = T3_LEVELS[level]
    L = 100.0
    args = (ng, L, 2.0 / L, rel_cut, rec_cut, rel_cut + 1.0, rec_cut + 2.0)
    engine.build_table_t3(*args)
    tab = engine.get_table_t3(ng)
    ref = port.t3_table(*args)
    np.testing.assert_allclose(tab, ref, rtol=0, atol=TABLE_TOL * np.abs(ref).max())
    ps = W.t3_clumpy(3000, L, seed=40 + level, n_clumps=12)
    engine.set_particles(ps.m, ps.eps)
    for order in (2, 4):
        p = S.params(S.T3, is_periodic=level, L=L, rsim=L / 2, ewald_order=order)
        F64 = engine.forces(ps.x, p, S.FP64)
        s = port.system(1, ps.m, ps.eps, port_params(O, is_periodic=level, L=L, rsim=L / 2), table=tab, ngrid=ng,
                        order=order)
        Fo = port.forces(s, ps.x, 0, 191)
        assert rel_err(F64[:192], Fo).max() < FP64_TOL, order
        st = err_stats(engine.forces(ps.x, p, S.MIXED), F64)
        assert st["p99"] < MIXED_P99, (level, order, st)


@pytest.mark.parametrize("level", [3, 4])
def test_s1r2_table_levels(engine, port, level):
    nz, alpha_l, nmax, mmax = S1_LEVELS[level]
    L, rsim = 200.0, 600.0
    nrho = int(math.floor(nz * 2.25 * rsim / L))
    args = (nrho, nz, 2.25 * rsim, L, alpha_l / L, nmax, mmax)
    engine.build_table_s1r2(*args)
    tab = engine.get_table_s1r2(nrho, nz)
    ref = port.s1r2_table(*args)
    np.testing.assert_allclose(tab, ref, rtol=0, atol=TABLE_TOL * np.abs(ref).max())
    ps = W.s1r2_cylindrical(4000, L, rsim, seed=50 + level)
    engine.set_particles(ps.m, ps.eps)
    for order in (0, 2, 4):
        p = S.params(S.S1R2, is_periodic=level, L=L, rsim=rsim, s1r2_images=0, ewald_order=order)
        F64 = engine.forces(ps.x, p, S.FP64)
        s = port.system(2, ps.m, ps.eps, port_params(O, is_periodic=level, L=L, rsim=rsim), table=tab, nrho=nrho,
                        nz=nz, order=order)
        Fo = port.forces(s, ps.x, 0, 255)
        assert rel_err(F64[:256], Fo).max() < FP64_TOL, order
        st = err_stats(engine.forces(ps.x, p, S.MIXED), F64)
        assert st["p99"] < MIXED_P99, (level, order, st)
