"""S1xR2 and T^3 forces and Ewald tables on the GPU through the C-ABI,
against the reference's golden vectors and the plain-C oracle."""
import math
import os

import numpy as np
import pyoracle as O
import pytest

import steps_gb300 as S
from helpers import GOLDEN, err_stats, golden, port_params, rel_err
from steps_gb300 import workloads as W

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12
MIXED_P99 = 1e-5


def s1_params(g, isp=2, images=1, order=4, **kw):
    return S.params(S.S1R2, is_periodic=isp, L=float(g["L"]), rsim=float(g["rsim"]), s1r2_images=images,
                    ewald_order=order, **kw)


def test_s1r2_images_fp64(engine):
    g = golden("s1r2_images")
    engine.set_particles(g["m"], g["eps"])
    assert rel_err(engine.forces(g["x"], s1_params(g, 2), S.FP64), g["F_is2"]).max() < FP64_TOL
    assert rel_err(engine.forces(g["x"], s1_params(g, 1), S.FP64), g["F_is1"]).max() < FP64_TOL
    assert rel_err(engine.forces(g["x"], s1_params(g, 4), S.FP64, 0, 255), g["F_is4_head"]).max() < FP64_TOL
    engine.set_radial_table(g["radial"])
    p = s1_params(g, 2, cosmology=1, comoving=1, mius=float(g["mius"]))
    assert rel_err(engine.forces(g["x"], p, S.FP64), g["F_comoving"]).max() < FP64_TOL


def test_s1r2_images_mixed(engine):
    g = golden("s1r2_images")
    engine.set_particles(g["m"], g["eps"])
    for isp, key in ((2, "F_is2"), (1, "F_is1")):
        st = err_stats(engine.forces(g["x"], s1_params(g, isp), S.MIXED), g[key])
        assert st["p99"] < MIXED_P99, (isp, st)
    st = err_stats(engine.forces(g["x"], s1_params(g, 4), S.MIXED, 0, 255), g["F_is4_head"])
    assert st["p99"] < MIXED_P99, st
    engine.set_radial_table(g["radial"])
    p = s1_params(g, 2, cosmology=1, comoving=1, mius=float(g["mius"]))
    assert err_stats(engine.forces(g["x"], p, S.MIXED), g["F_comoving"])["p99"] < MIXED_P99


@pytest.mark.parametrize("key", ["F_is1_comoving", "F_is2_de", "F_table_comoving", "F_table_de"])
def test_s1r2_background_terms(engine, key):
    """Comoving with the radial correction at IS_PERIODIC = 1, non-comoving
    H0^2 Omega_L x (image sum and table), and the table mode's plain
    mass_in_unit_sphere x, against the reference's golden vectors."""
    g, b, t = golden("s1r2_images"), golden("s1r2_background"), golden("s1r2_table_o2")
    cosmo = dict(cosmology=1, comoving=1, mius=float(b["mius"])) if key.endswith("comoving") else \
        dict(cosmology=1, comoving=0, h0=float(b["h0"]), oml=float(b["oml"]))
    engine.set_particles(g["m"], g["eps"])
    engine.set_radial_table(g["radial"])
    if key.startswith("F_table"):
        nrho, nz = (int(v) for v in t["shape"])
        engine.set_table_s1r2(t["table"], nrho, nz)
        p = s1_params(g, 2, images=0, order=2, **cosmo)
    else:
        p = s1_params(g, 1 if key == "F_is1_comoving" else 2, **cosmo)
    assert rel_err(engine.forces(g["x"], p, S.FP64), b[key]).max() < FP64_TOL
    assert err_stats(engine.forces(g["x"], p, S.MIXED), b[key])["p99"] < MIXED_P99


@pytest.mark.parametrize("isp", [3, 15])
def test_s1r2_other_image_counts(engine, port, isp):
    ps = W.s1r2_cylindrical(3000, 200.0, 600.0, seed=20 + isp)
    engine.set_particles(ps.m, ps.eps)
    s = port.system(3, ps.m, ps.eps, port_params(O, is_periodic=isp, L=200.0, rsim=600.0))
    Fo = port.forces(s, ps.x, 0, 511)
    p = S.params(S.S1R2, is_periodic=isp, L=200.0, rsim=600.0, s1r2_images=1)
    assert rel_err(engine.forces(ps.x, p, S.FP64, 0, 511), Fo).max() < FP64_TOL
    assert err_stats(engine.forces(ps.x, p, S.MIXED, 0, 511), Fo)["p99"] < MIXED_P99


def test_s1r2_images_mixed_large(engine):
    """The S1xR2 workload's geometry at N = 2^18: at this density some pairs
    sit within FP32 rounding of the image cut |dz + mL| = 2.6 L; mixed must
    still agree with FP64 (full-range mixed against an FP64 i subset)."""
    ps = W.s1r2_cylindrical(1 << 18, 200.0, 600.0, seed=12)
    engine.set_particles(ps.m, ps.eps)
    p = S.params(S.S1R2, is_periodic=2, L=200.0, rsim=600.0, s1r2_images=1)
    Fm = engine.forces(ps.x, p, S.MIXED)
    lo, hi = 100000, 100767
    F64 = engine.forces(ps.x, p, S.FP64, lo, hi)
    st = err_stats(Fm[lo:hi + 1], F64)
    assert st["p99"] < MIXED_P99, st


def test_s1r2_many_images_mixed(engine):
    """IS_PERIODIC = 15 (33 images, the cylindrical example's setting): the
    runtime image loop of the far path and its per-pair cut tests, full range
    against an FP64 i subset."""
    ps = W.s1r2_cylindrical(1 << 16, 100.0, 1000.0, seed=14)
    engine.set_particles(ps.m, ps.eps)
    p = S.params(S.S1R2, is_periodic=15, L=100.0, rsim=1000.0, s1r2_images=1)
    Fm = engine.forces(ps.x, p, S.MIXED)
    lo, hi = 30000, 30767
    st = err_stats(Fm[lo:hi + 1], engine.forces(ps.x, p, S.FP64, lo, hi))
    assert st["p99"] < MIXED_P99, st


@pytest.mark.parametrize("order", [0, 2, 4])
def test_s1r2_table_fp64(engine, order):
    g = golden(f"s1r2_table_o{order}")
    nrho, nz = (int(v) for v in g["shape"])
    engine.set_particles(g["m"], g["eps"])
    engine.set_table_s1r2(g["table"], nrho, nz)
    F = engine.forces(g["x"], s1_params(g, 2, images=0, order=order), S.FP64)
    assert rel_err(F, g["F"]).max() < FP64_TOL


@pytest.mark.parametrize("order", [0, 2, 4])
def test_s1r2_table_mixed(engine, order):
    """The (rho, z) table mode in mixed precision against the reference, every
    kernel shape, full range and an i subset."""
    g = golden(f"s1r2_table_o{order}")
    nrho, nz = (int(v) for v in g["shape"])
    engine.set_particles(g["m"], g["eps"])
    engine.set_table_s1r2(g["table"], nrho, nz)
    p = s1_params(g, 2, images=0, order=order)
    try:
        for threads, ipt in ((64, 1), (64, 2), (128, 1), (128, 2), (256, 1)):
            engine.set_tuning(threads, ipt, 0)
            st = err_stats(engine.forces(g["x"], p, S.MIXED), g["F"])
            assert st["p99"] < MIXED_P99, (order, threads, ipt, st)
    finally:
        engine.set_tuning(128, 2, 0)
    st = err_stats(engine.forces(g["x"], p, S.MIXED, 500, 1200), g["F"][500:1201])
    assert st["p99"] < MIXED_P99, st


def test_s1r2_table_builder(engine):
    g = golden("s1r2_table_o2")
    nrho, nz = (int(v) for v in g["shape"])
    alpha, nmax, mmax = g["ewald"]
    engine.build_table_s1r2(nrho, nz, 2.25 * float(g["rsim"]), float(g["L"]), float(alpha), int(nmax), int(mmax))
    tab = engine.get_table_s1r2()
    np.testing.assert_allclose(tab, g["table"], rtol=0, atol=1e-12 * np.abs(g["table"]).max())


def test_s1r2_table_builder_direct_sum(engine):
    """alpha = 0 and mmax = 0 (what the reference's PERIODIC_Z_RSPACELOOKUP
    build passes) build the table from direct real-space image sums in the
    reference's order: IEEE-exact operations only, so equal to its table."""
    g = golden("s1r2_table_rspace")
    nrho, nz = (int(v) for v in g["shape"])
    engine.build_table_s1r2(nrho, nz, 2.25 * float(g["rsim"]), float(g["L"]), 0.0, int(g["nmax"]), 0)
    tab = engine.get_table_s1r2()
    np.testing.assert_allclose(tab, g["table"], rtol=0, atol=1e-15 * np.abs(g["table"]).max())


@pytest.mark.parametrize("order", [2, 4])
def test_t3_fp64(engine, order):
    g = golden(f"t3_o{order}")
    ng, L = int(g["ngrid"]), float(g["L"])
    engine.set_particles(g["m"], g["eps"])
    engine.set_table_t3(g["table"], ng)
    p = S.params(S.T3, is_periodic=2, L=L, rsim=L / 2, ewald_order=order)
    assert rel_err(engine.forces(g["x"], p, S.FP64), g["F"]).max() < FP64_TOL
    p = S.params(S.T3, is_periodic=1, L=L, rsim=L / 2, ewald_order=order)
    assert rel_err(engine.forces(g["x"], p, S.FP64), g["F_nearest"]).max() < FP64_TOL


def test_t3_table_builder(engine):
    g = golden("t3_o4")
    ng, L = int(g["ngrid"]), float(g["L"])
    engine.build_table_t3(ng, L, *[float(v) for v in g["ewald"]])
    tab = engine.get_table_t3()
    np.testing.assert_allclose(tab, g["table"], rtol=0, atol=1e-13 * np.abs(g["table"]).max())
    g = golden("t3_table63_sample")
    engine.build_table_t3(63, 100.0, *[float(v) for v in g["ewald"]])
    tab = engine.get_table_t3()
    np.testing.assert_allclose(tab[g["idx"]], g["val"], rtol=0, atol=1e-13 * np.abs(g["val"]).max())
    # odd symmetry D(-r) = -D(r) of the table (StePS/src/ewald_space.cc:365-376)
    t = tab.reshape(63, 63, 63, 3)
    np.testing.assert_array_equal(t[::-1, ::-1, ::-1], -t)


def test_t3_lattice_forces_vanish(engine):
    g = golden("t3_o4")
    ng, L = int(g["ngrid"]), float(g["L"])
    k = 5
    c = (np.arange(k) + 0.5) * L / k
    x = np.stack(np.meshgrid(c, c, c, indexing="ij"), -1).reshape(-1, 3)
    n = x.shape[0]
    engine.set_particles(np.full(n, 1.0), np.full(n, 0.02))
    engine.set_table_t3(g["table"], ng)
    F = engine.forces(x, S.params(S.T3, is_periodic=2, L=L, rsim=L / 2, ewald_order=4), S.FP64)
    assert np.abs(F).max() < 1e-12 * (n / (0.2 * L) ** 2)


def test_table_errors(engine):
    g = golden("t3_o4")
    engine.set_particles(g["m"], g["eps"])
    with pytest.raises(S.StepsError) as e:
        engine.build_table_t3(16, 100.0, 0.02, 2.0, 0.3, 3.0, 6.0)  # even grid
    assert e.value.code == S.STEPS_E_ARG
    with pytest.raises(S.StepsError) as e:
        engine.forces(g["x"], S.params(S.T3, is_periodic=2, L=100.0, ewald_order=3), S.FP64)
    assert e.value.code == S.STEPS_E_ARG


@pytest.mark.parametrize("order", [2, 4])
def test_t3_mixed(engine, order):
    g = golden(f"t3_o{order}")
    ng, L = int(g["ngrid"]), float(g["L"])
    engine.set_particles(g["m"], g["eps"])
    engine.set_table_t3(g["table"], ng)
    p = S.params(S.T3, is_periodic=2, L=L, rsim=L / 2, ewald_order=order)
    st = err_stats(engine.forces(g["x"], p, S.MIXED), g["F"])
    assert st["p99"] < MIXED_P99, st
    st = err_stats(engine.forces(g["x"], p, S.MIXED, 300, 1000), g["F"][300:1001])
    assert st["p99"] < MIXED_P99, st
    p = S.params(S.T3, is_periodic=1, L=L, rsim=L / 2, ewald_order=order)
    st = err_stats(engine.forces(g["x"], p, S.MIXED), g["F_nearest"])
    assert st["p99"] < MIXED_P99, st


@pytest.mark.parametrize("order", [2, 4])
def test_t3_mixed_shapes_and_workload_table(engine, port, order):
    """The T^3 workload's own table (Ng = 63, built on the GPU) on a clumpy
    set: every kernel shape against the FP64 kernel, with the window fallback
    exercised by the larger tiles."""
    g = golden("t3_table63_sample")
    ps = W.t3_clumpy(6000, 100.0, seed=31, n_clumps=24)
    engine.set_particles(ps.m, ps.eps)
    engine.build_table_t3(63, 100.0, *[float(v) for v in g["ewald"]])
    p = S.params(S.T3, is_periodic=2, L=100.0, rsim=50.0, ewald_order=order)
    F64 = engine.forces(ps.x, p, S.FP64)
    tab = engine.get_table_t3(63)
    s = port.system(1, ps.m, ps.eps, port_params(O, is_periodic=2, L=100.0, rsim=50.0), table=tab, ngrid=63,
                    order=order)
    Fo = port.forces(s, ps.x, 0, 255)
    assert rel_err(F64[:256], Fo).max() < FP64_TOL
    try:
        # table reads: haloed copy / wrapped (tile pairs wider than the halo) /
        # shared-memory windows of two capacities
        for cells in (0, 1024, 4096):
            engine.set_t3_window(cells)
            for threads, ipt in ((64, 1), (64, 2), (128, 1), (128, 2), (256, 1)):
                engine.set_tuning(threads, ipt, 0)
                st = err_stats(engine.forces(ps.x, p, S.MIXED), F64)
                assert st["p99"] < MIXED_P99, (cells, threads, ipt, st)
        # quad lanes (trilinear; tricubic falls back to one i per lane)
        engine.set_t3_window(0)
        engine.set_variant(1)
        for threads in (64, 128, 256):
            engine.set_tuning(threads, 1, 0)
            st = err_stats(engine.forces(ps.x, p, S.MIXED), F64)
            assert st["p99"] < MIXED_P99, ("quad", threads, st)
    finally:
        engine.set_variant(0)
        engine.set_tuning(128, 2, 0)
        engine.set_t3_window(0)


def half_box_pairs(x, L, axes, seed, npairs):
    """Places particle 2p+1 at particle 2p's position shifted by L/2 + delta
    along one axis, delta within a few FP32 ulps of L/2: the reference's
    nearest-image test |d| > L/2 then sits inside FP32 rounding."""
    rng = np.random.default_rng(seed)
    x = x.copy()
    ulp = np.spacing(np.float32(L / 2))
    for p in range(npairs):
        i, j = 2 * p, 2 * p + 1
        ax = axes[p % len(axes)]
        x[j] = x[i]
        x[j, ax] = np.mod(x[i, ax] + L / 2 + rng.uniform(-3.0, 3.0) * ulp, L)
    return x


@pytest.mark.parametrize("isp", [1, 2])
def test_t3_nearest_image_at_half_box(engine, isp):
    """Pairs at |dx| = L/2 within FP32 rounding along every axis: mixed takes
    the same image as the FP64 kernel (a different one reverses the pair's
    direct force, ~1e-2 of these particles' forces)."""
    g = golden("t3_o2")
    ng, L = int(g["ngrid"]), float(g["L"])
    rng = np.random.default_rng(5)
    n = 4096
    x = half_box_pairs(rng.uniform(0.0, L, (n, 3)), L, (0, 1, 2), 6, 1024)
    m = np.full(n, 1.0 / n)
    eps = np.full(n, 0.01 * L / 16)
    engine.set_particles(m, eps)
    engine.set_table_t3(g["table"], ng)
    p = S.params(S.T3, is_periodic=isp, L=L, rsim=L / 2, ewald_order=2)
    F64 = engine.forces(x, p, S.FP64)
    try:
        for variant in (0, 1):  # one i per lane; quad lanes
            engine.set_variant(variant)
            engine.set_tuning(128, 1 if variant else 2, 0)
            e = rel_err(engine.forces(x, p, S.MIXED), F64)
            assert np.percentile(e[:2048], 99) < MIXED_P99 and np.percentile(e, 99) < MIXED_P99, (
                variant, np.percentile(e[:2048], [50, 99, 100]))
    finally:
        engine.set_variant(0)
        engine.set_tuning(128, 2, 0)


@pytest.mark.parametrize("mode", ["nearest", "table"])
def test_s1r2_nearest_image_at_half_period(engine, mode):
    """The same along the periodic z axis of S1xR2: IS_PERIODIC = 1 (nearest
    image only) and the (rho, z) table mode, both wrap dz at L/2."""
    g = golden("s1r2_table_o2")
    L = float(g["L"])
    n = g["x"].shape[0] - g["x"].shape[0] % 2
    x = half_box_pairs(g["x"][:n], L, (2,), 8, n // 4)
    engine.set_particles(g["m"][:n], g["eps"][:n])
    if mode == "table":
        nrho, nz = (int(v) for v in g["shape"])
        engine.set_table_s1r2(g["table"], nrho, nz)
        p = s1_params(g, 2, images=0, order=2)
    else:
        p = s1_params(g, 1)
    F64 = engine.forces(x, p, S.FP64)
    e = rel_err(engine.forces(x, p, S.MIXED), F64)
    assert np.percentile(e[:n // 2], 99) < MIXED_P99, np.percentile(e[:n // 2], [50, 99, 100])


def test_s1r2_ngp_at_cell_faces(engine):
    """NGP (order 0) picks a table cell, a hard decision. Pairs are planted
    with their (rho, z) separation within +-4e-7 (relative) of a cell face:
    rho = (K - 1/2) drho, or dz + L/2 = K dz_cell. At these offsets FP32
    rounding alone takes the wrong cell for about 6 % (rho) and 14 % (z) of
    the pairs. A wrong cell moves the pair force by ~1e-3 relative, so the
    mixed kernel must take these decisions on the FP64 separation."""
    g = golden("s1r2_table_o0")
    nrho, nz = (int(v) for v in g["shape"])
    L, rsim = float(g["L"]), float(g["rsim"])
    drho, dzc = 2.25 * rsim / (nrho - 1), L / nz
    rng = np.random.default_rng(17)
    npair = 384
    base = np.column_stack([rng.uniform(-300, 300, npair), rng.uniform(-300, 300, npair), rng.uniform(0, L, npair)])
    kind = np.arange(npair) % 3  # 0: rho face, 1: z face, 2: both
    K = rng.integers(1, 24, npair)
    rho = np.where(kind != 1, (K - 0.5) * drho * (1 + rng.uniform(-4e-7, 4e-7, npair)),
                   (rng.integers(1, 24, npair) + rng.uniform(-0.3, 0.3, npair)) * drho)
    Kz = rng.integers(nz // 4, 3 * nz // 4 + 1, npair)
    dz = np.where(kind != 0, Kz * dzc - L / 2 + L * rng.uniform(-4e-7, 4e-7, npair),
                  (rng.integers(nz // 4, 3 * nz // 4, npair) + 0.5 + rng.uniform(-0.3, 0.3, npair)) * dzc - L / 2)
    phi = rng.uniform(0, 2 * np.pi, npair)
    sep = np.column_stack([rho * np.cos(phi), rho * np.sin(phi), dz])
    x = np.empty((2 * npair, 3))
    x[0::2], x[1::2] = base, base + sep
    x[:, 2] %= L
    m = np.ones(2 * npair)
    eps = np.full(2 * npair, 0.05)
    engine.set_particles(m, eps)
    engine.set_table_s1r2(g["table"], nrho, nz)
    p = s1_params(g, 2, images=0, order=0)
    F64 = engine.forces(x, p, S.FP64)
    for threads, ipt in ((128, 1), (64, 2)):
        engine.set_tuning(threads, ipt, 0)
        try:
            e = rel_err(engine.forces(x, p, S.MIXED), F64)
        finally:
            engine.set_tuning(128, 2, 0)
        assert e.max() < 1e-4 and np.percentile(e, 99) < MIXED_P99, (threads, ipt, np.percentile(e, [50, 99, 100]))


MODES = ["t3_o2", "t3_o4", "s1_images", "s1_table_o0", "s1_table_o2", "s1_table_o4"]


def _mode_setup(engine, mode, n):
    """The first n particles of the mode's golden set, the golden table
    uploaded, and (library params, oracle system factory)."""
    if mode.startswith("t3"):
        order = int(mode[-1])
        g = golden(f"t3_o{order}")
        ng, L = int(g["ngrid"]), float(g["L"])
        engine.set_table_t3(g["table"], ng)
        p = S.params(S.T3, is_periodic=2, L=L, rsim=L / 2, ewald_order=order)
        sysf = lambda port, m, e: port.system(1, m, e, port_params(O, is_periodic=2, L=L, rsim=L / 2),  # noqa: E731
                                              table=g["table"], ngrid=ng, order=order)
    elif mode == "s1_images":
        g = golden("s1r2_images")
        L, rsim = float(g["L"]), float(g["rsim"])
        p = s1_params(g, 2)
        sysf = lambda port, m, e: port.system(3, m, e, port_params(O, is_periodic=2, L=L, rsim=rsim))  # noqa: E731
    else:
        order = int(mode[-1])
        g = golden(f"s1r2_table_o{order}")
        L, rsim = float(g["L"]), float(g["rsim"])
        nrho, nz = (int(v) for v in g["shape"])
        engine.set_table_s1r2(g["table"], nrho, nz)
        p = s1_params(g, 2, images=0, order=order)
        sysf = lambda port, m, e: port.system(2, m, e, port_params(O, is_periodic=2, L=L, rsim=rsim),  # noqa: E731
                                              table=g["table"], nrho=nrho, nz=nz, order=order)
    x, m, eps = g["x"][:n], g["m"][:n], g["eps"][:n]
    engine.set_particles(m, eps)
    return x, m, eps, p, sysf, float(g["L"])


@pytest.mark.parametrize("n", [1, 2, 3, 129, 1000])
@pytest.mark.parametrize("mode", MODES)
def test_periodic_edge_sizes(engine, port, mode, n):
    """Tiny and ragged particle counts (one particle, a pair, partial tiles)
    in every periodic mode: FP64 against the oracle to 1e-12, mixed against
    FP64, and single-particle i ranges at both ends. A lone particle's force
    (its own images and table correction) is ~0, so forces below 1e-9 of the
    set's scale m_total / L^2 are compared in absolute terms."""
    x, m, eps, p, sysf, L = _mode_setup(engine, mode, n)
    Fo = port.forces(sysf(port, m, eps), x)
    scale = float(m.sum()) / L ** 2
    big = np.linalg.norm(Fo, axis=1) > 1e-9 * scale

    def check(F, Fref, sel, tol_rel, tol_abs):
        assert np.abs(F[~sel] - Fref[~sel]).max(initial=0.0) <= tol_abs * scale
        if sel.any():
            e = rel_err(F[sel], Fref[sel])
            assert (e.max() if tol_rel == FP64_TOL else np.percentile(e, 99)) < tol_rel, np.percentile(e, [50, 99, 100])

    F64 = engine.forces(x, p, S.FP64)
    check(F64, Fo, big, FP64_TOL, 1e-12)
    Fm = engine.forces(x, p, S.MIXED)
    check(Fm, F64, big, MIXED_P99, 1e-6)
    for lo in {0, n - 1}:
        Fl = engine.forces(x, p, S.FP64, lo, lo)
        check(Fl, Fo[lo:lo + 1], big[lo:lo + 1], FP64_TOL, 1e-12)
        Fl = engine.forces(x, p, S.MIXED, lo, lo)
        check(Fl, Fo[lo:lo + 1], big[lo:lo + 1], 1e-4, 1e-6)


def test_radial_table_builder(engine, port):
    """The GPU builder of the cylindrical background multiplier
    (get_cylindrical_force_table, StePS/src/utils.cc:162-228) against the
    reference build's own table in the golden set, then used in a comoving
    S1xR2 evaluation against the reference's forces; and at the reference's
    default size and accuracy (1000 x 1000) against the oracle."""
    g = golden("s1r2_images")
    L, rsim = float(g["L"]), float(g["rsim"])
    ewald_cut = 3 - 0.4  # IS_PERIODIC = 2 (StePS/src/main.cc:1270-1271)
    engine.build_radial_table(200, rsim, L * ewald_cut, 400)
    tab = engine.get_radial_table(200)
    np.testing.assert_allclose(tab, g["radial"], rtol=1e-12, atol=1e-14)
    engine.set_particles(g["m"], g["eps"])
    p = s1_params(g, 2, cosmology=1, comoving=1, mius=float(g["mius"]))
    assert rel_err(engine.forces(g["x"], p, S.FP64), g["F_comoving"]).max() < FP64_TOL
    for lz in (0.5 * L, 5.6 * L):
        engine.build_radial_table(1000, rsim, lz, 1000)
        np.testing.assert_allclose(engine.get_radial_table(1000), port.cyl_table(rsim, lz, 1000, 1000), rtol=1e-12,
                                   atol=1e-14)


def test_load_tables_from_hdf5(engine):
    """Table files in the reference's HDF5 layout (StePS/src/inputoutput.cc:
    1792, 2102; tests/golden/make_h5_tables.py) loaded into the GPU context:
    the tables arrive bit for bit and give the reference's FP64 forces."""
    g = golden("t3_o2")
    L = float(g["L"])
    ng = engine.load_table_t3_hdf5(os.path.join(GOLDEN, "t3_table_ng17.h5"))
    assert ng == int(g["ngrid"]) and np.array_equal(engine.get_table_t3(ng), g["table"])
    engine.set_particles(g["m"], g["eps"])
    p = S.params(S.T3, is_periodic=2, L=L, rsim=L / 2, ewald_order=2)
    assert rel_err(engine.forces(g["x"], p, S.FP64), g["F"]).max() < FP64_TOL
    # a single-precision build's file holds floats: loaded exactly, as doubles
    engine.load_table_t3_hdf5(os.path.join(GOLDEN, "t3_table_ng17_f32.h5"))
    assert np.array_equal(engine.get_table_t3(ng), np.float32(g["table"]).astype(np.float64))
    g = golden("s1r2_table_o2")
    nrho, nz = engine.load_table_s1r2_hdf5(os.path.join(GOLDEN, "s1r2_table.h5"))
    assert (nrho, nz) == tuple(int(v) for v in g["shape"])
    assert np.array_equal(engine.get_table_s1r2(nrho, nz), g["table"])
    engine.set_particles(g["m"], g["eps"])
    assert rel_err(engine.forces(g["x"], s1_params(g, 2, images=0, order=2), S.FP64), g["F"]).max() < FP64_TOL
    with pytest.raises(S.StepsError) as e:  # the T3 loader rejects an S1xR2 file
        engine.load_table_t3_hdf5(os.path.join(GOLDEN, "s1r2_table.h5"))
    assert e.value.code == S.STEPS_E_ARG
