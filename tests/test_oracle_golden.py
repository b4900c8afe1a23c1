"""The plain-C oracle (oracle/steps_oracle.c) against the golden vectors that
the reference StePS CPU path produced (tests/golden/make_golden.py).

These run on CPU anywhere (no GPU, no reference tree): they pin the oracle
that the GPU parity tests use at sizes the golden set does not cover."""
import math

import numpy as np
import pyoracle as O
import pytest

from helpers import golden, port_params, rel_err

TOL = 1e-13  # same algorithm, same order of summation: rounding-level agreement


def test_softening_kernel(port):
    g = golden("softening")
    w = np.array([port.softening(r, 1.0) for r in g["r"]])
    np.testing.assert_allclose(w, g["w_beta1"], rtol=1e-14, atol=0)
    w2 = np.array([port.softening(r * 0.37, 0.37) for r in g["r"]])
    np.testing.assert_allclose(w2, g["w_beta037"], rtol=1e-14, atol=0)


def test_spline_continuity(port):
    # The cubic spline meets 1/r^3 at r = beta and its two branches meet at beta/2.
    for b in (0.1, 1.0, 3.7):
        for r0 in (b, 0.5 * b):
            lo, hi = port.softening(r0 * (1 - 1e-9), b), port.softening(r0 * (1 + 1e-9), b)
            assert abs(lo - hi) <= 1e-6 * abs(hi)
    assert abs(port.softening(2.0, 1.0) - 1 / 8.0) < 1e-15


def test_r3(port):
    g = golden("r3_n2048")
    np.testing.assert_allclose(g["eps"], g["eps_ref"], rtol=1e-14)
    s = port.system(0, g["m"], g["eps"], port_params(O))
    F = port.forces(s, g["x"])
    assert rel_err(F, g["F"]).max() < TOL
    lo, hi = g["sub"]
    assert rel_err(port.forces(s, g["x"], int(lo), int(hi)), g["F_sub"]).max() < TOL
    s = port.system(0, g["m"], g["eps"], port_params(O, cosmology=1, comoving=1, mius=float(g["mius"])))
    assert rel_err(port.forces(s, g["x"]), g["F_comoving"]).max() < TOL
    s = port.system(0, g["m"], g["eps"], port_params(O, cosmology=1, comoving=0, h0=float(g["h0"]), oml=float(g["oml"])))
    assert rel_err(port.forces(s, g["x"]), g["F_de"]).max() < TOL


def test_r3_kdk(port):
    g = golden("r3_kdk4")
    s = port.system(0, g["m"], g["eps"], port_params(O))
    F0 = port.forces(s, g["x"])
    assert rel_err(F0, g["F0"]).max() < TOL
    x, v, F, e = port.kdk(s, 4, float(g["dt"]), g["x"], np.zeros_like(g["x"]), F0, rho_part=float(g["rho_part"]))
    np.testing.assert_allclose(x, g["x4"], rtol=0, atol=1e-12)
    assert rel_err(v, g["v4"]).max() < 1e-11
    assert rel_err(F, g["F4"]).max() < 1e-11
    assert abs(e - float(g["errmax"])) <= 1e-11 * abs(float(g["errmax"]))


@pytest.mark.parametrize("order", [2, 4])
def test_t3(port, order):
    g = golden(f"t3_o{order}")
    ng, L = int(g["ngrid"]), float(g["L"])
    a = g["ewald"]
    tab = port.t3_table(ng, L, *a)
    np.testing.assert_allclose(tab, g["table"], rtol=0, atol=1e-13 * np.abs(g["table"]).max())
    D = np.array([port.t3_interp(ng, L, g["table"], p, order) for p in g["probes"]])
    np.testing.assert_allclose(D, g["D"], rtol=0, atol=1e-15 * np.abs(g["D"]).max())
    s = port.system(1, g["m"], g["eps"], port_params(O, is_periodic=2, L=L, rsim=L / 2), table=g["table"], ngrid=ng,
                    order=order)
    assert rel_err(port.forces(s, g["x"]), g["F"]).max() < 1e-12
    s = port.system(1, g["m"], g["eps"], port_params(O, is_periodic=1, L=L, rsim=L / 2), table=g["table"], ngrid=ng,
                    order=order)
    assert rel_err(port.forces(s, g["x"]), g["F_nearest"]).max() < TOL


def test_t3_lattice(port):
    g = golden("t3_lattice")
    for key, r in zip(("real", "rec"), g["radii"]):
        np.testing.assert_array_equal(port.lattice(float(r))[:, :3], g[key][:, :3])


def test_t3_table63_sample(port):
    g = golden("t3_table63_sample")
    tab = port.t3_table(63, 100.0, *g["ewald"])
    np.testing.assert_allclose(tab[g["idx"]], g["val"], rtol=0, atol=1e-13 * np.abs(g["val"]).max())


def test_s1r2_images(port):
    g = golden("s1r2_images")
    L, rsim = float(g["L"]), float(g["rsim"])
    for isp, key in ((2, "F_is2"), (1, "F_is1")):
        s = port.system(3, g["m"], g["eps"], port_params(O, is_periodic=isp, L=L, rsim=rsim))
        assert rel_err(port.forces(s, g["x"]), g[key]).max() < TOL, key
    s = port.system(3, g["m"], g["eps"], port_params(O, is_periodic=4, L=L, rsim=rsim))
    assert rel_err(port.forces(s, g["x"], 0, 255), g["F_is4_head"]).max() < TOL
    radial = port.cyl_table(rsim, L * 2.6, 200, 400)
    np.testing.assert_allclose(radial, g["radial"], rtol=1e-13, atol=1e-15)
    s = port.system(3, g["m"], g["eps"], port_params(O, is_periodic=2, L=L, rsim=rsim, cosmology=1, comoving=1,
                                                     mius=float(g["mius"])), radial=g["radial"])
    assert rel_err(port.forces(s, g["x"]), g["F_comoving"]).max() < TOL


@pytest.mark.parametrize("order", [0, 2, 4])
def test_s1r2_table(port, order):
    g = golden(f"s1r2_table_o{order}")
    nrho, nz = (int(v) for v in g["shape"])
    L, rsim = float(g["L"]), float(g["rsim"])
    alpha, nmax, mmax = g["ewald"]
    tab = port.s1r2_table(nrho, nz, 2.25 * rsim, L, alpha, int(nmax), int(mmax))
    np.testing.assert_allclose(tab, g["table"], rtol=0, atol=1e-13 * np.abs(g["table"]).max())
    pair = np.array([port.s1r2_pair(p, L, alpha, int(nmax), int(mmax)) for p in g["probes"][:16]])
    np.testing.assert_allclose(pair, g["pair"], rtol=1e-12, atol=1e-18)
    D = np.array([port.s1r2_interp(g["table"], nrho, nz, 2.25 * rsim, L, p, order) for p in g["probes"]])
    np.testing.assert_allclose(D, g["D"], rtol=0, atol=1e-15 * np.abs(g["D"]).max())
    s = port.system(2, g["m"], g["eps"], port_params(O, is_periodic=2, L=L, rsim=rsim), table=g["table"], nrho=nrho,
                    nz=nz, order=order)
    assert rel_err(port.forces(s, g["x"]), g["F"]).max() < TOL


def test_s1r2_table_direct_sum(port):
    """The (rho, z) table of the reference's PERIODIC_Z_RSPACELOOKUP build
    (direct real-space image sums, selected by alpha = 0 and mmax = 0):
    the same terms in the same order, so bit-identical."""
    g = golden("s1r2_table_rspace")
    nrho, nz = (int(v) for v in g["shape"])
    L, rsim = float(g["L"]), float(g["rsim"])
    tab = port.s1r2_table(nrho, nz, 2.25 * rsim, L, 0.0, int(g["nmax"]), 0)
    assert np.array_equal(tab, g["table"])


def test_s1r2_background_terms(port):
    """The S1xR2 background terms: comoving with the radial correction at
    IS_PERIODIC = 1, non-comoving H0^2 Omega_L x, and the table mode's plain
    mass_in_unit_sphere x."""
    g, b, t = golden("s1r2_images"), golden("s1r2_background"), golden("s1r2_table_o2")
    L, rsim = float(g["L"]), float(g["rsim"])
    mius, h0, oml = float(b["mius"]), float(b["h0"]), float(b["oml"])
    nrho, nz = (int(v) for v in t["shape"])
    cases = [
        (3, dict(is_periodic=1, cosmology=1, comoving=1, mius=mius), {}, "F_is1_comoving"),
        (3, dict(is_periodic=2, cosmology=1, comoving=0, h0=h0, oml=oml), {}, "F_is2_de"),
        (2, dict(is_periodic=2, cosmology=1, comoving=1, mius=mius), dict(table=t["table"], nrho=nrho, nz=nz, order=2),
         "F_table_comoving"),
        (2, dict(is_periodic=2, cosmology=1, comoving=0, h0=h0, oml=oml),
         dict(table=t["table"], nrho=nrho, nz=nz, order=2), "F_table_de"),
    ]
    for topo, pkw, skw, key in cases:
        s = port.system(topo, g["m"], g["eps"], port_params(O, L=L, rsim=rsim, **pkw), radial=g["radial"], **skw)
        assert rel_err(port.forces(s, g["x"]), b[key]).max() < TOL, key


def test_two_body_analytic(port):
    # Beyond the softening support the pair force is Newton's m / r^2.
    x = np.array([[0.0, 0.0, 0.0], [3.0, 4.0, 0.0]])
    m = np.array([2.0, 5.0])
    eps = np.array([0.1, 0.2])
    s = port.system(0, m, eps, port_params(O))
    F = port.forces(s, x)
    np.testing.assert_allclose(F[0], 5.0 / 25.0 * np.array([0.6, 0.8, 0.0]), rtol=1e-15)
    np.testing.assert_allclose(F[1], -2.0 / 25.0 * np.array([0.6, 0.8, 0.0]), rtol=1e-15)


def test_momentum_conservation(port):
    # Without the background term pairwise forces are antisymmetric (beta_ij = beta_ji).
    g = golden("r3_n2048")
    s = port.system(0, g["m"], g["eps"], port_params(O))
    F = port.forces(s, g["x"])
    p = (g["m"][:, None] * F).sum(0)
    assert np.abs(p).max() < 1e-12 * (g["m"][:, None] * np.abs(F)).sum()


def test_t3_lattice_forces_vanish(port):
    # On a perfect cubic lattice every particle sits at a symmetry centre of T^3.
    # An odd lattice keeps every separation strictly inside (-L/2, L/2): at
    # exactly L/2 the nearest-image rule (forces.cc:812-817) is one-sided.
    g = golden("t3_o4")
    ng, L = int(g["ngrid"]), float(g["L"])
    k = 5
    c = (np.arange(k) + 0.5) * L / k
    x = np.stack(np.meshgrid(c, c, c, indexing="ij"), -1).reshape(-1, 3)
    n = x.shape[0]
    s = port.system(1, np.full(n, 1.0), np.full(n, 0.02), port_params(O, is_periodic=2, L=L, rsim=L / 2),
                    table=g["table"], ngrid=ng, order=4)
    F = port.forces(s, x)
    assert np.abs(F).max() < 1e-12 * (n / (0.2 * L) ** 2)


def test_r3_n32768_subset(port):
    """The N = 32,768 compactified workload, regenerated from its seed, against
    the reference FP64 build on an i range (the fixture of the FP32 floor)."""
    from steps_gb300 import workloads as W

    g = golden("ref_fp32")
    ps = W.r3_compactified(int(g["r3_n"]), float(g["r3_rmax"]), seed=int(g["r3_seed"]))
    lo, hi = (int(v) for v in g["r3_sub"])
    s = port.system(0, ps.m, ps.eps, port_params(O))
    assert rel_err(port.forces(s, ps.x, lo, hi), g["r3_F64"]).max() < TOL


def test_s1r2_pair_line_mass_limit(port):
    """Far from the axis (rho >> L) the singly periodic sum tends to a line of
    mass m / L: radial force 2 m / (L rho), no z force. The oracle's pair force
    and the reference's own values (golden probes with rho > 3 L, where the
    first Fourier mode is down by exp(-2 pi rho / L) < 1e-8) both reach it."""
    L = 200.0
    alpha = 0.787875 / L
    for rho in (2000.0, 4000.0):
        for dz in (0.0, 37.0, -99.0):
            F = port.s1r2_pair((0.6 * rho, 0.8 * rho, dz), L, alpha, 4, 10)
            assert abs(math.hypot(F[0], F[1]) * L * rho / 2 - 1) < 1e-12
            assert abs(F[2]) < 1e-20
    g = golden("s1r2_table_o2")
    probes, pair = g["probes"][: len(g["pair"])], g["pair"]
    rho = np.hypot(probes[:, 0], probes[:, 1])
    far = rho > 3 * float(g["L"])
    assert far.sum() >= 3
    radial = np.hypot(pair[far, 0], pair[far, 1]) * float(g["L"]) * rho[far] / 2
    assert np.abs(radial - 1).max() < 1e-6


def test_t3_table_odd_symmetry(port):
    """The Ewald correction is odd, D(-r) = -D(r) (StePS/src/ewald_space.cc:365-376):
    on the cell-centred grid cell i mirrors to ng - 1 - i. The reference's table
    holds it exactly; so does the oracle's builder."""
    g = golden("t3_o2")
    ng = int(g["ngrid"])
    T = g["table"].reshape(ng, ng, ng, 3)
    assert np.abs(T + T[::-1, ::-1, ::-1]).max() == 0.0
    e = [float(v) for v in g["ewald"]]
    To = port.t3_table(ng, float(g["L"]), *e).reshape(ng, ng, ng, 3)
    assert np.abs(To + To[::-1, ::-1, ::-1]).max() <= 1e-15 * np.abs(To).max()
