"""The plain-C oracle against the reference's own CPU force path, compiled
unmodified from the reference tree into oracle/_ref, on fresh seeded inputs
(other seeds, sizes and i ranges than the golden vectors): R^3 with its three
background modes, T^3 at orders 2 and 4 and nearest image, S1xR2 image sums
at three IS_PERIODIC values and the (rho, z) table at orders 0/2/4, and both
table builders at other grid sizes. Runs where the reference build exists
(it does not travel to machines without the reference tree)."""
import math

import numpy as np
import pyoracle as O
import pytest

from helpers import golden, port_params, rel_err
from steps_gb300 import workloads as W

pytestmark = pytest.mark.skipif(not all(O.ref_available(v) for v in ("r3", "t3o2", "t3o4", "s1nl", "s1o0")),
                                reason="reference build (oracle/_ref) not present")

TOL = 1e-13


def _ref(variant, ps, **params):
    ref = O.Ref(variant)
    ref.set_particles(ps.x, ps.m, ps.eps)
    ref.set_params(**params)
    return ref


@pytest.mark.parametrize("bg", ["none", "comoving", "de"])
def test_r3(port, bg):
    ps = W.r3_compactified(3001, 700.0, seed=301, displace=True)
    kw = {"none": {}, "comoving": dict(cosmology=1, comoving=1, mius=0.23),
          "de": dict(cosmology=1, comoving=0, h0=0.068, oml=0.7)}[bg]
    ref = _ref("r3", ps, **kw)
    s = port.system(0, ps.m, ps.eps, port_params(O, **kw))
    for lo, hi in ((0, 3000), (17, 2900), (3000, 3000)):
        # same operations in the same order: bit-identical
        assert np.array_equal(port.forces(s, ps.x, lo, hi), ref.forces(lo, hi)), (lo, hi)


@pytest.mark.parametrize("order", [2, 4])
@pytest.mark.parametrize("isp", [1, 2])
def test_t3(port, order, isp):
    g = golden(f"t3_o{order}")
    ng, L = int(g["ngrid"]), float(g["L"])
    ps = W.t3_clumpy(1777, L, seed=302, n_clumps=9)
    ref = _ref(f"t3o{order}", ps, is_periodic=isp, L=L, rsim=L / 2)
    ref.set_t3_table(g["table"], ng)
    s = port.system(1, ps.m, ps.eps, port_params(O, is_periodic=isp, L=L, rsim=L / 2), table=g["table"], ngrid=ng,
                    order=order)
    for lo, hi in ((0, 1776), (5, 1000)):
        assert rel_err(port.forces(s, ps.x, lo, hi), ref.forces(lo, hi)).max() < TOL, (lo, hi)


@pytest.mark.parametrize("isp", [1, 2, 3])
def test_s1r2_images(port, isp):
    ps = W.s1r2_cylindrical(1500, 150.0, 450.0, seed=303)
    ref = _ref("s1nl", ps, is_periodic=isp, L=150.0, rsim=450.0)
    s = port.system(3, ps.m, ps.eps, port_params(O, is_periodic=isp, L=150.0, rsim=450.0))
    assert rel_err(port.forces(s, ps.x), ref.forces()).max() < TOL


@pytest.mark.parametrize("order", [0, 2, 4])
def test_s1r2_table(port, order):
    g = golden(f"s1r2_table_o{order}")
    nrho, nz = (int(v) for v in g["shape"])
    L, rsim = float(g["L"]), float(g["rsim"])
    ps = W.s1r2_cylindrical(1500, L, rsim, seed=304)
    ref = _ref(f"s1o{order}", ps, is_periodic=2, L=L, rsim=rsim)
    ref.set_s1r2_table(g["table"], nrho, nz)
    s = port.system(2, ps.m, ps.eps, port_params(O, is_periodic=2, L=L, rsim=rsim), table=g["table"], nrho=nrho,
                    nz=nz, order=order)
    assert rel_err(port.forces(s, ps.x), ref.forces()).max() < TOL


@pytest.mark.skipif(not O.ref_available("s1rs"), reason="reference build (oracle/_ref) not present")
def test_s1r2_direct_sum_table_other_size(port):
    """The direct real-space table (PERIODIC_Z_RSPACELOOKUP build) at another
    grid, period and image count: bit-identical."""
    lz, rmax = 90.0, 2.25 * 250.0
    want = O.Ref("s1rs").build_s1r2_table(25, 10, rmax, lz, 0.0, 3000, 0)
    assert np.array_equal(port.s1r2_table(25, 10, rmax, lz, 0.0, 3000, 0), want)


def test_table_builders_other_sizes(port):
    """Both Ewald table builders at grid sizes the golden set does not use."""
    L = 80.0
    args = (2.0 / L, 2.0, 5.0 * 2.0 * math.pi / L, 3.0, 6.0)
    want = O.Ref("t3o2").build_t3_table(19, L, *args)
    got = port.t3_table(19, L, *args)
    np.testing.assert_allclose(got, want, rtol=0, atol=1e-13 * np.abs(want).max())
    lz, rmax = 120.0, 2.25 * 300.0
    want = O.Ref("s1o2").build_s1r2_table(40, 12, rmax, lz, 0.787875 / lz, 4, 10)
    got = port.s1r2_table(40, 12, rmax, lz, 0.787875 / lz, 4, 10)
    np.testing.assert_allclose(got, want, rtol=0, atol=1e-13 * np.abs(want).max())


def _kdk_case(topo):
    """(variant, particle set, reference params, port system factory, moving axes)
    for a periodic KDK run; velocities move particles up to 2 % of L per step
    so that many cross the boundary."""
    if topo == "t3":
        g = golden("t3_o2")
        L, ng = float(g["L"]), int(g["ngrid"])
        ps = W.t3_clumpy(1200, L, seed=305, n_clumps=6)
        kw = dict(is_periodic=2, L=L, rsim=L / 2)
        return ("t3o2", ps, kw, g["table"], ng, 3, L,
                lambda port, eps: port.system(1, ps.m, eps, port_params(O, **kw), table=g["table"], ngrid=ng, order=2))
    g = golden("s1r2_table_o2") if topo == "s1tab" else golden("s1r2_images")
    L, rsim = float(g["L"]), float(g["rsim"])
    ps = W.s1r2_cylindrical(1200, L, rsim, seed=306)
    kw = dict(is_periodic=2, L=L, rsim=rsim)
    if topo == "s1tab":
        nrho, nz = (int(v) for v in g["shape"])
        return ("s1o2", ps, kw, g["table"], (nrho, nz), 1, L,
                lambda port, eps: port.system(2, ps.m, eps, port_params(O, **kw), table=g["table"], nrho=nrho, nz=nz,
                                              order=2))
    return ("s1nl", ps, kw, None, None, 1, L, lambda port, eps: port.system(3, ps.m, eps, port_params(O, **kw)))


@pytest.mark.parametrize("topo", ["t3", "s1img", "s1tab"])
def test_kdk_periodic_against_reference_step(port, topo):
    """The oracle's KDK (the checker of the GPU KDK tests) against the
    reference's own step() (StePS/src/step.cc:100-312) on a periodic
    topology, with the boundary wrap exercised: positions, velocities,
    forces and errmax after 3 fixed-dt steps."""
    var, ps, kw, table, shape, axes, L, sysf = _kdk_case(topo)
    ref = O.Ref(var)
    ref.set_particles(ps.x, ps.m, ps.eps)
    eps = ref.softening(W.PARTICLE_RADII)  # the reference's law; also sets rho_part for errmax
    ref.set_params(**kw)
    if var.startswith("t3"):
        ref.set_t3_table(table, shape)
    elif var == "s1o2":
        ref.set_s1r2_table(table, *shape)
    h, nsteps = 1e-3, 3
    v = np.zeros_like(ps.x)
    v[:, 3 - axes:] = np.random.default_rng(12).uniform(-1.0, 1.0, (ps.n, axes)) * (0.02 * L / h)
    ref.set_velocities(v)
    ref.forces_full()
    for _ in range(nsteps):
        ref.step(h)
    xr, vr, Fr = ref.state()
    er = ref.errmax()
    s = sysf(port, eps)
    rho_part = float(ps.m.min()) / (4.0 * math.pi * W.PARTICLE_RADII ** 3 / 3.0)
    xo, vo, Fo, eo = port.kdk(s, nsteps, h, ps.x, v, port.forces(s, ps.x), rho_part=rho_part)
    moved = np.abs(xr - ps.x)[:, 3 - axes:] > 0.5 * L
    assert moved.any()  # some particles wrapped
    np.testing.assert_allclose(xo, xr, rtol=0, atol=1e-12 * L)
    assert rel_err(vo, vr).max() < 1e-12
    assert rel_err(Fo, Fr).max() < 1e-11
    assert abs(eo - er) <= 1e-12 * abs(er)


@pytest.mark.parametrize("order", [0, 2, 4])
def test_s1r2_table_beyond_radial_extent(port, order):
    """Pairs whose rho separation passes the table's radial extent
    (2.25 Rsim): the reference clamps rho to the last table row; the
    oracle must do the same."""
    g = golden(f"s1r2_table_o{order}")
    nrho, nz = (int(v) for v in g["shape"])
    L, rsim = float(g["L"]), float(g["rsim"])
    ps = W.s1r2_cylindrical(800, L, rsim, seed=307)
    x = ps.x.copy()
    x[:200, :2] *= 2.0  # out to 2 Rsim from the axis: separations up to 3 Rsim
    rho = np.hypot(x[:, 0], x[:, 1])
    assert rho.max() + np.hypot(ps.x[:, 0], ps.x[:, 1]).max() > 2.25 * rsim
    ref = O.Ref(f"s1o{order}")
    ref.set_particles(x, ps.m, ps.eps)
    ref.set_params(is_periodic=2, L=L, rsim=rsim)
    ref.set_s1r2_table(g["table"], nrho, nz)
    s = port.system(2, ps.m, ps.eps, port_params(O, is_periodic=2, L=L, rsim=rsim), table=g["table"], nrho=nrho,
                    nz=nz, order=order)
    assert rel_err(port.forces(s, x), ref.forces()).max() < TOL


@pytest.mark.parametrize("size,accuracy,lz_over_L", [(1000, 1000, 0.5), (1000, 1000, 2.6), (257, 64, 5.6)])
def test_cylindrical_force_table(port, size, accuracy, lz_over_L):
    """The finite-cylinder radial multiplier (get_cylindrical_force_table,
    StePS/src/utils.cc:162-228) at the reference's default size and accuracy
    (1000, 1000; StePS/src/read_paramfile.cc:128-129) and at the half
    lengths its driver passes (L/2 at IS_PERIODIC = 1, L (IS_PERIODIC + 0.6)
    above; StePS/src/main.cc:905-917)."""
    rsim, L = 450.0, 150.0
    ref = port.cyl_table(rsim, lz_over_L * L, size, accuracy)
    theirs = O.Ref("s1nl").cyl_table(rsim, lz_over_L * L, size, accuracy)
    np.testing.assert_allclose(ref, theirs, rtol=TOL, atol=1e-15)
