"""The oracle restatement against the reference's own kernels run on the
host (oracle/_ref, built from the reference tree by oracle/build_ref.sh).

Only runs where oracle/_ref exists (the build container); the committed
golden fixtures in tests/golden/ carry the same pin to other machines.
"""
import numpy as np
import pytest

from thesis_gb300 import lattice

pytestmark = pytest.mark.skipif(
    __import__("oracle.pyoracle", fromlist=["x"]).ref_lib() is None,
    reason="oracle/_ref (reference kernels built for the host) not present")

CASES_2D = [(16, 16, 1), (16, 16, 2), (16, 16, 3), (24, 12, 1)]


@pytest.mark.parametrize("n,m,coll", CASES_2D)
@pytest.mark.parametrize("fp64", [False, True])
def test_cavity2d_bit_exact(oracle, n, m, coll, fp64):
    lat = lattice.cavity2d(n, m)
    kw = dict(u=0.1, viscosity=0.128, collision_model=coll, outlet_profile=1)
    ref = oracle.run_reference(lat, 25, fp64=fp64, **kw)
    orc = oracle.run_oracle(lat, 25, fp64=fp64, **kw)
    assert ref.rc == 0 and orc.rc == 0
    np.testing.assert_array_equal(ref.mask, orc.mask)
    np.testing.assert_array_equal(ref.stream, orc.stream)
    assert ref.count == orc.count
    tol = 0.0 if not fp64 else 1e-14
    for a, b in ((ref.f, orc.f), (ref.fc, orc.fc), (ref.rho, orc.rho), (ref.u, orc.u), (ref.v, orc.v)):
        assert np.abs(a - b).max() <= tol
    np.testing.assert_allclose(ref.resid[:25], orc.resid[:25], rtol=1e-12)


@pytest.mark.parametrize("coll", [1, 3])
@pytest.mark.parametrize("fp64", [False, True])
def test_cavity3d_bit_exact(oracle, coll, fp64):
    lat = lattice.cavity3d(10, 9, 8)
    kw = dict(u=0.05, viscosity=0.1, collision_model=coll)
    ref = oracle.run_reference(lat, 12, fp64=fp64, **kw)
    orc = oracle.run_oracle(lat, 12, fp64=fp64, **kw)
    assert ref.rc == 0 and orc.rc == 0
    np.testing.assert_array_equal(ref.mask, orc.mask)
    np.testing.assert_array_equal(ref.stream, orc.stream)
    tol = 0.0 if not fp64 else 1e-12
    for a, b in ((ref.f, orc.f), (ref.fc, orc.fc), (ref.rho, orc.rho), (ref.u, orc.u), (ref.w, orc.w)):
        assert np.abs(a - b).max() <= tol * max(1.0, np.abs(a).max())


def test_symmetry_and_gravity_3d(oracle):
    """Symmetry planes (GpuBoundaries.cu:2086-2168) and the g/omega force."""
    lat = lattice.cavity3d(8, 8, 10)
    bc = lat.bc.copy()
    # make the y- face a symmetry plane
    sel = (bc[:, 1] == 0) & (bc[:, 4] == 1)
    bc[sel, 4] = 5
    lat = lattice.Lattice(3, lat.n, lat.m, lat.h, lat.node_type, bc)
    kw = dict(u=0.05, viscosity=0.1, collision_model=1, g=1e-5)
    ref = oracle.run_reference(lat, 8, **kw)
    orc = oracle.run_oracle(lat, 8, **kw)
    np.testing.assert_array_equal(ref.mask, orc.mask)
    assert np.abs(ref.f - orc.f).max() == 0.0
    assert np.abs(ref.u - orc.u).max() == 0.0


def test_reference_lid_cavity_golden_mesh(oracle):
    """The 30^3 lid cavity the reference generator ships (latticegen2_W8/
    lidvalidation_{Node,BC}.dat): masks, stream flags and 5 MRT steps."""
    import os
    from oracle.pyoracle import reference_file
    g = reference_file("Source code", "latticegen2_W8")
    if g is None or not os.path.exists(os.path.join(g, "lidvalidation_Node.dat")):
        pytest.skip("reference tree not mounted")
    g += os.sep
    lat = lattice.from_files(g + "lidvalidation_Node.dat", g + "lidvalidation_BC.dat")
    kw = dict(u=0.05, viscosity=0.1, collision_model=3, delta=1 / 29)
    ref = oracle.run_reference(lat, 5, **kw)
    orc = oracle.run_oracle(lat, 5, **kw)
    np.testing.assert_array_equal(ref.mask, orc.mask)
    np.testing.assert_array_equal(ref.stream, orc.stream)
    assert np.abs(ref.f - orc.f).max() == 0.0


@pytest.mark.parametrize("coll", [1, 3])
@pytest.mark.parametrize("fp64", [False, True])
def test_hh_wall_and_periodic_copies_3d(oracle, coll, fp64):
    """HH walls (GpuBoundaries.cu:492-1560) on a cavity's faces, edges and
    corners, and periodic copies (:2025-2084) on a channel periodic in x,
    with straight and with HH walls."""
    cases = [(lattice.cavity3d(10, 9, 8), 2), (lattice.periodic_channel3d(10, 9, 8), 1),
             (lattice.periodic_channel3d(10, 9, 8), 2)]
    for lat, wm in cases:
        kw = dict(u=0.05, viscosity=0.1, collision_model=coll, bc_wall_model=wm)
        ref = oracle.run_reference(lat, 12, fp64=fp64, **kw)
        orc = oracle.run_oracle(lat, 12, fp64=fp64, **kw)
        assert ref.rc == 0 and orc.rc == 0
        np.testing.assert_array_equal(ref.mask, orc.mask)
        tol = 0.0 if not fp64 else 1e-12
        for a, b in ((ref.f, orc.f), (ref.fc, orc.fc), (ref.rho, orc.rho)):
            assert np.abs(a - b).max() <= tol * max(1.0, np.abs(a).max())
        if not fp64:
            assert np.abs(ref.u - orc.u).max() == 0.0 and np.abs(ref.w - orc.w).max() == 0.0


def test_two_periodic_axes_race_is_confined_to_their_edges(oracle):
    """Where two periodic faces meet, the reference's periodic copies race
    (each thread reads partners another thread may already have rewritten);
    the host replay runs them in boundary-list order, the oracle reads every
    partner from before the copies.  The two agree until the first step at
    which those edge nodes' copies feed back, and differ only there."""
    lat = lattice.periodic_channel3d(10, 9, 8, periodic_axes=(0, 1))
    kw = dict(u=0.05, viscosity=0.1, collision_model=1)
    ref = oracle.run_reference(lat, 2, **kw)
    orc = oracle.run_oracle(lat, 2, **kw)
    assert np.abs(ref.f - orc.f).max() == 0.0
    ref = oracle.run_reference(lat, 3, **kw)
    orc = oracle.run_oracle(lat, 3, **kw)
    diff = np.nonzero(np.abs(ref.f - orc.f).max(0) > 0)[0]
    x, y = diff % 10, (diff // 10) % 9
    assert diff.size > 0 and np.all((x == 0) | (x == 9)) and np.all((y == 0) | (y == 8))


CURVED = {
    "cylinder2d": (lambda: lattice.cylinder_channel2d(48, 24, outer_q=0.3), (1, 2, 3), 30),
    "sphere3d": (lambda: lattice.sphere_cavity3d(14, 12, 12, outer_q=0.3), (1, 3), 12),
}


@pytest.mark.parametrize("case", sorted(CURVED))
@pytest.mark.parametrize("fp64", [False, True])
def test_curved_walls_bit_exact(oracle, case, fp64):
    """Curved walls (gpuBcWall2D / gpuBcSimpleWall3D, CURVED): the reference
    derives each link's q from the BC file's boundary point; the oracle takes
    the same q as the reference computes it (reference_q) and matches its
    kernels bit for bit in FP32, both interpolation branches, including the
    first coefficient read one table entry ahead."""
    make, colls, steps = CURVED[case]
    lat = make()
    assert (lat.link_q < 0.5).sum() > 10 and (lat.link_q >= 0.5).sum() > 10
    qr = oracle.reference_q(lat, lat.link_q, fp64=fp64)
    for coll in colls:
        kw = dict(u=0.05, viscosity=0.05 if lat.dims == 2 else 0.1, collision_model=coll,
                  outlet_profile=1, boundary_type=1)
        ref = oracle.run_reference(lat, steps, fp64=fp64, link_q=lat.link_q, **kw)
        orc = oracle.run_oracle(lat, steps, fp64=fp64, link_q=qr, **kw)
        straight = oracle.run_oracle(lat, steps, fp64=fp64, **dict(kw, boundary_type=2))
        assert ref.rc == 0 and orc.rc == 0
        # FP64: the reference's 3D MRT from its zero start grows velocities
        # to O(100) within these steps, so rounding differences of the two
        # builds' libm-free arithmetic grow with it
        tol = 0.0 if not fp64 else 1e-10
        for a, b in ((ref.f, orc.f), (ref.fc, orc.fc), (ref.rho, orc.rho), (ref.u, orc.u), (ref.v, orc.v)):
            assert np.abs(a - b).max() <= tol * max(1.0, np.abs(a).max())
        assert np.abs(straight.f - orc.f).max() > 1e-3
