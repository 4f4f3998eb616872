"""The library's host-side lattice set-up (lbm_build_flags, no GPU) against
the oracle: the reference BC masks must match bit for bit, and the flag words
must encode the reference streaming flags (reference mode) or the solid /
out-of-domain links (physics mode)."""
import numpy as np
import pytest

from thesis_gb300 import lattice
from thesis_gb300 import native as N
from thesis_gb300.solver import Arguments, build_flags


def _lattices():
    yield "cav2d", lattice.cavity2d(12, 9)
    yield "cav3d", lattice.cavity3d(7, 6, 5)
    yield "duct", lattice.sphere_duct(24, 20, 40, porosity=0.8, rmin=3, rmax=5, seed=1)
    yield "channel", lattice.channel2d(96, 40, seed=3)


@pytest.mark.parametrize("name,lat", list(_lattices()), ids=[n for n, _ in _lattices()])
def test_reference_masks_bit_exact(native_lib, oracle, name, lat):
    # 3D outlets are refused in reference mode; the duct's masks are checked
    # through a physics-mode build (the masks do not depend on the mode)
    phys = name == "duct"
    args = Arguments(collision_model=N.BGKW, mode=N.MODE_PHYSICS if phys else N.MODE_REFERENCE,
                     outlet_profile=N.OUTLET_PRESSURE if phys else N.OUTLET_ZOUHE)
    mask, word, slot, nbc = build_flags(lat, args)
    r = oracle.run_oracle(lat, 0, mode=1 if phys else 0, outlet_profile=5 if phys else 1)
    assert r.rc == 0
    np.testing.assert_array_equal(mask, r.mask)
    assert nbc == r.count
    if phys:
        return
    nn = lat.num_nodes
    fluid = lat.node_type == 1
    assert np.array_equal((word & 1) == 1, fluid)
    stream = r.stream.reshape(lat.q - 1, nn)
    for d in range(1, lat.q):
        blocked = ((word >> d) & 1) == 1
        np.testing.assert_array_equal(blocked[fluid], (stream[d - 1] == 0)[fluid])


def test_physics_words_block_solid_and_outside(native_lib):
    lat = lattice.sphere_duct(20, 16, 32, porosity=0.8, rmin=3, rmax=4, seed=2)
    _, word, slot, _ = build_flags(lat, Arguments(mode=N.MODE_PHYSICS, collision_model=N.MRT,
                                                  inlet_profile=N.INLET_PRESSURE,
                                                  outlet_profile=N.OUTLET_PRESSURE))
    n, m, h = lat.n, lat.m, lat.h
    nt = lat.node_type.reshape(h, m, n)
    idx = np.arange(lat.num_nodes)
    x, y, z = idx % n, (idx // n) % m, idx // (n * m)
    for d in range(1, 19):
        sx, sy, sz = x - lattice.CX3[d], y - lattice.CY3[d], z - lattice.CZ3[d]
        out = (sx < 0) | (sx >= n) | (sy < 0) | (sy >= m) | (sz < 0) | (sz >= h)
        solid = np.zeros_like(out)
        ok = ~out
        solid[ok] = nt[sz[ok], sy[ok], sx[ok]] == 0
        expect = (out | solid) & (lat.node_type == 1)
        got = (((word >> d) & 1) == 1) & (lat.node_type == 1)
        np.testing.assert_array_equal(got, expect)
    # the pressure faces are the only special nodes
    special = ((word >> 19) & 1) == 1
    assert special.sum() > 0
    assert set(np.unique(z[special])) <= {0, h - 1}


def test_unsupported_reference_features_are_refused(native_lib):
    lat = lattice.cavity3d(6)
    with pytest.raises(N.LbmError) as e:
        build_flags(lat, Arguments(boundary_type=N.CURVED, mode=N.MODE_PHYSICS))
    assert e.value.code == N.LBM_ERR_UNSUPPORTED
    with pytest.raises(N.LbmError) as e:
        build_flags(lat, Arguments(boundary_type=7))
    assert e.value.code == N.LBM_ERR_INVALID
    bc = lat.bc.copy()
    bc[bc[:, 4] == 2, 4] = 3  # lid links become outlet links
    lat2 = lattice.Lattice(3, 6, 6, 6, lat.node_type, bc)
    with pytest.raises(N.LbmError) as e:
        build_flags(lat2, Arguments())
    assert e.value.code == N.LBM_ERR_UNSUPPORTED


def test_hh_walls_and_periodic_links_reference_mode(native_lib):
    """Reference mode takes the HH wall model (every boundary node gets a
    slot, so the wall kernel's face/edge/corner cases can run) and periodic
    links; physics mode refuses the HH model; 2D ignores it, as the
    reference's 2D loop does."""
    lat = lattice.cavity3d(7, 6, 5)
    mask, word, slot, nbc = build_flags(lat, Arguments(bc_wall_model=N.WALL_COMPLEX))
    special = ((word >> 19) & 1) == 1
    assert special.sum() == np.count_nonzero(mask) == nbc
    _, word_s, _, _ = build_flags(lat, Arguments())
    assert (((word_s >> 19) & 1) == 1).sum() < special.sum()
    with pytest.raises(N.LbmError) as e:
        build_flags(lat, Arguments(bc_wall_model=N.WALL_COMPLEX, mode=N.MODE_PHYSICS))
    assert e.value.code == N.LBM_ERR_UNSUPPORTED
    lat2 = lattice.cavity2d(8)
    w_hh = build_flags(lat2, Arguments(bc_wall_model=N.WALL_COMPLEX))[1]
    np.testing.assert_array_equal(w_hh, build_flags(lat2, Arguments())[1])
    per = lattice.periodic_channel3d(8, 7, 6)
    mask_p, word_p, _, _ = build_flags(per, Arguments())
    cycl = (mask_p >> np.uint64(54)) & np.uint64(4)
    assert np.all(((word_p >> 19) & 1)[cycl != 0] == 1)


def test_curved_walls_give_every_wall_node_a_slot(native_lib):
    """Reference curved walls: every fluid node with a wall link takes the
    boundary path (a slot), the masks stay the reference's; with the HH wall
    model the reference has no curved branch and the words equal the HH
    build's."""
    for lat in (lattice.cylinder_channel2d(32, 16), lattice.sphere_cavity3d(10, 9, 9)):
        mask, word, slot, nbc = build_flags(lat, Arguments(boundary_type=N.CURVED, outlet_profile=N.OUTLET_ZOUHE))
        mask_s, word_s, _, _ = build_flags(lat, Arguments(outlet_profile=N.OUTLET_ZOUHE))
        np.testing.assert_array_equal(mask, mask_s)
        special = ((word >> 19) & 1) == 1
        bits, wall = (2, 1) if lat.dims == 2 else (3, 1)
        has_wall = np.zeros(lat.num_nodes, bool)
        for d in range(1, lat.q):
            t = (mask >> np.uint64((d - 1) * bits)) & np.uint64((1 << bits) - 1)
            has_wall |= t == wall
        fluid = lat.node_type == 1
        assert np.all(special[has_wall & fluid])
        assert special.sum() > (((word_s >> 19) & 1) == 1).sum()
        assert np.all(slot[special] >= 0)
    lat = lattice.sphere_cavity3d(10, 9, 9)
    w_hh = build_flags(lat, Arguments(boundary_type=N.CURVED, bc_wall_model=N.WALL_COMPLEX))[1]
    np.testing.assert_array_equal(w_hh, build_flags(lat, Arguments(bc_wall_model=N.WALL_COMPLEX))[1])


def test_link_q_from_coordinates(native_lib, oracle):
    """lbm_link_q restates the reference's q = |B - X| / (delta |c_dir|)
    (GpuInit.cu:1086-1088, :1203-1207) in FP64: the fractions of BC points
    placed at q along each link come back to FP32 coordinate rounding."""
    from thesis_gb300.solver import link_q
    for lat, delta in ((lattice.cylinder_channel2d(32, 16), 0.01), (lattice.sphere_cavity3d(10, 9, 9), 1 / 9)):
        bx, by, bz = oracle.curved_bc_points(lat, lat.link_q, delta)
        x, y, z = lat.coords(delta)
        cols = (np.stack([bx, by], 1), np.stack([x, y], 1)) if lat.dims == 2 else \
            (np.stack([bx, by, bz], 1), np.stack([x, y, z], 1))
        q = link_q(lat, cols[0], cols[1], delta)
        np.testing.assert_allclose(q, lat.link_q, atol=2e-5)
        np.testing.assert_allclose(q, oracle.reference_q(lat, lat.link_q, delta, fp64=False), rtol=1e-5, atol=1e-6)
    lat = lattice.cylinder_channel2d(32, 16)
    with pytest.raises(N.LbmError) as e:
        link_q(lat, np.zeros((lat.bc.shape[0], 2)), np.zeros((lat.num_nodes, 2)), 0.0)
    assert e.value.code == N.LBM_ERR_INVALID


def test_invalid_links_are_rejected(native_lib):
    lat = lattice.cavity2d(6)
    bc = lat.bc.copy()
    bc[0, 0] = 99
    with pytest.raises(N.LbmError) as e:
        build_flags(lattice.Lattice(2, 6, 6, 1, lat.node_type, bc), Arguments())
    assert e.value.code == N.LBM_ERR_INVALID


def test_reference_generator_mesh_masks(native_lib, oracle):
    import os
    from oracle.pyoracle import reference_file
    g = reference_file("Source code", "latticegen2_W8")
    if g is None or not os.path.exists(os.path.join(g, "lidvalidation_Node.dat")):
        pytest.skip("reference tree not mounted")
    g += os.sep
    lat = lattice.from_files(g + "lidvalidation_Node.dat", g + "lidvalidation_BC.dat")
    mask, _, _, _ = build_flags(lat, Arguments())
    ref = oracle.run_reference(lat, 0)
    np.testing.assert_array_equal(mask, ref.mask)
