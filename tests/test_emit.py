"""Lattice emitters (lattice_emit.cpp): the sphere-packed duct, the obstacle
channel and the cavities written as reference-format Node and BC files by
the library equal, byte for byte, the files the Python builders
(thesis_gb300/lattice.py, which draw the same SplitMix64 sequence) write for
the same lattice, and the library's readers turn them back into the same
flags and BC links.  CPU only: nothing here touches a GPU."""
import ctypes as C
import filecmp

import numpy as np
import pytest

from thesis_gb300 import lattice


def _same_lattice(a, b):
    assert (a.dims, a.n, a.m, a.h) == (b.dims, b.n, b.m, b.h)
    np.testing.assert_array_equal(a.node_type, b.node_type)
    np.testing.assert_array_equal(a.bc, b.bc)


def test_splitmix64_known_values():
    # SplitMix64 from seed 0: the published first outputs of the generator
    g = lattice.SplitMix64(0)
    assert [g.next() for _ in range(3)] == [0xE220A8397B1DCDAF, 0x6E789E6AA1B965F4, 0x06C45D188009454F]


@pytest.mark.parametrize("dims,porosity,rmin,rmax,seed", [((24, 20, 40), 0.75, 3.0, 5.0, 7),
                                                          ((40, 32, 64), 0.70, 4.0, 9.0, 0),
                                                          ((30, 30, 48), 0.60, 2.0, 6.0, 12345)])
def test_pack_spheres_matches_python(native_lib, dims, porosity, rmin, rmax, seed):
    n, m, h = dims
    solid = np.zeros(n * m * h, np.uint8)
    sph = np.zeros((4096, 4))
    k = C.c_longlong(0)
    rc = native_lib.lbm_pack_spheres(n, m, h, porosity, rmin, rmax, seed, 2, 2.0, 2000000,
                                     solid.ctypes.data_as(C.c_void_p), sph.ctypes.data_as(C.c_void_p), 4096,
                                     C.byref(k))
    assert rc == 0
    want, spheres = lattice.pack_spheres((n, m, h), porosity, rmin, rmax, seed)
    np.testing.assert_array_equal(solid.reshape(h, m, n).astype(bool), want)
    np.testing.assert_array_equal(sph[:k.value], spheres)
    assert k.value > 3


def test_emit_sphere_duct_files(native_lib, tmp_path):
    n, m, h, seed = 24, 20, 40, 7
    node, bc = str(tmp_path / "duct_Node.dat"), str(tmp_path / "duct_BC.dat")
    k = C.c_longlong(0)
    assert native_lib.lbm_emit_sphere_duct(n, m, h, 0.75, 3.0, 5.0, seed, node.encode(), bc.encode(), C.byref(k)) == 0
    lat = lattice.sphere_duct(n, m, h, porosity=0.75, rmin=3.0, rmax=5.0, seed=seed)
    pnode, pbc = str(tmp_path / "py_Node.dat"), str(tmp_path / "py_BC.dat")
    lattice.write_files(lat, pnode, pbc)
    assert filecmp.cmp(node, pnode, shallow=False)
    assert filecmp.cmp(bc, pbc, shallow=False)
    _same_lattice(lattice.from_files_native(node, bc), lat)
    assert k.value == len(lat.spheres)


@pytest.mark.parametrize("n,m,seed,k,scale", [(256, 64, 3, -1, 0.25), (256, 64, 17, 6, 0.25),
                                              (1024, 256, 1, -1, 1.0)])
def test_emit_channel2d_files(native_lib, tmp_path, n, m, seed, k, scale):
    node, bc = str(tmp_path / "ch_Node.dat"), str(tmp_path / "ch_BC.dat")
    assert native_lib.lbm_emit_channel2d(n, m, seed, k, scale, node.encode(), bc.encode()) == 0
    lat = lattice.channel2d(n, m, seed=seed, n_obstacles=None if k < 0 else k, size_scale=scale)
    pnode, pbc = str(tmp_path / "py_Node.dat"), str(tmp_path / "py_BC.dat")
    lattice.write_files(lat, pnode, pbc)
    assert filecmp.cmp(node, pnode, shallow=False)
    assert filecmp.cmp(bc, pbc, shallow=False)
    _same_lattice(lattice.from_files_native(node, bc), lat)
    assert lat.num_fluid < n * m  # at least one obstacle


@pytest.mark.parametrize("dims,size", [(2, (33, 17, 1)), (3, (12, 10, 9))])
def test_emit_cavity_files(native_lib, tmp_path, dims, size):
    n, m, h = size
    node, bc = str(tmp_path / "cav_Node.dat"), str(tmp_path / "cav_BC.dat")
    assert native_lib.lbm_emit_cavity(dims, n, m, h, node.encode(), bc.encode()) == 0
    lat = lattice.cavity2d(n, m) if dims == 2 else lattice.cavity3d(n, m, h)
    pnode, pbc = str(tmp_path / "py_Node.dat"), str(tmp_path / "py_BC.dat")
    lattice.write_files(lat, pnode, pbc)
    assert filecmp.cmp(node, pnode, shallow=False)
    assert filecmp.cmp(bc, pbc, shallow=False)
    _same_lattice(lattice.from_files_native(node, bc), lat)


def test_emit_refuses_bad_arguments(native_lib, tmp_path):
    p = str(tmp_path / "x.dat").encode()
    assert native_lib.lbm_emit_cavity(4, 10, 10, 10, p, p) != 0
    assert b"invalid" in native_lib.lbm_emit_last_error()
    assert native_lib.lbm_emit_sphere_duct(1, 1, 1, 0.7, 3.0, 5.0, 0, p, p, None) != 0
