"""Lattice generator (lbm_latticegen) against the reference generator: the
Node and BC files must be byte-identical.  Hashes of the reference's output
for this project's geometries are committed (tests/golden/
latticegen_golden.json); where the reference tree is mounted, its own golden
lid-cavity files and its generator are compared directly too.  No GPU."""
import filecmp
import json
import os
import subprocess
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
import latticegen_cases as LC  # noqa: E402

from thesis_gb300 import lattice  # noqa: E402

from oracle.pyoracle import reference_file  # noqa: E402

REF_TREE = reference_file("Source code", "latticegen2_W8") or "reference tree not mounted"


@pytest.mark.parametrize("case", LC.CASES, ids=lambda c: "%s_%d_%d" % c)
def test_generator_matches_reference_hashes(native_lib, tmp_path, case):
    name, n, mode = case
    golden = json.load(open(LC.GOLDEN))["%s_%d_%d" % case]
    prefix, seed = LC.write_geometry(str(tmp_path), name)
    node, bc, dims = lattice.generate(prefix + ".vrt", prefix + ".bnd", n, seed, mode,
                                      str(tmp_path / ("out_%d_%d" % (n, mode))))
    assert LC.sha(node) == golden["node_sha256"]
    assert LC.sha(bc) == golden["bc_sha256"]


def test_generated_lattice_loads_and_has_links(native_lib, tmp_path):
    prefix, seed = LC.write_geometry(str(tmp_path), "duct_obstacle")
    node, bc, dims = lattice.generate(prefix + ".vrt", prefix + ".bnd", 21, seed, 1, str(tmp_path / "o"))
    lat = lattice.from_files(node, bc)
    assert (lat.n, lat.m, lat.h) == dims
    assert lat.bc.shape[0] > 0
    types = set(np.unique(lat.bc[:, 4]))
    assert {1, 2, 3} <= types
    # the obstacle is solid
    assert lat.num_fluid < lat.num_nodes


def test_bad_geometry_is_an_error_not_a_crash(native_lib, tmp_path):
    v, f = lattice.box_geometry((0, 0, 0), (1, 1, 1), {})
    f[0] = ((1, 2, 3, 99), 1, "WALL")  # vertex 99 does not exist
    lattice.write_starcd(str(tmp_path / "bad"), v, f)
    from thesis_gb300 import native as N
    with pytest.raises(N.LbmError):
        lattice.generate(str(tmp_path / "bad.vrt"), str(tmp_path / "bad.bnd"), 8, (0.5, 0.5, 0.5), 1,
                         str(tmp_path / "o"))


@pytest.mark.skipif(not os.path.isdir(REF_TREE), reason="reference tree not mounted")
@pytest.mark.parametrize("mode", [1, 2])
def test_reference_golden_lid_cavity(native_lib, tmp_path, mode):
    """latticegen2_W8/lidvalidation_{Node,BC}.dat, reproduced byte for byte."""
    g = os.path.join(REF_TREE, "STARCDfiles", "lid3D")
    node, bc, _ = lattice.generate(g + ".vrt", g + ".bnd", 30, (0.5, 0.5, 0.5), mode, str(tmp_path / "lid"))
    assert filecmp.cmp(node, os.path.join(REF_TREE, "lidvalidation_Node.dat"), shallow=False)
    assert filecmp.cmp(bc, os.path.join(REF_TREE, "lidvalidation_BC.dat"), shallow=False)


@pytest.mark.skipif(not (os.path.isdir(REF_TREE) and os.path.exists(os.path.join(
    LC.ROOT, "oracle", "_ref", "latticegen"))), reason="reference generator not built")
@pytest.mark.parametrize("geom,seed", [("rLid3D", (0.513, 1.507, 0.511)), ("channel_8", (4.013, 0.007, 0.011)),
                                       ("channel3D_4", (2.013, 0.007, 0.011)),
                                       ("ChannelWithObj", (4.013, 0.507, 0.511))])
def test_reference_geometries_vs_reference_generator(native_lib, tmp_path, geom, seed):
    ref = os.path.join(LC.ROOT, "oracle", "_ref", "latticegen")
    os.symlink(os.path.join(REF_TREE, "STARCDfiles"), tmp_path / "STARCDfiles")
    for mode in (1, 2):
        subprocess.run([ref, geom, "17", *map(repr, seed), "ref", str(mode)], cwd=tmp_path, check=True,
                       stdout=subprocess.DEVNULL)
        g = os.path.join(REF_TREE, "STARCDfiles", geom)
        node, bc, _ = lattice.generate(g + ".vrt", g + ".bnd", 17, seed, mode, str(tmp_path / "ours"))
        assert filecmp.cmp(node, tmp_path / "ref_Node.dat", shallow=False)
        assert filecmp.cmp(bc, tmp_path / "ref_BC.dat", shallow=False)
