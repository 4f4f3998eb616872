"""STAR-CD geometries of this project for the lattice-generator parity tests
and the hashes of what the reference generator writes for them.

make_latticegen_golden() runs the reference generator (oracle/_ref/latticegen,
built from the reference tree by oracle/build_ref.sh) and stores sha256 hashes
of its Node and BC files in latticegen_golden.json.
"""
import hashlib
import json
import os
import subprocess
import sys
import tempfile

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from thesis_gb300 import lattice  # noqa: E402

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "latticegen_golden.json")


def geometries():
    """name -> (vertices, faces, seed)."""
    g = {}
    v, f = lattice.box_geometry((0, 0, 0), (1, 1, 1), {"z+": "INLE"})
    g["lid_box"] = (v, f, (0.503, 0.497, 0.511))
    v, f = lattice.box_geometry((0, -0.5, -0.5), (4, 0.5, 0.5), {"x-": "INLE", "x+": "OUTL"})
    g["duct"] = (v, f, (2.01, 0.013, -0.007))
    v, f = lattice.box_geometry((0, -0.5, -0.5), (4, 0.5, 0.5), {"x-": "INLE", "x+": "OUTL"})
    v2, f2 = lattice.box_geometry((1.5, -0.2, -0.25), (2.0, 0.2, 0.25), {}, first_vertex=9, first_bcid=7)
    g["duct_obstacle"] = (v + v2, f + f2, (0.71, 0.013, -0.007))
    v, f = lattice.box_geometry((0, 0, 0), (1, 2, 1), {"x-": "CYCL", "x+": "CYCL", "z+": "SYMP"})
    g["periodic_box"] = (v, f, (0.51, 1.03, 0.49))
    return g


CASES = [(name, n, mode) for name in ("lid_box", "duct", "duct_obstacle", "periodic_box")
         for n in (8, 13, 21) for mode in (1, 2)]


def write_geometry(dirname, name):
    v, f, seed = geometries()[name]
    prefix = os.path.join(dirname, name)
    lattice.write_starcd(prefix, v, f)
    return prefix, seed


def sha(path):
    return hashlib.sha256(open(path, "rb").read()).hexdigest()


def make_latticegen_golden():
    ref = os.path.join(ROOT, "oracle", "_ref", "latticegen")
    if not os.path.exists(ref):
        sys.exit("oracle/_ref/latticegen not built")
    out = {}
    with tempfile.TemporaryDirectory() as d:
        os.makedirs(os.path.join(d, "STARCDfiles"))
        for name in geometries():
            write_geometry(os.path.join(d, "STARCDfiles"), name)
        for name, n, mode in CASES:
            seed = geometries()[name][2]
            tag = "%s_%d_%d" % (name, n, mode)
            subprocess.run([ref, name, str(n), repr(seed[0]), repr(seed[1]), repr(seed[2]), tag, str(mode)],
                           cwd=d, check=True, stdout=subprocess.DEVNULL)
            out[tag] = {"node_sha256": sha(os.path.join(d, tag + "_Node.dat")),
                        "bc_sha256": sha(os.path.join(d, tag + "_BC.dat"))}
    with open(GOLDEN, "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)
    print("wrote", GOLDEN, len(out), "cases")


if __name__ == "__main__":
    make_latticegen_golden()
