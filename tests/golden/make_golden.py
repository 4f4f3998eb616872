"""Generate tests/golden/reference_runs.npz from the reference's own kernels.

Runs the reference solver's kernels compiled for the host (oracle/_ref, built
by oracle/build_ref.sh from the reference tree) on lattices from
thesis_gb300.lattice and stores their outputs, so machines without the
reference tree can still pin the oracle.  Usage:
    oracle/build_ref.sh && python tests/golden/make_golden.py [--cavity128]
"""
import hashlib
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import pyoracle  # noqa: E402
from thesis_gb300 import lattice  # noqa: E402


def cases():
    """(name, lattice builder args, run kwargs, steps)."""
    out = []
    for coll, tag in ((1, "bgk"), (2, "trt"), (3, "mrt")):
        out.append(("cav2d_16_" + tag, ("cavity2d", (16, 16)),
                    dict(u=0.1, viscosity=0.128, collision_model=coll, outlet_profile=1), 25))
    for coll, tag in ((1, "bgk"), (3, "mrt")):
        out.append(("cav3d_10x9x8_" + tag, ("cavity3d", (10, 9, 8)),
                    dict(u=0.05, viscosity=0.1, collision_model=coll), 12))
    out.append(("cav2d_40x24_bgk_long", ("cavity2d", (40, 24)),
                dict(u=0.1, viscosity=0.05, collision_model=1, outlet_profile=1), 200))
    # HH walls (gpuBcComplexWall3D) and periodic copies (gpuBcPeriodic3D)
    for coll, tag in ((1, "bgk"), (3, "mrt")):
        out.append(("hh_cav3d_10x9x8_" + tag, ("cavity3d", (10, 9, 8)),
                    dict(u=0.05, viscosity=0.1, collision_model=coll, bc_wall_model=2), 12))
    out.append(("per_x_chan3d_10x9x8_bgk", ("periodic_channel3d", (10, 9, 8)),
                dict(u=0.05, viscosity=0.1, collision_model=1), 12))
    out.append(("per_x_chan3d_10x9x8_hh_mrt", ("periodic_channel3d", (10, 9, 8)),
                dict(u=0.05, viscosity=0.1, collision_model=3, bc_wall_model=2), 12))
    # curved (q-interpolated) walls: BC points at the exact cylinder / sphere
    # intersections, q = 0.3 on the outer walls
    for coll, tag in ((1, "bgk"), (2, "trt"), (3, "mrt")):
        out.append(("curved_cyl2d_48x24_" + tag, ("cylinder_channel2d", (48, 24, None, None, 0.3)),
                    dict(u=0.05, viscosity=0.05, collision_model=coll, outlet_profile=1, boundary_type=1), 30))
    for coll, tag in ((1, "bgk"), (3, "mrt")):
        out.append(("curved_sph3d_14x12x12_" + tag, ("sphere_cavity3d", (14, 12, 12, None, None, 0.3)),
                    dict(u=0.05, viscosity=0.1, collision_model=coll, boundary_type=1), 12))
    # 2D extrapolation outlets (second and first order) and HEmodel, which the
    # 2D outlet kernel has no case for
    for prof, ptag, coll, tag, bt in ((2, "2nd", 1, "bgk", 2), (3, "1st", 3, "mrt", 2), (4, "he", 2, "trt", 2),
                                      (2, "2nd_curved", 3, "mrt", 1)):
        out.append(("outlet%s_cyl2d_48x24_%s" % (ptag, tag), ("cylinder_channel2d", (48, 24, None, None, 0.3)),
                    dict(u=0.05, viscosity=0.05, collision_model=coll, outlet_profile=prof, boundary_type=bt), 40))
    return out


def link_q_kwargs(lat, kw, oracle_side, fp64=False):
    """Curved cases: the reference gets the BC points of lat.link_q, the
    oracle the fractions the reference computes from them."""
    if kw.get("boundary_type") != 1:
        return {}
    if oracle_side:
        return dict(link_q=pyoracle.reference_q(lat, lat.link_q, fp64=fp64))
    return dict(link_q=lat.link_q)


def make_lattice(spec):
    name, args = spec
    return getattr(lattice, name)(*args)


def bc_hash(lat):
    extra = np.ascontiguousarray(lat.link_q).tobytes() if hasattr(lat, "link_q") else b""
    return hashlib.sha256(np.ascontiguousarray(lat.bc).tobytes() + lat.node_type.tobytes() + extra).hexdigest()


def main():
    if pyoracle.ref_lib() is None:
        sys.exit("oracle/_ref not built; run oracle/build_ref.sh first")
    store = {}
    for name, spec, kw, steps in cases():
        lat = make_lattice(spec)
        r = pyoracle.run_reference(lat, steps, fp64=False, **kw, **link_q_kwargs(lat, kw, False))
        assert r.rc == 0, name
        store[name + "/f"] = r.f.astype(np.float32)
        store[name + "/fc"] = r.fc.astype(np.float32)
        for k in ("rho", "u", "v", "w"):
            store[name + "/" + k] = getattr(r, k).astype(np.float32)
        store[name + "/mask"] = r.mask
        store[name + "/stream"] = r.stream
        store[name + "/resid"] = r.resid[:steps]
        store[name + "/lattice_sha256"] = np.frombuffer(bc_hash(lat).encode(), np.uint8)
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_runs.npz")
    np.savez_compressed(path, **store)
    print("wrote", path, os.path.getsize(path), "bytes")


def main_cavity128():
    """The D2Q9 BGK lid-driven cavity 128x128, u_lid 0.1, Re 100
    (nu = 0.128), 20,000 steps, FP32, by the reference's kernels; the final
    rho, u, v and the centre lines go to cavity128_bgk_20000.npz."""
    if pyoracle.ref_lib() is None:
        sys.exit("oracle/_ref not built; run oracle/build_ref.sh first")
    lat = lattice.cavity2d(128)
    steps = 20000
    r = pyoracle.run_reference(lat, steps, fp64=False, u=0.1, viscosity=0.128, collision_model=1, outlet_profile=1)
    assert r.rc == 0
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "cavity128_bgk_20000.npz")
    np.savez_compressed(path, rho=r.rho.astype(np.float32), u=r.u.astype(np.float32), v=r.v.astype(np.float32),
                        resid=r.resid[-100:], steps=np.int64(steps),
                        lattice_sha256=np.frombuffer(bc_hash(lat).encode(), np.uint8))
    print("wrote", path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    if "--cavity128" in sys.argv:
        main_cavity128()
    else:
        main()
