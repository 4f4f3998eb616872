"""Parity of the kernel the duct benchmark times, on a lattice large enough
that its blocks cross many tiles and for hundreds of steps.

The autotuner keeps, on the 256x256x512 sphere-packed duct (F16S), the
storage-unit kernel walking 8 nodes along z with 64-thread blocks and a
20-blocks-per-SM register cap (THESIS_LBM_KERNEL=jithz8b64m20).  This test
pins that variant, a second z-walk shape and the z-walk that updates two
nodes at a time on packed FP32x2, on a 96x96x192 duct with the
benchmark's sphere radii (6-14 nodes), porosity 0.70, pressure faces and
tau 0.8, runs 300 steps and compares with the FP32 oracle run on the host
cores: F32 storage within 2e-5 absolute (populations, density, velocity),
F16S within 5e-3 relative L2 (velocity, rho - 1, f - w), the tolerances of
the other parity tests."""
import numpy as np
import pytest

from thesis_gb300 import lattice
from thesis_gb300 import native as N
from thesis_gb300.solver import Arguments, Solver

pytestmark = pytest.mark.gpu

DIMS = (96, 96, 192)
STEPS = 300
VARIANTS = ["jithz8b64m20", "jithz4b128m10", "jithz8b64m10q"]

_cache = {}


def _lattice():
    if "lat" not in _cache:
        _cache["lat"] = lattice.sphere_duct(*DIMS, porosity=0.70, rmin=6.0, rmax=14.0, seed=11)
    return _cache["lat"]


def _args(storage):
    return Arguments(viscosity=(0.8 - 0.5) / 3, collision_model=N.MRT, mode=N.MODE_PHYSICS, storage=storage,
                     init_equilibrium=1, inlet_profile=N.INLET_PRESSURE, outlet_profile=N.OUTLET_PRESSURE,
                     rho_in=1.005, rho_out=1.0)


def _oracle(oracle):
    if "ref" not in _cache:
        lat = _lattice()
        a = _args(N.STORE_F32)
        nn = lat.num_nodes
        init = (np.ones(nn), np.zeros(nn), np.zeros(nn), np.zeros(nn))
        r = oracle.run_oracle(lat, STEPS, fp64=False, mode=a.mode, init_kind=1, rho_in=a.rho_in,
                              rho_out=a.rho_out, extra_collide=True, init=init, viscosity=a.viscosity,
                              collision_model=a.collision_model, inlet_profile=a.inlet_profile,
                              outlet_profile=a.outlet_profile)
        assert r.rc == 0
        _cache["ref"] = r
    return _cache["ref"]


@pytest.mark.parametrize("storage", [N.STORE_F32, N.STORE_F16S])
@pytest.mark.parametrize("variant", VARIANTS)
def test_bench_kernel_matches_oracle_at_scale(oracle, monkeypatch, variant, storage):
    from test_gpu_parity import compare
    monkeypatch.setenv("THESIS_LBM_KERNEL", variant)
    lat = _lattice()
    nn = lat.num_nodes
    with Solver(lat, _args(storage)) as s:
        assert N.lib().lbm_kernel_variant(s._h) == 4
        block, hint, pred = s.kernel_config()
        zw = int(variant[5])
        assert hint >> 2 == zw and block == int(variant.split("b")[1].split("m")[0])
        assert (pred >> 10) & 1 == ("q" in variant)
        s.init(np.ones(nn), np.zeros(nn), np.zeros(nn), np.zeros(nn))
        s.step(STEPS, write_macro=True)
        rho, u, v, w = s.macro()
        f = s.populations()
    r = _oracle(oracle)
    g = dict(rho=rho.astype(np.float64), u=u.astype(np.float64), v=v.astype(np.float64),
             w=w.astype(np.float64), f=f)
    errs = compare(g, r, lat.node_type == 1, storage, 3)
    print("%s %s: %s" % (variant, "F32" if storage == N.STORE_F32 else "F16S",
                         ", ".join("%s %.2e" % kv for kv in errs.items())))
