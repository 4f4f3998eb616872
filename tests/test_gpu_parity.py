"""CUDA time step (through the C ABI) against the CPU oracle on the same
seeded inputs.

Tolerances (stated per storage type):
  * F64 storage vs the FP64 oracle: 1e-10 absolute on populations (FP64
    arithmetic in a different operation order); the macroscopic fields are
    returned as FP32, so 3e-7 absolute on them.
  * F32 storage vs the FP32 oracle: 2e-5 absolute on populations, density and
    velocity (FP32 with fused multiply-adds and another summation order; the
    oracle follows the reference's expression order without contraction).
  * F16S storage vs the FP32 oracle: relative L2 errors of 5e-3 on the
    velocity, on the density deviation rho - 1 and on the post-collision
    deviation f - w (half precision keeps 11 bits of the deviation from the
    collision model's rest state).
The GPU state after k steps is the post-collision field the next step
streams, i.e. the oracle's state after k steps followed by one collision.
"""
import dataclasses

import numpy as np
import pytest

from thesis_gb300 import lattice
from thesis_gb300 import native as N
from thesis_gb300.solver import Arguments, Solver

pytestmark = pytest.mark.gpu

TOL = {N.STORE_F64: 1e-10, N.STORE_F32: 2e-5}


def run_pair(oracle, lat, args, steps, init=None, link_q=None):
    """Run GPU and oracle; return (gpu dict, oracle Result).  link_q: the
    curved walls' link fractions (boundary_type CURVED)."""
    fluid = lat.node_type == 1
    with Solver(lat, args) as s:
        if link_q is not None:
            s.set_link_q(link_q)
        if init is not None:
            s.init(*init)
        else:
            s.init()
        s.step(steps, write_macro=True)
        rho, u, v, w = s.macro()
        f = s.populations()
    okw = dict(u=args.u, v=args.v, w=args.w, rho=args.rho, viscosity=args.viscosity, g=args.g,
               inlet_profile=args.inlet_profile, outlet_profile=args.outlet_profile,
               collision_model=args.collision_model, update_inlet_outlet=args.update_inlet_outlet,
               bc_wall_model=args.bc_wall_model, boundary_type=args.boundary_type)
    r = oracle.run_oracle(lat, steps, fp64=args.storage == N.STORE_F64, mode=args.mode,
                          init_kind=args.init_equilibrium, rho_in=args.rho_in, rho_out=args.rho_out,
                          extra_collide=True, init=init, periodic=args.periodic, link_q=link_q, **okw)
    assert r.rc == 0
    g = dict(rho=rho.astype(np.float64), u=u.astype(np.float64), v=v.astype(np.float64),
             w=w.astype(np.float64), f=f)
    return g, r, fluid


def compare(g, r, fluid, storage, dims):
    errs = {}
    keys = ["rho", "u", "v"] + (["w"] if dims == 3 else [])
    for k in keys:
        a, b = g[k][fluid], getattr(r, k)[fluid]
        errs[k] = float(np.abs(a - b).max())
    errs["f"] = float(np.abs(g["f"][:, fluid] - r.fc[:, fluid]).max())
    if storage in (N.STORE_F16S, N.STORE_F16C):
        vel = ["u", "v"] + (["w"] if dims == 3 else [])
        du = np.sqrt(sum(((g[k] - getattr(r, k))[fluid] ** 2).sum() for k in vel))
        uu = np.sqrt(sum((getattr(r, k)[fluid] ** 2).sum() for k in vel))
        drho = np.linalg.norm((g["rho"] - r.rho)[fluid]) / max(np.linalg.norm((r.rho - 1)[fluid]), 1e-12)
        w = (lattice.W2 if dims == 2 else lattice.W3)[:, None]
        df = np.linalg.norm(g["f"][:, fluid] - r.fc[:, fluid]) / np.linalg.norm(r.fc[:, fluid] - w)
        rel = {"u": du / max(uu, 1e-12), "rho-1": drho, "f-w": df}
        bad = {k: v for k, v in rel.items() if v > 5e-3}
        errs = rel
    elif storage == N.STORE_F64:
        bad = {k: v for k, v in errs.items() if v > (TOL[storage] if k == "f" else 3e-7)}
    else:
        bad = {k: v for k, v in errs.items() if v > TOL[storage]}
    assert not bad, (bad, errs)
    return errs


@pytest.mark.parametrize("coll", [N.BGKW, N.TRT, N.MRT])
def test_reference_cavity2d(oracle, coll):
    lat = lattice.cavity2d(32, 24)
    args = Arguments(u=0.1, viscosity=0.128, collision_model=coll, outlet_profile=N.OUTLET_ZOUHE)
    g, r, fl = run_pair(oracle, lat, args, 60)
    compare(g, r, fl, N.STORE_F32, 2)


@pytest.mark.parametrize("coll", [N.BGKW, N.MRT])
def test_reference_cavity2d_fp64(oracle, coll):
    lat = lattice.cavity2d(20)
    args = Arguments(u=0.1, viscosity=0.128, collision_model=coll, storage=N.STORE_F64,
                     outlet_profile=N.OUTLET_ZOUHE)
    g, r, fl = run_pair(oracle, lat, args, 40)
    compare(g, r, fl, N.STORE_F64, 2)


@pytest.mark.parametrize("coll", [N.BGKW, N.MRT])
def test_reference_cavity3d(oracle, coll):
    lat = lattice.cavity3d(12, 10, 9)
    args = Arguments(u=0.05, viscosity=0.1, collision_model=coll)
    g, r, fl = run_pair(oracle, lat, args, 25)
    compare(g, r, fl, N.STORE_F32, 3)


REF3_CASES = {
    "hh_cavity": (lambda: lattice.cavity3d(14, 12, 10), N.WALL_COMPLEX),
    "periodic_x": (lambda: lattice.periodic_channel3d(14, 12, 10), N.WALL_SIMPLE),
    "periodic_x_hh": (lambda: lattice.periodic_channel3d(14, 12, 10), N.WALL_COMPLEX),
    "periodic_xy_hh": (lambda: lattice.periodic_channel3d(14, 12, 10, periodic_axes=(0, 1)), N.WALL_COMPLEX),
}


@pytest.mark.parametrize("case", sorted(REF3_CASES))
@pytest.mark.parametrize("coll", [N.BGKW, N.MRT])
@pytest.mark.parametrize("storage", [N.STORE_F32, N.STORE_F64])
def test_reference_hh_walls_and_periodic_copies(oracle, case, coll, storage):
    """The reference's HH wall (faces, edges, corners) and its 3D periodic
    copies from the opposite face, against the oracle (which matches the
    reference's kernels bit for bit on these lattices, one periodic axis)."""
    make, wm = REF3_CASES[case]
    # equilibrium start: from the reference's zero populations the density
    # passes near 0 at some nodes and u = j / rho magnifies FP32 rounding
    args = Arguments(u=0.05, viscosity=0.1, collision_model=coll, bc_wall_model=wm, storage=storage,
                     init_equilibrium=1)
    g, r, fl = run_pair(oracle, make(), args, 20)
    compare(g, r, fl, storage, 3)


@pytest.mark.parametrize("variant", ["pair", "jith", "jiths", "scalar", "jit2"])
def test_reference_periodic_hh_every_kernel_form(oracle, monkeypatch, variant):
    """Partner pulls and HH walls are shared by the one-node, storage-unit and
    two-node kernels."""
    monkeypatch.setenv("THESIS_LBM_KERNEL", variant)
    args = Arguments(u=0.05, viscosity=0.1, collision_model=N.MRT, bc_wall_model=N.WALL_COMPLEX,
                     init_equilibrium=1)
    g, r, fl = run_pair(oracle, lattice.periodic_channel3d(14, 12, 10), args, 20)
    monkeypatch.delenv("THESIS_LBM_KERNEL", raising=False)
    compare(g, r, fl, N.STORE_F32, 3)


CURVED_CASES = {
    "cylinder2d": lambda: lattice.cylinder_channel2d(48, 24, outer_q=0.3),
    "sphere3d": lambda: lattice.sphere_cavity3d(14, 12, 12, outer_q=0.3),
}


@pytest.mark.parametrize("case", sorted(CURVED_CASES))
@pytest.mark.parametrize("coll", [N.BGKW, N.TRT, N.MRT])
@pytest.mark.parametrize("storage", [N.STORE_F32, N.STORE_F64, N.STORE_F16S])
def test_reference_curved_walls(oracle, case, coll, storage):
    """The reference's q-interpolated walls (both branches, q from the exact
    cylinder / sphere intersections, q = 0.3 on the outer walls) against the
    oracle, which matches the reference's kernels bit for bit on these
    lattices."""
    lat = CURVED_CASES[case]()
    if lat.dims == 3 and coll == N.TRT:
        pytest.skip("the reference has no 3D TRT")
    args = Arguments(u=0.05, viscosity=0.05 if lat.dims == 2 else 0.1, collision_model=coll,
                     outlet_profile=N.OUTLET_ZOUHE, boundary_type=N.CURVED, storage=storage,
                     init_equilibrium=1)
    g, r, fl = run_pair(oracle, lat, args, 30, link_q=lat.link_q)
    compare(g, r, fl, storage, lat.dims)


@pytest.mark.parametrize("variant", ["jith", "jiths", "jitf", "scalar", "jithz4", "pair"])
def test_reference_curved_walls_every_kernel_form(oracle, monkeypatch, variant):
    """The interpolation runs in the shared boundary code of the one-node
    f-space, storage-unit and z-walk kernels; the two-node kernels have no
    curved path, so a request for them falls back to a one-node kernel."""
    monkeypatch.setenv("THESIS_LBM_KERNEL", variant)
    lat = CURVED_CASES["sphere3d"]()
    args = Arguments(u=0.05, viscosity=0.1, collision_model=N.MRT, boundary_type=N.CURVED, init_equilibrium=1)
    g, r, fl = run_pair(oracle, lat, args, 20, link_q=lat.link_q)
    monkeypatch.delenv("THESIS_LBM_KERNEL", raising=False)
    compare(g, r, fl, N.STORE_F32, 3)


def test_reference_curved_walls_default_q_and_update(oracle):
    """Before lbm_set_link_q every fraction is 1/2 (the reference's fill
    value); new fractions take effect from the next step."""
    lat = CURVED_CASES["cylinder2d"]()
    args = Arguments(u=0.05, viscosity=0.05, collision_model=N.BGKW, outlet_profile=N.OUTLET_ZOUHE,
                     boundary_type=N.CURVED, init_equilibrium=1)
    g, r, fl = run_pair(oracle, lat, args, 20)
    compare(g, r, fl, N.STORE_F32, 2)
    half = np.full(lat.bc.shape[0], 0.5)
    with Solver(lat, args) as s:
        s.set_link_q(half)
        s.init()
        s.step(20, write_macro=True)
        fa = s.populations()
    assert np.array_equal(fa, g["f"])
    with Solver(lat, dataclasses.replace(args, boundary_type=N.STRAIGHT)) as s:
        s.init()
        s.step(20, write_macro=True)
        fs = s.populations()
    # q = 1/2 returns the node's own post-collision population, the straight
    # wall the streamed one
    assert np.abs(fs - fa).max() > 1e-4


def test_reference_curved_walls_l2_residual(oracle):
    """The L2 residual recomputes the boundary conditions, curved walls
    included."""
    lat = CURVED_CASES["cylinder2d"]()
    args = Arguments(u=0.05, viscosity=0.05, collision_model=N.MRT, outlet_profile=N.OUTLET_ZOUHE,
                     boundary_type=N.CURVED, init_equilibrium=1)
    k = 30
    with Solver(lat, args) as s:
        s.set_link_q(lat.link_q)
        s.init()
        s.step(k, write_macro=True)
        r_gpu, rc = s.residual_l2()
        assert rc == N.LBM_OK
    r = oracle.run_oracle(lat, k + 1, init_kind=1, link_q=lat.link_q, u=args.u, viscosity=args.viscosity,
                          outlet_profile=args.outlet_profile, collision_model=args.collision_model,
                          boundary_type=N.CURVED)
    assert r.rc == 0
    assert abs(r_gpu - r.resid[k]) <= 1e-4 * r.resid[k] + 1e-6, (r_gpu, r.resid[k])


@pytest.mark.parametrize("profile", [N.OUTLET_SECOND, N.OUTLET_FIRST, N.OUTLET_HEMODEL])
@pytest.mark.parametrize("boundary", [N.STRAIGHT, N.CURVED])
@pytest.mark.parametrize("storage", [N.STORE_F32, N.STORE_F64])
def test_reference_extrapolation_outlets_2d(oracle, profile, boundary, storage):
    """The reference's 2D east outlets: second- and first-order
    extrapolation of f1, f5, f8 from the post-stream, post-wall values of the
    two western neighbours (recomputed by the outlet node's thread), and
    HEmodel, which the 2D outlet kernel leaves without a case."""
    lat = CURVED_CASES["cylinder2d"]()
    args = Arguments(u=0.05, viscosity=0.05, collision_model=N.MRT, outlet_profile=profile,
                     boundary_type=boundary, storage=storage, init_equilibrium=1)
    g, r, fl = run_pair(oracle, lat, args, 40, link_q=lat.link_q if boundary == N.CURVED else None)
    compare(g, r, fl, storage, 2)


@pytest.mark.parametrize("variant", ["jith", "scalar", "pair", "jit2"])
def test_reference_extrapolation_outlet_kernel_forms(oracle, monkeypatch, variant):
    monkeypatch.setenv("THESIS_LBM_KERNEL", variant)
    lat = CURVED_CASES["cylinder2d"]()
    args = Arguments(u=0.05, viscosity=0.05, collision_model=N.BGKW, outlet_profile=N.OUTLET_SECOND,
                     init_equilibrium=1)
    g, r, fl = run_pair(oracle, lat, args, 30)
    monkeypatch.delenv("THESIS_LBM_KERNEL", raising=False)
    compare(g, r, fl, N.STORE_F32, 2)


def test_reference_cavity3d_gravity_no_inlet_update(oracle):
    lat = lattice.cavity3d(9, 8, 7)
    args = Arguments(u=0.05, viscosity=0.1, collision_model=N.BGKW, g=1e-5, update_inlet_outlet=0)
    g, r, fl = run_pair(oracle, lat, args, 15)
    compare(g, r, fl, N.STORE_F32, 3)


@pytest.mark.parametrize("coll", [N.BGKW, N.TRT, N.MRT])
@pytest.mark.parametrize("storage", [N.STORE_F32, N.STORE_F64])
def test_physics_cavity2d(oracle, coll, storage):
    lat = lattice.cavity2d(32)
    args = Arguments(u=0.1, viscosity=0.128, collision_model=coll, mode=N.MODE_PHYSICS,
                     storage=storage, init_equilibrium=1, outlet_profile=N.OUTLET_ZOUHE)
    nn = lat.num_nodes
    init = (np.ones(nn), np.zeros(nn), np.zeros(nn), np.zeros(nn))
    g, r, fl = run_pair(oracle, lat, args, 80, init=init)
    compare(g, r, fl, storage, 2)


@pytest.mark.parametrize("coll", [N.BGKW, N.TRT, N.MRT])
@pytest.mark.parametrize("storage", [N.STORE_F32, N.STORE_F64, N.STORE_F16S])
def test_physics_sphere_duct(oracle, coll, storage):
    lat = lattice.sphere_duct(24, 20, 48, porosity=0.75, rmin=3, rmax=5, seed=7)
    args = Arguments(viscosity=(0.8 - 0.5) / 3, collision_model=coll, mode=N.MODE_PHYSICS,
                     storage=storage, init_equilibrium=1, inlet_profile=N.INLET_PRESSURE,
                     outlet_profile=N.OUTLET_PRESSURE, rho_in=1.005, rho_out=1.0)
    nn = lat.num_nodes
    init = (np.ones(nn), np.zeros(nn), np.zeros(nn), np.zeros(nn))
    g, r, fl = run_pair(oracle, lat, args, 40, init=init)
    compare(g, r, fl, storage, 3)


def test_physics_channel2d_velocity_inlet_pressure_outlet(oracle):
    lat = lattice.channel2d(160, 48, seed=5)
    args = Arguments(u=0.05, viscosity=0.05, collision_model=N.TRT, mode=N.MODE_PHYSICS,
                     init_equilibrium=1, outlet_profile=N.OUTLET_PRESSURE, rho_out=1.0)
    nn = lat.num_nodes
    init = (np.ones(nn), np.zeros(nn), np.zeros(nn), np.zeros(nn))
    g, r, fl = run_pair(oracle, lat, args, 60, init=init)
    compare(g, r, fl, N.STORE_F32, 2)


def test_macro_norms_fp64(oracle):
    lat = lattice.sphere_duct(20, 16, 32, porosity=0.8, rmin=3, rmax=4, seed=3)
    args = Arguments(viscosity=0.1, collision_model=N.MRT, mode=N.MODE_PHYSICS, init_equilibrium=1,
                     inlet_profile=N.INLET_PRESSURE, outlet_profile=N.OUTLET_PRESSURE,
                     rho_in=1.01, rho_out=1.0)
    nn = lat.num_nodes
    fl = lat.node_type == 1
    with Solver(lat, args) as s:
        s.init(np.ones(nn), np.zeros(nn), np.zeros(nn), np.zeros(nn))
        s.step(10, write_macro=True)
        n0, rc = s.norms()
        assert rc == N.LBM_OK
        rho, u, v, w = [a.astype(np.float64) for a in s.macro()]
        assert n0[3] == fl.sum()
        np.testing.assert_allclose(n0[2], rho[fl].sum(), rtol=1e-12)
        np.testing.assert_allclose(n0[1], (u[fl] ** 2 + v[fl] ** 2 + w[fl] ** 2).sum(), rtol=1e-12)
        s.step(10, write_macro=True)
        n1, _ = s.norms()
        rho2, u2, v2, w2 = [a.astype(np.float64) for a in s.macro()]
        du = ((u2 - u)[fl] ** 2 + (v2 - v)[fl] ** 2 + (w2 - w)[fl] ** 2).sum()
        np.testing.assert_allclose(n1[0], du, rtol=1e-10)
        # deterministic: same inputs, same bits
        s.step(0, write_macro=False)
    with Solver(lat, args) as s2:
        s2.init(np.ones(nn), np.zeros(nn), np.zeros(nn), np.zeros(nn))
        s2.step(10, write_macro=True)
        m0, _ = s2.norms()
    assert np.array_equal(m0, n0)


def test_divergence_is_reported_not_fatal(oracle):
    """A blown-up run (host-seeded NaN in the initial density) is reported as
    LBM_DIVERGED by the FP64 norms and the handle stays usable."""
    lat = lattice.cavity2d(16)
    args = Arguments(u=0.1, viscosity=0.1, collision_model=N.BGKW, mode=N.MODE_PHYSICS, init_equilibrium=1)
    nn = lat.num_nodes
    rho = np.ones(nn)
    rho[nn // 2] = np.nan
    with Solver(lat, args) as s:
        s.init(rho, np.zeros(nn), np.zeros(nn), np.zeros(nn))
        s.step(5, write_macro=True)
        _, rc = s.norms()
        assert rc == N.LBM_DIVERGED
        assert s.status == N.LBM_DIVERGED
        s.init(np.ones(nn), np.zeros(nn), np.zeros(nn), np.zeros(nn))
        s.step(5, write_macro=True)
        _, rc = s.norms()
        assert rc == N.LBM_OK
        assert s.status == N.LBM_OK


def test_graph_path_matches_single_launches(oracle):
    """lbm_step replays a captured two-step graph for long runs; the result
    must equal step-by-step launches bit for bit."""
    lat = lattice.cavity2d(24)
    args = Arguments(u=0.1, viscosity=0.1, collision_model=N.MRT, mode=N.MODE_PHYSICS, init_equilibrium=1)
    nn = lat.num_nodes
    init = (np.ones(nn), np.zeros(nn), np.zeros(nn), np.zeros(nn))
    with Solver(lat, args) as a:
        a.init(*init)
        a.step(41, write_macro=True)
        fa = a.populations()
    with Solver(lat, args) as b:
        b.init(*init)
        for _ in range(40):
            b.step(1, write_macro=False)
        b.step(1, write_macro=True)
        fb = b.populations()
    assert np.array_equal(fa, fb)


@pytest.mark.parametrize("storage", [N.STORE_F32, N.STORE_F16S])
def test_pair_kernel_matches_single_node_kernel(oracle, monkeypatch, storage):
    """The two-node kernel (default for even n with F32 storage, selectable
    for F16S) and the one-node kernel give the same results within the
    storage's tolerance."""
    lat = lattice.sphere_duct(24, 20, 40, porosity=0.8, rmin=3, rmax=5, seed=11)
    nn = lat.num_nodes
    init = (np.ones(nn), np.zeros(nn), np.zeros(nn), np.zeros(nn))
    out = {}
    for variant in ("pair", "scalar"):
        monkeypatch.setenv("THESIS_LBM_KERNEL", variant)
        args = Arguments(viscosity=0.1, collision_model=N.MRT, mode=N.MODE_PHYSICS, init_equilibrium=1,
                         inlet_profile=N.INLET_PRESSURE, outlet_profile=N.OUTLET_PRESSURE, rho_in=1.01,
                         storage=storage)
        with Solver(lat, args) as s:
            assert N.lib().lbm_kernel_variant(s._h) == (2 if variant == "pair" else 1)
            s.init(*init)
            s.step(30, write_macro=True)
            out[variant] = (s.populations(), s.macro())
    monkeypatch.delenv("THESIS_LBM_KERNEL", raising=False)
    tol = TOL[N.STORE_F32] if storage == N.STORE_F32 else 2e-3
    assert np.abs(out["pair"][0] - out["scalar"][0]).max() < tol
    for a, b in zip(out["pair"][1], out["scalar"][1]):
        assert np.abs(a - b).max() < tol


@pytest.mark.parametrize("case", ["cavity2d_ref", "cavity3d_ref", "duct_phys"])
def test_reference_l2_residual(oracle, case):
    """lbm_residual_l2 (the reference's sqrt(sum (f - fColl)^2)) against the
    oracle's per-iteration residual, which follows computeResidual2D/3D."""
    if case == "cavity2d_ref":
        lat = lattice.cavity2d(32, 24)
        args = Arguments(u=0.1, viscosity=0.128, collision_model=N.MRT, outlet_profile=N.OUTLET_ZOUHE)
        init = None
    elif case == "cavity3d_ref":
        lat = lattice.cavity3d(12, 10, 9)
        args = Arguments(u=0.05, viscosity=0.1, collision_model=N.BGKW)
        init = None
    else:
        lat = lattice.sphere_duct(24, 20, 40, porosity=0.8, rmin=3, rmax=5, seed=3)
        args = Arguments(viscosity=0.1, collision_model=N.MRT, mode=N.MODE_PHYSICS, init_equilibrium=1,
                         inlet_profile=N.INLET_PRESSURE, outlet_profile=N.OUTLET_PRESSURE, rho_in=1.01)
        nn = lat.num_nodes
        init = (np.ones(nn), np.zeros(nn), np.zeros(nn), np.zeros(nn))
    k = 30
    with Solver(lat, args) as s:
        s.init(*init) if init is not None else s.init()
        s.step(k, write_macro=True)
        r_gpu, rc = s.residual_l2()
        assert rc == N.LBM_OK
    okw = dict(u=args.u, v=args.v, w=args.w, rho=args.rho, viscosity=args.viscosity,
               inlet_profile=args.inlet_profile, outlet_profile=args.outlet_profile,
               collision_model=args.collision_model)
    r = oracle.run_oracle(lat, k + 1, mode=args.mode, init_kind=args.init_equilibrium, rho_in=args.rho_in,
                          rho_out=args.rho_out, init=init, **okw)
    assert r.rc == 0
    assert abs(r_gpu - r.resid[k]) <= 1e-4 * r.resid[k] + 1e-6, (r_gpu, r.resid[k])


@pytest.mark.parametrize("storage", [N.STORE_F64, N.STORE_F32])
def test_reference_fd_rel_diff_residual(oracle, storage):
    """lbm_residual_fd_rel_diff (the reference's max |f - f_prev| / f_first)
    against the same maximum over the oracle's post-stream fields.  The GPU
    state after k steps streams into the oracle's field after k + 1 steps."""
    lat = lattice.cavity3d(12, 10, 9)
    args = Arguments(u=0.05, viscosity=0.1, collision_model=N.MRT, storage=storage, init_equilibrium=1)
    okw = dict(u=args.u, viscosity=args.viscosity, collision_model=args.collision_model)
    ks = [10, 25, 45]
    got = []
    with Solver(lat, args) as s:
        s.init()
        done = 0
        for k in ks:
            s.step(k - done, write_macro=True)
            done = k
            got.append(s.residual_fd_rel_diff())
    fl = lat.node_type == 1
    snaps = [oracle.run_oracle(lat, k + 1, fp64=storage == N.STORE_F64, init_kind=1, **okw).f[:, fl] for k in ks]
    first = snaps[0]
    ok = first != 0
    want = [0.0] + [float((np.abs(snaps[i] - snaps[i - 1])[ok] / np.abs(first[ok])).max()) for i in (1, 2)]
    assert got[0] == 0.0
    rtol = 1e-7 if storage == N.STORE_F64 else 2e-2
    for g, w in zip(got[1:], want[1:]):
        assert abs(g - w) <= rtol * w, (got, want)


@pytest.mark.parametrize("storage", [N.STORE_F32, N.STORE_F64, N.STORE_F16S])
def test_checkpoint_restart(storage):
    """A raw state saved after 30 steps and loaded into a fresh handle gives,
    20 steps later, the populations and fields of 50 uninterrupted steps bit
    for bit; a restart from the FP64 population read-back agrees to within
    the deviations FP64 cannot carry next to the rest-state shift."""
    lat = lattice.sphere_duct(24, 20, 40, porosity=0.8, rmin=3, rmax=5, seed=3)
    args = Arguments(viscosity=0.1, collision_model=N.MRT, mode=N.MODE_PHYSICS, init_equilibrium=1,
                     inlet_profile=N.INLET_PRESSURE, outlet_profile=N.OUTLET_PRESSURE, rho_in=1.01, storage=storage)
    nn = lat.num_nodes
    init = (np.ones(nn), np.zeros(nn), np.zeros(nn), np.zeros(nn))
    with Solver(lat, args) as s:
        s.init(*init)
        s.step(30, write_macro=False)
        state = s.get_state()
        saved = s.populations()
        s.step(20, write_macro=True)
        f_run = s.populations()
        m_run = s.macro()
    with Solver(lat, args) as s:
        s.set_state(state)
        np.testing.assert_array_equal(s.get_state(), state)
        s.step(20, write_macro=True)
        np.testing.assert_array_equal(s.populations(), f_run)
        for a, b in zip(s.macro(), m_run):
            np.testing.assert_array_equal(a, b)
    with Solver(lat, args) as s:
        s.set_populations(saved)
        np.testing.assert_array_equal(s.populations(), saved)
        s.step(20, write_macro=True)
        # a last-bit difference in one tiny deviation grows to FP32 rounding
        # level (2e-8 measured after 20 steps)
        tol = {N.STORE_F16S: 1e-5, N.STORE_F32: 1e-6, N.STORE_F64: 1e-12}[storage]
        assert np.abs(s.populations() - f_run).max() < tol


def test_momentum_exchange_matches_host_sum(oracle):
    """lbm_momentum_exchange against the same link sum evaluated on the host
    from the read-back populations and flag words; drag along the flow."""
    from thesis_gb300.solver import build_flags
    lat = lattice.channel2d(160, 48, seed=5)
    args = Arguments(u=0.05, viscosity=0.05, collision_model=N.TRT, mode=N.MODE_PHYSICS, init_equilibrium=1,
                     outlet_profile=N.OUTLET_PRESSURE, rho_out=1.0)
    nn = lat.num_nodes
    box = (10, 150, 1, 46, 0, 0)  # the obstacles, not the channel walls (out-of-domain links)
    with Solver(lat, args) as s:
        s.init(np.ones(nn), np.zeros(nn), np.zeros(nn), np.zeros(nn))
        s.step(300, write_macro=True)
        F = s.momentum_exchange(box)
        f = s.populations()
    _, word, _, _ = build_flags(lat, args)
    n, m = lat.n, lat.m
    idx = np.arange(nn)
    x, y = idx % n, idx // n
    host = np.zeros(2)
    for d in range(1, 9):
        o = lattice.OPP2[d] if hasattr(lattice, "OPP2") else [0, 3, 4, 1, 2, 7, 8, 5, 6][d]
        sx, sy = x - lattice.CX2[d], y - lattice.CY2[d]
        sel = ((word & 1) == 1) & (((word >> d) & 1) == 1) & (sx >= box[0]) & (sx <= box[1]) & \
              (sy >= box[2]) & (sy <= box[3]) & (sx >= 0) & (sx < n) & (sy >= 0) & (sy < m)
        host[0] += 2 * lattice.CX2[o] * f[o, sel].sum()
        host[1] += 2 * lattice.CY2[o] * f[o, sel].sum()
    np.testing.assert_allclose(F[:2], host, rtol=1e-9, atol=1e-12)
    assert F[2] == 0.0 and F[0] > 0  # obstacles are dragged downstream


def test_full_cavity128_against_reference_golden():
    """The BGK lid-driven cavity of the plain-method configuration (128x128,
    u_lid 0.1, Re 100, 20,000 steps, FP32, reference semantics) against the
    reference's own kernels' result (tests/golden/cavity128_bgk_20000.npz,
    made by tests/golden/make_golden.py --cavity128).  FP32 in a different
    operation order over 20,000 steps: 5e-5 absolute on u, v, rho and the
    centre lines."""
    import hashlib
    import os
    g = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "cavity128_bgk_20000.npz"))
    lat = lattice.cavity2d(128)
    sha = hashlib.sha256(np.ascontiguousarray(lat.bc).tobytes() + lat.node_type.tobytes()).hexdigest()
    assert sha == bytes(g["lattice_sha256"]).decode()
    args = Arguments(u=0.1, viscosity=0.128, collision_model=N.BGKW, outlet_profile=N.OUTLET_ZOUHE)
    with Solver(lat, args) as s:
        s.init()
        s.step(int(g["steps"]), write_macro=True)
        rho, u, v, _ = s.macro()
    for a, b in ((rho, g["rho"]), (u, g["u"]), (v, g["v"])):
        assert np.abs(a.astype(np.float64) - b).max() < 5e-5
    U = u.reshape(128, 128)[:, 64]  # vertical centre line
    V = v.reshape(128, 128)[64, :]  # horizontal centre line
    np.testing.assert_allclose(U, g["u"].reshape(128, 128)[:, 64], atol=5e-5)
    np.testing.assert_allclose(V, g["v"].reshape(128, 128)[64, :], atol=5e-5)


def _rest(nn):
    return (np.ones(nn), np.zeros(nn), np.zeros(nn), np.zeros(nn))


@pytest.mark.parametrize("outlet", [N.OUTLET_SECOND, N.OUTLET_FIRST, N.OUTLET_HEMODEL])
@pytest.mark.parametrize("storage", [N.STORE_F32, N.STORE_F64, N.STORE_F16S])
def test_physics_open_outlets_3d(oracle, outlet, storage):
    """Physics-mode open outlets on a 3D face (the reference's second- and
    first-order extrapolation and HEmodel outlets, GpuBoundaries.cu:1723-1874,
    with every population addressed at its own node): a sphere-packed duct
    with a pressure inlet at z = 0 and the outlet at z = h-1, MRT, against the
    oracle."""
    lat = lattice.sphere_duct(20, 16, 32, porosity=0.8, rmin=3, rmax=4, seed=9)
    args = Arguments(viscosity=0.1, collision_model=N.MRT, mode=N.MODE_PHYSICS, storage=storage,
                     init_equilibrium=1, inlet_profile=N.INLET_PRESSURE, outlet_profile=outlet,
                     rho_in=1.01, rho_out=1.0)
    g, r, fl = run_pair(oracle, lat, args, 60, init=_rest(lat.num_nodes))
    compare(g, r, fl, storage, 3)


@pytest.mark.parametrize("outlet", [N.OUTLET_SECOND, N.OUTLET_FIRST, N.OUTLET_HEMODEL])
@pytest.mark.parametrize("coll", [N.TRT, N.MRT])
def test_physics_open_outlets_2d(oracle, outlet, coll):
    """The same outlets on the east face of a 2D obstacle channel with a
    Zou-He velocity inlet of constant u (F32 and F64 storage)."""
    lat = lattice.channel2d(96, 32, seed=5, n_obstacles=2, size_scale=0.3)
    for storage in (N.STORE_F32, N.STORE_F64):
        args = Arguments(u=0.04, viscosity=0.05, collision_model=coll, mode=N.MODE_PHYSICS, storage=storage,
                         init_equilibrium=1, inlet_profile=N.NO_INLET, outlet_profile=outlet)
        g, r, fl = run_pair(oracle, lat, args, 80, init=_rest(lat.num_nodes))
        compare(g, r, fl, storage, 2)
