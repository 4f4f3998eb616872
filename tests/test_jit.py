"""Run-time specialised step kernel (THESIS_LBM_KERNEL=jit): the embedded
sources compile with NVRTC (CPU, no GPU needed), and on the GPU the kernel
matches the oracle with the tolerances of test_gpu_parity."""
import numpy as np
import pytest

from thesis_gb300 import lattice
from thesis_gb300 import native as N
from thesis_gb300.solver import Arguments, Solver


@pytest.mark.parametrize("q,coll,storage,phys,wrap,dims,knobs", [
    (19, N.MRT, N.STORE_F16S, 1, 0, (256, 256, 512), (128, 0, 0)),
    (19, N.MRT, N.STORE_F16S, 1, 0, (256, 256, 512), (256, 1, 1)),
    (19, N.BGKW, N.STORE_F64, 0, 1, (12, 10, 9), (128, 1, 0)),
    (9, N.TRT, N.STORE_F32, 1, 1, (160, 48, 1), (256, 0, 1)),
    (9, N.MRT, N.STORE_F32, 0, 1, (32, 24, 1), (128, 0, 0)),
    (19, N.MRT, N.STORE_F16S, 1, 0, (256, 256, 512), (64, 0, 2)),
    (19, N.MRT, N.STORE_F16S, 1, 0, (256, 256, 512), (64, 0, 2 | (12 << 2))),
    (19, N.MRT, N.STORE_F32, 1, 0, (256, 256, 512), (128, 1, 1 | (12 << 2))),
    (19, N.MRT, N.STORE_F16S, 1, 0, (256, 256, 512), (128, 2, 0)),
    (9, N.TRT, N.STORE_F32, 0, 1, (160, 48, 1), (256, 2, 5 << 2)),
    (9, N.TRT, N.STORE_F32, 0, 1, (160, 48, 1), (128, 0, 2)),
    # reference-mode D3Q19 (HH walls, periodic copies) in every kernel form
    (19, N.MRT, N.STORE_F32, 0, 0, (64, 48, 40), (128, 0, 0)),
    (19, N.BGKW, N.STORE_F32, 0, 1, (64, 48, 40), (128, 2, 0)),
    (19, N.MRT, N.STORE_F32, 0, 0, (64, 48, 40), (64, 0, 2)),
    # storage-unit kernel with speculative loads, and walking 4 nodes along z
    (19, N.MRT, N.STORE_F16S, 1, 0, (256, 256, 512), (128, 2, 1 | (10 << 2))),
    (19, N.MRT, N.STORE_F16S, 1, 0, (256, 256, 512), (128, 2 | (4 << 2), 10 << 2)),
    (19, N.BGKW, N.STORE_F32, 0, 1, (20, 16, 21), (128, 2 | (8 << 2), 0)),
    (9, N.TRT, N.STORE_F32, 1, 1, (160, 48, 1), (128, 2, 1)),
    # storage-unit z-walk kernel, two z nodes at a time on FP32x2
    (19, N.MRT, N.STORE_F16S, 1, 0, (256, 256, 512), (64, 2 | (8 << 2), (10 << 2) | (1 << 10))),
    (19, N.MRT, N.STORE_F32, 1, 1, (20, 16, 22), (64, 1 | 2 | (4 << 2), (1 << 10))),
    # storage-unit z-walk kernel with predicated bounce-back loads
    (19, N.MRT, N.STORE_F16S, 1, 0, (256, 256, 512), (64, 1 | 2 | (8 << 2), 20 << 2)),
    # F16C storage, storage-unit kernels
    (19, N.MRT, N.STORE_F16C, 1, 0, (256, 256, 512), (64, 2 | (8 << 2), 20 << 2)),
    (9, N.MRT, N.STORE_F16C, 1, 1, (160, 48, 1), (128, 2, 0)),
])
def test_jit_sources_compile(native_lib, q, coll, storage, phys, wrap, dims, knobs):
    rc = native_lib.lbm_jit_check(q, coll, storage, phys, wrap, *dims, *knobs)
    assert rc == N.LBM_OK, native_lib.lbm_last_error().decode()


@pytest.fixture
def jit(monkeypatch):
    monkeypatch.setenv("THESIS_LBM_KERNEL", "jit")
    yield
    monkeypatch.delenv("THESIS_LBM_KERNEL", raising=False)


def _rest(nn):
    return (np.ones(nn), np.zeros(nn), np.zeros(nn), np.zeros(nn))


def _check(oracle, lat, args, steps, init, dims, storage):
    from test_gpu_parity import compare, run_pair
    with Solver(lat, args) as s:
        assert N.lib().lbm_kernel_variant(s._h) == 4
    g, r, fl = run_pair(oracle, lat, args, steps, init=init)
    compare(g, r, fl, storage, dims)


@pytest.mark.gpu
@pytest.mark.parametrize("coll", [N.BGKW, N.TRT, N.MRT])
@pytest.mark.parametrize("storage", [N.STORE_F32, N.STORE_F16S, N.STORE_F64, N.STORE_F16C])
def test_jit_sphere_duct(oracle, jit, coll, storage):
    lat = lattice.sphere_duct(24, 20, 48, porosity=0.75, rmin=3, rmax=5, seed=7)
    args = Arguments(viscosity=(0.8 - 0.5) / 3, collision_model=coll, mode=N.MODE_PHYSICS, storage=storage,
                     init_equilibrium=1, inlet_profile=N.INLET_PRESSURE, outlet_profile=N.OUTLET_PRESSURE,
                     rho_in=1.005, rho_out=1.0)
    _check(oracle, lat, args, 40, _rest(lat.num_nodes), 3, storage)


@pytest.mark.gpu
def test_jit_periodic_duct(oracle, jit):
    lat = lattice.sphere_duct(32, 24, 40, porosity=0.8, rmin=3, rmax=5, seed=4)
    args = Arguments(viscosity=0.1, collision_model=N.MRT, mode=N.MODE_PHYSICS, init_equilibrium=1,
                     inlet_profile=N.INLET_PRESSURE, outlet_profile=N.OUTLET_PRESSURE, rho_in=1.005,
                     periodic=(1, 1, 0))
    _check(oracle, lat, args, 40, _rest(lat.num_nodes), 3, N.STORE_F32)


@pytest.mark.gpu
@pytest.mark.parametrize("coll", [N.BGKW, N.MRT])
def test_jit_reference_cavities(oracle, jit, coll):
    lat = lattice.cavity2d(32, 24)
    args = Arguments(u=0.1, viscosity=0.128, collision_model=coll, outlet_profile=N.OUTLET_ZOUHE)
    _check(oracle, lat, args, 60, None, 2, N.STORE_F32)
    lat = lattice.cavity3d(12, 10, 9)
    args = Arguments(u=0.05, viscosity=0.1, collision_model=coll)
    _check(oracle, lat, args, 25, None, 3, N.STORE_F32)


@pytest.mark.gpu
def test_jit_channel2d(oracle, jit):
    lat = lattice.channel2d(160, 48, seed=5)
    args = Arguments(u=0.05, viscosity=0.05, collision_model=N.TRT, mode=N.MODE_PHYSICS,
                     init_equilibrium=1, outlet_profile=N.OUTLET_PRESSURE, rho_out=1.0)
    _check(oracle, lat, args, 60, _rest(lat.num_nodes), 2, N.STORE_F32)


@pytest.mark.gpu
@pytest.mark.parametrize("storage", [N.STORE_F32, N.STORE_F16S, N.STORE_F64])
def test_compiled_in_kernel_sphere_duct(oracle, monkeypatch, storage):
    """The compiled-in one-node kernel (the fallback when the run-time build
    is unavailable) against the oracle."""
    monkeypatch.setenv("THESIS_LBM_KERNEL", "scalar")
    lat = lattice.sphere_duct(24, 20, 48, porosity=0.75, rmin=3, rmax=5, seed=7)
    args = Arguments(viscosity=(0.8 - 0.5) / 3, collision_model=N.MRT, mode=N.MODE_PHYSICS, storage=storage,
                     init_equilibrium=1, inlet_profile=N.INLET_PRESSURE, outlet_profile=N.OUTLET_PRESSURE,
                     rho_in=1.005, rho_out=1.0)
    from test_gpu_parity import compare, run_pair
    with Solver(lat, args) as s:
        assert N.lib().lbm_kernel_variant(s._h) == 1
    g, r, fl = run_pair(oracle, lat, args, 40, init=_rest(lat.num_nodes))
    compare(g, r, fl, storage, 3)


@pytest.mark.gpu
def test_autotune_then_parity(oracle):
    """lbm_autotune keeps one of its variants; after lbm_init the run matches
    the oracle, and a second handle on the same lattice reuses the choice."""
    from test_gpu_parity import compare
    lat = lattice.sphere_duct(32, 24, 40, porosity=0.75, rmin=3, rmax=5, seed=9)
    args = Arguments(viscosity=0.1, collision_model=N.MRT, mode=N.MODE_PHYSICS, storage=N.STORE_F32,
                     init_equilibrium=1, inlet_profile=N.INLET_PRESSURE, outlet_profile=N.OUTLET_PRESSURE,
                     rho_in=1.005)
    nn = lat.num_nodes
    with Solver(lat, args) as s:
        knobs = s.autotune(6)
        assert knobs[0] in (64, 128, 256) and knobs[1] in (0, 1, 2) and (knobs[2] & 3) in (0, 1, 2)
        with pytest.raises(N.LbmError):
            s.step(1)  # populations undefined until init
        s.init(*_rest(nn))
        s.step(30, write_macro=True)
        rho, u, v, w = s.macro()
        f = s.populations()
        with Solver(lat, args) as s2:
            assert s2.kernel_config() == knobs
    r = oracle.run_oracle(lat, 30, mode=N.MODE_PHYSICS, init_kind=1, rho_in=1.005, rho_out=1.0,
                          extra_collide=True, init=_rest(nn), viscosity=0.1, collision_model=N.MRT,
                          inlet_profile=N.INLET_PRESSURE, outlet_profile=N.OUTLET_PRESSURE)
    g = dict(rho=rho.astype(np.float64), u=u.astype(np.float64), v=v.astype(np.float64),
             w=w.astype(np.float64), f=f)
    compare(g, r, lat.node_type == 1, N.STORE_F32, 3)


@pytest.mark.gpu
@pytest.mark.parametrize("coll", [N.BGKW, N.TRT, N.MRT])
@pytest.mark.parametrize("storage", [N.STORE_F32, N.STORE_F16S])
def test_jit_pair_sphere_duct(oracle, monkeypatch, coll, storage):
    """The run-time specialised two-node kernel (THESIS_LBM_KERNEL=jit2)."""
    monkeypatch.setenv("THESIS_LBM_KERNEL", "jit2")
    from test_gpu_parity import compare, run_pair
    lat = lattice.sphere_duct(24, 20, 48, porosity=0.75, rmin=3, rmax=5, seed=7)
    args = Arguments(viscosity=(0.8 - 0.5) / 3, collision_model=coll, mode=N.MODE_PHYSICS, storage=storage,
                     init_equilibrium=1, inlet_profile=N.INLET_PRESSURE, outlet_profile=N.OUTLET_PRESSURE,
                     rho_in=1.005, rho_out=1.0)
    with Solver(lat, args) as s:
        assert N.lib().lbm_kernel_variant(s._h) == 4 and s.kernel_config()[2] & 2
    g, r, fl = run_pair(oracle, lat, args, 40, init=_rest(lat.num_nodes))
    compare(g, r, fl, storage, 3)


@pytest.mark.gpu
def test_jit_pair_reference_cavity(oracle, monkeypatch):
    monkeypatch.setenv("THESIS_LBM_KERNEL", "jit2")
    from test_gpu_parity import compare, run_pair
    lat = lattice.cavity3d(12, 10, 9)
    args = Arguments(u=0.05, viscosity=0.1, collision_model=N.MRT)
    g, r, fl = run_pair(oracle, lat, args, 25)
    compare(g, r, fl, N.STORE_F32, 3)


@pytest.mark.gpu
@pytest.mark.parametrize("kernel", ["jith", "jiths", "jithz4", "jithz5", "jitf", "jithz4q", "jithz6pq"])
@pytest.mark.parametrize("storage", [N.STORE_F32, N.STORE_F16S])
def test_storage_unit_and_f_space_kernels(oracle, monkeypatch, kernel, storage):
    """Both one-node arithmetic forms (and the storage-unit kernel with
    speculative loads) against the oracle (physics mode)."""
    monkeypatch.setenv("THESIS_LBM_KERNEL", kernel)
    from test_gpu_parity import compare, run_pair
    lat = lattice.sphere_duct(24, 20, 48, porosity=0.75, rmin=3, rmax=5, seed=7)
    args = Arguments(viscosity=(0.8 - 0.5) / 3, collision_model=N.MRT, mode=N.MODE_PHYSICS, storage=storage,
                     init_equilibrium=1, inlet_profile=N.INLET_PRESSURE, outlet_profile=N.OUTLET_PRESSURE,
                     rho_in=1.005, rho_out=1.0)
    with Solver(lat, args) as s:
        assert (s.kernel_config()[1] >> 1) & 1 == (kernel != "jitf")
        assert s.kernel_config()[2] & 1 == (kernel == "jiths")
        zw = int(kernel[5:].rstrip("pq")) if kernel.startswith("jithz") else 0
        assert s.kernel_config()[1] >> 2 == zw
        assert (s.kernel_config()[2] >> 10) & 1 == ("q" in kernel)
    g, r, fl = run_pair(oracle, lat, args, 40, init=_rest(lat.num_nodes))
    compare(g, r, fl, storage, 3)


@pytest.mark.gpu
def test_fp32_cavity_reaches_1e6_residual(monkeypatch):
    """Physics-mode FP32 stores deviations and computes in storage units, so a
    steady cavity reaches a 1e-6 velocity residual (f-space FP32 arithmetic
    stalls near 3e-6 on the same case: cancelling O(w) sums)."""
    monkeypatch.delenv("THESIS_LBM_KERNEL", raising=False)
    n = 24
    lat = lattice.cavity2d(n)
    args = Arguments(u=0.1, viscosity=0.1 * n / 10.0, collision_model=N.MRT, mode=N.MODE_PHYSICS,
                     init_equilibrium=1, outlet_profile=N.OUTLET_ZOUHE)
    with Solver(lat, args) as s:
        s.init()
        res = []
        for _ in range(200):
            s.step(200, write_macro=True)
            r, rc = s.residual()
            assert rc == N.LBM_OK
            res.append(r)
            if r < 1e-6 and len(res) > 2:
                break
        assert res[-1] < 1e-6, res[-5:]


def _f16c_round_trip(x):
    """The F16C storage format restated in numpy: FP32 input rounded to 12
    significant bits (nearest even), exponent range [2^-14, 2) with subnormal
    steps of 2^-25 below, saturation at the largest value."""
    x = np.asarray(x, np.float32).astype(np.float64)
    a = np.abs(x)
    _, e = np.frexp(a)  # a = m 2^e, 1/2 <= m < 1: leading bit 2^(e-1)
    e = np.maximum(e.astype(np.float64) - 1.0, -14.0)
    step = 2.0 ** (e - 11)
    q = np.round(a / step) * step  # numpy rounds halves to even
    q = np.minimum(q, 2.0 - 2.0 ** -11)
    return np.sign(x) * q


@pytest.mark.gpu
def test_f16c_storage_round_trip(native_lib):
    """Populations written with F16C storage (lbm_set_populations) read back
    (lbm_get_populations) exactly as the format defines: w + q((f - w) S)/S
    with q the 1-4-11 rounding of the FP32 value."""
    lat = lattice.sphere_duct(16, 12, 20, porosity=0.8, rmin=3, rmax=4, seed=2)
    args = Arguments(viscosity=0.1, collision_model=N.BGKW, mode=N.MODE_PHYSICS, storage=N.STORE_F16C,
                     init_equilibrium=1, inlet_profile=N.INLET_PRESSURE, outlet_profile=N.OUTLET_PRESSURE,
                     rho_in=1.005, rho_out=1.0)
    nn = lat.num_nodes
    w = lattice.W3[:, None]
    rng = np.random.default_rng(4)
    # deviations spanning the subnormal range, the normal range and saturation
    dev = rng.choice([-1, 1], size=(19, nn)) * 10.0 ** rng.uniform(-12, -2.6, size=(19, nn))
    dev[0, :8] = [0.0, 3e-3, -3e-3, 2.0 ** -24, 2.0 ** -23 * 1.5, 1e-9, -1e-9, 0.0039]
    f = w + dev
    with Solver(lat, args) as s:
        s.set_populations(f)
        g = s.populations()
    S = 256.0  # the F16C default scale
    w32 = w.astype(np.float32).astype(np.float64)  # the shift as the kernels hold it
    want = w32 + _f16c_round_trip((f - w32) * S) / S
    fl = lat.node_type == 1
    np.testing.assert_array_equal(g[:, fl], want[:, fl])
