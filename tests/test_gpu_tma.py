"""Row-staged step kernel (bulk copies into shared memory, THESIS_LBM_KERNEL=tma)
against the oracle, with the tolerances of test_gpu_parity, and against the
one-node kernel on a larger lattice."""
import numpy as np
import pytest

from test_gpu_parity import TOL, compare, run_pair
from thesis_gb300 import lattice
from thesis_gb300 import native as N
from thesis_gb300.solver import Arguments, Solver

pytestmark = pytest.mark.gpu


@pytest.fixture
def tma(monkeypatch):
    monkeypatch.setenv("THESIS_LBM_KERNEL", "tma")
    yield
    monkeypatch.delenv("THESIS_LBM_KERNEL", raising=False)


def _rest(nn):
    return (np.ones(nn), np.zeros(nn), np.zeros(nn), np.zeros(nn))


def _duct_args(coll, storage, periodic=(0, 0, 0)):
    return Arguments(viscosity=(0.8 - 0.5) / 3, collision_model=coll, mode=N.MODE_PHYSICS, storage=storage,
                     init_equilibrium=1, inlet_profile=N.INLET_PRESSURE, outlet_profile=N.OUTLET_PRESSURE,
                     rho_in=1.005, rho_out=1.0, periodic=periodic)


def _variant(lat, args):
    with Solver(lat, args) as s:
        return N.lib().lbm_kernel_variant(s._h)


@pytest.mark.parametrize("coll", [N.BGKW, N.TRT, N.MRT])
@pytest.mark.parametrize("storage", [N.STORE_F32, N.STORE_F16S])
def test_tma_sphere_duct(oracle, tma, coll, storage):
    lat = lattice.sphere_duct(24, 20, 48, porosity=0.75, rmin=3, rmax=5, seed=7)
    args = _duct_args(coll, storage)
    assert _variant(lat, args) == 3
    g, r, fl = run_pair(oracle, lat, args, 40, init=_rest(lat.num_nodes))
    compare(g, r, fl, storage, 3)


@pytest.mark.parametrize("coll", [N.BGKW, N.MRT])
def test_tma_periodic_xy_duct(oracle, tma, coll):
    """Periodic side faces: pull rows wrap in y, the x shift wraps inside
    shared memory."""
    lat = lattice.sphere_duct(32, 24, 40, porosity=0.8, rmin=3, rmax=5, seed=4)
    args = _duct_args(coll, N.STORE_F32, periodic=(1, 1, 0))
    assert _variant(lat, args) == 3
    g, r, fl = run_pair(oracle, lat, args, 40, init=_rest(lat.num_nodes))
    compare(g, r, fl, N.STORE_F32, 3)


@pytest.mark.parametrize("storage", [N.STORE_F32, N.STORE_F16S])
def test_tma_channel2d(oracle, tma, storage):
    lat = lattice.channel2d(160, 48, seed=5)
    args = Arguments(u=0.05, viscosity=0.05, collision_model=N.TRT, mode=N.MODE_PHYSICS, storage=storage,
                     init_equilibrium=1, outlet_profile=N.OUTLET_PRESSURE, rho_out=1.0)
    assert _variant(lat, args) == 3
    g, r, fl = run_pair(oracle, lat, args, 60, init=_rest(lat.num_nodes))
    compare(g, r, fl, storage, 2)


def test_tma_ineligible_falls_back(tma):
    """Rows that are not a multiple of 16 bytes, F64 storage and the
    reference mode keep the one-node kernel."""
    lat = lattice.sphere_duct(22, 20, 24, porosity=0.8, rmin=3, rmax=4, seed=2)  # 22 * 2 B rows
    assert _variant(lat, _duct_args(N.MRT, N.STORE_F16S)) != 3
    lat = lattice.sphere_duct(24, 20, 24, porosity=0.8, rmin=3, rmax=4, seed=2)
    assert _variant(lat, _duct_args(N.MRT, N.STORE_F64)) == 1
    assert _variant(lattice.cavity3d(16, 12, 10), Arguments(u=0.05, viscosity=0.1, collision_model=N.MRT)) != 3


@pytest.mark.parametrize("storage", [N.STORE_F32, N.STORE_F16S])
def test_tma_matches_one_node_kernel_large(monkeypatch, storage):
    """Size-independent check at a size the oracle would be slow on: the
    row-staged and one-node kernels agree after 200 steps."""
    lat = lattice.sphere_duct(128, 96, 160, porosity=0.7, rmin=5, rmax=9, seed=1)
    args = _duct_args(N.MRT, storage)
    out = {}
    for v in ("tma", "scalar"):
        monkeypatch.setenv("THESIS_LBM_KERNEL", v)
        with Solver(lat, args) as s:
            assert N.lib().lbm_kernel_variant(s._h) == (3 if v == "tma" else 1)
            s.init(*_rest(lat.num_nodes))
            s.step(200, write_macro=True)
            out[v] = s.macro()
            nm, rc = s.norms()
            assert rc == N.LBM_OK
    monkeypatch.delenv("THESIS_LBM_KERNEL", raising=False)
    tol = TOL[N.STORE_F32] if storage == N.STORE_F32 else 1e-3
    for a, b in zip(out["tma"], out["scalar"]):
        assert np.abs(a.astype(np.float64) - b).max() < tol
