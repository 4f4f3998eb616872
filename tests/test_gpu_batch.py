"""Batched independent domains (lbm_batch_*): every domain of a batch matches
the same lattice run alone through lbm_create with the one-node storage-unit
kernel (the code the batch runs), retirement by residual, and buffer parity
when a retired domain rejoins."""
import numpy as np
import pytest

from thesis_gb300 import lattice
from thesis_gb300 import native as N
from thesis_gb300.batch import Batch, cavity_args
from thesis_gb300.solver import Solver

pytestmark = pytest.mark.gpu

SIZES = [(24, 24), (40, 32), (64, 48)]


def _alone(monkeypatch, lat, args, steps):
    monkeypatch.setenv("THESIS_LBM_KERNEL", "jith")
    with Solver(lat, args) as s:
        s.init()
        s.step(steps, write_macro=True)
        out = s.macro(), s.populations()
    monkeypatch.delenv("THESIS_LBM_KERNEL", raising=False)
    return out


@pytest.mark.parametrize("storage,coll", [(N.STORE_F32, N.MRT), (N.STORE_F16S, N.MRT), (N.STORE_F32, N.TRT)])
def test_batch_matches_single_domains(monkeypatch, storage, coll):
    lats = [lattice.cavity2d(n, m) for n, m in SIZES]
    args = [cavity_args(n, re, collision_model=coll, storage=storage) for (n, _), re in zip(SIZES, (50, 200, 800))]
    with Batch(lats, args) as b:
        info = b.info()
        assert info["domains"] == 3 and info["nodes"] == sum(n * m for n, m in SIZES)
        b.init()
        b.step(150, write_macro=True)
        got = [(b.macro(d), b.populations(d)) for d in range(3)]
    for d, (lat, a) in enumerate(zip(lats, args)):
        (m_ref, f_ref) = _alone(monkeypatch, lat, a, 150)
        (m_b, f_b) = got[d]
        # same kernel code on the same inputs: equal to FP32 rounding
        for x, y in zip(m_b, m_ref):
            assert np.abs(x.astype(np.float64) - y).max() <= 1e-6
        assert np.abs(f_b - f_ref).max() <= 1e-6


def test_batch_run_to_tolerance_retires_domains():
    sizes = [16, 24, 32, 40]
    lats = [lattice.cavity2d(n) for n in sizes]
    args = [cavity_args(n, 10.0, storage=N.STORE_F32) for n in sizes]
    with Batch(lats, args) as b:
        b.init()
        steps, res, rc = b.run_to_tolerance(1e-6, 200, 200000)
        assert rc == N.LBM_OK
        assert np.all(res < 1e-6) and np.all(steps > 0) and np.all(steps % 200 == 0)
        # larger cavities (longer diffusion time) need at least as many steps
        assert steps[0] <= steps[-1]
        assert b.info()["active_tiles"] == 0
        rho, u, v, _ = b.macro(3)
        assert np.isfinite(u).all() and np.abs(u).max() <= 0.1 + 1e-6


def test_batch_rejoin_keeps_state(monkeypatch):
    lats = [lattice.cavity2d(n) for n in (20, 28)]
    args = [cavity_args(n, 100.0, storage=N.STORE_F32) for n in (20, 28)]
    with Batch(lats, args) as b:
        b.init()
        b.step(10, write_macro=True)
        b.set_active([1, 0])
        b.step(7, write_macro=True)   # domain 0 only; domain 1's state stays in the other buffer
        b.set_active([1, 1])
        b.step(10, write_macro=True)
        m1 = b.macro(1)
    ref, _ = _alone(monkeypatch, lats[1], args[1], 20)
    for x, y in zip(m1, ref):
        assert np.abs(x.astype(np.float64) - y).max() <= 1e-6


def test_batch_refusals():
    lat = lattice.cavity2d(16)
    a = cavity_args(16, 10.0, storage=N.STORE_F64)
    with pytest.raises(N.LbmError):
        Batch([lat], [a])
    a2 = cavity_args(16, 10.0)
    a3 = cavity_args(16, 10.0, collision_model=N.BGKW)
    with pytest.raises(N.LbmError):
        Batch([lat, lat], [a2, a3])
