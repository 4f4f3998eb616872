"""lbm_fluid_norms_noalloc: the norms entry point for callers that may not
allocate device memory while the solver runs (a host framework with a fixed
device arena, say).  It keeps its scratch in a static device array, so this
test checks, through the C ABI, that it returns what the allocating entry
point lbm_macro_norms returns on the same fields, on two calls in a row (the
second call also checks that it carries the previous velocity forward).
It sits in its own file, collected last, and runs alone or after the rest."""
import ctypes as C

import numpy as np
import pytest

from thesis_gb300 import lattice
from thesis_gb300 import native as N
from thesis_gb300.solver import Arguments, Solver, build_flags

pytestmark = pytest.mark.gpu

RTOL = 1e-12  # same FP64 tolerance as the norms test in test_gpu_parity.py


def _noalloc_fn(lib):
    fn = lib.lbm_fluid_norms_noalloc
    fn.restype = C.c_int
    fn.argtypes = [C.c_void_p] * 8 + [C.c_longlong, C.c_void_p, C.c_void_p]
    lib.lbm_noalloc_last_error.restype = C.c_char_p
    lib.lbm_noalloc_max_nodes.restype = C.c_longlong
    return fn


# one block of partial sums covers 16,384 nodes: 20x16x32 fits one block;
# 40x32x70 (89,600 nodes) needs six, the last one partly filled
@pytest.mark.parametrize("dims", [(20, 16, 32), (40, 32, 70)])
def test_noalloc_norms_match_allocating_norms(native_lib, dims):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    fn = _noalloc_fn(native_lib)
    lat = lattice.sphere_duct(*dims, porosity=0.8, rmin=3, rmax=4, seed=3)
    args = Arguments(viscosity=0.1, collision_model=N.MRT, mode=N.MODE_PHYSICS, init_equilibrium=1,
                     inlet_profile=N.INLET_PRESSURE, outlet_profile=N.OUTLET_PRESSURE,
                     rho_in=1.01, rho_out=1.0)
    nn = lat.num_nodes
    _, word, _, _ = build_flags(lat, args)
    dev = torch.device("cuda", 0)
    word_t = torch.from_numpy(word.view(np.int32).copy()).to(dev)
    prev = [torch.zeros(nn, dtype=torch.float32, device=dev) for _ in range(3)]
    out = torch.zeros(N.NORMS, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev)
    with Solver(lat, args) as s:
        s.init(np.ones(nn), np.zeros(nn), np.zeros(nn), np.zeros(nn))
        for call in range(2):
            s.step(10, write_macro=True)
            expect, rc = s.norms()
            assert rc == N.LBM_OK
            fields = [torch.from_numpy(a).to(dev) for a in s.macro()]
            torch.cuda.synchronize(dev)
            rc = fn(word_t.data_ptr(), *[t.data_ptr() for t in fields], *[t.data_ptr() for t in prev],
                    nn, out.data_ptr(), stream.cuda_stream)
            assert rc == N.LBM_OK, native_lib.lbm_noalloc_last_error()
            torch.cuda.synchronize(dev)
            got = out.cpu().numpy()
            np.testing.assert_allclose(got, expect, rtol=RTOL, atol=0.0)
            # at fluid nodes the previous-velocity arrays now hold this call's velocity
            fl = lat.node_type == 1
            for k in range(3):
                np.testing.assert_array_equal(prev[k].cpu().numpy()[fl], fields[1 + k].cpu().numpy()[fl])


def test_noalloc_rejects_oversized_calls(native_lib):
    fn = _noalloc_fn(native_lib)
    too_many = native_lib.lbm_noalloc_max_nodes() + 1
    dummy = C.c_void_p(16)  # never dereferenced: the size check comes first
    rc = fn(*([dummy] * 8), too_many, dummy, None)
    assert rc == N.LBM_ERR_INVALID
    assert b"exceed the maximum" in native_lib.lbm_noalloc_last_error()
