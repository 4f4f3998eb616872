"""Batched independent domains (include/thesis_lbm.h lbm_batch_*): many
lattices of uneven sizes advanced by one persistent launch per step.  The
compute runs in the CUDA library; this module marshals arrays."""
import ctypes as C

import numpy as np

from . import native as N
from .solver import Arguments, lattice_desc


def _sig(L):
    vp, dp, fp = C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_float)
    ll = C.POINTER(C.c_longlong)
    sig = {
        "lbm_batch_create": (C.c_int, [C.POINTER(C.POINTER(N.LatticeDesc)), C.POINTER(N.Params), C.c_int,
                                       C.POINTER(vp)]),
        "lbm_batch_init": (C.c_int, [vp]),
        "lbm_batch_set_inlet_velocity": (C.c_int, [vp, C.c_int, fp, fp, fp]),
        "lbm_batch_init_fields": (C.c_int, [vp, C.c_int, fp, fp, fp, fp]),
        "lbm_batch_step": (C.c_int, [vp, C.c_int, C.c_int, vp]),
        "lbm_batch_residuals": (C.c_int, [vp, dp]),
        "lbm_batch_set_active": (C.c_int, [vp, C.POINTER(C.c_int)]),
        "lbm_batch_run_to_tolerance": (C.c_int, [vp, C.c_double, C.c_int, C.c_longlong, ll, dp]),
        "lbm_batch_get_macro": (C.c_int, [vp, C.c_int, fp, fp, fp, fp]),
        "lbm_batch_get_populations": (C.c_int, [vp, C.c_int, dp]),
        "lbm_batch_info": (C.c_int, [vp, C.POINTER(C.c_int), ll, ll, C.POINTER(C.c_int)]),
        "lbm_batch_active_fluid_nodes": (C.c_longlong, [vp]),
        "lbm_batch_last_error": (C.c_char_p, []),
        "lbm_batch_destroy": (None, [vp]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    return L


def check(lib, rc):
    if rc != N.LBM_OK:
        raise N.LbmError(rc, lib.lbm_batch_last_error().decode(errors="replace"))
    return rc


def _fptr(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_float))


class Batch:
    """Usage: b = Batch([lat, ...], [Arguments, ...]); b.init();
    steps, res = b.run_to_tolerance(1e-6, 1000, 10**6)."""

    def __init__(self, lattices, args):
        self._lib = _sig(N.lib())
        self.lattices = list(lattices)
        self.count = len(self.lattices)
        descs, self._keep = [], []
        for lat in self.lattices:
            d, keep = lattice_desc(lat)
            descs.append(d)
            self._keep.append(keep)
        self._descs = descs
        ptrs = (C.POINTER(N.LatticeDesc) * self.count)(*[C.pointer(d) for d in descs])
        params = (N.Params * self.count)(*[a.to_c() for a in args])
        h = C.c_void_p()
        check(self._lib, self._lib.lbm_batch_create(ptrs, params, self.count, C.byref(h)))
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            self._lib.lbm_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def init(self):
        check(self._lib, self._lib.lbm_batch_init(self._h))

    def set_inlet_velocity(self, d, u=None, v=None, w=None):
        arrs = [None if a is None else np.ascontiguousarray(a, np.float32).reshape(-1) for a in (u, v, w)]
        check(self._lib, self._lib.lbm_batch_set_inlet_velocity(self._h, int(d), *[_fptr(a) for a in arrs]))

    def init_fields(self, d, rho=None, u=None, v=None, w=None):
        """Equilibrium start of domain d from fields (after init, before any step)."""
        arrs = [None if a is None else np.ascontiguousarray(a, np.float32).reshape(-1) for a in (rho, u, v, w)]
        check(self._lib, self._lib.lbm_batch_init_fields(self._h, int(d), *[_fptr(a) for a in arrs]))

    def step(self, nsteps, write_macro=True, stream=None):
        check(self._lib, self._lib.lbm_batch_step(self._h, int(nsteps), int(bool(write_macro)),
                                                  None if stream is None else C.c_void_p(stream)))

    def residuals(self):
        r = np.zeros(self.count)
        rc = self._lib.lbm_batch_residuals(self._h, r.ctypes.data_as(C.POINTER(C.c_double)))
        if rc not in (N.LBM_OK, N.LBM_DIVERGED):
            check(self._lib, rc)
        return r, rc

    def set_active(self, active):
        a = np.ascontiguousarray(active, np.int32)
        check(self._lib, self._lib.lbm_batch_set_active(self._h, a.ctypes.data_as(C.POINTER(C.c_int))))

    def run_to_tolerance(self, tol, check_every, max_steps):
        steps = np.zeros(self.count, np.int64)
        res = np.zeros(self.count)
        rc = self._lib.lbm_batch_run_to_tolerance(self._h, float(tol), int(check_every), int(max_steps),
                                                  steps.ctypes.data_as(C.POINTER(C.c_longlong)),
                                                  res.ctypes.data_as(C.POINTER(C.c_double)))
        if rc not in (N.LBM_OK, N.LBM_DIVERGED):
            check(self._lib, rc)
        return steps, res, rc

    def macro(self, d):
        nn = self.lattices[d].num_nodes
        out = [np.empty(nn, np.float32) for _ in range(4)]
        fp = lambda a: a.ctypes.data_as(C.POINTER(C.c_float))
        check(self._lib, self._lib.lbm_batch_get_macro(self._h, int(d), *[fp(a) for a in out]))
        return out

    def populations(self, d):
        lat = self.lattices[d]
        f = np.empty(lat.q * lat.num_nodes)
        check(self._lib, self._lib.lbm_batch_get_populations(self._h, int(d),
                                                             f.ctypes.data_as(C.POINTER(C.c_double))))
        return f.reshape(lat.q, -1)

    def info(self):
        nd, nodes, fl, tiles = C.c_int(), C.c_longlong(), C.c_longlong(), C.c_int()
        check(self._lib, self._lib.lbm_batch_info(self._h, C.byref(nd), C.byref(nodes), C.byref(fl),
                                                  C.byref(tiles)))
        return dict(domains=nd.value, nodes=nodes.value, fluid_nodes=fl.value, active_tiles=tiles.value)

    @property
    def active_fluid_nodes(self):
        return int(self._lib.lbm_batch_active_fluid_nodes(self._h))


def cavity_args(n, re, u_lid=0.1, collision_model=N.MRT, storage=N.STORE_F16S):
    """Physics-mode lid-driven cavity parameters: nu = u_lid * n / Re."""
    return Arguments(u=u_lid, viscosity=u_lid * n / re, collision_model=collision_model, mode=N.MODE_PHYSICS,
                     storage=storage, init_equilibrium=1, outlet_profile=N.OUTLET_ZOUHE)
