"""Python host mirror of the reference's time-step entry points.

`Arguments` carries the fields of the reference's Arguments struct
(Source code/lbm-solver_final/include/Arguments.h:86-135) that the time-step
loop reads; `Solver` wraps one libthesis_lbm handle.  All compute runs in the
CUDA library; this module only marshals arrays.
"""
import ctypes as C
import warnings
from dataclasses import dataclass, field

import numpy as np

from . import native as N
from .lattice import Lattice


@dataclass
class Arguments:
    u: float = 0.0
    v: float = 0.0
    w: float = 0.0
    rho: float = 1.0
    viscosity: float = 0.1
    g: float = 0.0
    inlet_profile: int = N.NO_INLET
    outlet_profile: int = N.OUTLET_SECOND
    collision_model: int = N.BGKW
    boundary_type: int = N.STRAIGHT
    bc_wall_model: int = N.WALL_SIMPLE
    update_inlet_outlet: int = 1
    # engine options
    mode: int = N.MODE_REFERENCE
    storage: int = N.STORE_F32
    rho_in: float = 1.0
    rho_out: float = 1.0
    f16_scale: float = 0.0
    periodic: tuple = (0, 0, 0)
    init_equilibrium: int = 0

    def to_c(self):
        p = N.Params()
        for k in ("u", "v", "w", "rho", "viscosity", "g", "rho_in", "rho_out", "f16_scale"):
            setattr(p, k, float(getattr(self, k)))
        for k in ("inlet_profile", "outlet_profile", "collision_model", "boundary_type",
                  "bc_wall_model", "update_inlet_outlet", "mode", "storage", "init_equilibrium"):
            setattr(p, k, int(getattr(self, k)))
        for i in range(3):
            p.periodic[i] = int(self.periodic[i])
        return p

    @property
    def omega(self):
        return 1.0 / (3.0 * self.viscosity + 0.5)


def _iptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_int))


def _fptr(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_float))


def lattice_desc(lat: Lattice):
    """Fill an lbm_lattice_desc; the returned tuple keeps the arrays alive."""
    bc = lat.bc
    cols = [np.ascontiguousarray(bc[:, k], dtype=np.int32) for k in range(6)]
    d = N.LatticeDesc()
    d.dims, d.n, d.m, d.h = lat.dims, lat.n, lat.m, lat.h
    d.node_type = _iptr(lat.node_type)
    d.num_conns = int(bc.shape[0])
    d.bc_i, d.bc_j = _iptr(cols[0]), _iptr(cols[1])
    d.bc_k = _iptr(cols[2]) if lat.dims == 3 else None
    d.bc_dir, d.bc_type, d.bc_id = _iptr(cols[3]), _iptr(cols[4]), _iptr(cols[5])
    return d, cols


def build_flags(lat: Lattice, args: Arguments):
    """Reference masks, flag words and slots computed by the library on the
    host (no GPU).  Returns (mask uint64, word uint32, slot int32, n_bc)."""
    L = N.lib()
    d, keep = lattice_desc(lat)
    p = args.to_c()
    nn = lat.num_nodes
    mask = np.zeros(nn, np.uint64)
    word = np.zeros(nn, np.uint32)
    slot = np.zeros(nn, np.int32)
    nbc = C.c_int(0)
    N.check(L.lbm_build_flags(C.byref(d), C.byref(p), mask.ctypes.data_as(C.POINTER(C.c_uint64)),
                              word.ctypes.data_as(C.POINTER(C.c_uint32)),
                              slot.ctypes.data_as(C.POINTER(C.c_int32)), C.byref(nbc)))
    del keep
    return mask, word, slot, nbc.value


def link_q(lat: Lattice, bc_xyz, node_xyz, delta):
    """The reference's link fractions |B - X| / (delta |c_dir|) (lbm_link_q):
    bc_xyz the BC file's boundary points (num_conns x 2 or 3), node_xyz the
    Node file's coordinates by node index (num_nodes x 2 or 3)."""
    L = N.lib()
    bc = lat.bc
    cols = [np.ascontiguousarray(bc[:, k], dtype=np.int32) for k in range(4)]
    b = [np.ascontiguousarray(np.asarray(bc_xyz, np.float32)[:, k]) for k in range(lat.dims)]
    x = [np.ascontiguousarray(np.asarray(node_xyz, np.float32)[:, k]) for k in range(lat.dims)]
    if lat.dims == 2:
        b.append(None)
        x.append(None)
    q = np.zeros(bc.shape[0], np.float64)
    N.check(L.lbm_link_q(lat.dims, lat.n, lat.m, lat.h, int(bc.shape[0]), _iptr(cols[0]), _iptr(cols[1]),
                         _iptr(cols[2]) if lat.dims == 3 else None, _iptr(cols[3]), *[_fptr(a) for a in b],
                         *[_fptr(a) for a in x], float(delta), q.ctypes.data_as(C.POINTER(C.c_double))))
    return q


class Solver:
    """One lattice on the GPU.  Usage: s = Solver(lat, args); s.init();
    s.step(100, write_macro=True); rho, u, v, w = s.macro()."""

    def __init__(self, lat: Lattice, args: Arguments):
        self.lat = lat
        self.args = args
        self._lib = N.lib()
        d, keep = lattice_desc(lat)
        p = args.to_c()
        h = C.c_void_p()
        N.check(self._lib.lbm_create(C.byref(d), C.byref(p), C.byref(h)))
        del keep
        self._h = h
        warn = self._lib.lbm_kernel_warning(h)
        if warn:
            warnings.warn(warn.decode(), RuntimeWarning, stacklevel=2)

    def close(self):
        if getattr(self, "_h", None):
            self._lib.lbm_destroy(self._h)
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

    def set_inlet_velocity(self, u=None, v=None, w=None):
        arrs = [None if a is None else np.ascontiguousarray(a, np.float32).reshape(-1) for a in (u, v, w)]
        N.check(self._lib.lbm_set_inlet_velocity(self._h, *[_fptr(a) for a in arrs]))

    def set_link_q(self, q):
        """Curved walls: the wall's fraction along each BC link, in the
        lattice's link order (lbm_set_link_q)."""
        a = np.ascontiguousarray(q, np.float64).reshape(-1)
        if a.size != self.lat.bc.shape[0]:
            raise ValueError("expected %d link fractions, got %d" % (self.lat.bc.shape[0], a.size))
        N.check(self._lib.lbm_set_link_q(self._h, a.ctypes.data_as(C.POINTER(C.c_double))))

    def autotune(self, trial_steps=20):
        """Pick the fastest variant of the specialised step kernel (block size,
        load form, bounce-back form); leaves the populations undefined, so
        call init() afterwards.  Returns (block, hint, pred)."""
        b, h, p = C.c_int(), C.c_int(), C.c_int()
        N.check(self._lib.lbm_autotune(self._h, int(trial_steps), C.byref(b), C.byref(h), C.byref(p)))
        return b.value, h.value, p.value

    def kernel_config(self):
        b, h, p = C.c_int(), C.c_int(), C.c_int()
        N.check(self._lib.lbm_kernel_config(self._h, C.byref(b), C.byref(h), C.byref(p)))
        return b.value, h.value, p.value

    def init(self, rho=None, u=None, v=None, w=None):
        arrs = [None if a is None else np.ascontiguousarray(a, np.float32).reshape(-1) for a in (rho, u, v, w)]
        N.check(self._lib.lbm_init(self._h, *[_fptr(a) for a in arrs]))

    def step(self, nsteps, write_macro=True, stream=None):
        N.check(self._lib.lbm_step(self._h, int(nsteps), int(bool(write_macro)),
                                   None if stream is None else C.c_void_p(stream)))

    def macro(self, out=None):
        """rho, u, v, w of the last step that stored them; `out` may hold four
        contiguous float32 arrays of num_nodes (pinned ones are filled by
        direct copies) that receive them."""
        nn = self.lat.num_nodes
        if out is None:
            out = [np.empty(nn, np.float32) for _ in range(4)]
        elif len(out) != 4 or any(a.dtype != np.float32 or a.size != nn or not a.flags.c_contiguous for a in out):
            raise ValueError("out must be four contiguous float32 arrays of %d values" % nn)
        N.check(self._lib.lbm_get_macro(self._h, *[_fptr(a) for a in out]))
        return out

    def populations(self):
        q = self.lat.q
        f = np.empty(q * self.lat.num_nodes, np.float64)
        N.check(self._lib.lbm_get_populations(self._h, f.ctypes.data_as(C.POINTER(C.c_double))))
        return f.reshape(q, -1)

    def norms(self):
        out = np.zeros(N.NORMS, np.float64)
        rc = self._lib.lbm_macro_norms(self._h, out.ctypes.data_as(C.POINTER(C.c_double)))
        if rc not in (N.LBM_OK, N.LBM_DIVERGED):
            N.check(rc)
        return out, rc

    def macro_diff(self):
        """The reference's MaxMacroDiff residual: (max|du|, max|dv|, max|dw|,
        max|drho|, non-finite count) against the previous call (the initial
        fields before the first), and the status code."""
        out = np.zeros(5, np.float64)
        rc = self._lib.lbm_macro_diff(self._h, out.ctypes.data_as(C.POINTER(C.c_double)))
        if rc not in (N.LBM_OK, N.LBM_DIVERGED):
            N.check(rc)
        return out, rc

    def reference_drag_lift(self, boundary_id, x, y):
        """The reference's 2D drag and lift sums over the fluid nodes of a
        boundary id (lbm_reference_drag_lift); x, y: node coordinates."""
        xs = np.ascontiguousarray(x, np.float32).reshape(-1)
        ys = np.ascontiguousarray(y, np.float32).reshape(-1)
        out = np.zeros(2, np.float64)
        N.check(self._lib.lbm_reference_drag_lift(self._h, int(boundary_id), _fptr(xs), _fptr(ys),
                                                  out.ctypes.data_as(C.POINTER(C.c_double))))
        return out

    def momentum_exchange(self, box):
        """Force (fx, fy, fz) on the solid nodes inside box = (x0, x1, y0, y1,
        z0, z1) by momentum exchange."""
        b = np.ascontiguousarray(box, np.int32)
        out = np.zeros(3)
        N.check(self._lib.lbm_momentum_exchange(self._h, b.ctypes.data_as(C.POINTER(C.c_int)),
                                                out.ctypes.data_as(C.POINTER(C.c_double))))
        return out

    def set_populations(self, f):
        """Restart from a population field in the populations() layout."""
        f = np.ascontiguousarray(f, np.float64).reshape(-1)
        N.check(self._lib.lbm_set_populations(self._h, f.ctypes.data_as(C.POINTER(C.c_double))))

    def get_state(self):
        """Exact checkpoint: the stored populations as raw bytes."""
        buf = np.empty(int(self._lib.lbm_state_bytes(self._h)), np.uint8)
        N.check(self._lib.lbm_get_state(self._h, buf.ctypes.data_as(C.c_void_p)))
        return buf

    def set_state(self, buf):
        buf = np.ascontiguousarray(buf, np.uint8)
        assert buf.size == int(self._lib.lbm_state_bytes(self._h))
        N.check(self._lib.lbm_set_state(self._h, buf.ctypes.data_as(C.c_void_p)))

    def residual_fd_rel_diff(self):
        """The reference's FdRelDiff residual (first call after init: 0)."""
        out = C.c_double()
        N.check(self._lib.lbm_residual_fd_rel_diff(self._h, C.byref(out)))
        return out.value

    def residual_l2(self):
        """The reference's L2 residual sqrt(sum (f - fColl)^2) of the current
        state, and the status code."""
        out = C.c_double()
        rc = self._lib.lbm_residual_l2(self._h, C.byref(out))
        if rc not in (N.LBM_OK, N.LBM_DIVERGED):
            N.check(rc)
        return out.value, rc

    def residual(self):
        """Velocity residual sqrt(sum|u - u_prev|^2) / sqrt(sum|u|^2) over
        fluid nodes (FP64), relative to the field at the previous call."""
        nm, rc = self.norms()
        return (np.sqrt(nm[0]) / np.sqrt(nm[1]) if nm[1] > 0 else np.inf), rc

    @property
    def fluid_nodes(self):
        return int(self._lib.lbm_fluid_nodes(self._h))

    @property
    def bytes_per_update(self):
        return int(self._lib.lbm_bytes_per_update(self._h))

    @property
    def status(self):
        return int(self._lib.lbm_status(self._h))
