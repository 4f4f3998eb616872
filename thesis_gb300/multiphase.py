"""Host side of the colour-gradient two-phase D2Q9 path.

Mirrors the reference's multiphase 2D driver pieces around the time step:
`create_bubble` is createBubble test case 1 (Multiphase.cu:325-356),
`predicted_surface_tension` the prediction of Iterate.cu:163-168 and
`surface_tension_error` calculateSurfaceTension (Multiphase.cu:1082-1091)
applied to the Laplace-law sums (Iterate.cu:496-499).  The step itself runs
in the CUDA library (`lbm_cg_*` in include/thesis_lbm.h); this module only
marshals arrays.
"""
import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import native as N


@dataclass
class CgArguments:
    """The multiphase fields of the reference's Arguments
    (include/Arguments.h:112-131)."""
    r_density: float = 1.0
    b_density: float = 1.0
    r_alpha: float = 4.0 / 9.0
    b_alpha: float = 4.0 / 9.0
    r_viscosity: float = 1.0 / 6.0
    b_viscosity: float = 1.0 / 6.0
    beta: float = 0.7
    A: float = 0.005
    g_limit: float = 0.0
    control_param: float = 0.9
    high_order: bool = False
    enhanced_distrib: bool = False
    bubble_radius: float = 0.2
    # engine option: population storage, N.STORE_F32, N.STORE_F16S (summed
    # population as a shifted FP16 deviation plus the colour difference in
    # FP16, FP32 arithmetic) or N.STORE_F64 (FP64 storage and arithmetic)
    storage: int = N.STORE_F32

    def to_c(self):
        return N.CgParams(self.r_alpha, self.b_alpha, self.r_viscosity, self.b_viscosity, self.beta,
                          self.A, self.g_limit, self.control_param, int(bool(self.high_order)),
                          int(bool(self.enhanced_distrib)), int(self.storage))


def rest_weights(alpha):
    """phi_k of a colour at rest (GpuInit.cu:323-360): alpha, (1-alpha)/5 on
    the axes, (1-alpha)/20 on the diagonals."""
    return np.array([alpha] + [(1 - alpha) / 5] * 4 + [(1 - alpha) / 20] * 4)


def create_bubble(n, m, args: CgArguments, x=None, y=None):
    """Red bubble of radius `args.bubble_radius` (in the node coordinates'
    units) centred at (0.5, 0.5), blue around it, both at rest.  x, y default
    to i/(n-1), j/(m-1).  Returns post-streaming red and blue populations,
    (9, n*m) float64 each, in SoA order."""
    if x is None or y is None:
        j, i = np.divmod(np.arange(n * m), n)
        x, y = i / (n - 1), j / (m - 1)
    inside = np.sqrt((np.asarray(x) - 0.5) ** 2 + (np.asarray(y) - 0.5) ** 2) <= args.bubble_radius
    r = np.where(inside[None, :], (args.r_density * rest_weights(args.r_alpha))[:, None], 0.0)
    b = np.where(~inside[None, :], (args.b_density * rest_weights(args.b_alpha))[:, None], 0.0)
    return np.ascontiguousarray(r), np.ascontiguousarray(b)


def rest_weights3d(alpha):
    """D3Q19 phi_k + theta_k alpha of a colour at rest (GpuInit.cu:905-913):
    alpha, (1-alpha)/12 on the axes, (1-alpha)/24 on the diagonals."""
    return np.array([alpha] + [(1 - alpha) / 12] * 6 + [(1 - alpha) / 24] * 12)


def create_bubble3d(n, m, h, args: CgArguments, radius_nodes=None):
    """Red sphere of radius `args.bubble_radius` * n nodes (or radius_nodes)
    centred in the box, blue around it (initCGBubble3D test case 1,
    GpuInit.cu:536-600): each colour's populations are its density times
    phi_k (1/12 on the axes, 1/24 on the diagonals, 0 at rest), as the
    reference starts them whatever alpha.  Returns (19, n*m*h) float64
    each."""
    R = args.bubble_radius * n if radius_nodes is None else radius_nodes
    idx = np.arange(n * m * h)
    x, y, z = idx % n, (idx // n) % m, idx // (n * m)
    inside = (x - (n - 1) / 2) ** 2 + (y - (m - 1) / 2) ** 2 + (z - (h - 1) / 2) ** 2 <= R * R
    phi = rest_weights3d(0.0)
    r = np.where(inside[None, :], (args.r_density * phi)[:, None], 0.0)
    b = np.where(~inside[None, :], (args.b_density * phi)[:, None], 0.0)
    return np.ascontiguousarray(r), np.ascontiguousarray(b)


def predicted_surface_tension(args: CgArguments):
    """sigma = 4 A / (9 omega_eff) with omega_eff from the density-weighted
    harmonic mean viscosity (Iterate.cu:163-168)."""
    rd, bd = args.r_density, args.b_density
    mean_nu = 1.0 / (rd / ((rd + bd) * args.r_viscosity) + bd / ((rd + bd) * args.b_viscosity))
    omega_eff = 1.0 / (3.0 * mean_nu + 0.5)
    return 4.0 * args.A / 9.0 / omega_eff


def laplace_pressure_jump3d(laplace, args: CgArguments):
    """Mean pressures inside and outside a 3D drop from the Laplace sums,
    p = (1/2)(1 - alpha) rho_colour (calculateSurfaceTension3D,
    Multiphase.cu:1093-1102); returns p_in - p_out."""
    p_in = laplace[0] / laplace[1] if laplace[1] > 0 else 0.0
    p_out = laplace[2] / laplace[3] if laplace[3] > 0 else 0.0
    return 0.5 * (1.0 - args.r_alpha) * p_in - 0.5 * (1.0 - args.b_alpha) * p_out


def surface_tension_error(laplace, args: CgArguments, radius_nodes):
    """Percent error of the Laplace-law surface tension R (p_in - p_out),
    p = (3/5)(1 - alpha) rho_colour averaged over each phase
    (Multiphase.cu:1082-1091), against the prediction."""
    p_in = laplace[0] / laplace[1] if laplace[1] > 0 else 0.0
    p_out = laplace[2] / laplace[3] if laplace[3] > 0 else 0.0
    p_in *= 3.0 / 5.0 * (1.0 - args.r_alpha)
    p_out *= 3.0 / 5.0 * (1.0 - args.b_alpha)
    st = radius_nodes * (p_in - p_out)
    pred = predicted_surface_tension(args)
    return abs(pred - st) / pred * 100.0


def _fp(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_float))


class CgSolver:
    """One periodic n x m (D2Q9) or n x m x h (D3Q19, h given)
    colour-gradient lattice on the GPU."""

    def __init__(self, n, m, args: CgArguments, h=None):
        self.n, self.m, self.args = n, m, args
        self.h = 1 if h is None else int(h)
        self.q = 9 if h is None else 19
        self._lib = N.lib()
        hd = C.c_void_p()
        p = args.to_c()
        if h is None:
            N.check_cg(self._lib.lbm_cg_create(n, m, C.byref(p), C.byref(hd)))
        else:
            N.check_cg(self._lib.lbm_cg_create3d(n, m, self.h, C.byref(p), C.byref(hd)))
        self._h = hd

    @property
    def num_nodes(self):
        return self.n * self.m * self.h

    def close(self):
        if getattr(self, "_h", None):
            self._lib.lbm_cg_destroy(self._h)
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

    def init(self, r_f, b_f):
        r = np.ascontiguousarray(r_f, np.float32).reshape(-1)
        b = np.ascontiguousarray(b_f, np.float32).reshape(-1)
        if r.size != self.q * self.num_nodes or b.size != r.size:
            raise ValueError("populations must hold %d values per node and colour" % self.q)
        N.check_cg(self._lib.lbm_cg_init(self._h, _fp(r), _fp(b)))

    def step(self, nsteps, write_macro=True, stream=None):
        N.check_cg(self._lib.lbm_cg_step(self._h, int(nsteps), int(bool(write_macro)),
                                         None if stream is None else C.c_void_p(stream)))

    def macro(self):
        """rho_r, rho_b, u, v (and w in 3D)."""
        out = [np.empty(self.num_nodes, np.float32) for _ in range(4 if self.q == 9 else 5)]
        if self.q == 9:
            N.check_cg(self._lib.lbm_cg_get_macro(self._h, *[_fp(a) for a in out]))
        else:
            N.check_cg(self._lib.lbm_cg_get_macro3d(self._h, *[_fp(a) for a in out]))
        return out

    def populations(self):
        r = np.empty(self.q * self.num_nodes, np.float32)
        b = np.empty_like(r)
        N.check_cg(self._lib.lbm_cg_get_populations(self._h, _fp(r), _fp(b)))
        return r.reshape(self.q, -1), b.reshape(self.q, -1)

    def laplace(self):
        out = np.zeros(5, np.float64)
        rc = self._lib.lbm_cg_laplace(self._h, out.ctypes.data_as(C.POINTER(C.c_double)))
        if rc not in (N.LBM_OK, N.LBM_DIVERGED):
            N.check_cg(rc)
        return out, rc
