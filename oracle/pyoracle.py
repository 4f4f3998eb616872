"""ctypes binding of the oracle restatement (oracle/lbm_oracle.cpp) and of the
reference kernels run on the host (oracle/_ref/libreflbm_*.so, built here from
the reference tree by oracle/build_ref.sh; absent on machines without it).

TEST INFRASTRUCTURE ONLY.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
ORACLE_SO = os.path.join(BUILD, "liboracle_lbm.so")
REF_DIR = os.path.join(HERE, "_ref")

ORC_OK, ORC_UNSUPPORTED, ORC_BAD_INPUT = 0, 3, 4


def reference_root():
    """Root of the reference project's tree when it is mounted (environment
    variable THESIS_REFERENCE_ROOT, else its usual mount point), or None."""
    root = os.environ.get("THESIS_REFERENCE_ROOT", "/root/reference")
    return root if os.path.isdir(root) else None


def reference_file(*parts):
    """Path of a file inside the reference tree, or None when it is absent."""
    root = reference_root()
    if root is None:
        return None
    path = os.path.join(root, *parts)
    return path if os.path.exists(path) else None

_RP = ["u", "v", "w", "rho", "viscosity", "g"]
_RI = ["inlet_profile", "outlet_profile", "collision_model", "boundary_type", "bc_wall_model",
       "update_inlet_outlet", "boundary_id"]
_RD = ["delta", "min_inlet_y", "max_inlet_y", "min_inlet_z", "max_inlet_z"]


class RefParams(C.Structure):
    _fields_ = [(k, C.c_double) for k in _RP] + [(k, C.c_int) for k in _RI] + [(k, C.c_double) for k in _RD]


class OrcParams(C.Structure):
    _fields_ = RefParams._fields_ + [("mode", C.c_int), ("init_kind", C.c_int),
                                     ("rho_in", C.c_double), ("rho_out", C.c_double),
                                     ("periodic", C.c_int * 3), ("link_q", C.POINTER(C.c_double))]


def build_oracle(force=False):
    """Compile the oracle with g++ (OpenMP, no FMA contraction)."""
    src = os.path.join(HERE, "lbm_oracle.cpp")
    if not force and os.path.exists(ORACLE_SO) and os.path.getmtime(ORACLE_SO) >= os.path.getmtime(src):
        return ORACLE_SO
    os.makedirs(BUILD, exist_ok=True)
    tmp = ORACLE_SO + ".tmp"
    subprocess.run(["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-fopenmp",
                    src, "-o", tmp], check=True)
    os.replace(tmp, ORACLE_SO)
    return ORACLE_SO


_orc = None


def oracle_lib():
    global _orc
    if _orc is None:
        _orc = C.CDLL(build_oracle())
    return _orc


def ref_lib(fp64=False):
    path = os.path.join(REF_DIR, "libreflbm_f64.so" if fp64 else "libreflbm_f32.so")
    if not os.path.exists(path):
        return None
    return C.CDLL(path)


def _vp(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _params(cls, kw):
    p = cls()
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def default_params(**kw):
    base = dict(u=0.0, v=0.0, w=0.0, rho=1.0, viscosity=0.1, g=0.0, inlet_profile=2,
                outlet_profile=2, collision_model=1, boundary_type=2, bc_wall_model=1,
                update_inlet_outlet=1, boundary_id=0, delta=1.0, min_inlet_y=0.0,
                max_inlet_y=0.0, min_inlet_z=0.0, max_inlet_z=0.0)
    base.update(kw)
    return base


def _cols(lat):
    return [np.ascontiguousarray(lat.bc[:, k], dtype=np.int32) for k in range(6)]


class Result:
    pass


def run_oracle(lat, steps, fp64=False, mode=0, init_kind=0, rho_in=1.0, rho_out=1.0,
               extra_collide=False, init=None, periodic=(0, 0, 0), link_q=None, **kw):
    """Run the oracle restatement; returns a Result with f, fc (q, N), rho,
    u, v, w (N), mask, stream, count, resid, rc.  link_q: curved walls' link
    fractions, one per BC link (boundary_type=1)."""
    L = oracle_lib()
    q = lat.q
    nn = lat.num_nodes
    p = _params(OrcParams, dict(default_params(**kw), mode=mode, init_kind=init_kind,
                                rho_in=rho_in, rho_out=rho_out))
    for a in range(3):
        p.periodic[a] = int(periodic[a])
    lq = None
    if link_q is not None:
        lq = np.ascontiguousarray(link_q, np.float64)
        p.link_q = lq.ctypes.data_as(C.POINTER(C.c_double))
    cols = _cols(lat)
    r = Result()
    r.f, r.fc = np.zeros(q * nn), np.zeros(q * nn)
    r.rho, r.u, r.v, r.w = (np.zeros(nn) for _ in range(4))
    r.mask = np.zeros(nn, np.uint64)
    r.stream = np.zeros((q - 1) * nn, np.uint8)
    r.resid = np.zeros(max(steps, 1))
    cnt = C.c_int(0)
    ini = [None] * 4
    if init is not None:
        ini = [None if a is None else np.ascontiguousarray(a, np.float64) for a in init]
    r.rc = L.orc_run(int(fp64), lat.dims, lat.n, lat.m, lat.h, _vp(lat.node_type), int(lat.bc.shape[0]),
                     _vp(cols[0]), _vp(cols[1]), _vp(cols[2]) if lat.dims == 3 else None,
                     _vp(cols[3]), _vp(cols[4]), _vp(cols[5]), C.byref(p),
                     _vp(ini[1]), _vp(ini[2]), _vp(ini[3]), _vp(ini[0]), int(steps), int(extra_collide),
                     _vp(r.f), _vp(r.fc), _vp(r.rho), _vp(r.u), _vp(r.v), _vp(r.w), _vp(r.mask),
                     _vp(r.stream), C.byref(cnt), _vp(r.resid))
    r.count = cnt.value
    r.f, r.fc = r.f.reshape(q, nn), r.fc.reshape(q, nn)
    return r


def curved_bc_points(lat, link_q, delta=1.0):
    """BC-file boundary points that give the links the fractions link_q:
    node + q delta c_dir (the reference's q = |B - X| / (delta |c_dir|))."""
    from thesis_gb300.lattice import CX2, CX3, CY2, CY3, CZ3
    cols = _cols(lat)
    x, y, z = lat.coords(delta)
    ind = cols[0] + lat.n * (cols[1] + lat.m * cols[2])
    d = cols[3]
    if lat.q == 9:
        cx, cy, cz = CX2[d], CY2[d], np.zeros(d.size)
    else:
        cx, cy, cz = CX3[d], CY3[d], CZ3[d]
    qv = np.asarray(link_q, np.float64) * delta
    return x[ind] + qv * cx, y[ind] + qv * cy, z[ind] + qv * cz


def reference_q(lat, link_q, delta=1.0, fp64=False):
    """The link fractions the reference derives from the BC points that
    curved_bc_points writes: sqrt(dx^2 + dy^2 [+ dz^2]) / (delta qLat) in its
    FLOAT_TYPE (GpuInit.cu:1084-1088, :1199-1207), qLat = sqrt(2) rounded
    to FLOAT_TYPE on the diagonals."""
    from thesis_gb300.lattice import CX2, CX3, CY2, CY3, CZ3
    t = np.float64 if fp64 else np.float32
    cols = _cols(lat)
    x, y, z = lat.coords(delta)
    ind = cols[0] + lat.n * (cols[1] + lat.m * cols[2])
    bx, by, bz = curved_bc_points(lat, link_q, delta)
    dx = t(bx) - t(x[ind])
    dy = t(by) - t(y[ind])
    s2 = dx * dx + dy * dy
    if lat.dims == 3:
        dz = t(bz) - t(z[ind])
        s2 = s2 + dz * dz
        diag = (np.abs(CX3) + np.abs(CY3) + np.abs(CZ3))[cols[3]] == 2
    else:
        diag = (np.abs(CX2) + np.abs(CY2))[cols[3]] == 2
    qlat = np.where(diag, t(np.sqrt(2.0)), t(1.0)).astype(t)
    return (np.sqrt(s2).astype(t) / (t(delta) * qlat)).astype(np.float64)


def run_reference(lat, steps, fp64=False, link_q=None, **kw):
    """Run the reference's own kernels on the host (oracle/_ref).  Returns
    None when oracle/_ref has not been built on this machine.  link_q: curved
    walls' link fractions, passed as BC-file boundary points."""
    L = ref_lib(fp64)
    if L is None:
        return None
    q = lat.q
    nn = lat.num_nodes
    p = _params(RefParams, default_params(**kw))
    cols = _cols(lat)
    x, y, z = lat.coords(kw.get("delta", 1.0))
    x, y, z = (np.ascontiguousarray(a, np.float64) for a in (x, y, z))
    bx = np.ascontiguousarray(x[cols[0] + lat.n * (cols[1] + lat.m * cols[2])] if len(cols[0]) else np.zeros(0))
    by = np.ascontiguousarray(y[cols[0] + lat.n * (cols[1] + lat.m * cols[2])] if len(cols[0]) else np.zeros(0))
    bz = np.ascontiguousarray(z[cols[0] + lat.n * (cols[1] + lat.m * cols[2])] if len(cols[0]) else np.zeros(0))
    if link_q is not None:
        bx, by, bz = (np.ascontiguousarray(a, np.float64) for a in curved_bc_points(lat, link_q, kw.get("delta", 1.0)))
    r = Result()
    r.f, r.fc = np.zeros(q * nn), np.zeros(q * nn)
    r.rho, r.u, r.v, r.w = (np.zeros(nn) for _ in range(4))
    r.resid = np.zeros(max(steps, 1))
    cnt = C.c_int(0)
    if lat.dims == 2:
        r.mask32 = np.zeros(nn, np.int32)
        r.stream32 = np.zeros(8 * nn, np.int32)
        r.rc = L.ref_run2d(lat.n, lat.m, _vp(lat.node_type), _vp(x), _vp(y), int(lat.bc.shape[0]),
                           _vp(cols[0]), _vp(cols[1]), _vp(cols[3]), _vp(cols[4]), _vp(cols[5]),
                           _vp(bx), _vp(by), C.byref(p), int(steps), _vp(r.f), _vp(r.fc), _vp(r.rho),
                           _vp(r.u), _vp(r.v), _vp(r.mask32), _vp(r.stream32), C.byref(cnt), _vp(r.resid))
        r.mask = r.mask32.astype(np.uint32).astype(np.uint64)
        r.stream = r.stream32.astype(np.uint8)
    else:
        r.mask = np.zeros(nn, np.uint64)
        r.stream = np.zeros(18 * nn, np.uint8)
        r.rc = L.ref_run3d(lat.n, lat.m, lat.h, _vp(lat.node_type), _vp(x), _vp(y), _vp(z),
                           int(lat.bc.shape[0]), *[_vp(c) for c in cols[:5]], _vp(cols[5]),
                           _vp(bx), _vp(by), _vp(bz), C.byref(p), int(steps), _vp(r.f), _vp(r.fc),
                           _vp(r.rho), _vp(r.u), _vp(r.v), _vp(r.w), _vp(r.mask), _vp(r.stream),
                           C.byref(cnt), _vp(r.resid))
    r.count = cnt.value
    r.f, r.fc = r.f.reshape(q, nn), r.fc.reshape(q, nn)
    return r


class CgParams(C.Structure):
    _fields_ = [(k, C.c_double) for k in ("r_density", "b_density", "r_alpha", "b_alpha", "r_viscosity",
                                          "b_viscosity", "beta", "A", "g_limit", "control_param", "g")] + \
               [(k, C.c_int) for k in ("high_order", "enhanced", "external_force")]


def cg_params(**kw):
    base = dict(r_density=1.0, b_density=1.0, r_alpha=4 / 9, b_alpha=4 / 9, r_viscosity=1 / 6,
                b_viscosity=1 / 6, beta=0.7, A=0.005, g_limit=0.0, control_param=0.9, g=0.0,
                high_order=0, enhanced=0, external_force=0)
    base.update(kw)
    return _params(CgParams, base)


def cg_rest_populations(alpha, density):
    """Colour populations of a fluid at rest (GpuInit.cu:323-360):
    density * (alpha, (1-alpha)/5 x4, (1-alpha)/20 x4)."""
    return density * np.array([alpha] + [(1 - alpha) / 5] * 4 + [(1 - alpha) / 20] * 4)


def droplet(n, m, radius, p, centre=None):
    """Red droplet in blue at rest: per-colour populations (9, N) each."""
    cx, cy = centre if centre is not None else ((n - 1) / 2, (m - 1) / 2)
    idx = np.arange(n * m)
    x, y = idx % n, idx // n
    inside = (x - cx) ** 2 + (y - cy) ** 2 <= radius ** 2
    r = np.where(inside[None, :], cg_rest_populations(p.r_alpha, p.r_density)[:, None], 0.0)
    b = np.where(~inside[None, :], cg_rest_populations(p.b_alpha, p.b_density)[:, None], 0.0)
    return np.ascontiguousarray(r), np.ascontiguousarray(b)


def run_oracle_cg(n, m, p, r0, b0, steps, fp64=False, extra_collide=False):
    L = oracle_lib()
    nn = n * m
    r = Result()
    r.rf, r.bf, r.rfc, r.bfc = (np.zeros(9 * nn) for _ in range(4))
    r.rr, r.br, r.u, r.v = (np.zeros(nn) for _ in range(4))
    r.laplace = np.zeros(5)
    r0 = np.ascontiguousarray(r0, np.float64).reshape(-1)
    b0 = np.ascontiguousarray(b0, np.float64).reshape(-1)
    r.rc = L.orc_run_cg2d(int(fp64), n, m, C.byref(p), _vp(r0), _vp(b0), int(steps), int(extra_collide),
                          _vp(r.rf), _vp(r.bf), _vp(r.rfc), _vp(r.bfc), _vp(r.rr), _vp(r.br), _vp(r.u),
                          _vp(r.v), _vp(r.laplace))
    for k in ("rf", "bf", "rfc", "bfc"):
        setattr(r, k, getattr(r, k).reshape(9, nn))
    return r


def cg_collide_pair(n, m, p, rho, r_rho, b_rho, u, v, f, fp64=False):
    """One colour-gradient collision by the oracle and, where oracle/_ref
    exists, by the reference kernel; returns (oracle (rfc, bfc), reference
    (rfc, bfc, cg_dir) or None)."""
    arrs = [np.ascontiguousarray(a, np.float64).reshape(-1) for a in (rho, r_rho, b_rho, u, v, f)]
    nn = n * m
    orc = (np.zeros(9 * nn), np.zeros(9 * nn))
    rc = oracle_lib().orc_cg2d_collide(int(fp64), n, m, C.byref(p), *[_vp(a) for a in arrs],
                                       _vp(orc[0]), _vp(orc[1]))
    assert rc == 0
    ref = None
    L = ref_lib(fp64)
    if L is not None:
        rr, bb, cd = np.zeros(9 * nn), np.zeros(9 * nn), np.zeros(nn, np.int32)
        L.ref_cg2d_collide(n, m, C.byref(p), *[_vp(a) for a in arrs], _vp(rr), _vp(bb), _vp(cd))
        ref = (rr.reshape(9, nn), bb.reshape(9, nn), cd)
    return (orc[0].reshape(9, nn), orc[1].reshape(9, nn)), ref


def cg3_rest_populations(alpha, density):
    """D3Q19 colour populations at rest (initCGBubble3D, GpuInit.cu:536-600,
    with phi3D + theta3D alpha): density * (alpha, (1-alpha)/12 x6,
    (1-alpha)/24 x12)."""
    return density * np.array([alpha] + [(1 - alpha) / 12] * 6 + [(1 - alpha) / 24] * 12)


def droplet3d(n, m, h, radius, p, centre=None):
    """Red droplet in blue at rest on an n x m x h lattice: (19, N) each."""
    c = centre if centre is not None else ((n - 1) / 2, (m - 1) / 2, (h - 1) / 2)
    idx = np.arange(n * m * h)
    x, y, z = idx % n, (idx // n) % m, idx // (n * m)
    inside = (x - c[0]) ** 2 + (y - c[1]) ** 2 + (z - c[2]) ** 2 <= radius ** 2
    r = np.where(inside[None, :], cg3_rest_populations(p.r_alpha, p.r_density)[:, None], 0.0)
    b = np.where(~inside[None, :], cg3_rest_populations(p.b_alpha, p.b_density)[:, None], 0.0)
    return np.ascontiguousarray(r), np.ascontiguousarray(b)


def run_oracle_cg3(n, m, h, p, r0, b0, steps, fp64=False, extra_collide=False):
    """The D3Q19 colour-gradient loop in the oracle: Result with rfc, bfc
    (19, N), rr, br, u, v, w (N), laplace (5), rc."""
    L = oracle_lib()
    nn = n * m * h
    r = Result()
    r.rfc, r.bfc = np.zeros(19 * nn), np.zeros(19 * nn)
    r.rr, r.br, r.u, r.v, r.w = (np.zeros(nn) for _ in range(5))
    r.laplace = np.zeros(5)
    r0 = np.ascontiguousarray(r0, np.float64).reshape(-1)
    b0 = np.ascontiguousarray(b0, np.float64).reshape(-1)
    r.rc = L.orc_run_cg3d(int(fp64), n, m, h, C.byref(p), _vp(r0), _vp(b0), int(steps), int(extra_collide),
                          _vp(r.rfc), _vp(r.bfc), _vp(r.rr), _vp(r.br), _vp(r.u), _vp(r.v), _vp(r.w),
                          _vp(r.laplace))
    r.rfc, r.bfc = r.rfc.reshape(19, nn), r.bfc.reshape(19, nn)
    return r


def cg3_collide_pair(n, m, h, p, rho, r_rho, b_rho, u, v, w, f, fp64=False):
    """One D3Q19 colour-gradient collision by the oracle and, where
    oracle/_ref exists, by the reference kernel; as cg_collide_pair."""
    arrs = [np.ascontiguousarray(a, np.float64).reshape(-1) for a in (rho, r_rho, b_rho, u, v, w, f)]
    nn = n * m * h
    orc = (np.zeros(19 * nn), np.zeros(19 * nn))
    rc = oracle_lib().orc_cg3d_collide(int(fp64), n, m, h, C.byref(p), *[_vp(a) for a in arrs],
                                       _vp(orc[0]), _vp(orc[1]))
    assert rc == 0
    ref = None
    L = ref_lib(fp64)
    if L is not None:
        rr, bb, cd = np.zeros(19 * nn), np.zeros(19 * nn), np.zeros(nn, np.int32)
        L.ref_cg3d_collide(n, m, h, C.byref(p), *[_vp(a) for a in arrs], _vp(rr), _vp(bb), _vp(cd))
        ref = (rr.reshape(19, nn), bb.reshape(19, nn), cd)
    return (orc[0].reshape(19, nn), orc[1].reshape(19, nn)), ref


class RefCpuCgParams(C.Structure):
    _fields_ = [(k, C.c_double) for k in ("r_density", "b_density", "r_alpha", "b_alpha", "r_viscosity",
                                          "b_viscosity", "beta", "A", "g_limit", "control_param", "bubble_radius")]


def run_reference_cpu_cg(n, m, steps, **kw):
    """The reference's serial CPU colour-gradient loop (Multiphase.cu through
    oracle/ref_shim/ref_cpu_cg.cpp) from its test-case-1 bubble; returns
    (r_rho, b_rho, seconds), or None where oracle/_ref is absent."""
    import time
    path = os.path.join(REF_DIR, "libref_multiphase.so")
    if not os.path.exists(path):
        return None
    L = C.CDLL(path)
    base = dict(r_density=1.0, b_density=1.0, r_alpha=4 / 9, b_alpha=4 / 9, r_viscosity=1 / 6, b_viscosity=1 / 6,
                beta=0.7, A=0.005, g_limit=0.0, control_param=0.9, bubble_radius=0.25)
    base.update(kw)
    p = _params(RefCpuCgParams, base)
    rr, bb = np.zeros(n * m), np.zeros(n * m)
    t0 = time.perf_counter()
    rc = L.ref_cpu_cg2d(n, m, C.byref(p), int(steps), _vp(rr), _vp(bb))
    dt = time.perf_counter() - t0
    assert rc == 0
    return rr, bb, dt
