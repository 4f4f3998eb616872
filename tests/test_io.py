"""The reference's file formats (include/thesis_lbm_io.h): init file, Node/BC
files, result writers/readers and the comparison, checked on CPU with files
written in those layouts."""
import ctypes as C
import os

import numpy as np
import pytest

from thesis_gb300 import lattice
from thesis_gb300 import native as N

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")

# An init file in the reference's 23-line layout (FilesReading.cu:60-222):
# "name = value" lines in fixed order, quoted lattice and initial-file names.
INIT = """Lattice = "duct_64x48"
U= 0.04
V= 0.0
W= 0.01
Density = 1.0
viscosity = 0.0333333
InletProfile = INLET_PROF
CollisionModel = MRT
Walls = STRAIGHT
BCwallModel = BBack
BCoutlet = 2ndE
Number of iterations = 2500
AutosaveAfter = 100
AutosaveEach = 500
MinMacroDiffs(u_v_w_rho)(StopCond) = 1.0e-9 2.0e-9 3.0e-9 4.0e-9
OutputFormat = CSV
InitialConditionFromFile = yes
InitialFile = "Restart/state.csv"
ResidualModel = MaxMacroDiff
ResidualsAndMacroDiffsAfter = 50
Force = 0.0001
DragAndLift = 3
UpdateInltOutl = no
"""


def _fp(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def _ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int))


def test_read_init_file(native_lib, tmp_path):
    p = tmp_path / "SetUpData.ini"
    p.write_text(INIT)
    cfg = N.RunConfig()
    assert native_lib.lbm_read_init_file(str(p).encode(), C.byref(cfg)) == N.LBM_OK
    assert cfg.unparsed_lines == 0
    assert cfg.problem_name == b"duct_64x48"
    assert cfg.initial_conditions_name == b"Restart/state.csv"
    assert cfg.u == float(np.float32(0.04)) and cfg.w == float(np.float32(0.01))
    assert cfg.viscosity == float(np.float32(0.0333333))
    assert (cfg.inlet_profile, cfg.collision_model, cfg.boundary_type, cfg.bc_wall_model) == (1, N.MRT, 2, 1)
    assert cfg.outlet_profile == 3  # "2ndE" as the reference maps it
    assert (cfg.iterations, cfg.autosave_after, cfg.autosave_every) == (2500, 100, 500)
    assert list(cfg.stop_condition) == [float(np.float32(v)) for v in (1e-9, 2e-9, 3e-9, 4e-9)]
    assert cfg.output_format == 1 and cfg.use_initial_conditions_file == 1
    assert cfg.residual_model == 3 and cfg.show_macro_diff == 50 and cfg.update_inlet_outlet == 0
    assert cfg.g == float(np.float32(1e-4)) and cfg.boundary_id == 3
    # a broken line is counted, the rest still parses
    p.write_text(INIT.replace("CollisionModel = MRT", "CollisionModel MRT"))
    assert native_lib.lbm_read_init_file(str(p).encode(), C.byref(cfg)) == N.LBM_OK
    assert cfg.unparsed_lines == 1 and cfg.collision_model == N.MRT
    assert native_lib.lbm_read_init_file(str(tmp_path / "missing.ini").encode(), C.byref(cfg)) == N.LBM_ERR_FILE


def test_line_count_counts_cr_and_lf(native_lib, tmp_path):
    p = tmp_path / "a.txt"
    p.write_bytes(b"a\nb\r\nc\n")
    assert native_lib.lbm_count_lines(str(p).encode()) == 4  # '\r' and '\n' both count
    assert native_lib.lbm_count_lines(str(tmp_path / "none").encode()) == -1


@pytest.mark.parametrize("dims", [2, 3])
def test_node_bc_round_trip(native_lib, tmp_path, dims):
    lat = lattice.cavity2d(12, 9) if dims == 2 else lattice.cavity3d(7, 6, 5)
    node, bc = str(tmp_path / "L_Node.dat"), str(tmp_path / "L_BC.dat")
    lattice.write_files(lat, node, bc)
    assert native_lib.lbm_node_file_dims(node.encode()) == dims
    nn = native_lib.lbm_count_lines(node.encode())
    nc = native_lib.lbm_count_lines(bc.encode())
    assert nn == lat.num_nodes and nc == len(lat.bc)
    ni, nj, nk, nt = (np.zeros(nn, np.int32) for _ in range(4))
    x, y, z = (np.zeros(nn, np.float32) for _ in range(3))
    assert native_lib.lbm_read_node_file(node.encode(), dims, nn, _ip(ni), _ip(nj), _ip(nk), _fp(x), _fp(y),
                                         _fp(z), _ip(nt)) == 0
    idx = np.arange(nn)
    assert np.array_equal(ni, idx % lat.n) and np.array_equal(nt, lat.node_type)
    if dims == 3:
        assert np.array_equal(nk, idx // (lat.n * lat.m))
    bi, bj, bk, bd, bt, bid = (np.zeros(nc, np.int32) for _ in range(6))
    bx, by, bz = (np.zeros(nc, np.float32) for _ in range(3))
    assert native_lib.lbm_read_bc_file(bc.encode(), dims, nc, _ip(bi), _ip(bj), _ip(bk), _ip(bd), _ip(bt), _fp(bx),
                                       _fp(by), _fp(bz), _ip(bid)) == 0
    got = np.stack([bi, bj, bk, bd, bt, bid], 1)
    assert np.array_equal(got, lat.bc)
    # the Python reader agrees
    lat2 = lattice.from_files(node, bc)
    assert np.array_equal(lat2.bc, lat.bc) and np.array_equal(lat2.node_type, lat.node_type)


def _fields(n, m, h, seed=0):
    rng = np.random.default_rng(seed)
    N_ = n * m * h
    return [rng.standard_normal(N_).astype(np.float32) * s for s in (0.05, 0.05, 0.02)] + \
        [(1 + 0.01 * rng.standard_normal(N_)).astype(np.float32)]


@pytest.mark.parametrize("fmt", [1, 2, 3])
def test_results_write_read_compare(native_lib, tmp_path, fmt):
    n, m, h = 9, 7, 3
    u, v, w, rho = _fields(n, m, h)
    lat = lattice.cavity3d(n, m, h)
    x, y, z = (a.astype(np.float32) for a in lat.coords())
    ext = {1: "csv", 2: "dat", 3: "vti"}[fmt]
    p1 = str(tmp_path / ("a." + ext))
    assert native_lib.lbm_write_results(p1.encode(), fmt, n, m, h, _fp(x), _fp(y), _fp(z), _fp(u), _fp(v), _fp(w),
                                        _fp(rho)) == 0
    N_ = n * m * h
    lines = native_lib.lbm_count_lines(p1.encode())
    assert lines == {1: N_ + 1, 2: N_ + 3, 3: 3 * N_ + 18}[fmt]
    cols = np.zeros(9 * N_)
    rows = native_lib.lbm_read_results(p1.encode(), N_, cols.ctypes.data_as(C.POINTER(C.c_double)))
    assert rows == N_
    cols = cols.reshape(9, N_)
    np.testing.assert_allclose(cols[3], u, atol=1e-9)
    np.testing.assert_allclose(cols[7], rho, atol=1e-9)
    if fmt != 3:
        np.testing.assert_allclose(cols[6], np.sqrt(u.astype(np.float64) ** 2 + v.astype(np.float64) ** 2 +
                                                    w.astype(np.float64) ** 2), atol=1e-9)
        np.testing.assert_allclose(cols[8], rho / np.float32(3), atol=1e-9)
    # restart input: the same file read back as initial conditions
    ru, rv, rw, rr = (np.zeros(N_, np.float32) for _ in range(4))
    assert native_lib.lbm_read_initial_conditions(p1.encode(), N_, n, m, h, _fp(ru), _fp(rv), _fp(rw), _fp(rr)) == 0
    np.testing.assert_allclose(ru, u, atol=1e-9)
    np.testing.assert_allclose(rr, rho, atol=1e-9)
    # comparison: identical files match, a perturbed one does not
    p2 = str(tmp_path / ("b." + ext))
    u2 = u.copy()
    u2[5] += 0.01
    native_lib.lbm_write_results(p2.encode(), fmt, n, m, h, _fp(x), _fp(y), _fp(z), _fp(u2), _fp(v), _fp(w),
                                 _fp(rho))
    s, mx = np.zeros(9), np.zeros(9)
    dp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
    assert native_lib.lbm_compare_results(p1.encode(), p1.encode(), dp(s), dp(mx)) == 0
    assert native_lib.lbm_compare_results(p1.encode(), p2.encode(), dp(s), dp(mx)) == 1
    assert abs(mx[3] - 0.01) < 1e-6 and s[4] == 0.0


def test_csv_layout_matches_reference_writer(native_lib, tmp_path):
    """The CSV line layout of WriteResults3D (FilesWriting.cu:156-171)."""
    one = lambda v: np.array([v], np.float32)
    p = str(tmp_path / "r.csv")
    native_lib.lbm_write_results(p.encode(), 1, 1, 1, 1, _fp(one(0.5)), _fp(one(0.25)), _fp(one(0.0)),
                                 _fp(one(0.1)), _fp(one(-0.2)), _fp(one(0.0)), _fp(one(1.0)))
    lines = open(p).read().splitlines()
    assert lines[0] == "x,y,z,u,v,w,vel_mag,rho,press"
    f32 = lambda v: float(np.float32(v))
    vm = np.sqrt(f32(0.1) ** 2 + f32(-0.2) ** 2)
    expect = "%.10f, %.10f, %.10f, %.10f, %.10f, %.10f, %.10f, %.10f, %.10f" % (
        0.5, 0.25, 0.0, f32(0.1), f32(-0.2), 0.0, vm, 1.0, f32(np.float32(1.0) / np.float32(3)))
    assert lines[1] == expect


def test_compare_line_mismatch(native_lib, tmp_path):
    a, b = tmp_path / "a.csv", tmp_path / "b.csv"
    a.write_text("x,y,z,u,v,w,vel_mag,rho,press\n0, 0, 0, 0, 0, 0, 0, 1, 0.3\n")
    b.write_text("x,y,z,u,v,w,vel_mag,rho,press\n")
    assert native_lib.lbm_compare_results(str(a).encode(), str(b).encode(), None, None) == N.LBM_ERR_FILE


def test_midlines_and_cross_section(native_lib, tmp_path):
    n, m, h = 9, 7, 5
    lat = lattice.cavity3d(n, m, h)
    x, y, z = (a.astype(np.float32) for a in lat.coords())
    u, v, w, _ = _fields(n, m, h, 3)
    p = str(tmp_path / "midLines.txt")
    assert native_lib.lbm_write_midlines(p.encode(), 3, n, m, h, _fp(x), _fp(y), _fp(z), _fp(u), _fp(v), _fp(w),
                                         0.1) == 0
    lines = open(p).read().splitlines()
    assert lines[0] == "CASE: Ulid = 0.100000 Nx = %d" % n and lines[1] == "U/Ulid\tZ\tX\tW/Ulid"
    rows = np.array([[float(c) for c in ln.split("\t")] for ln in lines[2:]])
    assert rows.shape == (h, 4)
    ids = (n // 2) + n * ((m // 2) + m * np.arange(h))
    np.testing.assert_allclose(rows[:, 0], u[ids] / np.float32(0.1), atol=1e-7)
    np.testing.assert_allclose(rows[:, 1], z[ids], atol=1e-7)
    # 2D: u along x = n/2, v along y = m/2
    lat2 = lattice.cavity2d(8, 6)
    x2, y2, z2 = (a.astype(np.float32) for a in lat2.coords())
    u2, v2, w2, _ = _fields(8, 6, 1, 4)
    p2 = str(tmp_path / "mid2d.txt")
    assert native_lib.lbm_write_midlines(p2.encode(), 2, 8, 6, 1, _fp(x2), _fp(y2), _fp(z2), _fp(u2), _fp(v2),
                                         _fp(w2), 0.1) == 0
    r2 = np.array([[float(c) for c in ln.split("\t")] for ln in open(p2).read().splitlines()[2:]])
    np.testing.assert_allclose(r2[:6, 0], u2[4 + 8 * np.arange(6)] / np.float32(0.1), atol=1e-7)
    np.testing.assert_allclose(r2[:8, 3], v2[np.arange(8) + 8 * 3] / np.float32(0.1), atol=1e-7)
    # cross-section at x = 3n/4
    p3 = str(tmp_path / "channelPlane.txt")
    assert native_lib.lbm_write_cross_section(p3.encode(), n, m, h, _fp(x), _fp(y), _fp(z), _fp(u), _fp(v),
                                              _fp(w), 0.05) == 0
    l3 = open(p3).read().splitlines()
    assert l3[1] == "X\tY\tZ\tU\tV\tW" and len(l3) == 2 + m * h
    first = [float(c) for c in l3[2].split()]
    assert abs(first[3] - u[int(0.75 * n)]) < 1e-9
