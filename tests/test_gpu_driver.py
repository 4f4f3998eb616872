"""The file-driven drop-in (thesis_lbm_run): init file + Mesh/ files in the
reference's formats in, FinalData and MacroDiffs out, on the GPU; and the
MaxMacroDiff residual."""
import os
import subprocess

import numpy as np
import pytest

from thesis_gb300 import build, lattice
from thesis_gb300 import native as N
from thesis_gb300.solver import Arguments, Solver

pytestmark = pytest.mark.gpu

INIT = """Lattice = "cav"
U= 0.1
V= 0.0
W= 0.0
Density = 1.0
viscosity = 0.128
InletProfile = INLET_CTE
CollisionModel = {coll}
Walls = STRAIGHT
BCwallModel = BBack
BCoutlet = Vout
Number of iterations = {iters}
AutosaveAfter = 0
AutosaveEach = 0
MinMacroDiffs(u_v_w_rho)(StopCond) = {stop}
OutputFormat = {fmt}
InitialConditionFromFile = {ic}
InitialFile = "{icfile}"
ResidualModel = {resmodel}
ResidualsAndMacroDiffsAfter = 100
Force = 0
DragAndLift = {dl}
UpdateInltOutl = yes
"""


def _setup(tmp_path, lat, **kw):
    (tmp_path / "Mesh").mkdir(exist_ok=True)
    lattice.write_files(lat, str(tmp_path / "Mesh" / "cav_Node.dat"), str(tmp_path / "Mesh" / "cav_BC.dat"))
    d = dict(coll="SRT", iters=400, stop="0 0 0 0", fmt="CSV", ic="no", icfile="none", resmodel="MaxMacroDiff",
             dl=0)
    d.update(kw)
    (tmp_path / "SetUpData.ini").write_text(INIT.format(**d))


def _run(tmp_path, *args):
    build.build()
    exe = build.tool_path("thesis_lbm_run")
    return subprocess.run([exe] + list(args), cwd=str(tmp_path), capture_output=True, text=True, timeout=600)


def test_driver_matches_api_run(tmp_path):
    lat = lattice.cavity2d(40, 32)
    _setup(tmp_path, lat)
    r = _run(tmp_path)
    assert r.returncode == 0, r.stderr
    out = tmp_path / "Results" / "FinalData.csv"
    rows = np.loadtxt(out, delimiter=",", skiprows=1)
    assert rows.shape == (lat.num_nodes, 9)
    # the init file's values are parsed into FP32, as the reference does
    f32 = lambda v: float(np.float32(v))
    with Solver(lat, Arguments(u=f32(0.1), viscosity=f32(0.128), collision_model=N.BGKW, outlet_profile=1)) as s:
        s.init()
        s.step(400, write_macro=True)
        rho, u, v, w = s.macro()
    # same library, same steps: equal up to the %.10f formatting of the file
    np.testing.assert_allclose(rows[:, 3], u, atol=6e-11)
    np.testing.assert_allclose(rows[:, 7], rho, atol=6e-11)
    md = (tmp_path / "Results" / "MacroDiffs.txt").read_text().splitlines()
    assert md[0].startswith("iteration") and len(md) == 1 + 4  # checks at 100, 200, 300, 400
    # compare subcommand: identical files agree, an edited one does not
    assert _run(tmp_path, "compare", str(out), str(out)).returncode == 0
    edited = tmp_path / "edited.csv"
    lines = out.read_text().splitlines()
    parts = lines[5].split(", ")
    parts[3] = "%.10f" % (float(parts[3]) + 0.01)
    lines[5] = ", ".join(parts)
    edited.write_text("\n".join(lines) + "\n")
    assert _run(tmp_path, "compare", str(out), str(edited)).returncode == 1


def test_driver_stop_condition_and_restart(tmp_path):
    lat = lattice.cavity2d(24)
    # changes per 100 steps below 1e-6 (physics mode: the lid is a moving
    # wall, which conserves mass, so the density settles too)
    stop = "1e-6 1e-6 1e-6 1e-6"
    _setup(tmp_path, lat, iters=100000, stop=stop, coll="MRT")
    r = _run(tmp_path, "--physics")
    md = (tmp_path / "Results" / "MacroDiffs.txt").read_text().splitlines()
    assert r.returncode == 0 and "converged" in r.stdout, (r.stderr, md[-3:])
    last = [float(x) for x in md[-1].split()[1:]]
    assert len(md) < 1000 and max(last) < 1e-6
    # restart from the converged field (physics mode starts from f_eq of the
    # given fields): far fewer checks until the stop test holds
    (tmp_path / "Restart").mkdir()
    os.replace(tmp_path / "Results" / "FinalData.csv", tmp_path / "Restart" / "s.csv")
    _setup(tmp_path, lat, iters=100000, stop=stop, coll="MRT", ic="yes", icfile="Restart/s.csv")
    r = _run(tmp_path, "-o", "Run2", "--physics")
    assert r.returncode == 0, r.stderr
    md2 = (tmp_path / "Run2" / "MacroDiffs.txt").read_text().splitlines()
    assert len(md2) < len(md)


def test_driver_fd_rel_diff_residual_model(tmp_path):
    """ResidualModel MaxRelativeFdDiff: the residual is written every 100
    steps to Residuals.txt, decreases as the cavity settles, and the run stops
    once it is below StopCondition[0]."""
    lat = lattice.cavity2d(24)
    _setup(tmp_path, lat, iters=200000, stop="1e-5 0 0 0", coll="MRT", resmodel="MaxRelativeFdDiff")
    r = _run(tmp_path, "--physics")
    assert r.returncode == 0 and "converged" in r.stdout, r.stderr
    rows = _residual_rows(tmp_path, 200000)
    # the file is the reference's: one row per iteration, in 2D the L2 norm
    # at the checks (every 100 steps until the FdRelDiff stop test held)
    chk = rows[rows[:, 1] != 0]
    assert 2 <= len(chk) < 2000 and chk[-1, 1] < chk[0, 1]
    assert np.all(chk[:, 0] % 100 == 99)


def test_driver_l2_residual_model(tmp_path):
    """ResidualModel L2: sqrt(sum (f - fColl)^2) every 100 steps in
    Residuals.txt, equal to the API's value at the end of the same run (it
    settles at the size of the steady streaming step, not at zero)."""
    lat = lattice.cavity2d(24)
    _setup(tmp_path, lat, iters=1000, stop="0 0 0 0", coll="MRT", resmodel="L2")
    r = _run(tmp_path, "--physics")
    assert r.returncode == 0, r.stderr
    rows = _residual_rows(tmp_path, 1000)
    chk = rows[rows[:, 1] != 0]
    assert len(chk) == 10 and np.array_equal(chk[:, 0], np.arange(99, 1000, 100))
    np.testing.assert_allclose(chk[:, 2], chk[:, 1] / lat.num_nodes, rtol=2e-4)
    f32 = lambda v: float(np.float32(v))
    args = Arguments(u=f32(0.1), viscosity=f32(0.128), collision_model=N.MRT, mode=N.MODE_PHYSICS, init_equilibrium=1)
    with Solver(lat, args) as s:
        s.init()
        s.step(1000, write_macro=True)
        want, rc = s.residual_l2()
    assert abs(rows[999, 1] - want) <= 1e-4 * want  # %5.4e in the file


def _residual_rows(tmp_path, iterations):
    lines = (tmp_path / "Results" / "Residuals.txt").read_text().splitlines()
    assert lines[0] == "Iter L2_norm L2_norm_weighted Drag Lift"
    rows = np.array([[float(v) for v in ln.split()] for ln in lines[1:]])
    assert rows.shape == (iterations, 5) and np.array_equal(rows[:, 0], np.arange(iterations))
    return rows


def test_driver_reference_drag_lift_columns(tmp_path):
    """BoundaryId (init file line 22): the Drag and Lift columns hold the
    reference's sums 0.33333333 rho (20 - x) 0.2 and (20 - y) over the fluid
    nodes of that boundary id at every check (gpuUpdateMacro2D, computeDragLift2D),
    equal at the last check to the sums over the final density."""
    lat = lattice.cylinder_channel2d(48, 24)
    bc = lat.bc.copy()
    # the cylinder's links (their target node lies inside the lattice) get id 1
    tx = bc[:, 0] + lattice.CX2[bc[:, 3]]
    ty = bc[:, 1] + lattice.CY2[bc[:, 3]]
    obstacle = (tx >= 0) & (tx < lat.n) & (ty >= 0) & (ty < lat.m)
    bc[obstacle, 5] = 1
    lat = lattice.Lattice(2, lat.n, lat.m, 1, lat.node_type, bc)
    _setup(tmp_path, lat, iters=300, dl=1)
    r = _run(tmp_path)
    assert r.returncode == 0, r.stderr
    rows = _residual_rows(tmp_path, 300)
    chk = rows[rows[:, 1] != 0]
    assert len(chk) == 3 and np.all(chk[:, 3] > 0) and np.all(chk[:, 4] > 0)
    data = np.loadtxt(tmp_path / "Results" / "FinalData.csv", delimiter=",", skiprows=1)
    x, y, rho = data[:, 0].astype(np.float32), data[:, 1].astype(np.float32), data[:, 7]
    nodes = np.unique(bc[obstacle, 0] + lat.n * bc[obstacle, 1])
    nodes = nodes[lat.node_type[nodes] == 1]
    drag = np.float32(0.33333333 * rho[nodes] * (np.float32(20) - x[nodes]).astype(np.float64) * 0.2).sum()
    lift = np.float32(0.33333333 * rho[nodes] * (np.float32(20) - y[nodes]).astype(np.float64) * 0.2).sum()
    np.testing.assert_allclose(rows[299, 3], drag, rtol=1e-6)
    np.testing.assert_allclose(rows[299, 4], lift, rtol=1e-6)


def test_driver_missing_lattice(tmp_path):
    (tmp_path / "SetUpData.ini").write_text(INIT.format(coll="SRT", iters=10, stop="0 0 0 0", fmt="CSV", ic="no",
                                                        icfile="x", resmodel="MaxMacroDiff", dl=0))
    assert _run(tmp_path).returncode == 2


def test_macro_diff_semantics():
    lat = lattice.cavity2d(20)
    with Solver(lat, Arguments(u=0.1, viscosity=0.1, collision_model=N.BGKW, mode=N.MODE_PHYSICS,
                               init_equilibrium=1)) as s:
        s.init()
        s.step(10, write_macro=True)
        _, u0, v0, _ = [a.astype(np.float64) for a in s.macro()]
        d, rc = s.macro_diff()
        assert rc == N.LBM_OK
        # first call: against the initial fields (u = 0.1 everywhere, from params)
        assert abs(d[0] - np.abs(u0 - np.float32(0.1)).max()) < 1e-7
        assert abs(d[1] - np.abs(v0).max()) < 1e-7
        s.step(10, write_macro=True)
        _, u1, v1, _ = [a.astype(np.float64) for a in s.macro()]
        d, rc = s.macro_diff()
        assert abs(d[0] - np.abs(u1 - u0).max()) < 1e-7 and d[4] == 0
