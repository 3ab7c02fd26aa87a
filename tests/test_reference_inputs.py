"""The reference's own input files through the command line.

The reference ships input files beside its sources (heat.lua, scalar_wave.lua,
scalar_wave_1d.lua, eigenvalues.lua, lua-configs/brady_livescu_4_3*.lua).
tests/golden/reference_inputs.json holds their `simulation` tables as the command line's Lua
reader evaluates them, with the exit status of `shoccs --check` on each.

* CPU, where the reference tree is present: `shoccs --check` on the unchanged files exits as
  recorded (0; 1 for the driver template brady_livescu_4_3.lua, whose unfilled markers are
  not Lua), and the reader still gives the recorded tables.
* CPU: a table written back out as Lua source reads back as the same table.
* GPU: heat.lua (2-D heat, E2, a Floating circle, the gaussian manufactured solution,
  diffusivity 1/30, to t = 0.3), brady_livescu_4_3_n61.lua (the Brady-Livescu radial wave
  with E4u, shortened to t = 0.2 by --script) and scalar_wave.lua (the radial wave with the
  E2-poly scheme around a Dirichlet and a Floating quarter circle, its 20 steps) run through
  the command line from their recorded tables; every step's Linf error in logs/system.csv
  equals the oracle's (the reference's heat / scalar_wave RK4 restated) within 1e-10 of the
  solution's scale; scalar_wave.lua also in mixed precision (`system.precision = "mixed"`),
  within 2e-5 of the FP64 oracle's.
"""
import json
import os
import subprocess

import numpy as np
import pytest

from tests.reference_inputs import lua_input, parse_dump

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
GOLD = os.path.join(HERE, "golden", "reference_inputs.json")
CLI = os.path.join(ROOT, "shoccs_gb300", "_build", "shoccs")
REF = os.environ.get("SHOCCS_REFERENCE_ROOT", os.path.join(os.path.dirname(ROOT), "reference"))


def _inputs():
    with open(GOLD) as f:
        return json.load(f)["inputs"]


@pytest.fixture(scope="module")
def lua_eval(tmp_path_factory):
    d = tmp_path_factory.mktemp("lua_eval_ref")
    exe = d / "lua_eval"
    r = subprocess.run(["g++", "-std=c++20", "-O2", "-I" + os.path.join(ROOT, "shoccs_gb300", "app"),
                        os.path.join(HERE, "cpp", "lua_eval.cpp"), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    return str(exe)


def _strkeys(t):
    return {str(k): _strkeys(v) for k, v in t.items()} if isinstance(t, dict) else t


@pytest.mark.parametrize("name", sorted(_inputs()))
def test_reference_input_files_check_and_read(name, lua_eval, tmp_path):
    path = os.path.join(REF, name)
    if not os.path.exists(path):
        pytest.skip("the reference tree is not here")
    if not os.path.exists(CLI):
        pytest.fail("command line not built: " + CLI)
    rec = _inputs()[name]
    r = subprocess.run([CLI, "--check", path], capture_output=True, text=True, cwd=str(tmp_path))
    assert r.returncode == rec["check_rc"], r.stderr
    r = subprocess.run([lua_eval, path, "result = simulation"], capture_output=True, text=True)
    if rec["table"] is None:
        assert r.returncode != 0
    else:
        assert _strkeys(parse_dump(r.stdout)) == rec["table"]


@pytest.mark.parametrize("name", sorted(n for n, v in _inputs().items() if v["table"]))
def test_recorded_tables_write_back_as_lua(name, lua_eval, tmp_path):
    table = _inputs()[name]["table"]
    if "__function__" in json.dumps(table):
        pytest.skip("the table holds functions")
    f = tmp_path / "in.lua"
    f.write_text(lua_input(table))
    r = subprocess.run([lua_eval, str(f), "result = simulation"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout
    assert _strkeys(parse_dump(r.stdout)) == table


def _run_cli(table, tmp_path, *script):
    f = tmp_path / "input.lua"
    f.write_text(lua_input(table))
    args = [CLI, str(f)]
    for s in script:
        args += ["--script", s]
    r = subprocess.run(args, cwd=str(tmp_path), capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    assert "[error]" not in r.stderr, r.stderr
    rows = [l.split(",") for l in open(str(tmp_path / "logs" / "system.csv")).read().splitlines()[1:]]
    return [(float(row[1]), float(row[3])) for row in rows]


def _compare(rows, step, stats, u0, scale_tol=1e-10):
    """rows: (time, Linf) per logged step; step(u, t, dt) advances the oracle one RK4 step;
    stats(t, u) its Linf error"""
    assert len(rows) >= 3 and rows[0][0] == 0.0
    u, scale = u0, np.abs(u0[0]).max()
    assert abs(rows[0][1] - stats(0.0, u)) <= scale_tol * scale
    for k in range(1, len(rows)):
        t0, t1 = rows[k - 1][0], rows[k][0]
        u = step(u, t0, t1 - t0)
        want = stats(t1, u)
        assert abs(rows[k][1] - want) <= scale_tol * max(scale, np.abs(u[0]).max()), (k, rows[k], want)
    return u


def _scalar_wave_case(table):
    m, sc = table["mesh"], table["scheme"]
    n = (int(m["index_extents"]["1"]), int(m["index_extents"]["2"]), 1)
    hi = (m["domain_bounds"]["1"], m["domain_bounds"]["2"], 0.0)
    arr = lambda t: [t[str(i + 1)] for i in range(len(t))]
    alpha = arr(sc["floating_alpha"]) + arr(sc["dirichlet_alpha"]) + arr(sc["interpolant_alpha"])
    shapes = [table["shapes"][k] for k in sorted(table["shapes"], key=int)]
    spheres = [((s_["center"]["1"], s_["center"]["2"], 0.0), s_["radius"], s_["boundary_condition"])
               for s_ in shapes]
    return dict(n=n, lo=(0, 0, 0), hi=hi, spheres=spheres,
                grid_bc=("dirichlet", "floating", "dirichlet", "floating", "floating", "floating"),
                scheme="polyE2_1", alpha=alpha)


@pytest.mark.gpu
def test_reference_scalar_wave_input_runs_mixed(tmp_path):
    """The reference's scalar_wave.lua (E2-poly, a Dirichlet and a Floating quarter circle) in
    mixed precision -- the unfused whole-field step with FP32 stage fields at the grid points
    and FP64 cut points and state: every logged step's error equals the FP64 oracle's to 2e-5
    of max |u| (the case itself moves its errors by 5e-8 of max |u| when its initial data is
    rounded to FP32)"""
    from oracle.oracle import OracleProblem
    table = _inputs()["scalar_wave.lua"]["table"]
    rows = _run_cli(table, tmp_path, 'simulation.system.precision = "mixed"')
    sy = table["system"]
    c = (sy["center"]["1"], sy["center"]["2"], 0.0)
    sol = list(c) + [sy["radius"]]
    o = OracleProblem(**_scalar_wave_case(table))
    assert len(rows) == 21
    _compare(rows, lambda u, t, dt: o.wave_rk4(1, (0, 0, 0), c, 3, sol, t, dt, 1, u),
             lambda t, u: o.stats(3, sol, t, u)[0], o.initialize(3, sol, 0.0), scale_tol=2e-5)


@pytest.mark.gpu
def test_reference_heat_input_runs(tmp_path):
    from oracle.oracle import OracleProblem
    table = _inputs()["heat.lua"]["table"]
    rows = _run_cli(table, tmp_path)
    m, sh = table["mesh"], table["shapes"]["1"]
    n = (int(m["index_extents"]["1"]), int(m["index_extents"]["2"]), 1)
    hi = (m["domain_bounds"]["1"], m["domain_bounds"]["2"], 0.0)
    case = dict(n=n, lo=(0, 0, 0), hi=hi,
                spheres=[((sh["center"]["1"], sh["center"]["2"], 0.0), sh["radius"], "floating")],
                grid_bc=("dirichlet",) * 4 + ("floating",) * 2, scheme="E2_2")
    g = table["manufactured_solution"]["1"]
    terms = [((g["center"]["1"], g["center"]["2"], 0.0), (g["variance"]["1"], g["variance"]["2"], 0.0),
              g["amplitude"], g["frequency"])]
    k = table["system"]["diffusivity"]
    o = OracleProblem(**case)
    # the cycle runs to max_time = 0.3 (dt = 0.5 h^2 / (4 k) = 0.006: 50 steps)
    assert rows[-1][0] >= table["step_controller"]["max_time"] - 1e-9 and len(rows) in (51, 52)
    _compare(rows, lambda u, t, dt: o.heat_rk4(k, 4, terms, t, dt, 1, u),
             lambda t, u: o.stats(4, terms, t, u)[0], o.initialize(4, terms, 0.0))
    # the field writer's schedule: write_every_time = 0.01
    assert os.path.exists(str(tmp_path / "io" / "view.xmf"))


@pytest.mark.gpu
def test_reference_brady_livescu_input_runs(tmp_path):
    from oracle.oracle import OracleProblem
    table = _inputs()["lua-configs/brady_livescu_4_3_n61.lua"]["table"]
    rows = _run_cli(table, tmp_path, "simulation.step_controller.max_time = 0.2")
    m, sc, sy = table["mesh"], table["scheme"], table["system"]
    n = (int(m["index_extents"]["1"]), int(m["index_extents"]["2"]), 1)
    hi = (m["domain_bounds"]["1"], m["domain_bounds"]["2"], 0.0)
    case = dict(n=n, lo=(0, 0, 0), hi=hi, spheres=[],
                grid_bc=("dirichlet", "floating", "dirichlet", "floating", "floating", "floating"),
                scheme="E4u_1", alpha=(sc["alpha"]["1"], sc["alpha"]["2"]))
    c = (sy["center"]["1"], sy["center"]["2"], sy["center"]["3"])
    sol = list(c) + [sy["radius"]]
    o = OracleProblem(**case)
    assert rows[-1][0] >= 0.2 - 1e-12 and len(rows) > 5
    _compare(rows, lambda u, t, dt: o.wave_rk4(1, (0, 0, 0), c, 3, sol, t, dt, 1, u),
             lambda t, u: o.stats(3, sol, t, u)[0], o.initialize(3, sol, 0.0))


@pytest.mark.gpu
def test_reference_scalar_wave_input_runs(tmp_path):
    from oracle.oracle import OracleProblem
    table = _inputs()["scalar_wave.lua"]["table"]
    rows = _run_cli(table, tmp_path)
    m, sc, sy = table["mesh"], table["scheme"], table["system"]
    n = (int(m["index_extents"]["1"]), int(m["index_extents"]["2"]), 1)
    hi = (m["domain_bounds"]["1"], m["domain_bounds"]["2"], 0.0)
    arr = lambda t: [t[str(i + 1)] for i in range(len(t))]
    alpha = arr(sc["floating_alpha"]) + arr(sc["dirichlet_alpha"]) + arr(sc["interpolant_alpha"])
    shapes = [table["shapes"][k] for k in sorted(table["shapes"], key=int)]
    spheres = [((s_["center"]["1"], s_["center"]["2"], 0.0), s_["radius"], s_["boundary_condition"])
               for s_ in shapes]
    case = dict(n=n, lo=(0, 0, 0), hi=hi, spheres=spheres,
                grid_bc=("dirichlet", "floating", "dirichlet", "floating", "floating", "floating"),
                scheme="polyE2_1", alpha=alpha)
    c = (sy["center"]["1"], sy["center"]["2"], 0.0)
    sol = list(c) + [sy["radius"]]
    o = OracleProblem(**case)
    # max_step = 20 ends the run (max_time = 500)
    assert len(rows) == 21
    _compare(rows, lambda u, t, dt: o.wave_rk4(1, (0, 0, 0), c, 3, sol, t, dt, 1, u),
             lambda t, u: o.stats(3, sol, t, u)[0], o.initialize(3, sol, 0.0))
