"""The shoccs command line on the GPU: an input file in the reference's Lua format runs the
simulation cycle and leaves what a driver script reads from the reference's binary.

* Radial wave on a 2-D box (tests/lua/wave_radial_2d.lua): logs/system.csv holds the
  header line and one line per step (initial state included); every step's time and Linf
  error equal, bit for bit, those of the Python binding's system stepped one rk4 call at a
  time with the same step size; the state dumped at the last dump step equals the binding's
  state bit for bit and the oracle's (src/systems/scalar_wave.cpp, src/temporal/rk4.cpp
  restated) to 1e-12 relative.
* Heat around a circle (tests/lua/heat_circle_2d.lua): the system log under the configured
  logging_dir, the field dumps on a simulation-time schedule, FP64 errors equal to the
  binding's; the same input with `--script 'simulation.system.precision = "mixed"'` ends at
  an error within 10 % of the FP64 one.
* A driver's template filled in by text substitution runs, and its system.csv parses the way
  such a driver parses it (rows that start with a digit: time in column 1, Linf in column 3).
"""
import os
import subprocess

import numpy as np
import pytest

import shoccs_gb300 as S
from oracle.oracle import OracleProblem
from tests.test_cli import LUA, fill_template
from tests.test_field_io import _d_interval_dumps

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CLI = os.path.join(ROOT, "shoccs_gb300", "_build", "shoccs")
DIR, FLT = "dirichlet", "floating"

WAVE = dict(n=(41, 41, 1), lo=(0, 0, 0), hi=(1.25, 1.25, 0), spheres=[],
            grid_bc=(DIR, FLT, DIR, FLT, FLT, FLT), scheme="E4u_1",
            alpha=(-0.7733323791884821, 0.1623961700641681))
WAVE_CENTER = (-0.3, -0.2, 0.0)
HEAT = dict(n=(65, 65, 1), lo=(0, 0, 0), hi=(1, 1, 0), spheres=[((0.51, 0.49, 0.0), 0.2, DIR)],
            grid_bc=(DIR,) * 4 + (FLT, FLT), scheme="E4_2")


def _run(args, cwd):
    r = subprocess.run([CLI] + args, cwd=str(cwd), capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    assert "[error]" not in r.stderr, r.stderr
    return r


def _system_csv(path):
    lines = open(path).read().splitlines()
    assert lines[0].startswith("Timestamp,Time,Step,Linf,Min,Max,Domain_Linf")
    rows = [l.split(",") for l in lines[1:]]
    assert all(len(r) == 15 for r in rows)
    return rows


def _stepwise(system, dt, nsteps):
    """the binding's system stepped like the cycle: one rk4 call per step at t += dt"""
    system.initialize(0.0)
    t, out = 0.0, [(0.0, system.stats(0.0)[0])]
    for _ in range(nsteps):
        system.rk4(t, dt, 1)
        t += dt
        out.append((t, system.stats(t)[0]))
    return out


@pytest.mark.gpu
def test_cli_radial_wave(tmp_path):
    r = _run([os.path.join(LUA, "wave_radial_2d.lua")], tmp_path)
    assert "cumulative wall time" in r.stdout
    rows = _system_csv(str(tmp_path / "logs" / "system.csv"))
    dt = 0.5 * 1.25 / 40  # hyperbolic cfl * h_min, exact in binary
    nsteps = 16  # t < 0.25 with dt = 1/64
    assert len(rows) == nsteps + 1 and [int(r[2]) for r in rows] == list(range(nsteps + 1))
    p = S.Problem(**WAVE)
    sol = list(WAVE_CENTER) + [0.0]
    w = S.ScalarWave(p, S.PREC_FP64, S.VEL_RADIAL, (0, 0, 0), WAVE_CENTER, S.SOL_RADIAL_SIN, sol, 10.0)
    ref = _stepwise(w, dt, nsteps)
    for row, (t, st) in zip(rows, ref):
        assert float(row[1]) == t
        assert [float(v) for v in row[3:14]] == list(st)
    # simulation_run's result: {time, Linf, Linf} of a run that reached its bound
    last = r.stdout.strip().splitlines()[-1].split()
    assert last[0] == "result" and [float(v) for v in last[1:]] == [ref[-1][0], ref[-1][1][0], ref[-1][1][0]]
    # dumps every 4 steps: 0, 4, ..., 16; the last holds the final state
    steps = list(range(0, nsteps + 1, 4))
    assert sorted(os.listdir(str(tmp_path / "out"))) == sorted(
        ["U.%06d" % k for k in range(len(steps))] + ["Error.%06d" % k for k in range(len(steps))]
        + ["rx", "ry", "rz", "view.xmf"])
    sizes = [p.size] + list(p.nR)
    u = np.split(np.fromfile(str(tmp_path / "out" / ("U.%06d" % (len(steps) - 1)))), np.cumsum(sizes)[:-1])
    got = [np.zeros(k) for k in sizes]
    w.get_state(S.ScalarField(*got))
    for a, b in zip(u, got):
        assert np.array_equal(a, b)
    o = OracleProblem(**WAVE)
    u0 = o.initialize(S.SOL_RADIAL_SIN, sol, 0.0)
    want = o.wave_rk4(S.VEL_RADIAL, (0, 0, 0), WAVE_CENTER, S.SOL_RADIAL_SIN, sol, 0.0, dt, nsteps, u0)
    assert np.abs(u[0] - want[0]).max() <= 1e-12 * np.abs(want[0]).max()


@pytest.mark.gpu
def test_cli_heat_fp64_and_mixed(tmp_path):
    _run([os.path.join(LUA, "heat_circle_2d.lua")], tmp_path)
    rows = _system_csv(str(tmp_path / "mylogs" / "system.csv"))
    assert len(rows) == 61
    p = S.Problem(**HEAT)
    h = S.Heat(p, 1.0, S.PREC_FP64, S.SOL_SINSIN, [1.0])
    dt = h.timestep(0.4)  # parabolic cfl * h_min^2 / (4 k)
    ref = _stepwise(h, dt, 60)
    for row, (t, st) in zip(rows, ref):
        assert float(row[1]) == t
        assert [float(v) for v in row[3:14]] == list(st)
    # field dumps every 7 dt of simulation time (one step size of slack)
    steps = _d_interval_dumps(7 * (0.4 * (1 / 64) ** 2 / 4), dt, 60)  # the input's 7 * dt
    files = os.listdir(str(tmp_path / "fields"))
    assert sorted(f for f in files if f.startswith("U.")) == ["U.%04d" % k for k in range(len(steps))]
    assert "heat.xmf" in files
    e64 = float(rows[-1][3])
    # mixed precision through the extension key, set by --script (runs after the file)
    mixed = tmp_path / "mixed"
    mixed.mkdir()
    _run([os.path.join(LUA, "heat_circle_2d.lua"), "--script", 'simulation.system.precision = "mixed"'], mixed)
    rows32 = _system_csv(str(mixed / "mylogs" / "system.csv"))
    assert len(rows32) == 61
    e32 = float(rows32[-1][3])
    assert e64 < 1e-3 and e32 <= 1.1 * e64


@pytest.mark.gpu
def test_cli_filled_template_runs_and_parses(tmp_path):
    f = tmp_path / "filled.lua"
    f.write_text(fill_template(31, 0.1, "E4u", WAVE["alpha"]))
    (tmp_path / "logs").mkdir()
    _run([str(f)], tmp_path)
    times, linfs = [], []
    for row in open(str(tmp_path / "logs" / "system.csv")).read().splitlines():
        fields = row.split(",")
        if not fields or not fields[0] or not fields[0][0].isdigit():
            continue
        times.append(float(fields[1]))
        linfs.append(float(fields[3]))
    assert len(times) >= 2 and times[0] == 0.0 and times[-1] >= 0.1
    assert np.isfinite(linfs).all() and linfs[-1] < 10.0
