"""The forward Euler integrator (integrators::euler, src/temporal/euler.cpp:11-27) on the GPU
against the oracle's restatement: u <- u + dt rhs(u, t), then the boundary data at t + dt.

FP64 heat on the fused operator path (Dirichlet circle), FP64 heat on the unfused path (Neumann
faces, Floating object), and the FP64 wave (E4u_1 box, Gaussian pulse): the state after the
steps to 1e-12 (fused heat, wave) / 1e-10 (unfused) relative max-norm.  Mixed-precision
systems reject the integrator.  The command line runs it for `integrator.type = "euler"`,
every logged step bit-equal to the binding's one-call-per-step run.
"""
import os
import subprocess

import numpy as np
import pytest

import shoccs_gb300 as S
from oracle.oracle import OracleProblem
from shoccs_gb300 import workloads as W
from tests.cases import cases
from tests.test_cli import LUA
from tests.test_cli_gpu import WAVE, WAVE_CENTER, _system_csv


def rel(got, want):
    want = np.asarray(want)
    if want.size == 0:
        return 0.0
    return float(np.abs(np.asarray(got) - want).max() / max(np.abs(want).max(), 1e-300))


def _state(h, p):
    u = [np.zeros(p.size)] + [np.zeros(k) for k in p.nR]
    h.get_state(S.ScalarField(*u))
    return u


@pytest.mark.gpu
@pytest.mark.parametrize("name,tol", [("c0_circle_2d", 1e-12), ("neumann_e22", 1e-10)])
def test_heat_euler_matches_oracle(name, tol):
    c = cases()[name]
    p, o = S.Problem(**c), OracleProblem(**c)
    h = S.Heat(p, 1.0, S.PREC_FP64, S.SOL_SINSIN, [1.0])
    h.initialize(0.0)
    u0 = _state(h, p)
    dt = W.heat_dt(max(c["n"]))
    h.euler(0.0, dt, 40)
    got = _state(h, p)
    want = o.heat_euler(1.0, S.SOL_SINSIN, [1.0], 0.0, dt, 40, u0)
    for k, (g, w) in enumerate(zip(got, want)):
        assert rel(g, w) <= tol, (name, k)
    st, ok = h.stats(40 * dt)
    ref = o.stats(S.SOL_SINSIN, [1.0], 40 * dt, want)
    assert ok and abs(st[0] - ref[0]) <= 1e-8 * ref[0]


@pytest.mark.gpu
def test_wave_euler_matches_oracle():
    c = cases()["box_e4u"]
    p, o = S.Problem(**c), OracleProblem(**c)
    vel, center = W.WAVE_VEL, (0.0, 0.0, 0.0)
    w = S.ScalarWave(p, S.PREC_FP64, S.VEL_CONSTANT, vel, center, S.SOL_GAUSS_PULSE, W.WAVE_PULSE)
    w.initialize(0.0)
    u0 = _state(w, p)
    dt = 0.2 / (min(c["n"]) - 1)
    w.euler(0.0, dt, 20)
    got = _state(w, p)
    want = o.wave_euler(S.VEL_CONSTANT, vel, center, S.SOL_GAUSS_PULSE, W.WAVE_PULSE, 0.0, dt, 20, u0)
    assert rel(got[0], want[0]) <= 1e-12


@pytest.mark.gpu
def test_euler_rejects_mixed_precision():
    p = S.Problem(**cases()["c0_circle_2d"])
    h = S.Heat(p, 1.0, S.PREC_MIXED, S.SOL_SINSIN, [1.0])
    h.initialize(0.0)
    with pytest.raises(S.ShoccsError):
        h.euler(0.0, 1e-5, 1)


@pytest.mark.gpu
def test_cli_euler(tmp_path):
    cli = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "shoccs_gb300", "_build", "shoccs")
    r = subprocess.run([cli, os.path.join(LUA, "wave_radial_2d.lua"), "--script",
                        'simulation.integrator.type = "euler"; simulation.step_controller.max_time = 0.1'],
                       cwd=str(tmp_path), capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and "[error]" not in r.stderr, r.stderr
    rows = _system_csv(str(tmp_path / "logs" / "system.csv"))
    dt = 0.5 * 1.25 / 40
    p = S.Problem(**WAVE)
    sol = list(WAVE_CENTER) + [0.0]
    w = S.ScalarWave(p, S.PREC_FP64, S.VEL_RADIAL, (0, 0, 0), WAVE_CENTER, S.SOL_RADIAL_SIN, sol, 10.0)
    w.initialize(0.0)
    t = 0.0
    assert [float(v) for v in rows[0][3:14]] == list(w.stats(0.0)[0])
    for row in rows[1:]:
        w.euler(t, dt, 1)
        t += dt
        assert float(row[1]) == t
        assert [float(v) for v in row[3:14]] == list(w.stats(t)[0])
    assert len(rows) == 8  # t < 0.1 with dt = 1/64: 7 steps


@pytest.mark.gpu
def test_cli_without_integrator_keeps_the_state(tmp_path):
    """no integrator table: the reference's empty integrator, the state stays the initial one
    while the cycle advances the time and logs the statistics"""
    cli = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "shoccs_gb300", "_build", "shoccs")
    r = subprocess.run([cli, os.path.join(LUA, "wave_radial_2d.lua"), "--script",
                        "simulation.integrator = nil; simulation.step_controller.max_time = 0.05"],
                       cwd=str(tmp_path), capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and "[error]" not in r.stderr, r.stderr
    assert "Defaulting to empty" in r.stdout
    rows = _system_csv(str(tmp_path / "logs" / "system.csv"))
    assert len(rows) == 5  # t < 0.05 with dt = 1/64: 4 steps
    p = S.Problem(**WAVE)
    sol = list(WAVE_CENTER) + [0.0]
    w = S.ScalarWave(p, S.PREC_FP64, S.VEL_RADIAL, (0, 0, 0), WAVE_CENTER, S.SOL_RADIAL_SIN, sol, 10.0)
    w.initialize(0.0)
    t = 0.0
    for k, row in enumerate(rows):
        assert float(row[1]) == t
        assert [float(v) for v in row[3:14]] == list(w.stats(t)[0])  # the initial state at time t
        t += 0.5 * 1.25 / 40
