"""Heat systems with the reference's "gaussian" manufactured solution (src/mms/gauss2d.cpp,
gauss3d.cpp) on the GPU, against the oracle: the right-hand side (its source is
ddt - k lap of the Gaussian sum, its Neumann data the sum's gradient), 10 RK4 steps and the
statistics.  These systems run on the unfused FP64 whole-field step; mixed precision, the
wave system and batched solves reject the kind.  The command line reads the kind from an
input file's manufactured_solution table.

Tolerances as for the other unfused cases: rhs 1e-11, state 1e-10 (relative max-norm),
errors / min / max 1e-8.
"""
import os
import subprocess

import numpy as np
import pytest

import shoccs_gb300 as S
from oracle.oracle import OracleProblem
from shoccs_gb300 import workloads as W
from tests.test_cli import LUA

TERMS = [((0.4, 0.55, 0.5), (0.18, 0.22, 0.2), 1.3, 2.0),
         ((0.7, 0.3, 0.45), (0.15, 0.12, 0.17), -0.6, 5.0)]
CASES = {
    "circle65_neumann_faces": dict(n=(65, 65, 1), lo=(0, 0, 0), hi=(1, 1, 0),
                                   spheres=[((0.51, 0.49, 0.0), 0.2, "dirichlet")],
                                   grid_bc=("neumann", "dirichlet", "dirichlet", "neumann",
                                            "floating", "floating"), scheme="E4_2"),
    "sphere24_floating": dict(n=(24, 24, 24), lo=(0, 0, 0), hi=(1, 1, 1),
                              spheres=[((0.5, 0.5, 0.5), 0.25, "floating")],
                              grid_bc=("dirichlet",) * 6, scheme="E4_2"),
    "sphere26_neumann_e22": dict(n=(26, 24, 28), lo=(0, 0, 0), hi=(1, 1, 1),
                                 spheres=[((0.3, 0.33, 0.36), 0.14, "neumann"),
                                          ((0.66, 0.64, 0.62), 0.14, "dirichlet")],
                                 grid_bc=("dirichlet", "floating", "neumann", "dirichlet",
                                          "floating", "dirichlet"), scheme="E2_2"),
}


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
@pytest.mark.parametrize("name", sorted(CASES))
def test_gaussian_heat_matches_oracle(name):
    import torch
    c = CASES[name]
    p, o = S.Problem(**c), OracleProblem(**c)
    h = S.Heat(p, 0.7, S.PREC_FP64, S.SOL_GAUSSIAN, TERMS)
    assert h.stage_kernel == "unfused"
    h.initialize(0.0)
    u0 = _state(h, p)
    want0 = o.initialize(S.SOL_GAUSSIAN, TERMS, 0.0)
    for g, w in zip(u0, want0):
        assert rel(g, w) <= 1e-14
    t = 0.013
    got = h.rhs(t, p.zeros(torch.float64))
    want = o.heat_rhs(0.7, S.SOL_GAUSSIAN, TERMS, t, u0)
    for k, (g, w) in enumerate(zip(got, want)):
        assert rel(g.cpu().numpy(), w) <= 1e-11, (name, k)
    # 10 steps: the Floating sphere's closure grows without bound after ~15 steps, with the
    # sin-sin solution as well (a property of the reference's scheme on this geometry)
    dt = W.heat_dt(max(c["n"]), k=0.7)
    h.rk4(0.0, dt, 10)
    got = _state(h, p)
    want = o.heat_rk4(0.7, S.SOL_GAUSSIAN, TERMS, 0.0, dt, 10, u0)
    for k, (g, w) in enumerate(zip(got, want)):
        assert rel(g, w) <= 1e-10, (name, k)
    st, ok = h.stats(10 * dt)
    ref = o.stats(S.SOL_GAUSSIAN, TERMS, 10 * dt, want)
    assert ok
    for k in (0, 1, 2, 3, 5, 7, 9):
        assert abs(st[k] - ref[k]) <= 1e-8 * max(abs(ref[k]), 1e-12), (name, k, st[k], ref[k])


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(CASES))
def test_gaussian_heat_mixed_close_to_oracle(name):
    """mixed precision on the unfused step (FP32 stage fields, FP64 state): 10 RK4 steps
    against the FP64 oracle within 1e-4 of the max norm"""
    c = CASES[name]
    p, o = S.Problem(**c), OracleProblem(**c)
    h = S.Heat(p, 0.7, S.PREC_MIXED, S.SOL_GAUSSIAN, TERMS)
    assert h.stage_kernel == "unfused"
    h.initialize(0.0)
    u0 = _state(h, p)
    dt = W.heat_dt(max(c["n"]), k=0.7)
    h.rk4(0.0, dt, 10)
    got = _state(h, p)
    want = o.heat_rk4(0.7, S.SOL_GAUSSIAN, TERMS, 0.0, dt, 10, u0)
    for k, (g, w) in enumerate(zip(got, want)):
        assert rel(g, w) <= 1e-4, (name, k, rel(g, w))


@pytest.mark.gpu
def test_gaussian_unsupported_combinations():
    q = S.Problem(**dict(CASES["circle65_neumann_faces"], grid_bc=("dirichlet",) * 4 + ("floating",) * 2))
    with pytest.raises(S.ShoccsError):
        S.ScalarWave(q, S.PREC_FP64, S.VEL_CONSTANT, (1, 0, 0), (0, 0, 0), S.SOL_GAUSSIAN, TERMS)
    h = S.Heat(q, 1.0, S.PREC_FP64, S.SOL_GAUSSIAN, TERMS)
    with pytest.raises(S.ShoccsError):
        S.Batch([h])


@pytest.mark.gpu
def test_cli_heat_with_gaussian_solution(tmp_path):
    cli = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "shoccs_gb300", "_build", "shoccs")
    script = ('simulation.manufactured_solution = {type = "gaussian", '
              '{center = {0.4, 0.55}, variance = {0.18, 0.22}, amplitude = 1.3, frequency = 2}, '
              '{center = {0.7, 0.3}, variance = {0.15, 0.12}, amplitude = -0.6, frequency = 5}}; '
              'simulation.step_controller.max_step = 20; simulation.io = nil')
    r = subprocess.run([cli, os.path.join(LUA, "heat_circle_2d.lua"), "--script", script], cwd=str(tmp_path),
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and "[error]" not in r.stderr, r.stderr
    rows = [l.split(",") for l in open(str(tmp_path / "mylogs" / "system.csv")).read().splitlines()[1:]]
    assert len(rows) == 21
    c = dict(n=(65, 65, 1), lo=(0, 0, 0), hi=(1, 1, 0), spheres=[((0.51, 0.49, 0.0), 0.2, "dirichlet")],
             grid_bc=("dirichlet",) * 4 + ("floating",) * 2, scheme="E4_2")
    terms2 = [((0.4, 0.55, 0.0), (0.18, 0.22, 0.0), 1.3, 2.0), ((0.7, 0.3, 0.0), (0.15, 0.12, 0.0), -0.6, 5.0)]
    h = S.Heat(S.Problem(**c), 1.0, S.PREC_FP64, S.SOL_GAUSSIAN, terms2)
    h.initialize(0.0)
    dt, t = h.timestep(0.4), 0.0
    for _ in range(20):
        h.rk4(t, dt, 1)
        t += dt
    st, _ = h.stats(t)
    assert float(rows[-1][1]) == t and [float(v) for v in rows[-1][3:14]] == list(st)
