"""Heat systems with Floating or Neumann objects, or Neumann faces.  The cut-point values of a
non-Dirichlet object are state, so the RK4 step advances the whole field {D, Rx, Ry, Rz}
(src/temporal/rk4.cpp:16-47), their right-hand side comes from the Laplacian's R-space rows plus
the source (heat::rhs adds it at every non-Dirichlet cut point; a Neumann object's closure
carries no Neumann data, the object part of the reference's Neumann data is never assigned),
and the statistics include them (compute_scalar_stats visits the non-Dirichlet cut points).  On Neumann faces the Laplacian's N rows take the solution's gradient component as
Neumann data, evaluated at each right-hand side's time (heat::update_boundary,
src/systems/heat.cpp:324-352).  The FP64 heat system runs these cases on its unfused path;
everything is checked against the oracle's heat rhs, rk4 and stats.

The FP64 scalar wave with Floating objects takes the same unfused path (right-hand side
gG . grad u over the whole field) and is checked against the oracle's wave rhs, rk4 and stats,
with constant and radial velocity.

Tolerances (max-norm, relative to the oracle array's max-norm): rhs 1e-11, RK4 state 1e-10
(FP64 arithmetic in a different order); errors, min and max to 1e-8; each argmax index must
carry the maximum error (ties to rounding on symmetric geometries).
"""
import numpy as np
import pytest

import shoccs_gb300 as S
from oracle.oracle import OracleProblem
from shoccs_gb300 import workloads as W
from tests.cases import cases

CASES = {
    "circle65_floating": dict(n=(65, 65, 1), lo=(0, 0, 0), hi=(1, 1, 0),
                              spheres=[((0.51, 0.49, 0.0), 0.2, "floating")],
                              grid_bc=("dirichlet",) * 4 + ("floating",) * 2, scheme="E4_2"),
    "sphere24_floating": dict(n=(24, 24, 24), lo=(0, 0, 0), hi=(1, 1, 1),
                              spheres=[((0.5, 0.5, 0.5), 0.25, "floating")],
                              grid_bc=("dirichlet",) * 6, scheme="E4_2"),
    "two_objects": dict(n=(49, 49, 1), lo=(0, 0, 0), hi=(1, 1, 0),
                        spheres=[((0.3, 0.3, 0.0), 0.12, "floating"),
                                 ((0.7, 0.68, 0.0), 0.15, "dirichlet")],
                        grid_bc=("dirichlet",) * 4 + ("floating",) * 2, scheme="E2_2"),
    "neumann_x_circle65": dict(n=(65, 65, 1), lo=(0, 0, 0), hi=(1, 1, 0),
                               spheres=[((0.51, 0.49, 0.0), 0.2, "dirichlet")],
                               grid_bc=("neumann", "neumann", "dirichlet", "dirichlet",
                                        "floating", "floating"), scheme="E4_2"),
    "neumann_faces24_floating": dict(n=(24, 24, 24), lo=(0, 0, 0), hi=(1, 1, 1),
                                     spheres=[((0.5, 0.5, 0.5), 0.25, "floating")],
                                     grid_bc=("neumann", "dirichlet", "dirichlet", "neumann",
                                              "neumann", "neumann"), scheme="E4_2"),
    "neumann_e22": dict(n=(41, 41, 1), lo=(0, 0, 0), hi=(1, 1, 0),
                        spheres=[((0.5, 0.5, 0.0), 0.2, "dirichlet")],
                        grid_bc=("dirichlet", "neumann", "neumann", "dirichlet",
                                 "floating", "floating"), scheme="E2_2"),
    "neumann_circle49_e22": dict(n=(49, 49, 1), lo=(0, 0, 0), hi=(1, 1, 0),
                                 spheres=[((0.52, 0.47, 0.0), 0.21, "neumann")],
                                 grid_bc=("dirichlet",) * 4 + ("floating",) * 2, scheme="E2_2"),
    "neumann_and_dirichlet_spheres26": dict(n=(26, 24, 28), lo=(0, 0, 0), hi=(1, 1, 1),
                                            spheres=[((0.3, 0.33, 0.36), 0.14, "neumann"),
                                                     ((0.66, 0.64, 0.62), 0.14, "dirichlet")],
                                            grid_bc=("dirichlet", "floating", "neumann",
                                                     "dirichlet", "floating", "dirichlet"),
                                            scheme="E4_2"),
}
SOL = [1.0]  # sin(2 pi x) sin(2 pi y) (sin 2 pi z) e^-t


def rel(got, want):
    want = np.asarray(want)
    if want.size == 0:
        return 0.0
    return float(np.abs(np.asarray(got) - want).max() / max(np.abs(want).max(), 1e-300))


def _system(c):
    p = S.Problem(**c)
    h = S.Heat(p, 1.0, S.PREC_FP64, S.SOL_SINSIN, SOL)
    h.initialize(0.0)
    return p, h


def _state(h, p):
    u = [np.zeros(p.size)] + [np.zeros(k) for k in p.nR]
    h.get_state(S.ScalarField(*u))
    return u


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(CASES))
def test_floating_rhs_matches_oracle(name):
    import torch
    c = CASES[name]
    p, h = _system(c)
    assert h.stage_kernel == "unfused"
    o = OracleProblem(**c)
    u = _state(h, p)
    t = 0.013
    want = o.heat_rhs(1.0, S.SOL_SINSIN, SOL, t, u)
    got = h.rhs(t, p.zeros(torch.float64))
    for k, (g, w) in enumerate(zip(got, want)):
        assert rel(g.cpu().numpy(), w) <= 1e-11, (name, k)
    if any(s_[2] != "dirichlet" for s_ in c["spheres"]):
        # the non-Dirichlet cut points have a nonzero right-hand side (they evolve)
        assert any(np.abs(w).max() > 0 for w in want[1:])


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(CASES))
def test_floating_rk4_and_stats_match_oracle(name):
    c = CASES[name]
    p, h = _system(c)
    o = OracleProblem(**c)
    u0 = _state(h, p)
    n = max(c["n"])
    dt = W.heat_dt(n)
    steps = 20
    h.rk4(0.0, dt, steps)
    got = _state(h, p)
    want = o.heat_rk4(1.0, S.SOL_SINSIN, SOL, 0.0, dt, steps, u0)
    for k, (g, w) in enumerate(zip(got, want)):
        assert rel(g, w) <= 1e-10, (name, k)
    t = steps * dt
    st, ok = h.stats(t)
    ref = o.stats(S.SOL_SINSIN, SOL, t, want)
    assert ok
    for k in (0, 1, 2, 3, 5, 7, 9):  # errors, min, max
        assert abs(st[k] - ref[k]) <= 1e-8 * max(abs(ref[k]), 1e-12), (name, k, st[k], ref[k])
    # argmax of each R array: on a symmetric geometry several cut points share the largest
    # error to rounding, so the oracle's error at the index returned must be that maximum
    ex = o.exact(S.SOL_SINSIN, SOL, t)
    for d, k in ((0, 6), (1, 8), (2, 10)):
        err = np.abs(want[1 + d] - ex[1 + d])
        if err.size == 0 or ref[k - 1] == 0:
            continue
        assert err[int(st[k])] >= err.max() * (1 - 1e-8), (name, k, st[k], ref[k])


# ---- mixed precision on the unfused step --------------------------------------------------
# FP32 stage inputs, right-hand sides and stage accumulator, FP64 state.  The right-hand side
# of an FP32-representable state against the oracle's: 2e-5 of the max norm (FP32
# arithmetic on k lap and the source, each about 40x the right-hand side they sum to); the
# RK4 state after 20 steps against the FP64 oracle's: within max(1e-4, 4 s) of the max norm,
# s the case's own sensitivity -- how far the FP64 oracle's 20 steps move when only the
# initial data is rounded to FP32 (a 3e-8 change).  The reference's Floating heat cases
# amplify that change up to 1e5-fold (s = 3.9e-3 for circle65_floating's cut points, 1.5e-4
# for the 24^3 spheres; 1e-8 for the stable cases); on the stable Neumann-face cases the
# error against the exact solution equals the FP64 system's within 10 % (equal accuracy).
def _round32(u):
    return [np.asarray(a, dtype=np.float32).astype(np.float64) for a in u]


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(CASES))
def test_floating_mixed_rhs_matches_oracle(name):
    import torch
    c = CASES[name]
    p = S.Problem(**c)
    h = S.Heat(p, 1.0, S.PREC_MIXED, S.SOL_SINSIN, SOL)
    h.initialize(0.0)
    assert h.stage_kernel == "unfused"
    o = OracleProblem(**c)
    u = _round32(_state(h, p))
    h.set_state(S.ScalarField(*[a.copy() for a in u]))
    t = 0.013
    want = o.heat_rhs(1.0, S.SOL_SINSIN, SOL, t, u)
    got = h.rhs(t, p.zeros(torch.float64))
    scale = max(np.abs(w).max() for w in want if w.size)
    for k, (g, w) in enumerate(zip(got, want)):
        if w.size:
            assert np.abs(g.cpu().numpy() - w).max() <= 2e-5 * scale, (name, k)


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(CASES))
def test_floating_mixed_rk4_close_to_fp64_oracle(name):
    c = CASES[name]
    p = S.Problem(**c)
    o = OracleProblem(**c)
    h = S.Heat(p, 1.0, S.PREC_MIXED, S.SOL_SINSIN, SOL)
    h.initialize(0.0)
    u0 = _state(h, p)
    dt, steps = W.heat_dt(max(c["n"])), 20
    h.rk4(0.0, dt, steps)
    got = _state(h, p)
    want = o.heat_rk4(1.0, S.SOL_SINSIN, SOL, 0.0, dt, steps, u0)
    moved = o.heat_rk4(1.0, S.SOL_SINSIN, SOL, 0.0, dt, steps, _round32(u0))
    for k, (g, w, m) in enumerate(zip(got, want, moved)):
        sens = rel(m, w)
        assert rel(g, w) <= max(1e-4, 4 * sens), (name, k, rel(g, w), sens)
    with pytest.raises(S.ShoccsError):  # forward Euler steps FP64 systems
        h.euler(0.0, dt, 1)


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["neumann_x_circle65", "neumann_e22"])
def test_neumann_faces_mixed_equal_accuracy(name):
    c = CASES[name]
    p = S.Problem(**c)
    dt, steps = W.heat_dt(max(c["n"])), 100
    err = {}
    for prec in (S.PREC_FP64, S.PREC_MIXED):
        h = S.Heat(p, 1.0, prec, S.SOL_SINSIN, SOL)
        h.initialize(0.0)
        h.rk4(0.0, dt, steps)
        st, ok = h.stats(steps * dt)
        assert ok
        err[prec] = st[0]
    assert abs(err[S.PREC_MIXED] - err[S.PREC_FP64]) <= 0.1 * err[S.PREC_FP64], err


# the scalar wave with Floating objects (FP64, unfused): the cut-point values of a Floating
# object evolve by gG . grad u from the gradient's R-space rows (scalar_wave.cpp:241-321);
# Dirichlet faces and Dirichlet cut points take the exact solution (scalar_wave.cpp:329-355)
# (the first-derivative schemes E4_1 and E4u_1 have no cross-direction interpolant, so the
# reference takes Floating objects with the E2-poly scheme; cases of tests/cases.py)
WAVE_CASES = {name: cases()[name] for name in ("poly_scalar_wave_2d", "poly_spheres_3d")}
VEL = (1.0, 0.7, 0.4)
PULSE = [0.3, 0.3, 0.3, 1.0, 0.7, 0.4, 0.08]  # Gaussian pulse (x0, a, sigma)


WAVE_CENTER = (-1.0, -1.0, 0.0)  # the radial velocity's centre, outside both domains


def _wave(c, vel_kind):
    p = S.Problem(**c)
    w = S.ScalarWave(p, S.PREC_FP64, vel_kind, VEL, WAVE_CENTER, 2, PULSE)
    w.initialize(0.0)
    return p, w


@pytest.mark.gpu
@pytest.mark.parametrize("vel_kind", [S.VEL_CONSTANT, S.VEL_RADIAL])
@pytest.mark.parametrize("name", sorted(WAVE_CASES))
def test_wave_floating_rhs_matches_oracle(name, vel_kind):
    import torch
    c = WAVE_CASES[name]
    p, w = _wave(c, vel_kind)
    assert w.stage_kernel == "unfused"
    o = OracleProblem(**c)
    u = _state(w, p)
    want = o.wave_rhs(vel_kind, VEL, WAVE_CENTER, u)
    got = w.rhs(0.01, p.zeros(torch.float64))
    for k, (g, wv) in enumerate(zip(got, want)):
        assert rel(g.cpu().numpy(), wv) <= 1e-11, (name, k)
    # the Floating object's cut points have a nonzero right-hand side (they evolve)
    assert any(np.abs(wv).max() > 0 for wv in want[1:])


@pytest.mark.gpu
@pytest.mark.parametrize("vel_kind", [S.VEL_CONSTANT, S.VEL_RADIAL])
@pytest.mark.parametrize("name", sorted(WAVE_CASES))
def test_wave_floating_rk4_and_stats_match_oracle(name, vel_kind):
    c = WAVE_CASES[name]
    p, w = _wave(c, vel_kind)
    o = OracleProblem(**c)
    u0 = _state(w, p)
    h = min((c["hi"][a] - c["lo"][a]) / (c["n"][a] - 1) for a in range(3) if c["n"][a] > 1)
    dt, steps = 0.4 * h, 20
    w.rk4(0.0, dt, steps)
    got = _state(w, p)
    want = o.wave_rk4(vel_kind, VEL, WAVE_CENTER, 2, PULSE, 0.0, dt, steps, u0)
    for k, (g, wv) in enumerate(zip(got, want)):
        assert rel(g, wv) <= 1e-10, (name, k)
    t = steps * dt
    st, ok = w.stats(t)
    ref = o.stats(2, PULSE, t, want)
    for k in (0, 1, 2, 3, 5, 7, 9):  # errors, min, max
        assert abs(st[k] - ref[k]) <= 1e-8 * max(abs(ref[k]), 1e-12), (name, k, st[k], ref[k])


@pytest.mark.gpu
@pytest.mark.parametrize("vel_kind", [S.VEL_CONSTANT, S.VEL_RADIAL])
@pytest.mark.parametrize("name", sorted(WAVE_CASES))
def test_wave_floating_mixed_matches_oracle(name, vel_kind):
    """the mixed unfused wave: right-hand side of an FP32-representable state (2e-6 of the
    max norm), 20 RK4 steps against the FP64 oracle (2e-5), statistics (1e-3)"""
    import torch
    c = WAVE_CASES[name]
    p = S.Problem(**c)
    w = S.ScalarWave(p, S.PREC_MIXED, vel_kind, VEL, WAVE_CENTER, 2, PULSE)
    w.initialize(0.0)
    assert w.stage_kernel == "unfused"
    o = OracleProblem(**c)
    u = _round32(_state(w, p))
    w.set_state(S.ScalarField(*[a.copy() for a in u]))
    want = o.wave_rhs(vel_kind, VEL, WAVE_CENTER, u)
    got = w.rhs(0.0, p.zeros(torch.float64))
    scale = max(np.abs(x).max() for x in want if x.size)
    for k, (g, wv) in enumerate(zip(got, want)):
        if wv.size:
            assert np.abs(g.cpu().numpy() - wv).max() <= 2e-6 * scale, (name, k)
    h = min((c["hi"][a] - c["lo"][a]) / (c["n"][a] - 1) for a in range(3) if c["n"][a] > 1)
    dt, steps = 0.4 * h, 20
    w.rk4(0.0, dt, steps)
    got = _state(w, p)
    want = o.wave_rk4(vel_kind, VEL, WAVE_CENTER, 2, PULSE, 0.0, dt, steps, u)
    for k, (g, wv) in enumerate(zip(got, want)):
        assert rel(g, wv) <= 2e-5, (name, k, rel(g, wv))
    t = steps * dt
    st, ok = w.stats(t)
    ref = o.stats(2, PULSE, t, want)
    assert ok
    for k in (0, 1, 2):
        assert abs(st[k] - ref[k]) <= 1e-3 * max(abs(ref[k]), 1e-12), (name, k, st[k], ref[k])


@pytest.mark.gpu
@pytest.mark.parametrize("prec", [S.PREC_FP64, S.PREC_MIXED])
def test_wave_poly_e2_dirichlet_fused_matches_oracle(prec):
    """E2-poly (3-point antisymmetric interior) with Dirichlet objects only: the fused stage
    kernels, FP64 and mixed, against the oracle's RK4"""
    c = dict(WAVE_CASES["poly_spheres_3d"])
    c["spheres"] = [(cc, r, "dirichlet") for cc, r, _ in c["spheres"]]
    p = S.Problem(**c)
    o = OracleProblem(**c)
    w = S.ScalarWave(p, prec, S.VEL_CONSTANT, VEL, (0, 0, 0), 2, PULSE)
    w.initialize(0.0)
    assert w.stage_kernel != "unfused"
    u0 = o.initialize(2, PULSE, 0.0)
    h = 1.0 / (max(c["n"]) - 1)
    dt, steps = 0.4 * h, 20
    w.rk4(0.0, dt, steps)
    got = _state(w, p)
    want = o.wave_rk4(S.VEL_CONSTANT, VEL, (0, 0, 0), 2, PULSE, 0.0, dt, steps, u0)
    assert rel(got[0], want[0]) <= (1e-10 if prec == S.PREC_FP64 else 2e-5)


@pytest.mark.gpu
def test_floating_systems_that_stay_unsupported():
    c = dict(CASES["circle65_floating"])
    p = S.Problem(**c)
    assert S.Heat(p, 1.0, S.PREC_MIXED, S.SOL_SINSIN, SOL).stage_kernel == "unfused"
    pw = S.Problem(**WAVE_CASES["poly_scalar_wave_2d"])
    assert S.ScalarWave(pw, S.PREC_FP64).stage_kernel == "unfused"
    assert S.ScalarWave(pw, S.PREC_MIXED).stage_kernel == "unfused"
    h = S.Heat(p, 1.0, S.PREC_FP64, S.SOL_SINSIN, SOL)
    with pytest.raises(S.ShoccsError):  # the adjoint covers Dirichlet objects
        h.forward(0.0, 1e-5, 2)
    with pytest.raises(S.ShoccsError):  # and so do batched solves
        S.Batch([h])
    pno = S.Problem(**CASES["neumann_circle49_e22"])
    assert S.Heat(pno, 1.0, S.PREC_FP64, S.SOL_SINSIN, SOL).stage_kernel == "unfused"
    assert S.Heat(pno, 1.0, S.PREC_MIXED, S.SOL_SINSIN, SOL).stage_kernel == "unfused"
    with pytest.raises(S.ShoccsError):  # Neumann objects: no first-derivative closures
        S.ScalarWave(pno, S.PREC_FP64)
    with pytest.raises(S.ShoccsError):
        S.ScalarWave(pno, S.PREC_MIXED)
