"""The benchmarked mixed-precision stage kernel on cut-cell geometry, and convergence of the
GPU solutions under grid refinement.

* The vectorised mixed stage kernel (`vec`, four z points per thread, the kernel the
  autotuner picks on the benchmark grids) against the FP64 oracle trajectory on a 3-D heat
  problem around a Dirichlet sphere (E4_2 cut-cell rows, Dirichlet walls), 60 RK4 steps.
  Tolerance: 2e-5 relative in max norm (FP32 stage fields and interior stencils; the
  measured difference is printed).
* Manufactured-solution convergence (the reference's simulation_cycle test pattern,
  src/simulation/simulation_cycle.t.cpp:22-100, taken to three grids): the 2-D heat
  configuration (circle, E4_2, sin 2 pi x sin 2 pi y e^-t, dt = 0.1 h^2) on 33^2, 65^2,
  129^2, and a 3-D heat problem around an off-grid sphere on 32^3, 64^3, 128^3, to the same
  final time.  E4_2 is fourth order in the interior with third-order closures; the observed
  order of the max-norm error must be >= 3.5 for FP64 and for mixed precision, and the
  mixed error within 1.1x of the FP64 error on every grid (the equal-accuracy criterion).
"""
import math

import numpy as np
import pytest

import shoccs_gb300 as S
from oracle.oracle import OracleProblem

T_END = 100 * 0.1 / 64 ** 2  # the 2-D configuration's 100 steps on 65^2

SPHERE3D = dict(lo=(0, 0, 0), hi=(1, 1, 1), spheres=[((0.51, 0.49, 0.503), 0.27, "dirichlet")],
                grid_bc=("dirichlet",) * 6, scheme="E4_2")


def _circle2d(npts):
    return dict(n=(npts, npts, 1), lo=(0, 0, 0), hi=(1, 1, 0),
                spheres=[((0.51, 0.49, 0.0), 0.2, "dirichlet")],
                grid_bc=("dirichlet",) * 4 + ("floating",) * 2, scheme="E4_2")


def _state(sys_, p):
    u = [np.zeros(p.size)] + [np.zeros(k) for k in p.nR]
    sys_.get_state(S.ScalarField(*u))
    return u


def _solve(case, prec, kernel=None, monkeypatch=None):
    p = S.Problem(**case)
    if kernel:
        monkeypatch.setenv("SHOCCS_STAGE_KERNEL", kernel)
    hs = S.Heat(p, 1.0, prec, S.SOL_SINSIN, [1.0])
    if kernel:
        assert hs.stage_kernel == kernel
        monkeypatch.delenv("SHOCCS_STAGE_KERNEL")
    h = min((case["hi"][a] - case["lo"][a]) / (case["n"][a] - 1) for a in range(3)
            if case["n"][a] > 1)
    n = int(round(T_END / (0.1 * h * h)))
    hs.initialize(0.0)
    hs.rk4(0.0, T_END / n, n)
    st, valid = hs.stats(T_END)
    assert valid
    return st[0], h


def _orders(errs, hs):
    return [math.log(errs[i - 1] / errs[i]) / math.log(hs[i - 1] / hs[i])
            for i in range(1, len(errs))]


@pytest.mark.gpu
def test_vec_stage_kernel_on_sphere_matches_fp64_oracle(monkeypatch):
    case = dict(SPHERE3D, n=(40, 38, 48))
    p, o = S.Problem(**case), OracleProblem(**case)
    h = 1.0 / 47  # the finest axis
    dt, n = 0.4 * h * h / 4, 60
    monkeypatch.setenv("SHOCCS_STAGE_KERNEL", "vec")
    hs = S.Heat(p, 1.0, S.PREC_MIXED, S.SOL_SINSIN, [1.0])
    assert hs.stage_kernel == "vec"
    assert sum(p.nR) > 0
    hs.initialize(0.0)
    hs.rk4(0.0, dt, n)
    got = _state(hs, p)
    want = o.heat_rk4(1.0, 1, [1.0], 0.0, dt, n, o.initialize(1, [1.0], 0.0))
    scale = np.abs(want[0]).max()
    err = np.abs(got[0] - want[0]).max() / scale
    print("vec stage kernel vs FP64 oracle, 60 steps: %.3e relative" % err)
    assert err <= 2e-5
    # the statistics of the mixed state against the oracle's of the same state
    st, valid = hs.stats(n * dt)
    assert valid
    assert st[0] == pytest.approx(o.stats(1, [1.0], n * dt, got)[0], rel=1e-6)


@pytest.mark.gpu
def test_mms_convergence_circle_2d():
    errs = {S.PREC_FP64: [], S.PREC_MIXED: []}
    hs = []
    for npts in (33, 65, 129):
        for prec in errs:
            e, h = _solve(_circle2d(npts), prec)
            errs[prec].append(e)
        hs.append(h)
    for prec, e in errs.items():
        orders = _orders(e, hs)
        print("2-D circle", "fp64" if prec == S.PREC_FP64 else "mixed",
              ["%.3e" % v for v in e], ["%.2f" % q for q in orders])
        assert min(orders) >= 3.5, (prec, orders)
    for a, b in zip(errs[S.PREC_MIXED], errs[S.PREC_FP64]):
        assert a <= 1.1 * b


@pytest.mark.gpu
def test_mms_convergence_sphere_3d(monkeypatch):
    errs = {S.PREC_FP64: [], S.PREC_MIXED: []}
    hs = []
    for npts in (32, 64, 128):
        case = dict(SPHERE3D, n=(npts,) * 3)
        e, h = _solve(case, S.PREC_FP64)
        errs[S.PREC_FP64].append(e)
        e, _ = _solve(case, S.PREC_MIXED, "vec", monkeypatch)
        errs[S.PREC_MIXED].append(e)
        hs.append(h)
    for prec, e in errs.items():
        orders = _orders(e, hs)
        print("3-D sphere", "fp64" if prec == S.PREC_FP64 else "mixed (vec)",
              ["%.3e" % v for v in e], ["%.2f" % q for q in orders])
        assert min(orders) >= 3.5, (prec, orders)
    for a, b in zip(errs[S.PREC_MIXED], errs[S.PREC_FP64]):
        assert a <= 1.1 * b
