"""The Error field of system::write on the GPU (shoccs_system_error_field) against the oracle's
restatement of write_scalar_error (src/systems/detail/scalar_system_utils.hpp:224-296):
|u - exact(t)| at the fluid D points and the non-Dirichlet cut points, 0 on the Dirichlet
faces, the solid points and the Dirichlet cut points.

Both sides take the same state u (the GPU system's, read back as FP64); the exact solution is
evaluated by the device and by the host math library, which may differ in the last bit, so
the tolerance is 1e-14 of the state's max-norm.  Zeros must be exact zeros, and the device-
buffer and host-buffer calls must give the same bits.
"""
import numpy as np
import pytest

import shoccs_gb300 as S
from oracle.oracle import OracleProblem
from shoccs_gb300 import workloads as W
from tests.cases import cases

FLOATING_3D = dict(n=(24, 24, 24), lo=(0, 0, 0), hi=(1, 1, 1),
                   spheres=[((0.5, 0.5, 0.5), 0.25, "floating")],
                   grid_bc=("dirichlet", "floating", "dirichlet", "dirichlet", "neumann", "dirichlet"),
                   scheme="E4_2")


def _host(p):
    return [np.zeros(p.size)] + [np.zeros(k) for k in p.nR]


def _check(c, system, steps, dt, sol_kind, params):
    import torch
    p = S.Problem(**c)
    h = system(p)
    h.initialize(0.0)
    h.rk4(0.0, dt, steps)
    t = steps * dt
    u = _host(p)
    h.get_state(S.ScalarField(*u))
    got = h.error_field(t, S.ScalarField(*_host(p)))
    want = OracleProblem(**c).error_field(sol_kind, params, t, u)
    scale = max(max(np.abs(a).max() for a in u if a.size), 1e-300)
    for g, w in zip(got, want):
        assert np.array_equal(g == 0, w == 0)
        assert np.abs(g - w).max(initial=0.0) <= 1e-14 * scale
    dev = h.error_field(t, S.ScalarField(*[torch.zeros(a.size, dtype=torch.float64, device="cuda")
                                           for a in u]))
    for g, d in zip(got, dev):
        assert np.array_equal(g, d.cpu().numpy())
    return got


@pytest.mark.gpu
def test_error_field_fp64_floating_object_and_neumann_face():
    got = _check(FLOATING_3D, lambda p: S.Heat(p, 1.0, S.PREC_FP64, S.SOL_SINSIN, [1.0]), 20,
                 W.heat_dt(24), S.SOL_SINSIN, [1.0])
    # the Floating object's cut points evolve, so their error is not zero
    assert all(np.abs(r).max() > 0 for r in got[1:])


@pytest.mark.gpu
@pytest.mark.parametrize("prec", [S.PREC_FP64, S.PREC_MIXED])
def test_error_field_heat_dirichlet_circle(prec):
    c = cases()["c0_circle_2d"]
    got = _check(c, lambda p: S.Heat(p, 1.0, prec, S.SOL_SINSIN, [1.0]), 50, W.heat_dt(65),
                 S.SOL_SINSIN, [1.0])
    assert np.abs(got[0]).max() > 0
    assert all(not r.any() for r in got[1:])  # Dirichlet cut points


@pytest.mark.gpu
def test_error_field_wave():
    c = cases()["box_e4u"]
    vel = (1.0, 0.7, 0.4)
    pulse = W.WAVE_PULSE
    got = _check(c, lambda p: S.ScalarWave(p, S.PREC_MIXED, S.VEL_CONSTANT, vel, (0, 0, 0),
                                           S.SOL_GAUSS_PULSE, pulse),
                 10, 0.2 / 33, S.SOL_GAUSS_PULSE, pulse)
    assert np.abs(got[0]).max() > 0
