"""The uniform-grid 6th- and 8th-order first derivatives E6u_1 (7-point interior, 5 x 8 wall
blocks; src/stencils/E6u_1.cpp) and E8u_1 (9-point interior, 7 x 11 wall blocks;
src/stencils/E8u_1.cpp) on the CUDA path.  The column, vectorised and TMA stage kernels keep
a five-point window, so systems with these schemes run on the per-point stage kernel, and
wall blocks wider than five rows by seven columns are stored as per-row closure records.

Tolerances (max-norm, relative to the oracle array's max-norm): FP64 right-hand side 1e-12,
FP64 derivative of a degree-6/8 polynomial at 150 x 144 x 160 5e-12 (7- and 9-term sums of
terms up to 1e3 times the result, summed in a different order), RK4
state 1e-10 (FP64 arithmetic in a different order); mixed right-hand side 2e-6, mixed RK4
state 2e-5 (FP32 fields).
"""
import numpy as np
import pytest

import shoccs_gb300 as S
from oracle.oracle import OracleProblem
from tests.cases import E6U_ALPHA, E8U_ALPHA, cases

WIDE = {name: cases()[name] for name in ("e6u_sphere_3d", "e8u_circle_2d")}
VEL = (1.0, 0.7, 0.4)
PULSE = [0.3, 0.3, 0.3, 1.0, 0.7, 0.4, 0.08]  # Gaussian pulse (x0, a, sigma)


def rel(got, want):
    want = np.asarray(want)
    if want.size == 0:
        return 0.0
    return float(np.abs(np.asarray(got) - want).max() / max(np.abs(want).max(), 1e-300))


def _state(w, p):
    u = [np.zeros(p.size)] + [np.zeros(k) for k in p.nR]
    w.get_state(S.ScalarField(*u))
    return u


@pytest.mark.gpu
@pytest.mark.parametrize("prec", [S.PREC_FP64, S.PREC_MIXED])
@pytest.mark.parametrize("name", sorted(WIDE))
def test_wide_wave_rhs_and_rk4_match_oracle(name, prec):
    """The alpha of the reference's own stencil tests do not make these closures stable
    under RK4 with Dirichlet inflow (the oracle's solution grows by orders of magnitude within
    twenty steps), so the right-hand side is compared, then a few RK4 steps."""
    import torch
    c = WIDE[name]
    p, o = S.Problem(**c), OracleProblem(**c)
    w = S.ScalarWave(p, prec, S.VEL_CONSTANT, VEL, (0, 0, 0), 2, PULSE)
    w.initialize(0.0)
    assert w.stage_kernel == "point"
    u0 = o.initialize(2, PULSE, 0.0)
    want = o.wave_rhs(S.VEL_CONSTANT, VEL, (0, 0, 0), u0)
    got = w.rhs(0.0, p.zeros(torch.float64))  # FP64 output for either precision
    assert rel(got.D.cpu().numpy(), want[0]) <= (1e-12 if prec == S.PREC_FP64 else 2e-6), name
    h = min((c["hi"][a] - c["lo"][a]) / (c["n"][a] - 1) for a in range(3) if c["n"][a] > 1)
    dt, steps = 0.2 * h, 3
    w.rk4(0.0, dt, steps)
    got = _state(w, p)
    want = o.wave_rk4(S.VEL_CONSTANT, VEL, (0, 0, 0), 2, PULSE, 0.0, dt, steps, u0)
    assert rel(got[0], want[0]) <= (1e-10 if prec == S.PREC_FP64 else 2e-5), name
    t = steps * dt
    st, ok = w.stats(t)
    ref = o.stats(2, PULSE, t, want)
    # E6u with these alpha has grown past the wave system's error bound (ScalarWave's
    # default max_error, 100) within the three steps: the status says so, the values are
    # still reported
    assert ok == (ref[0] <= 100.0), (name, ref[0])
    tol = 1e-8 if prec == S.PREC_FP64 else 1e-3
    for k in (0, 1, 2, 5, 7):  # errors, min, max
        assert abs(st[k] - ref[k]) <= tol * max(abs(ref[k]), 1e-12), (name, k, st[k], ref[k])


@pytest.mark.gpu
@pytest.mark.parametrize("scheme,alpha,deg", [("E6u_1", E6U_ALPHA, 6), ("E8u_1", E8U_ALPHA, 8)])
def test_wide_derivative_large_grid(scheme, alpha, deg):
    """At 150 x 144 x 160 with a Dirichlet sphere: the FP64 derivative along each axis equals
    the oracle's, and on points whose rows are interior along every axis (the 7- or 9-point
    stencil clear of walls and the sphere) it differentiates a polynomial of the interior
    stencil's degree exactly (to rounding)."""
    import torch
    c = dict(n=(150, 144, 160), lo=(0, 0, 0), hi=(1, 1, 1),
             spheres=[((0.5, 0.47, 0.53), 0.2, "dirichlet")],
             grid_bc=("dirichlet", "floating") * 3, scheme=scheme, alpha=alpha)
    p, o = S.Problem(**c), OracleProblem(**c)
    xs = [np.linspace(0, 1, n) for n in c["n"]]
    X, Y, Z = [g.ravel() for g in np.meshgrid(*xs, indexing="ij")]
    f = lambda x, y, z: (x - 0.4) ** deg + 0.5 * (y - 0.3) ** (deg - 1) + (z - 0.6) ** deg
    df = [lambda x, y, z: deg * (x - 0.4) ** (deg - 1),
          lambda x, y, z: 0.5 * (deg - 1) * (y - 0.3) ** (deg - 2),
          lambda x, y, z: deg * (z - 0.6) ** (deg - 1)]
    u = o.zeros()
    u[0][:] = f(X, Y, Z)
    for d in range(3):
        pos = o.cut_points(d)["position"]
        u[1 + d][:] = f(pos[:, 0], pos[:, 1], pos[:, 2])
    cls = p.classes()
    interior = (cls & 0x3F) == 0x15
    assert interior.sum() > 0.5 * p.size
    ud = S.ScalarField(*[torch.tensor(a, dtype=torch.float64, device="cuda") for a in u])
    for d in range(3):
        want = o.derivative(d, u, o.zeros())
        got = p.zeros(torch.float64)
        S.Derivative(p, d)(ud, got)
        g = got.D.cpu().numpy()
        assert rel(g, want[0]) <= 5e-12, (scheme, d)
        exact = df[d](X, Y, Z)
        assert np.abs(g[interior] - exact[interior]).max() <= 1e-9 * np.abs(exact).max(), (scheme, d)


@pytest.mark.gpu
def test_wide_batch_unsupported():
    """batched solves keep a five-point window along each axis"""
    p = S.Problem(**WIDE["e6u_sphere_3d"])
    with pytest.raises(S.ShoccsError):
        S.Batch([S.Heat(p, 1.0, S.PREC_MIXED, S.SOL_SINSIN, [1.0])])
