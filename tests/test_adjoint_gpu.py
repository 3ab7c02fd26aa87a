"""Discrete adjoint of the heat RK4 path (FP64): the transposed right-hand-side operator and
the vector-Jacobian product of an RK4 solve.

* A^T against the oracle: the dot-product identity <A^T x, y> = <x, A y> with A y from the
  oracle's heat_rhs (the reference algorithm), and the transpose of the operator assembled
  from the oracle by probing on a 24^3 copy of the adjoint configuration.
* The gradient of J(u0) = 1/2 ||u(T) - u_obs||^2 (fluid points) against central finite
  differences (eps = 1e-6) along seeded random directions: J is quadratic in u0, so central
  differences are exact up to rounding and the tolerance is 1e-6 relative.
* The torch.autograd wrapper, the tape's checkpoints, and the unsupported cases.
"""
import numpy as np
import pytest

import shoccs_gb300 as S
from shoccs_gb300 import workloads as W
from oracle.oracle import OracleProblem


def case(n):
    return dict(n=(n, n, n), lo=(0, 0, 0), hi=(1, 1, 1),
                spheres=[((0.5, 0.5, 0.5), 0.25, "dirichlet")],
                grid_bc=("dirichlet",) * 6, scheme="E4_2")


def _torch():
    import torch
    return torch


def _field(p, D):
    torch = _torch()
    return S.ScalarField(torch.as_tensor(D, dtype=torch.float64, device="cuda"),
                         *[torch.zeros(k, dtype=torch.float64, device="cuda") for k in p.nR])


def _masks(p):
    c = p.classes()
    evolving = ((c & 0x3F) != 0) & ((c & 0x40) == 0)
    fluid = (c & 0x80) != 0
    return evolving, fluid


def _grid_u0(n):
    x = np.linspace(0, 1, n)
    X, Y, Z = np.meshgrid(x, x, x, indexing="ij")
    return W.gaussian_sum(X, Y, Z, W.adjoint_gaussians()).ravel()


@pytest.mark.gpu
def test_rhs_transpose_dot_product_against_oracle():
    n = 24
    p, o = S.Problem(**case(n)), OracleProblem(**case(n))
    sys_ = S.Heat(p, 1.0, S.PREC_FP64, S.SOL_ZERO)
    rng = np.random.default_rng(5)
    for _ in range(4):
        x, y = rng.standard_normal(p.size), rng.standard_normal(p.size)
        Ay = o.heat_rhs(1.0, S.SOL_ZERO, [], 0.0, [y] + [np.zeros(k) for k in p.nR])[0]
        ATx = _field(p, np.zeros(p.size))
        sys_.rhs_transpose(_field(p, x), ATx)
        lhs = float(np.dot(ATx.D.cpu().numpy(), y))
        rhs = float(np.dot(x, Ay))
        assert abs(lhs - rhs) <= 1e-12 * max(abs(rhs), np.abs(x).dot(np.abs(Ay))), (lhs, rhs)


@pytest.mark.gpu
def test_rhs_transpose_matches_assembled_oracle_operator():
    """Assemble A column by column from the oracle's heat_rhs (probing with every 13th point
    along each axis at once: rows reach at most 6 points along one axis, so each response
    belongs to one probe) and compare A^T x with the library's transposed operator."""
    n, P = 24, 13
    p, o = S.Problem(**case(n)), OracleProblem(**case(n))
    sys_ = S.Heat(p, 1.0, S.PREC_FP64, S.SOL_ZERO)
    idx = np.arange(p.size)
    I, J, K = idx // (n * n), (idx // n) % n, idx % n
    rows, cols, vals = [], [], []
    zR = [np.zeros(k) for k in p.nR]
    for a in range(P):
        for b in range(P):
            for c in range(P):
                colr = (I % P == a) & (J % P == b) & (K % P == c)
                if not colr.any():
                    continue
                r = o.heat_rhs(1.0, S.SOL_ZERO, [], 0.0, [colr.astype(float)] + zR)[0]
                nz = np.nonzero(r)[0]
                for i in nz:
                    # the probe point on one of the axis lines through i within 6 points
                    ci = (I[i], J[i], K[i])
                    found = None
                    for d in range(3):
                        for m in range(-6, 7):
                            q = list(ci)
                            q[d] += m
                            if not 0 <= q[d] < n:
                                continue
                            j = (q[0] * n + q[1]) * n + q[2]
                            if colr[j]:
                                found = j
                    assert found is not None
                    rows.append(i)
                    cols.append(found)
                    vals.append(r[i])
    rows, cols, vals = np.array(rows), np.array(cols), np.array(vals)
    rng = np.random.default_rng(6)
    for _ in range(3):
        x = rng.standard_normal(p.size)
        want = np.zeros(p.size)
        np.add.at(want, cols, vals * x[rows])
        got = _field(p, np.zeros(p.size))
        sys_.rhs_transpose(_field(p, x), got)
        got = got.D.cpu().numpy()
        assert np.abs(got - want).max() <= 1e-12 * np.abs(want).max()


def _loss_and_grad(sys_, p, u0, obs, fluid, t0, dt, steps, need_grad=True):
    sys_.set_state(_field(p, u0))
    tape = sys_.forward(t0, dt, steps, checkpoint_every=10)
    uT = _field(p, np.zeros(p.size))
    sys_.get_state(uT)
    r = (uT.D.cpu().numpy() - obs) * fluid
    J = 0.5 * float(np.dot(r, r))
    if not need_grad:
        return J, r
    g = _field(p, np.zeros(p.size))
    sys_.backward(tape, _field(p, r), g)
    return J, g.D.cpu().numpy()


def _smooth_direction(n, rng, bumps=12):
    """a random sum of Gaussian bumps: the heat solve damps white noise below rounding, so
    directions must live in modes it keeps"""
    gs = [(tuple(rng.uniform(0.1, 0.9, 3)), rng.uniform(0.04, 0.1), rng.standard_normal())
          for _ in range(bumps)]
    x = np.linspace(0, 1, n)
    X, Y, Z = np.meshgrid(x, x, x, indexing="ij")
    v = W.gaussian_sum(X, Y, Z, gs).ravel()
    return v / np.linalg.norm(v)


@pytest.mark.gpu
def test_backward_matches_central_finite_differences():
    n, steps = 24, 40
    p = S.Problem(**case(n))
    sys_ = S.Heat(p, 1.0, S.PREC_FP64, S.SOL_ZERO)
    _, fluid = _masks(p)
    dt = W.heat_dt(n)
    u0 = _grid_u0(n)
    rng = np.random.default_rng(W.SEED_ADJOINT_DIRECTIONS)
    obs = 0.01 * rng.standard_normal(p.size)
    _, g = _loss_and_grad(sys_, p, u0, obs, fluid, 0.0, dt, steps)
    eps = 1e-6
    for _ in range(8):
        v = _smooth_direction(n, rng)
        _, rp = _loss_and_grad(sys_, p, u0 + eps * v, obs, fluid, 0.0, dt, steps, False)
        _, rm = _loss_and_grad(sys_, p, u0 - eps * v, obs, fluid, 0.0, dt, steps, False)
        # J(u0 + eps v) - J(u0 - eps v) = 1/2 (r+ - r-).(r+ + r-), without cancellation
        fd = 0.5 * float(np.dot(rp - rm, rp + rm)) / (2 * eps)
        gv = float(np.dot(g, v))
        assert abs(fd - gv) <= 1e-6 * abs(gv), (fd, gv)


@pytest.mark.gpu
@pytest.mark.parametrize("steps", [1, 2, 17])
def test_backward_is_the_transpose_of_the_solve(steps):
    """w . F(v) = F^T(w) . v for the RK4 solve F (Dirichlet faces and solid points included)"""
    n = 24
    p = S.Problem(**case(n))
    sys_ = S.Heat(p, 1.0, S.PREC_FP64, S.SOL_ZERO)
    rng = np.random.default_rng(11)
    dt = W.heat_dt(n)
    for _ in range(3):
        v, w = _smooth_direction(n, rng), _smooth_direction(n, rng)
        sys_.set_state(_field(p, v))
        tape = sys_.forward(0.0, dt, steps)
        Fv = _field(p, np.zeros(p.size))
        sys_.get_state(Fv)
        FTw = _field(p, np.zeros(p.size))
        sys_.backward(tape, _field(p, w), FTw)
        a = float(np.dot(w, Fv.D.cpu().numpy()))
        b = float(np.dot(FTw.D.cpu().numpy(), v))
        assert abs(a - b) <= 1e-13 * (abs(a) + 1e-300) + 1e-15, (a, b)


@pytest.mark.gpu
def test_torch_autograd_wrapper():
    torch = _torch()
    n, steps = 20, 12
    p = S.Problem(**case(n))
    sys_ = S.Heat(p, 1.0, S.PREC_FP64, S.SOL_ZERO)
    _, fluid = _masks(p)
    dt = W.heat_dt(n)
    u0 = torch.tensor(_grid_u0(n), dtype=torch.float64, device="cuda", requires_grad=True)
    obs = torch.zeros(p.size, dtype=torch.float64, device="cuda")
    fl = torch.tensor(fluid, dtype=torch.float64, device="cuda")
    uT = S.rk4_solve(sys_, u0, 0.0, dt, steps)
    L = 0.5 * (((uT - obs) * fl) ** 2).sum()
    L.backward()
    J, g = _loss_and_grad(sys_, p, u0.detach().cpu().numpy(), obs.cpu().numpy(), fluid, 0.0,
                          dt, steps)
    assert abs(L.item() - J) <= 1e-12 * J
    np.testing.assert_allclose(u0.grad.cpu().numpy(), g, rtol=0, atol=1e-14 * np.abs(g).max())


@pytest.mark.gpu
def test_tape_checkpoints_are_the_forward_states():
    torch = _torch()
    n, steps, every = 20, 25, 10
    p = S.Problem(**case(n))
    a = S.Heat(p, 1.0, S.PREC_FP64, S.SOL_ZERO)
    b = S.Heat(p, 1.0, S.PREC_FP64, S.SOL_ZERO)
    u0 = _grid_u0(n)
    dt = W.heat_dt(n)
    a.set_state(_field(p, u0))
    tape = a.forward(0.0, dt, steps, checkpoint_every=every)
    assert len(tape) == 4  # t0, after 10, 20, 25 steps
    b.set_state(_field(p, u0))
    done = 0
    for i, k in enumerate((0, 10, 10, 5)):
        if k:
            b.rk4(done * dt, dt, k)
        done += k
        want = _field(p, np.zeros(p.size))
        b.get_state(want)
        got = torch.empty(p.size, dtype=torch.float64, device="cuda")
        tape.checkpoint(i, got)
        assert torch.equal(got, want.D), i


@pytest.mark.gpu
def test_mixed_adjoint_matches_fp64_gradient():
    """A mixed system records its tape in FP64 and runs the reverse sweep in FP32: its
    gradient equals the FP64 system's to FP32 accuracy, and it is the transpose of the mixed
    solve to FP32 accuracy."""
    n, steps = 24, 30
    p = S.Problem(**case(n))
    s64 = S.Heat(p, 1.0, S.PREC_FP64, S.SOL_ZERO)
    s32 = S.Heat(p, 1.0, S.PREC_MIXED, S.SOL_ZERO)
    _, fluid = _masks(p)
    dt = W.heat_dt(n)
    u0 = _grid_u0(n)
    obs = np.zeros(p.size)
    _, g64 = _loss_and_grad(s64, p, u0, obs, fluid, 0.0, dt, steps)
    _, g32 = _loss_and_grad(s32, p, u0, obs, fluid, 0.0, dt, steps)
    assert np.linalg.norm(g32 - g64) <= 1e-5 * np.linalg.norm(g64)
    rng = np.random.default_rng(12)
    v, w = _smooth_direction(n, rng), _smooth_direction(n, rng)
    s32.set_state(_field(p, v))
    tape = s32.forward(0.0, dt, steps)
    Fv = _field(p, np.zeros(p.size))
    s32.get_state(Fv)
    FTw = _field(p, np.zeros(p.size))
    s32.backward(tape, _field(p, w), FTw)
    a, b = float(np.dot(w, Fv.D.cpu().numpy())), float(np.dot(FTw.D.cpu().numpy(), v))
    assert abs(a - b) <= 1e-5 * (np.linalg.norm(w) * np.linalg.norm(Fv.D.cpu().numpy())), (a, b)


@pytest.mark.gpu
def test_adjoint_rejects_unsupported_systems():
    p = S.Problem(**case(20))
    m = S.Heat(p, 1.0, S.PREC_MIXED, S.SOL_ZERO)
    with pytest.raises(S.ShoccsError):  # the transposed operator alone takes FP64 fields
        m.rhs_transpose(_field(p, np.zeros(p.size)), _field(p, np.zeros(p.size)))
    w = S.ScalarWave(S.Problem(**W.wave_3d(16, radius=0)), S.PREC_FP64, S.VEL_CONSTANT,
                     W.WAVE_VEL, (0, 0, 0), S.SOL_GAUSS_PULSE, W.WAVE_PULSE)
    with pytest.raises(S.ShoccsError):
        w.forward(0.0, 1e-4, 2)
