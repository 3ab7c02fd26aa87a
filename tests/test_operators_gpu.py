"""CUDA operators against the oracle: derivative (eq / plus_eq, with and without Neumann
data), Laplacian and gradient on every shared case.

Tolerance (max-norm, relative to the oracle's max-norm of the same array):
  FP64   1e-12   (the reference's own path and the CUDA path differ only by the order
                  and fusion of the FP64 operations)
  MIXED  2e-6    (FP32 field values and FP32 interior arithmetic; FP64 closure rows)
"""
import numpy as np
import pytest

import shoccs_gb300 as S
from oracle.oracle import OracleProblem
from tests.cases import cases

CASES = cases()
TOL64 = 1e-12
TOL32 = 2e-6


def _torch():
    import torch
    return torch


def rand_field(o, seed):
    rng = np.random.default_rng(seed)
    return [rng.uniform(-1, 1, o.size)] + [rng.uniform(-1, 1, n) for n in o.nR]


def to_dev(f, dtype):
    torch = _torch()
    return S.ScalarField(*[torch.tensor(a, dtype=dtype, device="cuda") for a in f])


def rel_err(got, want):
    got = np.asarray(got, dtype=np.float64)
    if want.size == 0:
        return 0.0
    scale = max(np.abs(want).max(), 1e-300)
    return float(np.abs(got - want).max() / scale)


def check(got_field, want, tol, what):
    for k, (g, w) in enumerate(zip(got_field, want)):
        e = rel_err(g.cpu().numpy(), w)
        assert e <= tol, "%s component %d: relative max-norm error %.3e > %.1e" % (what, k, e, tol)


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(CASES))
@pytest.mark.parametrize("prec", [S.PREC_FP64, S.PREC_MIXED])
def test_derivative(name, prec):
    torch = _torch()
    c = CASES[name]
    p, o = S.Problem(**c), OracleProblem(**c)
    dtype, tol = (torch.float64, TOL64) if prec == S.PREC_FP64 else (torch.float32, TOL32)
    u = rand_field(o, 1)
    if prec == S.PREC_MIXED:
        u = [a.astype(np.float32).astype(np.float64) for a in u]
    has_neumann = "neumann" in c.get("grid_bc", ())
    for d in range(3):
        for plus_eq in (False, True):
            for use_nu in ((False, True) if has_neumann else (False,)):
                du0 = rand_field(o, 10 + d)
                if prec == S.PREC_MIXED:
                    du0 = [a.astype(np.float32).astype(np.float64) for a in du0]
                nu = np.random.default_rng(5).uniform(-1, 1, o.size) if use_nu else None
                want = o.derivative(d, u, [a.copy() for a in du0], plus_eq=plus_eq, nu=nu)
                got = to_dev(du0, dtype)
                nu_dev = None
                if use_nu:
                    nu_dev = S.ScalarField(torch.tensor(nu, device="cuda"), None, None, None)
                S.Derivative(p, d, prec)(to_dev(u, dtype), got, plus_eq=plus_eq, nu=nu_dev)
                check(got, want, tol, "%s d=%d plus_eq=%s nu=%s" % (name, d, plus_eq, use_nu))


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(CASES))
@pytest.mark.parametrize("prec", [S.PREC_FP64, S.PREC_MIXED])
def test_laplacian(name, prec):
    torch = _torch()
    c = CASES[name]
    if c["scheme"] == "E4_1":
        pytest.skip("first-derivative scheme")
    p, o = S.Problem(**c), OracleProblem(**c)
    dtype, tol = (torch.float64, TOL64) if prec == S.PREC_FP64 else (torch.float32, TOL32)
    u = rand_field(o, 2)
    if prec == S.PREC_MIXED:
        u = [a.astype(np.float32).astype(np.float64) for a in u]
    nus = [None]
    if "neumann" in c.get("grid_bc", ()):
        nus.append(np.random.default_rng(6).uniform(-1, 1, o.size))
    for nu in nus:
        want = o.laplacian(u, o.zeros(), nu=nu)
        got = p.zeros(dtype)
        nu_dev = None if nu is None else S.ScalarField(torch.tensor(nu, device="cuda"), None,
                                                       None, None)
        S.Laplacian(p, prec)(to_dev(u, dtype), got, nu=nu_dev)
        check(got, want, tol, "%s laplacian nu=%s" % (name, nu is not None))


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(CASES))
@pytest.mark.parametrize("prec", [S.PREC_FP64, S.PREC_MIXED])
def test_gradient(name, prec):
    torch = _torch()
    c = CASES[name]
    p, o = S.Problem(**c), OracleProblem(**c)
    dtype, tol = (torch.float64, TOL64) if prec == S.PREC_FP64 else (torch.float32, TOL32)
    u = rand_field(o, 3)
    if prec == S.PREC_MIXED:
        u = [a.astype(np.float32).astype(np.float64) for a in u]
    want = o.gradient(u)
    got = [p.zeros(dtype) for _ in range(3)]
    S.Gradient(p, prec)(to_dev(u, dtype), *got)
    for d in range(3):
        check(got[d], want[d], tol, "%s gradient d=%d" % (name, d))


@pytest.mark.gpu
def test_derivative_smooth_function_large_grid():
    """Size-independent check at a larger grid: E4_2 Laplacian of a smooth field converges
    at 4th order in the interior and the FP64 kernel matches the oracle."""
    torch = _torch()
    c = dict(n=(96, 90, 100), lo=(0, 0, 0), hi=(1, 1, 1),
             spheres=[((0.5, 0.45, 0.55), 0.25, "dirichlet")],
             grid_bc=("dirichlet",) * 6, scheme="E4_2")
    p, o = S.Problem(**c), OracleProblem(**c)
    xs = [np.linspace(0, 1, n) for n in c["n"]]
    X, Y, Z = [g.ravel() for g in np.meshgrid(*xs, indexing="ij")]
    f = lambda x, y, z: np.sin(2 * x) * np.cos(3 * y) * np.exp(z)
    u = o.zeros()
    u[0][:] = f(X, Y, Z)
    for d in range(3):
        pos = o.cut_points(d)["position"]
        u[1 + d][:] = f(pos[:, 0], pos[:, 1], pos[:, 2])
    want = o.laplacian(u, o.zeros())
    got = p.zeros(torch.float64)
    S.Laplacian(p)(to_dev(u, torch.float64), got)
    check(got, want, TOL64, "smooth laplacian")
    exact = (-4 - 9 + 1) * f(X, Y, Z)
    cls = p.classes()
    interior = (cls & 0x3F) == 0x15
    err = np.abs(got.D.cpu().numpy()[interior] - exact[interior]).max()
    assert err < 1e-4 * np.abs(exact).max()
