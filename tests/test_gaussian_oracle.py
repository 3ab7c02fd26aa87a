"""The oracle's Gaussian manufactured solution (the reference's "gaussian" kind,
src/mms/gauss1d.cpp, gauss2d.cpp, gauss3d.cpp), on the host.

* Its value equals a transcription of the reference's gauss2d / gauss3d value expression
  (exp(sum_d -0.5 (x_d - c_d)^2 v_d^-2) A cos(t f), summed over terms) to 1e-14.
* Its time derivative, Laplacian and gradient are the derivatives of that value: the heat
  right-hand side of the exact solution, k lap_h(u) + (ddt - k lap), tends to du/dt (a central
  difference in time) as the grid is refined, at fourth order inside and at least second
  order on the Floating and Neumann boundary rows, whose Neumann data is the gradient.  The
  corner shared by two Neumann faces is left out: there the reference's Neumann array holds
  the later axis' gradient component (heat.cpp:324-352 assigns the axes in order), so the
  earlier axis' closure reads the other component, at any resolution.
"""
import numpy as np
import pytest

from oracle.oracle import OracleProblem

GAUSSIAN = 4
TERMS = [((0.4, 0.55, 0.5), (0.18, 0.22, 0.2), 1.3, 2.0),
         ((0.7, 0.3, 0.45), (0.15, 0.12, 0.17), -0.6, 5.0)]


def _reference_value(x, y, z, t, dims):
    """gauss2d / gauss3d operator() (src/mms/gauss2d.cpp:13-24, gauss3d.cpp:13-26), transcribed"""
    sol = 0.0
    for c, v, a, f in TERMS:
        e = -0.5 * (x - c[0]) ** 2 * v[0] ** -2 + -0.5 * (y - c[1]) ** 2 * v[1] ** -2
        if dims == 3:
            e = e + -0.5 * (z - c[2]) ** 2 * v[2] ** -2
        sol = sol + np.exp(e) * a * np.cos(t * f)
    return sol


@pytest.mark.parametrize("dims", [2, 3])
def test_gaussian_value_matches_reference_expression(dims):
    n = (21, 18, 16 if dims == 3 else 1)
    c = dict(n=n, lo=(0, 0, 0), hi=(1, 1.1, 0.9 if dims == 3 else 0), spheres=[((0.5, 0.5, 0.45 if dims == 3 else 0),
                                                                                0.2, "dirichlet")],
             grid_bc=("dirichlet",) * 4 + (("dirichlet",) * 2 if dims == 3 else ("floating",) * 2),
             scheme="E4_2")
    o = OracleProblem(**c)
    t = 0.37
    u = o.exact(GAUSSIAN, TERMS, t)
    x = np.linspace(0, 1, n[0])[:, None, None]
    y = np.linspace(0, 1.1, n[1])[None, :, None]
    z = np.linspace(0, 0.9, n[2])[None, None, :] if dims == 3 else np.zeros((1, 1, 1))
    want = _reference_value(x, y, z, t, dims).reshape(-1)
    assert np.abs(u[0] - want).max() <= 1e-14 * np.abs(want).max()
    for d in range(3):
        pos = o.cut_points(d)["position"]
        if len(pos):
            w = _reference_value(pos[:, 0], pos[:, 1], pos[:, 2], t, dims)
            assert np.abs(u[1 + d] - w).max() <= 1e-14 * np.abs(w).max()


def _rhs_error(n, dims):
    grid_bc = ("neumann", "dirichlet", "dirichlet", "neumann") + (("floating", "neumann") if dims == 3 else
                                                                  ("floating", "floating"))
    c = dict(n=(n, n, n if dims == 3 else 1), lo=(0, 0, 0), hi=(1, 1, 1 if dims == 3 else 0), spheres=[],
             grid_bc=grid_bc, scheme="E4_2")
    o = OracleProblem(**c)
    t, eps = 0.3, 1e-5
    u = o.exact(GAUSSIAN, TERMS, t)
    r = o.heat_rhs(1.0, GAUSSIAN, TERMS, t, u)
    dudt = (o.exact(GAUSSIAN, TERMS, t + eps)[0] - o.exact(GAUSSIAN, TERMS, t - eps)[0]) / (2 * eps)
    shape = (n, n, n) if dims == 3 else (n, n)
    E = np.abs(r[0] - dudt).reshape(shape)
    keep = np.ones(shape, bool)
    keep[-1, ...] = False  # Dirichlet x max
    keep[:, 0, ...] = False  # Dirichlet y min
    # points on two or more Neumann faces (x min, y max, and z max in 3-D)
    on = [np.zeros(shape, bool) for _ in range(3)]
    on[0][0, ...] = True
    on[1][:, -1, ...] = True
    if dims == 3:
        on[2][..., -1] = True
    keep &= (on[0].astype(int) + on[1] + on[2]) < 2
    inner = tuple([slice(3, -3)] * len(shape))
    return E[keep].max(), E[inner].max()


@pytest.mark.parametrize("dims", [2, 3])
def test_gaussian_heat_source_and_neumann_data_converge(dims):
    sizes = (17, 33) if dims == 3 else (33, 65)
    (b0, i0), (b1, i1) = [_rhs_error(n, dims) for n in sizes]
    assert i1 <= i0 / 12  # fourth order inside (16 for a grid twice as fine)
    assert b1 <= b0 / 3.5  # the boundary closures: at least second order
