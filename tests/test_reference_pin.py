"""Pin the oracle to the reference's own compiled code.

oracle/build_ref.sh compiles the reference's stencils, mesh and cut-point code, operator
assembly, block / CSR matvecs, derivative, laplacian, gradient, heat and scalar-wave systems
and RK4 integrator unmodified (against serial stand-ins for Kokkos, sol2 and spdlog) into
oracle/_ref.  The arrays of tests/golden/pins.py are compared two ways:

* live, where oracle/_ref exists (it is built wherever the reference tree is present):
  every array of the oracle equals the reference's, bit for bit, on every parity case of
  tests/cases.py -- cut points, line segments, fluid set, block metadata and coefficients,
  the eight CSR matrices per axis, derivative / laplacian / gradient applies, and the heat
  (sin-sin solution, Dirichlet / Floating / Neumann objects and faces) and radial scalar
  wave systems: initial state, right-hand side, RK4 steps, statistics;
* through tests/golden/reference_pins.json, SHA-256 digests of the same arrays made by the
  reference (tests/golden/make_golden.py), on any machine.

Plus the reference's own known-answer tests of the derivative operator
(src/operators/derivative.t.cpp) and the block metadata layout
(src/matrices/block.t.cpp:244-397), run against the oracle and the reference alike.
"""
import json
import os
import platform
import subprocess

import numpy as np
import pytest

from oracle import reference as ref
from oracle.oracle import OracleProblem
from tests.cases import cases
from tests.golden import pins

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "reference_pins.json")
CASES = cases()
REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def reflib():
    if not ref.available():
        script = os.path.join(REPO, "oracle", "build_ref.sh")
        subprocess.run(["sh", script], capture_output=True, check=False)
    if not ref.available():
        pytest.skip("the reference's code is not built here (no reference tree)")
    return ref


def _assert_same(a, b, where):
    assert set(a) == set(b), where
    for k in a:
        x, y = np.asarray(a[k]), np.asarray(b[k])
        assert x.shape == y.shape, (where, k, x.shape, y.shape)
        if x.dtype.kind == "f":
            assert np.array_equal(x.view(np.int64), y.astype(np.float64).view(np.int64)), \
                (where, k, np.abs(x - y).max() if x.size else 0)
        else:
            assert np.array_equal(x, y), (where, k)


def _heat_cases():
    return sorted(n for n, c in CASES.items() if c["scheme"] in pins.HEAT_SCHEMES)


def _shape_ids(p):
    return [p.cut_points(d)["shape_id"] for d in range(3)]


# ---------------------------------------------------------------------------------------
# live comparison with the reference's code
# ---------------------------------------------------------------------------------------
@pytest.mark.parametrize("name", sorted(CASES))
def test_setup_and_operators_equal_reference(reflib, name):
    c = CASES[name]
    r, o = reflib.RefProblem(**c), OracleProblem(**c)
    _assert_same(pins.setup_arrays(r), pins.setup_arrays(o), name)
    _assert_same(pins.operator_arrays(r, name), pins.operator_arrays(o, name), name)


@pytest.mark.parametrize("name", _heat_cases())
def test_heat_system_equals_reference(reflib, name):
    c = CASES[name]
    r = reflib.RefSystem("heat", **c, diffusivity=pins.KAPPA, sol_kind=1, sol=(pins.SINSIN_K,))
    o = OracleProblem(**c)
    sid = _shape_ids(o)
    n, dt = pins.heat_steps(c), pins.heat_dt(c)
    got = pins.system_arrays(pins.OracleHeat(o), name, n, dt,
                             lambda t, u: pins.dirichlet_update(c, sid, o.exact(1, (pins.SINSIN_K,), t), u))
    want = pins.system_arrays(r, name, n, dt, r.update_boundary)
    _assert_same(want, got, name)


@pytest.mark.parametrize("name", sorted(pins.WAVE_CASES))
def test_wave_system_equals_reference(reflib, name):
    c = CASES[name]
    cen, rad = pins.wave_center(c, name)
    r = reflib.RefSystem("wave", **c, center=cen, radius=rad)
    o = OracleProblem(**c)
    sid = _shape_ids(o)
    sol = list(cen) + [rad]
    got = pins.system_arrays(pins.OracleWave(o, cen, rad), name, 3, pins.wave_dt(c),
                             lambda t, u: pins.dirichlet_update(c, sid, o.exact(3, sol, t), u))
    want = pins.system_arrays(r, name, 3, pins.wave_dt(c), r.update_boundary)
    _assert_same(want, got, name)


def test_gaussian_heat_close_to_reference(reflib):
    """The reference's gaussian manufactured solution (src/mms/gauss2d.cpp, gauss3d.cpp) is
    written as generated expanded polynomials; the oracle (and the GPU) evaluate the same
    function in factored form, so heat states agree to rounding, not bit for bit."""
    terms = [((0.3, 0.4, 0.5), (0.02, 0.03, 0.05), 1.3, 0.7),
             ((0.6, 0.5, 0.45), (0.04, 0.02, 0.03), -0.8, 1.9)]
    for name in ("c0_circle_2d", "multi_sphere_e42", "neumann_z_e42"):
        c = CASES[name]
        r = reflib.RefSystem("heat", **c, diffusivity=pins.KAPPA, sol_kind=4, sol=terms)
        o = OracleProblem(**c)
        u0 = r.initialize(0.0)
        assert all(np.allclose(a, b, rtol=0, atol=1e-14)
                   for a, b in zip(u0, o.initialize(4, terms, 0.0)))
        dt = pins.heat_dt(c)
        a = r.rk4(0.0, dt, 4, u0)
        b = o.heat_rk4(pins.KAPPA, 4, terms, 0.0, dt, 4, u0)
        for x, y in zip(a, b):
            if len(y):
                assert np.abs(x - y).max() <= 1e-12 * max(1.0, np.abs(y).max()), name


# ---------------------------------------------------------------------------------------
# the same arrays against the committed digests (no reference tree needed)
# ---------------------------------------------------------------------------------------
def _gold():
    with open(GOLD) as f:
        return json.load(f)


def _check_digests(want, got, where, libm_dependent):
    assert set(want) == set(got), where
    exact_libm = platform.machine() in ("x86_64", "AMD64")
    for k, a in got.items():
        d = pins.digest(a)
        if d == want[k]["sha256"]:
            continue
        # values that went through sin / cos / exp may differ in the last bit on another
        # C library; everything else must match exactly
        assert libm_dependent and not exact_libm, (where, k)
        v = np.asarray(a, dtype=np.float64).ravel()
        assert v.size == want[k]["n"], (where, k)
        assert abs(float(np.abs(v).max(initial=0.0)) - want[k]["maxabs"]) <= \
            1e-12 * max(1.0, want[k]["maxabs"]), (where, k)


@pytest.mark.parametrize("name", sorted(CASES))
def test_setup_and_operators_match_reference_digests(name):
    g = _gold()["cases"][name]
    o = OracleProblem(**CASES[name])
    _check_digests(g["setup"], pins.setup_arrays(o), name, False)
    _check_digests(g["operators"], pins.operator_arrays(o, name), name, False)


def test_systems_match_reference_digests():
    g = _gold()["cases"]
    for name in _heat_cases():
        c = CASES[name]
        o = OracleProblem(**c)
        sid = _shape_ids(o)
        got = pins.system_arrays(
            pins.OracleHeat(o), name, pins.heat_steps(c), pins.heat_dt(c),
            lambda t, u: pins.dirichlet_update(c, sid, o.exact(1, (pins.SINSIN_K,), t), u))
        _check_digests(g[name]["heat"], got, name, True)
    for name in sorted(pins.WAVE_CASES):
        c = CASES[name]
        cen, rad = pins.wave_center(c, name)
        o = OracleProblem(**c)
        sid = _shape_ids(o)
        sol = list(cen) + [rad]
        got = pins.system_arrays(
            pins.OracleWave(o, cen, rad), name, 3, pins.wave_dt(c),
            lambda t, u: pins.dirichlet_update(c, sid, o.exact(3, sol, t), u))
        _check_digests(g[name]["wave"], got, name, True)


# ---------------------------------------------------------------------------------------
# the reference's own known-answer tests
# ---------------------------------------------------------------------------------------
def _f2(x, y, z):
    # src/operators/derivative.t.cpp:30-33
    return x * (y + z) + y * (x + z) + z * (x + y) + 3 * x * y * z


def _f2_dx(x, y, z):
    return 2.0 * (y + z) + 3.0 * y * z


def _eval(p, case, f):
    n = list(case["n"])
    lo, hi = case["lo"], case["hi"]
    xs = [np.array([lo[a] + i * (hi[a] - lo[a]) / (n[a] - 1) if n[a] > 1 else lo[a]
                    for i in range(n[a])]) for a in range(3)]
    X, Y, Z = np.meshgrid(*xs, indexing="ij")
    u = [f(X.ravel(), Y.ravel(), Z.ravel())]
    for d in range(3):
        pos = p.cut_points(d)["position"]
        u.append(f(pos[:, 0], pos[:, 1], pos[:, 2]) if len(pos) else np.zeros(0))
    return u


def _approx(a, b):
    """Catch::Approx with its default epsilon (100 float epsilons) after the tests' +1
    offset (derivative.t.cpp approx_D / approx_all)"""
    a, b = np.asarray(a) + 1.0, np.asarray(b) + 1.0
    return np.all(np.abs(a - b) <= 100 * np.finfo(np.float32).eps * np.maximum(np.abs(a), np.abs(b)))


KNOWN = {
    # derivative.t.cpp:235-261 "E2_2 FFFFFF"
    "E2_2 FFFFFF": dict(n=(5, 7, 6), lo=(0.1, 0.2, 0.3), hi=(1, 2, 2.2), spheres=[],
                        grid_bc=("floating",) * 6, scheme="E2_2"),
    # derivative.t.cpp:324-358 "E2 Mixed" DDFFFD
    "E2 Mixed DDFFFD": dict(n=(5, 7, 6), lo=(0.1, 0.2, 0.3), hi=(1, 2, 2.2), spheres=[],
                            grid_bc=("dirichlet", "dirichlet", "floating", "floating",
                                     "floating", "dirichlet"), scheme="E2_2"),
    # derivative.t.cpp:360-384 "E2 Mixed" FNDDDF (Neumann data = df2/dx)
    "E2 Mixed FNDDDF": dict(n=(5, 7, 6), lo=(0.1, 0.2, 0.3), hi=(1, 2, 2.2), spheres=[],
                            grid_bc=("floating", "neumann", "dirichlet", "dirichlet",
                                     "dirichlet", "floating"), scheme="E2_2"),
}


def _zero_dirichlet_faces(case, a):
    n = list(case["n"])
    A = a.reshape(n)
    for ax in range(3):
        for side, face in ((0, 0), (1, n[ax] - 1)):
            if case["grid_bc"][2 * ax + side] == "dirichlet":
                sl = [slice(None)] * 3
                sl[ax] = face
                A[tuple(sl)] = 0.0
    return a


@pytest.mark.parametrize("label", sorted(KNOWN))
def test_derivative_known_answers(label):
    """second derivatives of the quadratic-in-each-variable f2 are exactly zero, and zero
    at the Dirichlet faces (the rows the operator removes)"""
    c = KNOWN[label]
    impls = [OracleProblem(**c)]
    if ref.available():
        impls.append(ref.RefProblem(**c))
    for p in impls:
        u = _eval(p, c, _f2)
        nu = _eval(p, c, _f2_dx)[0] if "neumann" in c["grid_bc"] else None
        for d in range(3):
            du = p.derivative(d, u, p.zeros(), False, nu)
            want = _zero_dirichlet_faces(c, np.zeros(p.size))
            assert _approx(du[0], want), (label, type(p).__name__, d)
        if nu is None:
            # and a nonzero answer: d2/dx_d2 of x^2 + 2 y^2 + 3 z^2 is 2 (d + 1)
            q = _eval(p, c, lambda x, y, z: x * x + 2 * y * y + 3 * z * z)
            for d in range(3):
                du = p.derivative(d, q, p.zeros())
                want = _zero_dirichlet_faces(c, np.full(p.size, 2.0 * (d + 1)))
                assert _approx(du[0], want), (label, type(p).__name__, d)


def test_derivative_known_answers_with_floating_object():
    """derivative.t.cpp:515-568 "E2 with Objects": a Floating sphere, Neumann x faces and
    Dirichlet y faces; every D and R value of each second derivative of f2 is zero at fluid
    points and at non-Dirichlet cut points"""
    c = dict(n=(25, 26, 27), lo=(0.1, 0.2, 0.3), hi=(1, 2, 2.2),
             spheres=[((0.45, 1.011, 1.31), 0.25, "floating")],
             grid_bc=("neumann", "neumann", "dirichlet", "dirichlet", "floating", "floating"),
             scheme="E2_2")
    impls = [OracleProblem(**c)]
    if ref.available():
        impls.append(ref.RefProblem(**c))
    for p in impls:
        u = _eval(p, c, _f2)
        nu = _eval(p, c, _f2_dx)[0]
        for d in range(3):
            du = p.derivative(d, u, p.zeros(), False, nu if d == 0 else None)
            for k in range(4):
                assert _approx(du[k], np.zeros_like(du[k])), (type(p).__name__, d, k)


def test_block_metadata_known_answers():
    """src/matrices/block.t.cpp:244-397: the metadata fields of two hand-built line blocks
    (left 4x5, circulant width 3 over 10 rows, right 2x3, 16 columns, stride 1, at offsets
    1 and 20) and of two strided ones (left 3x5, width 5, right 2x3, 15 columns, stride 3,
    offsets 0 and 1)"""
    o = OracleProblem(n=(4, 1, 1), lo=(0, 0, 0), hi=(1, 0, 0))
    meta = o.block_layout([(16, 1, 1, 1, (4, 5), 10, 3, (2, 3)),
                           (16, 20, 20, 1, (4, 5), 10, 3, (2, 3))])
    per = 20 + 3 + 6
    assert meta[0].tolist() == [1, 1, 1, 4, 5, 0, 10, 20, 3, 2, 3, 23, 14]
    assert meta[1].tolist() == [20, 20, 1, 4, 5, per, 10, per + 20, 3, 2, 3, per + 23, 33]
    meta = o.block_layout([(15, 0, 0, 3, (3, 5), 10, 5, (2, 3)),
                           (15, 1, 1, 3, (3, 5), 10, 5, (2, 3))])
    assert meta[0][[0, 1, 2, 12]].tolist() == [0, 0, 3, 36]
    assert meta[1][[0, 1, 2, 12]].tolist() == [1, 1, 3, 37]
