"""Pin the CPU oracle against the reference's own golden vectors and code.

* stencils_ref.json / stencils_poly_ref.json / stencils_wide_ref.json / sphere_hits_ref.json:
  produced by the reference's own src/stencils/{E2_2,E4_2,E4_1,E4u_1,polyE2_1,E6u_1,
  E8u_1}.cpp and src/mesh/sphere.cpp (oracle/_ref) -> bit-exact.
* object_geometry_sphere.json: the expected values of src/mesh/object_geometry.t.cpp:11-330.
* line segmentation: the assertions of src/mesh/mesh.t.cpp:71-141.
* known-answer polynomial tests in the style of src/operators/derivative.t.cpp:235-261,
  515-568 and src/operators/laplacian.t.cpp:337-410 (quadratics are reproduced exactly).
"""
import ctypes
import json
import os

import numpy as np
import pytest

from oracle import oracle as orc

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
D = ctypes.c_double


def _hex(a):
    return np.array([float.fromhex(v) for v in a])


def test_stencils_bit_exact_vs_reference_code():
    g = json.load(open(os.path.join(GOLD, "stencils_ref.json")))
    L = orc.lib()
    alpha = (D * 2)(*g["alpha"])
    alpha_u = (D * 2)(*g["alpha_e4u"])
    for e in g["nbs"]:
        c, x = (D * 64)(), (D * 8)()
        L.orc_stencil_nbs(e["scheme"], alpha_u if e["scheme"] == 3 else alpha, D(e["h"]),
                          e["bc"], D(e["psi"]), e["right"], c, x)
        want = _hex(e["c"])
        got = np.array(c[:len(want)])
        assert np.array_equal(got.view(np.int64), want.view(np.int64)), e
        wx = _hex(e["x"])
        nx = {0: 2, 1: 3, 2: 0, 3: 0}[e["scheme"]] if e["bc"] == 2 else 0
        assert np.array_equal(np.array(x[:nx]), wx[:nx]), e
    for e in g["interior"]:
        c = (D * 8)()
        L.orc_stencil_interior(e["scheme"], D(e["h"]), c)
        want = _hex(e["c"])
        assert np.array_equal(np.array(c[:len(want)]).view(np.int64), want.view(np.int64))
    for e in g["interp"]:
        c = (D * 8)()
        if e["kind"] == "interior":
            n = L.orc_stencil_interp_interior(e["scheme"], D(e["y"]), c)
        else:
            n = L.orc_stencil_interp_wall(e["scheme"], None, e["i"], D(e["y"]), D(e["psi"]),
                                          e["right"], c)
        want = _hex(e["c"])
        assert n == len(want)
        assert np.array_equal(np.array(c[:n]).view(np.int64), want.view(np.int64)), e


def test_poly_e2_stencil_bit_exact_vs_reference_code():
    """E2-poly (polyE2_1): closure blocks (Dirichlet 2 x 4, Floating 3 x 4), interior row and
    interpolants of src/stencils/polyE2_1.cpp compiled in oracle/_ref, for the parameters of
    the reference's scalar_wave.lua and a random set."""
    g = json.load(open(os.path.join(GOLD, "stencils_poly_ref.json")))
    L = orc.lib()
    als = [(D * 13)(*a) for a in g["alpha"]]
    for e in g["nbs"]:
        c, x = (D * 64)(), (D * 8)()
        L.orc_stencil_nbs(5, als[e["alpha"]], D(e["h"]), e["bc"], D(e["psi"]), e["right"], c, x)
        want = _hex(e["c"])
        assert np.array_equal(np.array(c[:len(want)]).view(np.int64), want.view(np.int64)), e
    for e in g["interior"]:
        c = (D * 8)()
        L.orc_stencil_interior(5, D(e["h"]), c)
        want = _hex(e["c"])
        assert np.array_equal(np.array(c[:len(want)]).view(np.int64), want.view(np.int64)), e
    for e in g["interp"]:
        c = (D * 8)()
        if e["kind"] == "interior":
            n = L.orc_stencil_interp_interior(5, D(e["y"]), c)
        else:
            n = L.orc_stencil_interp_wall(5, als[e["alpha"]], e["i"], D(e["y"]), D(e["psi"]),
                                          e["right"], c)
        want = _hex(e["c"])
        assert n == len(want)
        assert np.array_equal(np.array(c[:n]).view(np.int64), want.view(np.int64)), e


def test_wide_uniform_stencils_bit_exact_vs_reference_code():
    """E6u_1 (7-point interior, 5 x 8 closures) and E8u_1 (9-point interior, 7 x 11) of
    src/stencils/E6u_1.cpp, E8u_1.cpp compiled in oracle/_ref, with the alpha of the
    reference's own tests"""
    g = json.load(open(os.path.join(GOLD, "stencils_wide_ref.json")))
    L = orc.lib()
    als = {int(k): (D * len(v))(*v) for k, v in g["alpha"].items()}
    for e in g["nbs"]:
        c, x = (D * 128)(), (D * 8)()
        L.orc_stencil_nbs(e["scheme"], als[e["scheme"]], D(e["h"]), e["bc"], D(1.0), e["right"], c, x)
        want = _hex(e["c"])
        assert np.array_equal(np.array(c[:len(want)]).view(np.int64), want.view(np.int64)), e
    for e in g["interior"]:
        c = (D * 16)()
        L.orc_stencil_interior(e["scheme"], D(e["h"]), c)
        want = _hex(e["c"])
        assert np.array_equal(np.array(c[:len(want)]).view(np.int64), want.view(np.int64)), e


def test_sphere_hits_bit_exact_vs_reference_code():
    g = json.load(open(os.path.join(GOLD, "sphere_hits_ref.json")))
    L = orc.lib()
    n_hit = 0
    for e in g["hits"]:
        direction = [0.0, 0.0, 0.0]
        direction[e["axis"]] = 1.0
        t, pos, ro, nrm = D(), (D * 3)(), ctypes.c_int(), (D * 3)()
        ok = L.orc_sphere_hit((D * 3)(*_hex(e["center"])), D(float.fromhex(e["radius"])),
                              (D * 3)(*_hex(e["origin"])), (D * 3)(*direction), D(0.0), D(3.0),
                              ctypes.byref(t), pos, ctypes.byref(ro), nrm)
        assert ok == e["hit"]
        if ok:
            n_hit += 1
            assert t.value == float.fromhex(e["t"])
            assert list(pos) == list(_hex(e["pos"]))
            assert ro.value == e["ray_outside"]
            assert list(nrm) == list(_hex(e["normal"]))
    assert n_hit > 200


def test_sphere_intersections_match_reference_test():
    g = json.load(open(os.path.join(GOLD, "object_geometry_sphere.json")))
    m = g["mesh"]
    p = orc.OracleProblem(m["n"], m["lo"], m["hi"],
                          spheres=[(g["sphere"]["center"], g["sphere"]["radius"], "dirichlet")])
    for d, name in enumerate("xyz"):
        exp = g["axes"][name]
        cp = p.cut_points(d)
        pos = np.array(exp["position"]).reshape(-1, 3)
        assert cp["position"].shape == pos.shape
        np.testing.assert_allclose(cp["position"], pos, rtol=0, atol=1e-14)
        assert np.array_equal(cp["solid_coord"], np.array(exp["solid_coord"]).reshape(-1, 3))
        np.testing.assert_allclose(cp["psi"], np.array(exp["psi"]), rtol=1.2e-5)


def test_lines_match_reference_test():
    # src/mesh/mesh.t.cpp:71-141 (X section)
    ext = (21, 22, 23)
    p = orc.OracleProblem(ext, (-1, -1, 0), (1, 2, 2.2),
                          spheres=[((0.01, -0.01, 0.5), 0.25, "dirichlet")])
    lines = p.lines(0)
    assert len(lines) == ext[1] * ext[2] + 26 // 2
    assert list(lines[0][:3]) == [0, 0, 0] and list(lines[0][4:7]) == [20, 0, 0]
    assert list(lines[1][:3]) == [0, 0, 1] and list(lines[1][4:7]) == [20, 0, 1]
    assert list(lines[-1][:3]) == [0, 21, 22] and list(lines[-1][4:7]) == [20, 21, 22]
    l = lines[6 * ext[2] + 3]
    assert list(l[:3]) == [0, 6, 3] and l[3] == -1
    assert list(l[4:7]) == [10, 6, 3] and l[7] == 0
    l = lines[6 * ext[2] + 3 + 1]
    assert list(l[:3]) == [10, 6, 3] and l[3] == 1
    assert list(l[4:7]) == [20, 6, 3] and l[7] == -1
    psi = p.cut_points(0)["psi"]
    assert psi[0] == pytest.approx(0.40365385103120377)
    assert psi[1] == pytest.approx(0.2036538510312047)


def _coords(p):
    n = p.n
    lo, hi = p._lo, p._hi
    xs = [np.array([lo[a] + i * (hi[a] - lo[a]) / (n[a] - 1) if n[a] > 1 else lo[a]
                    for i in range(n[a])]) for a in range(3)]
    X, Y, Z = np.meshgrid(*xs, indexing="ij")
    return X.ravel(), Y.ravel(), Z.ravel()


@pytest.mark.parametrize("scheme", ["E2_2", "E4_2"])
@pytest.mark.parametrize("obj_bc", ["dirichlet", "floating"])
def test_laplacian_quadratic_exact(scheme, obj_bc):
    """laplacian(x^2 + 2 y^2 + 3 z^2) = 12 at every row (laplacian.t.cpp:337-488 style)."""
    n, lo, hi = (19, 21, 17), (-1, -1, -1), (1, 1, 1)
    p = orc.OracleProblem(n, lo, hi, spheres=[((0.05, -0.02, 0.03), 0.45, obj_bc)],
                          grid_bc=("dirichlet", "floating", "floating", "dirichlet",
                                   "floating", "floating"), scheme=scheme)
    p._lo, p._hi = lo, hi
    X, Y, Z = _coords(p)
    f = lambda x, y, z: x * x + 2 * y * y + 3 * z * z
    u = p.zeros()
    u[0][:] = f(X, Y, Z)
    for d in range(3):
        pos = p.cut_points(d)["position"]
        u[1 + d][:] = f(pos[:, 0], pos[:, 1], pos[:, 2])
    du = p.laplacian(u, p.zeros())
    fl = p.fluid()
    # rows that exist along every axis: fluid points off the Dirichlet faces
    ijk = np.stack(np.unravel_index(fl, n), axis=1)
    keep = (ijk[:, 0] > 0) & (ijk[:, 1] < n[1] - 1)
    np.testing.assert_allclose(du[0][fl[keep]], 12.0, rtol=0, atol=2e-8)
    # The R-space rows of Floating objects are not exact for quadratics in the reference
    # either: its own "E2 with Floating Objects" test fails at the Rx assertion
    # (src/operators/laplacian.t.cpp:483, excluded from its CI).  The oracle reproduces the
    # reference's rows, so only their finiteness is asserted here.
    if obj_bc == "floating":
        for d in range(3):
            assert np.all(np.isfinite(du[1 + d]))
