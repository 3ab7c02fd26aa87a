"""The C++ classes of include/shoccs_gb300.hpp (ccs::derivative, laplacian, gradient,
systems::heat, integrators::rk4 ... with the reference's names and call shapes) over the C ABI.

CPU: the header compiles on its own, its enums map onto the C ABI's, and make_E4_1 rejects
alpha[1] < 197/288 with std::invalid_argument as src/stencils/E4_1.cpp:37-40 does.
GPU: tests/cpp/mirror_ops.cpp runs the 2-D heat case (65^2, circle, E4_2) and the three
operators through the classes; every array must equal, bit for bit, what the Python binding
gets from the same library on the same inputs, and the FP64 Laplacian must agree with the
oracle to 1e-12; simulation_cycle runs the case for 100 steps and writes the system log, and two cycles write
their fields through ccs::field_io (every 40 steps; every 3 dt of simulation time around a
Floating sphere): the U files must hold the Python binding's states at the dump steps, the
Error files the oracle's write_scalar_error of them, rx/ry/rz the cut-point positions.
"""
import os
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")
CASE = dict(n=(65, 65, 1), lo=(0, 0, 0), hi=(1, 1, 0),
            spheres=[((0.51, 0.49, 0.0), 0.2, "dirichlet")],
            grid_bc=("dirichlet",) * 4 + ("floating",) * 2, scheme="E4_2")


def _gxx(args, cwd):
    r = subprocess.run(["g++", "-std=c++20", "-O2", "-Wall", "-Wextra", "-I" + os.path.join(ROOT, "include"),
                        "-I" + os.path.join(CUDA, "include")] + args, cwd=cwd, capture_output=True,
                       text=True)
    assert r.returncode == 0, r.stderr[-3000:]


def test_header_compiles_and_maps_the_c_abi(tmp_path):
    src = tmp_path / "t.cpp"
    src.write_text(r'''
#include "shoccs_gb300.hpp"
static_assert(ccs::bcs::to_c(ccs::bcs::Dirichlet) == SHOCCS_BC_DIRICHLET);
static_assert(ccs::bcs::to_c(ccs::bcs::Floating) == SHOCCS_BC_FLOATING);
static_assert(ccs::bcs::to_c(ccs::bcs::Neumann) == SHOCCS_BC_NEUMANN);
static_assert((int)ccs::precision::mixed == SHOCCS_PREC_MIXED);
int main()
{
    const double ok[2] = {0.1, 0.7}, bad[2] = {0.1, 0.5};
    if (ccs::stencils::make_E4_1(ok).scheme != SHOCCS_SCHEME_E4_1) return 1;
    try {
        (void)ccs::stencils::make_E4_1(bad);
        return 2;
    } catch (const std::invalid_argument&) {
    }
    ccs::mesh m{ccs::index_extents{{5, 6, 7}}, ccs::domain_extents{{0, 0, 0}, {1, 1, 1}}};
    return m.size() == 210 && m.ic({1, 2, 3}) == 1 * 42 + 2 * 7 + 3 ? 0 : 3;
}
''')
    _gxx([str(src), "-o", str(tmp_path / "t")], str(tmp_path))
    assert subprocess.run([str(tmp_path / "t")]).returncode == 0


def _build_mirror(tmp_path):
    from shoccs_gb300 import _capi
    lib_dir = os.path.dirname(_capi.LIB_PATH)
    if not os.path.exists(_capi.LIB_PATH):
        pytest.fail("library not built: " + _capi.LIB_PATH)
    exe = tmp_path / "mirror_ops"
    _gxx([os.path.join(HERE, "cpp", "mirror_ops.cpp"), "-o", str(exe), "-L" + lib_dir,
          "-lshoccs_gb300", "-L" + os.path.join(CUDA, "lib64"), "-lcudart",
          "-Wl,-rpath," + lib_dir], str(tmp_path))
    return exe


@pytest.mark.gpu
def test_cpp_classes_match_the_python_binding(tmp_path):
    import torch
    import shoccs_gb300 as S
    from oracle.oracle import OracleProblem

    exe = _build_mirror(tmp_path)
    p = S.Problem(**CASE)
    sizes = [p.size] + list(p.nR)
    rng = np.random.default_rng(20261208)
    u = [rng.uniform(-1, 1, n) for n in sizes]
    np.concatenate(u).tofile(str(tmp_path / "u.f64"))
    r = subprocess.run([str(exe), str(tmp_path)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr

    def load(name, dtype=np.float64):
        a = np.fromfile(str(tmp_path / name), dtype=dtype)
        return np.split(a, np.cumsum(sizes)[:-1])

    dev = lambda arrs, dt=torch.float64: S.ScalarField(*[torch.tensor(a, dtype=dt, device="cuda") for a in arrs])
    host = lambda f: [t.cpu().numpy() for t in f]
    U = dev(u)
    # derivative along x, eq then plus_eq on the same output
    du = p.zeros()
    S.Derivative(p, 0)(U, du)
    for a, b in zip(load("dx.f64"), host(du)):
        assert np.array_equal(a, b)
    S.Derivative(p, 0)(U, du, plus_eq=True)
    for a, b in zip(load("dx_plus.f64"), host(du)):
        assert np.array_equal(a, b)
    # Laplacian, FP64 and mixed; gradient
    lap = S.Laplacian(p)(U, p.zeros())
    got_lap = load("lap.f64")
    for a, b in zip(got_lap, host(lap)):
        assert np.array_equal(a, b)
    want = OracleProblem(**CASE).laplacian(u, OracleProblem(**CASE).zeros())
    scale = max(np.abs(want[0]).max(), 1e-300)
    assert np.abs(got_lap[0] - want[0]).max() / scale <= 1e-12
    uf = dev([a.astype(np.float32) for a in u], torch.float32)
    lapf = S.Laplacian(p, S.PREC_MIXED)(uf, p.zeros(torch.float32))
    for a, b in zip(load("lap_mixed.f32", np.float32), host(lapf)):
        assert np.array_equal(a, b)
    g = S.Gradient(p)(U, p.zeros(), p.zeros(), p.zeros())
    for name, comp in (("gx.f64", g[0]), ("gy.f64", g[1])):
        for a, b in zip(load(name), host(comp)):
            assert np.array_equal(a, b)

    # heat, 100 RK4 steps, FP64 and mixed: the same state as the Python path
    stats = {}
    for line in (tmp_path / "stats.txt").read_text().splitlines():
        k, *rest = line.split()
        stats[k] = rest
    for key, prec in (("fp64", S.PREC_FP64), ("mixed", S.PREC_MIXED)):
        h = S.Heat(p, 1.0, prec, S.SOL_SINSIN, [1.0])
        h.initialize(0.0)
        dt = float(stats[key][5])
        h.rk4(0.0, dt, 100)
        st = [np.zeros(n) for n in sizes]
        h.get_state(S.ScalarField(*st))
        for a, b in zip(load("heat_%s.f64" % key), st):
            assert np.array_equal(a, b)
        assert stats[key][3] == "1"  # system::valid
    e64, e32 = float(stats["fp64"][1]), float(stats["mixed"][1])
    assert e64 < 1e-3 and e32 <= 1.1 * e64
    # one rk4 call per step gives the error of the fused multi-step call
    assert abs(float(stats["stepwise"][1]) - e64) <= 1e-12 * e64
    # simulation_cycle: 100 steps, one log line per step plus the initial one, each
    # timestamp,time,step,11 statistics,wall ms; the run ends in a valid state with the error
    # of 100 steps
    t_end, e_cycle, nstep = float(stats["cycle"][0]), float(stats["cycle"][1]), int(stats["cycle"][2])
    assert nstep == 100 and abs(e_cycle - e64) <= 1e-12 * e64
    assert abs(t_end - 100 * float(stats["fp64"][5])) <= 1e-12
    lines = (tmp_path / "system.csv").read_text().splitlines()
    assert len(lines) == 101
    for k, line in enumerate(lines):
        f = line.split(",")
        assert len(f) == 15 and int(f[2]) == k
    assert abs(float(lines[-1].split(",")[3]) - e_cycle) <= 1e-15 * e_cycle
    assert stats["e4_1_bound"] == ["invalid_argument"]
    # a mixed system with a Floating object steps by RK4; forward Euler refuses it
    assert stats["floating_object"] == ["status", "6"]  # SHOCCS_EUNSUPPORTED

    # the field writer of both simulation cycles (ccs::field_io through system::write)
    _check_cycle_io(tmp_path, p, float(stats["fp64"][5]), stats)


def _check_cycle_io(tmp_path, p, dt2, stats):
    import xml.etree.ElementTree as ET
    import shoccs_gb300 as S
    from oracle.oracle import OracleProblem
    from tests.test_field_io import _d_interval_dumps

    def times(steps, dt):
        t, out = 0.0, []
        for s in range(max(steps) + 1):
            if s in steps:
                out.append(t)
            t += dt
        return out

    def check_run(case, io, steps, dt, suffix, xmf, make, swap):
        q = S.Problem(**case)
        o = OracleProblem(**case)
        sizes = [q.size] + list(q.nR)
        root = ET.parse(str(io / xmf)).getroot()
        dom = root.find("Domain")
        grids = [g for g in dom.findall("Grid") if g.get("Name") == "TimeSeries"][0].findall("Grid")
        assert [g.get("Name") for g in grids] == [str(k) for k in range(len(steps))]
        assert [float(g.find("Time").get("Value")) for g in grids] == times(steps, dt)
        assert [t.get("NumberOfElements") for t in dom.findall("Topology")[1:]] == [str(k) for k in q.nR]
        for d, name in enumerate(("rx", "ry", "rz")):
            pos = np.fromfile(str(io / name)).reshape(-1, 3)
            want = q.cut_points(d)["position"]
            assert np.array_equal(pos, want[:, ::-1] if swap else want)
        for k, (s, t) in enumerate(zip(steps, times(steps, dt))):
            u = np.split(np.fromfile(str(io / ("U.%0*d" % (suffix, k)))), np.cumsum(sizes)[:-1])
            e = np.split(np.fromfile(str(io / ("Error.%0*d" % (suffix, k)))), np.cumsum(sizes)[:-1])
            h = make(q)
            h.initialize(0.0)
            if s:
                h.rk4(0.0, dt, s)
            ref = [np.zeros(m) for m in sizes]
            h.get_state(S.ScalarField(*ref))
            scale = max(np.abs(a).max() for a in ref if a.size)
            for a, b in zip(u, ref):
                assert np.abs(a - b).max(initial=0.0) <= 1e-12 * scale, (k, s)
            want = o.error_field(S.SOL_SINSIN, [1.0], t, u)
            for a, b in zip(e, want):
                assert np.array_equal(a == 0, b == 0)
                assert np.abs(a - b).max(initial=0.0) <= 1e-14 * scale
        return e

    # 2-D heat cycle: a dump every 40 steps of 100
    steps2 = [0, 40, 80]
    assert stats["io2d_dumps"] == [str(len(steps2))]
    check_run(CASE, tmp_path / "io2d", steps2, dt2, 6, "view.xmf",
              lambda q: S.Heat(q, 1.0, S.PREC_FP64, S.SOL_SINSIN, [1.0]), True)
    # 3-D Floating sphere: a dump every 3 dt of simulation time over 10 steps
    err3, nstep3, ndump3, dt3 = stats["io3d"]
    dt3 = float(dt3)
    steps3 = _d_interval_dumps(3 * dt3, dt3, 10)
    assert int(nstep3) == 10 and int(ndump3) == len(steps3)
    case3 = dict(n=(24, 24, 24), lo=(0, 0, 0), hi=(1, 1, 1), spheres=[((0.5, 0.5, 0.5), 0.25, "floating")],
                 grid_bc=("dirichlet",) * 6, scheme="E4_2")
    e = check_run(case3, tmp_path / "io3d", steps3, dt3, 4, "floating.xmf",
                  lambda q: S.Heat(q, 1.0, S.PREC_FP64, S.SOL_SINSIN, [1.0]), False)
    assert all(np.abs(r).max() > 0 for r in e[1:])  # Floating cut points evolve
