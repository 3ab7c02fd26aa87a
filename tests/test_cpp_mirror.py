"""The C++ classes of include/shoccs_gb300.hpp (ccs::derivative, laplacian, gradient,
systems::heat, integrators::rk4 ... with the reference's names and call shapes) over the C ABI.

CPU: the header compiles on its own, its enums map onto the C ABI's, and make_E4_1 rejects
alpha[1] < 197/288 with std::invalid_argument as src/stencils/E4_1.cpp:37-40 does.
GPU: tests/cpp/mirror_ops.cpp runs the 2-D heat case (65^2, circle, E4_2) and the three
operators through the classes; every array must equal, bit for bit, what the Python binding
gets from the same library on the same inputs, and the FP64 Laplacian must agree with the
oracle to 1e-12; simulation_cycle runs the case for 100 steps and writes the system log.
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
    assert stats["floating_object"] == ["status", "6"]  # SHOCCS_EUNSUPPORTED
