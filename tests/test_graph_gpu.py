"""Graph forms of the reference's API (derivative / laplacian / gradient add_graph_nodes,
build_graph, submit_graph; system build_rhs_graph / submit_rhs_graph) over captured CUDA
graphs, against the eager applies: equal bit for bit, the pattern of the reference's
"graph matches eager" tests (src/operators/derivative.t.cpp:423-513).

CPU: the C++ test program (tests/cpp/graph_ops.cpp) compiles against include/ and links
against the library.  GPU: it runs and every check holds (FP64 and vectorised FP32
operators on a 3-D Dirichlet sphere with Neumann faces, a Floating sphere's R-space rows,
the 2-D heat configuration; resubmits, plus_eq accumulation, a composite graph, right-hand
sides at changing times and states); and the Python binding's Graph gives the eager bits.
"""
import os
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")


def _build(tmp_path):
    from shoccs_gb300 import _capi
    lib_dir = os.path.dirname(_capi.LIB_PATH)
    if not os.path.exists(_capi.LIB_PATH):
        pytest.fail("library not built: " + _capi.LIB_PATH)
    exe = tmp_path / "graph_ops"
    r = subprocess.run(["g++", "-std=c++20", "-O2", "-Wall", "-Wextra",
                        "-I" + os.path.join(ROOT, "include"), "-I" + os.path.join(CUDA, "include"),
                        os.path.join(HERE, "cpp", "graph_ops.cpp"), "-o", str(exe), "-L" + lib_dir,
                        "-lshoccs_gb300", "-L" + os.path.join(CUDA, "lib64"), "-lcudart",
                        "-Wl,-rpath," + lib_dir], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    return exe


def test_graph_program_builds(tmp_path):
    _build(tmp_path)


@pytest.mark.gpu
def test_graphs_equal_eager_cpp(tmp_path):
    exe = _build(tmp_path)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    print(r.stdout)
    assert r.returncode == 0, r.stdout[-4000:] + r.stderr[-2000:]
    assert "0 failure(s)" in r.stdout


@pytest.mark.gpu
def test_graphs_equal_eager_python():
    import torch
    import shoccs_gb300 as S
    from tests.cases import cases

    c = cases()["micro_e42_96"]
    p = S.Problem(**c)
    rng = np.random.default_rng(5)
    for prec, dt in ((S.PREC_FP64, torch.float64), (S.PREC_MIXED, torch.float32)):
        u = S.ScalarField(*[torch.tensor(rng.uniform(-1, 1, n), dtype=dt, device="cuda")
                            for n in [p.size] + list(p.nR)])
        e1, e2, g1, g2 = (p.zeros(dt) for _ in range(4))
        S.Derivative(p, 1, prec)(u, e1)
        S.Laplacian(p, prec)(u, e2)
        g = S.Graph().add_derivative(p, 1, u, g1, prec=prec).add_laplacian(p, u, g2, prec=prec)
        g.submit()
        for a, b in ((e1, g1), (e2, g2)):
            for x, y in zip(a, b):
                assert torch.equal(x, y)
        assert g.info()[0] == 2 and g.info()[2] == 1
        g.submit()
        assert g.info()[2] == 1  # replayed, not captured again
