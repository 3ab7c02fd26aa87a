"""The field writer of include/shoccs_gb300.hpp (ccs::interval, d_interval, xdmf, field_data,
field_io), on the host: tests/cpp/field_io_host.cpp runs the cases of the reference's
src/io/interval.t.cpp, field_io.t.cpp and xdmf.t.cpp and a time schedule with cut points.

The binary files must hold exactly the bytes field_data::write / write_geom give
(src/io/field_data.cpp:8-57): D (nx*ny*nz doubles), then the nonempty Rx, Ry, Rz; positions as
3 doubles per cut point, (z, y, x) when nz == 1.  The XDMF index is checked by structure
(src/io/xdmf.cpp:20-179: the outline, one spatial grid per dump with the grid F and the
nonempty cut-point grids, Seek offsets where the cut-point parts follow D); the reference
saves it through pugixml, which is not available here, so the byte layout is not compared.
"""
import os
import subprocess
import xml.etree.ElementTree as ET

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")


@pytest.fixture(scope="module")
def run(tmp_path_factory):
    tmp_path = tmp_path_factory.mktemp("field_io")
    exe = tmp_path / "field_io_host"
    r = subprocess.run(["g++", "-std=c++20", "-O2", "-Wall", "-Wextra", "-I" + os.path.join(ROOT, "include"),
                        "-I" + os.path.join(CUDA, "include"), os.path.join(HERE, "cpp", "field_io_host.cpp"),
                        "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    r = subprocess.run([str(exe), str(tmp_path)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    out = {}
    for line in r.stdout.splitlines():
        k, *v = line.split()
        out[k] = v
    return tmp_path, out


def _grids(path):
    root = ET.parse(path).getroot()
    dom = root.find("Domain")
    series = [g for g in dom.findall("Grid") if g.get("Name") == "TimeSeries"]
    assert len(series) == 1 and series[0].get("CollectionType") == "Temporal"
    return root, dom, series[0].findall("Grid")


def _d_interval_dumps(every_time, dt, steps):
    """d_interval (src/io/interval.hpp:56-97) with a time interval only, restated: fires at step
    0 and when t - first >= every - dt; each firing moves first on by one interval"""
    first, t, fired = 0.0, 0.0, []
    for s in range(steps + 1):
        tol = 0.0 if s == 0 else dt
        ready = t - first >= every_time - tol
        if ready or s == 0:
            fired.append(s)
            if ready:
                first += every_time
        t += dt
    return fired


def test_interval_and_field_io_cases(run):
    tmp_path, out = run
    assert out["never_fire"] == ["1"]
    assert out["no_rollover"] == ["1"]
    assert out["rollover"] == ["1", "10"]
    assert out["default_writes"] == ["0"]
    assert out["data_writes"] == ["1", "1"]
    io = tmp_path / "io_test"
    u = np.fromfile(str(io / "U.000000"))
    v = np.fromfile(str(io / "V.000000"))
    assert np.array_equal(u, np.arange(24.0)) and np.array_equal(v, np.arange(24.0, 48.0))
    for r in ("rx", "ry", "rz"):
        assert (io / r).stat().st_size == 0
    _, dom, grids = _grids(str(io / "view.xmf"))
    assert dom.find("Topology").get("Dimensions") == "2 3 4"
    assert len(grids) == 1 and grids[0].get("Name") == "0"


def test_xdmf_outline_and_grids(run):
    tmp_path, _ = run
    root, dom, grids = _grids(str(tmp_path / "headertest.xmf"))
    assert root.tag == "Xdmf" and root.get("Version") == "3.0"
    topo = dom.findall("Topology")
    geom = dom.findall("Geometry")
    assert [t.get("TopologyType") for t in topo] == ["3DCoRectMesh"] + ["Polyvertex"] * 3
    assert topo[0].get("Dimensions") == "3 4 5"
    assert [t.get("NumberOfElements") for t in topo[1:]] == ["0", "0", "0"]
    origin, dxyz = [np.array(d.text.split(), dtype=float) for d in geom[0].findall("DataItem")]
    assert np.array_equal(origin, [0.1, 0.2, 0.3])
    ext = np.array([3, 4, 5.0])
    assert np.array_equal(dxyz, (np.array([1.1, 1.2, 1.3]) - np.array([0.1, 0.2, 0.3])) / (ext - 1))
    assert [g.find("DataItem").text for g in geom[1:]] == ["rx", "ry", "rz"]
    assert [g.get("Name") for g in grids] == ["0", "1"]
    for k, g in enumerate(grids):
        assert g.get("CollectionType") == "Spatial"
        assert float(g.find("Time").get("Value")) == [0.0, 0.1][k]
        sub = g.findall("Grid")
        assert [s.get("Name") for s in sub] == ["F"]  # no cut points: no RX / RY / RZ grid
        f = sub[0]
        assert f.find("Topology").get("Reference") == "/Xdmf/Domain/Topology[1]"
        assert f.find("Geometry").get("Reference") == "/Xdmf/Domain/Geometry[1]"
        attrs = f.findall("Attribute")
        assert [a.get("Name") for a in attrs] == ["U", "V"]
        for a, name in zip(attrs, ("U", "V")):
            item = a.find("DataItem")
            assert item.text == "%s.%05d" % (name, k)
            assert item.get("Dimensions") == "3 4 5" and item.get("Precision") == "8"
            assert item.get("Format") == "Binary" and item.get("Seek") is None


def test_time_schedule_and_cut_point_geometry(run):
    tmp_path, out = run
    want = _d_interval_dumps(0.25, 0.1, 10)
    assert [int(s) for s in out["time_dumps"]] == want
    io = tmp_path / "io_time"
    # positions: nz == 1, so (z, y, x) per point; an axis without cut points: empty file
    rx = np.fromfile(str(io / "rx")).reshape(-1, 3)
    assert np.array_equal(rx, [[0.0, 0.2, 0.1], [0.0, 0.4, 0.3], [0.0, 0.6, 0.5]])
    assert (io / "ry").stat().st_size == 0
    assert np.array_equal(np.fromfile(str(io / "rz")), [0.0, 0.8, 0.7])
    _, dom, grids = _grids(str(io / "t.xmf"))
    assert [t.get("NumberOfElements") for t in dom.findall("Topology")[1:]] == ["3", "0", "1"]
    assert len(grids) == len(want)
    for k, s in enumerate(want):
        data = np.fromfile(str(io / ("U.%03d" % k)))
        assert np.array_equal(data[:20], 100.0 * s + np.arange(20))
        assert np.array_equal(data[20:23], -(100.0 * s + np.arange(3)))
        assert np.array_equal(data[23:], [0.5 + s])
        g = grids[k]
        assert g.get("Name") == str(k)
        t = 0.0
        for _ in range(s):  # step_controller::advance: t += dt (sum() would compensate)
            t += 0.1
        assert float(g.find("Time").get("Value")) == t
        sub = g.findall("Grid")
        assert [x.get("Name") for x in sub] == ["F", "RX", "RZ"]
        seeks = [x.find("Attribute/DataItem").get("Seek") for x in sub]
        assert seeks == [None, str(20 * 8), str(23 * 8)]
        assert [x.find("Attribute/DataItem").get("Dimensions") for x in sub] == ["5 4 1", "3 1", "1 1"]
        assert [x.find("Topology").get("Reference") for x in sub] == [
            "/Xdmf/Domain/Topology[%d]" % i for i in (1, 2, 4)]
