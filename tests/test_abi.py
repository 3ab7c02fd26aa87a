"""The C-ABI library loads without a GPU, exports every symbol include/shoccs_gpu.h
declares, and rejects bad configurations on the host with the reference's error meaning."""
import ctypes
import os
import re

import pytest

import shoccs_gb300 as S
from shoccs_gb300 import _capi

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    src = open(os.path.join(REPO, "include", "shoccs_gpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(shoccs_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol():
    lib = ctypes.CDLL(_capi.LIB_PATH)
    names = header_functions()
    assert len(names) >= 20
    for n in names:
        assert hasattr(lib, n), n
    assert set(names) == set(_capi.SIGNATURES), "binding and header disagree"


def test_bad_configurations_are_rejected():
    with pytest.raises(S.ShoccsError, match="alpha"):
        S.Problem((16, 16, 16), (0, 0, 0), (1, 1, 1), scheme="E4_1", alpha=(0.1, 0.5))
    with pytest.raises(S.ShoccsError, match="EINVAL"):
        S.Problem((16, 0, 16), (0, 0, 0), (1, 1, 1))
    with pytest.raises(S.ShoccsError, match="Dirichlet"):
        S.Problem((40, 40, 40), (0, 0, 0), (1, 1, 1), spheres=[((0.5, 0.5, 0.5), 0.2, "floating")],
                  scheme="E4_1", alpha=(0.1, 0.7))
    with pytest.raises(S.ShoccsError, match="radius"):
        S.Problem((16, 16, 16), (0, 0, 0), (1, 1, 1), spheres=[((0.5, 0.5, 0.5), 0.0, "dirichlet")])


def test_last_error_message():
    lib = _capi.lib()
    st = lib.shoccs_problem_create(None, None)
    assert st == _capi.EINVAL
    buf = ctypes.create_string_buffer(128)
    n = lib.shoccs_last_error(buf, 128)
    assert n > 0 and b"null" in buf.value
