"""The allocation-free statistics entry point (shoccs_system_stats_noalloc).

Some callers cannot allocate device memory while they call in -- an application that has
handed the whole device memory to its own pool allocator, or a time loop that must never
block in the CUDA allocator between steps.  For them the library offers a statistics call
whose scratch lives in a fixed array inside the library's device image.  This test calls
it through the C ABI and checks it against the allocating shoccs_system_stats, twice in a
row (the array is shared and keeps the previous call's contents), and checks that grids
beyond its fixed capacity are refused.  It is collected last so that a failure here leaves
every other test already run.
"""
import ctypes

import numpy as np
import pytest

import shoccs_gb300 as S
from shoccs_gb300 import _capi

CASE = dict(n=(34, 30, 36), lo=(0, 0, 0), hi=(1, 1, 1),
            spheres=[((0.5, 0.48, 0.52), 0.18, "dirichlet")],
            grid_bc=("dirichlet", "floating") * 3, scheme="E4_2")


def _stats(fn, sys_, t):
    out = (ctypes.c_double * 11)()
    st = fn(sys_.handle, ctypes.c_double(t), out, None)
    return st, np.array(out[:])


@pytest.mark.gpu
@pytest.mark.parametrize("prec", [S.PREC_FP64, S.PREC_MIXED])
def test_noalloc_stats_match_allocating_entry_point(prec):
    lib = _capi.lib()
    p = S.Problem(**CASE)
    h = S.Heat(p, 1.0, prec, S.SOL_SINSIN, [1.0])
    h.initialize(0.0)
    dt = 0.4 * (1.0 / 33) ** 2 / 4
    t = 0.0
    for _ in range(2):  # two calls in a row, the second after more time steps
        h.rk4(t, dt, 7)
        t += 7 * dt
        st_ref, ref = _stats(lib.shoccs_system_stats, h, t)
        st_new, new = _stats(lib.shoccs_system_stats_noalloc, h, t)
        assert st_ref == _capi.OK and st_new == _capi.OK
        assert ref[0] > 0
        np.testing.assert_allclose(new, ref, rtol=1e-12, atol=0)


@pytest.mark.gpu
def test_noalloc_stats_rejects_grids_beyond_its_scratch():
    lib = _capi.lib()
    p = S.Problem((257, 256, 256), (0, 0, 0), (1, 1, 1),
                  grid_bc=("dirichlet", "floating") * 3, scheme="E4_2")
    h = S.Heat(p, 1.0, S.PREC_FP64, S.SOL_SINSIN, [1.0])
    st, _ = _stats(lib.shoccs_system_stats_noalloc, h, 0.0)
    assert st == _capi.EINVAL
    buf = ctypes.create_string_buffer(256)
    lib.shoccs_last_error(buf, 256)
    assert b"at most 65536" in buf.value
