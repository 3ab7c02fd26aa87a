"""Host setup of the product library against the oracle: cut points, line blocks,
closure sparsity (B, N, Bf, Br) and coefficients must be bit-identical (no GPU needed)."""
import numpy as np
import pytest

import shoccs_gb300 as S
from oracle.oracle import OracleProblem
from tests.cases import cases

CASES = cases()


@pytest.mark.parametrize("name", sorted(CASES))
def test_setup_bit_exact(name):
    c = CASES[name]
    p = S.Problem(**c)
    o = OracleProblem(**c)
    assert p.size == o.size
    assert p.nR == o.nR
    assert p.n_fluid == len(o.fluid())
    for d in range(3):
        a, b = p.cut_points(d), o.cut_points(d)
        for k in a:
            assert np.array_equal(a[k], b[k]), (d, k)
        ma, ca = p.block_meta(d)
        mb, cb = o.block_meta(d)
        assert np.array_equal(ma, mb), d
        assert np.array_equal(ca.view(np.int64), cb.view(np.int64)), d
        for w in range(8):
            ra, rb = p.csr(d, w), o.csr(d, w)
            assert ra[0] == rb[0], (d, w)
            assert np.array_equal(ra[1], rb[1]), (d, w)
            assert np.array_equal(ra[2], rb[2]), (d, w)
            assert np.array_equal(ra[3].view(np.int64), rb[3].view(np.int64)), (d, w)


def test_config0_cut_point_counts():
    # |Rx| = |Ry| = 52 for the 65x65 circle of the 2-D heat configuration
    p = S.Problem(**CASES["c0_circle_2d"])
    assert p.nR == (52, 52, 0)


def test_classes_cover_every_row():
    """Every reference row gets exactly one class per axis; fluid points off Dirichlet faces
    have a row along every active axis."""
    for name in ("wave_sphere_3d", "multi_sphere_e42", "c0_circle_2d"):
        c = CASES[name]
        p = S.Problem(**c)
        cls = p.classes()
        for d in range(3):
            meta, _ = p.block_meta(d)
            kinds = (cls >> (2 * d)) & 3
            n_rows = int(meta[:, 3].sum() + meta[:, 6].sum() + meta[:, 9].sum()) if len(meta) else 0
            assert int((kinds > 0).sum()) == n_rows
            assert int((kinds == 1).sum()) == int(meta[:, 6].sum()) if len(meta) else True
        fluid = (cls & 0x80) != 0
        dirface = (cls & 0x40) != 0
        act = [d for d in range(3) if p.n[d] > 1]
        for d in act:
            kinds = (cls >> (2 * d)) & 3
            assert np.all(kinds[fluid & ~dirface] > 0)
            assert np.all(kinds[~fluid] == 0)


def test_overlapping_closures_rejected():
    # a 6-point gap between a wall and a sphere is shorter than two E4_1 closures
    with pytest.raises(S.ShoccsError, match="overlap"):
        S.Problem(n=(30, 28, 26), lo=(0, 0, 0), hi=(1, 1, 1),
                  spheres=[((0.5, 0.5, 0.5), 0.3, "dirichlet")],
                  grid_bc=("dirichlet", "floating") * 3, scheme="E4_1", alpha=(0.1, 0.7))


@pytest.mark.parametrize("name", sorted(n for n, c in CASES.items() if c["n"][2] > 1))
def test_points_with_rows_have_a_row_on_every_axis(name):
    """The vectorised stage kernel evaluates the interior row at every point and lets only
    cut-cell and wall rows replace it: a point without a row along some axis must be a solid
    point (no row at all: right-hand side 0) or a Dirichlet face point (value replaced).  The
    host checks this before it offers that kernel; the cases here all satisfy it."""
    p = S.Problem(**CASES[name])
    cls = p.classes()
    used = ((cls & 0x3F) != 0) & ((cls & 0x40) == 0)
    for d in range(3):
        assert not np.any(used & (((cls >> (2 * d)) & 3) == 0)), (name, d)
