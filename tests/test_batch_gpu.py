"""Batched heat solves (shoccs_batch_*): independent 2-D heat instances of different grid
sizes and circle geometries advanced together under one captured CUDA graph.

The batch runs the single-system stage arithmetic with the same time points and boundary
products, so every instance must come out bit-identical to shoccs_system_rk4 run on that
instance alone -- in FP64 and in the mixed path, through the split 2-D stage (uniform tiles
and special points; the default), the same in one persistent launch for the whole solve
(SHOCCS_BATCH_PERSIST=1), the flat 2-D stage (SHOCCS_BATCH_KERNEL=flat) and the per-point
stage (SHOCCS_BATCH_KERNEL=point) with every tile shape, and across graph replays.  The instances are drawn by the batched configuration's own generator
(shoccs_gb300.workloads.batch_heat_2d) with smaller grids.
"""
import numpy as np
import pytest

import shoccs_gb300 as S
from shoccs_gb300 import workloads as W


def _instances(count=6, nmax=72):
    return W.batch_heat_2d(count=count, nmin=32, nmax=nmax)


def _make(insts, prec):
    probs = [S.Problem(**it["case"]) for it in insts]
    systems = [S.Heat(p, 1.0, prec, S.SOL_SINSIN, [float(it["k"])]) for p, it in zip(probs, insts)]
    for s in systems:
        s.initialize(0.0)
    return probs, systems


def _state(sys_, p):
    u = [np.zeros(p.size)] + [np.zeros(k) for k in p.nR]
    sys_.get_state(S.ScalarField(*u))
    return u


@pytest.mark.gpu
@pytest.mark.parametrize("kernel", ["split", "persist", "flat", "point"])
@pytest.mark.parametrize("prec", [S.PREC_FP64, S.PREC_MIXED])
def test_batch_matches_single_systems_bitwise(prec, kernel, monkeypatch):
    monkeypatch.setenv("SHOCCS_BATCH_KERNEL", "split" if kernel == "persist" else kernel)
    monkeypatch.setenv("SHOCCS_BATCH_PERSIST", "1" if kernel == "persist" else "0")
    insts = _instances()
    pb, sb = _make(insts, prec)
    ps, ss = _make(insts, prec)
    batch = S.Batch(sb)
    dts = [it["dt"] for it in insts]
    steps = 23
    batch.rk4(0.0, dts, steps)
    for s, dt in zip(ss, dts):
        s.rk4(0.0, dt, steps)
    for i in range(len(insts)):
        ub, us = _state(sb[i], pb[i]), _state(ss[i], ps[i])
        for a, b in zip(ub, us):
            assert np.array_equal(a, b), i
    info = batch.info()
    assert info["instances"] == len(insts) and info["graph_nodes"] > 0
    if kernel == "persist":  # the whole solve is one launch
        assert info["graph_nodes"] == 1 and info["grid"] % 8 == 0


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["one_group", "groups", "persist"])
@pytest.mark.parametrize("prec", [S.PREC_FP64, S.PREC_MIXED])
def test_split_batch_many_instances(prec, mode, monkeypatch):
    """96 instances: the split stage over the whole batch at once, over groups of a few
    instances each advanced through all its steps in turn (a 0.2 MB group budget), and the
    persistent launch whose clusters each own several instances of unequal work, give every
    instance its single-system solve bit for bit."""
    monkeypatch.setenv("SHOCCS_BATCH_KERNEL", "split")
    monkeypatch.setenv("SHOCCS_BATCH_PERSIST", "1" if mode == "persist" else "0")
    monkeypatch.setenv("SHOCCS_BATCH_GROUP_MB", "0.2" if mode == "groups" else "0")
    insts = W.batch_heat_2d(count=96, nmin=32, nmax=56)
    pb, sb = _make(insts, prec)
    ps, ss = _make(insts, prec)
    batch = S.Batch(sb)
    dts = [it["dt"] for it in insts]
    batch.rk4(0.0, dts, 9)
    info = batch.info()
    if mode == "persist":
        assert info["graph_nodes"] == 1 and info["grid"] // 8 < len(insts)
    if mode == "groups":  # two kernels per stage, and the groups one after another
        assert info["graph_nodes"] > 2 * 4 * 9 * 4
    for s, dt in zip(ss, dts):
        s.rk4(0.0, dt, 9)
    for i in range(len(insts)):
        for a, b in zip(_state(sb[i], pb[i]), _state(ss[i], ps[i])):
            assert np.array_equal(a, b), i


@pytest.mark.gpu
def test_batch_graph_replay_continues_the_solve():
    insts = _instances(count=4)
    pb, sb = _make(insts, S.PREC_MIXED)
    ps, ss = _make(insts, S.PREC_MIXED)
    batch = S.Batch(sb)
    dts = [it["dt"] for it in insts]
    batch.rk4(0.0, dts, 10)
    batch.rk4([10 * d for d in dts], dts, 10)  # same length: the captured graph is replayed
    for s, dt in zip(ss, dts):
        s.rk4(0.0, dt, 10)
        s.rk4(10 * dt, dt, 10)
    for i in range(len(insts)):
        for a, b in zip(_state(sb[i], pb[i]), _state(ss[i], ps[i])):
            assert np.array_equal(a, b), i


@pytest.mark.gpu
@pytest.mark.parametrize("warps", [1, 2, 4, 8])
def test_batch_tile_shapes_agree(warps, monkeypatch):
    insts = _instances(count=3, nmax=64)
    monkeypatch.setenv("SHOCCS_BATCH_KERNEL", "point")  # tile shapes belong to the per-point stage
    monkeypatch.setenv("SHOCCS_BATCH_TILE_WARPS", str(warps))
    pb, sb = _make(insts, S.PREC_MIXED)
    batch = S.Batch(sb)
    assert batch.info()["tile_warps"] == warps
    batch.rk4(0.0, [it["dt"] for it in insts], 7)
    monkeypatch.delenv("SHOCCS_BATCH_TILE_WARPS")
    monkeypatch.delenv("SHOCCS_BATCH_KERNEL")
    ps, ss = _make(insts, S.PREC_MIXED)
    for s, it in zip(ss, insts):
        s.rk4(0.0, it["dt"], 7)
    for i in range(len(insts)):
        for a, b in zip(_state(sb[i], pb[i]), _state(ss[i], ps[i])):
            assert np.array_equal(a, b), (warps, i)


@pytest.mark.gpu
def test_batch_manufactured_solution_error():
    """200 steps at dt = 0.1 h^2 (the batched configuration's step count): every instance of
    the mixed batch reaches the manufactured-solution error of the FP64 batch within 1.1x
    (the equal-accuracy criterion), and the errors are those of a converging scheme."""
    insts = _instances(count=4, nmax=96)
    dts = [it["dt"] for it in insts]
    err = {}
    for prec in (S.PREC_FP64, S.PREC_MIXED):
        pb, sb = _make(insts, prec)
        batch = S.Batch(sb)
        batch.rk4(0.0, dts, 200)
        err[prec] = []
        for s, dt in zip(sb, dts):
            st, ok = s.stats(200 * dt)
            assert ok
            err[prec].append(st[0])
    for e64, e32, it in zip(err[S.PREC_FP64], err[S.PREC_MIXED], insts):
        assert e32 <= 1.1 * e64, (e64, e32, it["case"]["n"], it["k"])
        assert e64 < 0.05, (e64, it["case"]["n"], it["k"])


@pytest.mark.gpu
def test_batch_rejects_unsupported_systems():
    it = _instances(count=1)[0]
    p = S.Problem(**it["case"])
    h = S.Heat(p, 1.0, S.PREC_MIXED, S.SOL_SINSIN, [1.0])
    with pytest.raises(S.ShoccsError):
        S.Batch([h, h])  # the same system twice
    with pytest.raises(S.ShoccsError):
        S.Batch([S.Heat(p, 1.0, S.PREC_MIXED, S.SOL_ZERO)])  # not the sin-sin solution
