"""Size-independent properties at the benchmark workloads' full sizes (the oracle checks the
same kernels on smaller grids; these run every path the benchmark times on its own grid).

* 256^3 wave (sphere r = 0.3, E4_1, constant velocity): with zero boundary data the RK4 step
  is linear and homogeneous, and scaling by 2 is exact in binary floating point, so
  rk4(2u) == 2 rk4(u) bit for bit, in FP64 and in the mixed path (FP32 stencils, compensated
  FP32-pair solution); and the vectorised stage kernel gives the per-point kernel's bits.
* 512^3 operators (8 spheres): the mixed operators agree with the FP64 ones on the same
  FP32-representable field to 2e-6 (the mixed operators' tolerance against the oracle), and
  D(2u) == 2 D(u) bit for bit.
* 128^3 heat (sphere r = 0.25): the transpose identity <A^T x, y> = <x, A y> of the adjoint's
  operator to 1e-11 relative.
* The 256-instance batch: sampled instances bit-identical to their single-system solves.
"""
import numpy as np
import pytest

import shoccs_gb300 as S
from shoccs_gb300 import workloads as W


def _torch():
    import torch
    return torch


def _dev_state(p, D, dtype=None):
    torch = _torch()
    dtype = dtype or torch.float64
    return S.ScalarField(D.to(dtype), *[torch.zeros(n, dtype=dtype, device="cuda") for n in p.nR])


def _pulse_field(p, c):
    """a smooth field on the grid (the headline Gaussian pulse), zero at the cut points"""
    s = S.ScalarWave(p, S.PREC_FP64, S.VEL_CONSTANT, W.WAVE_VEL, (0, 0, 0), S.SOL_GAUSS_PULSE,
                     W.WAVE_PULSE)
    s.initialize(0.0)
    u = p.zeros()
    s.get_state(u)
    del s
    return u.D.clone()


@pytest.mark.gpu
@pytest.mark.parametrize("prec", [S.PREC_FP64, S.PREC_MIXED])
def test_wave256_rk4_homogeneous_bitwise(prec):
    c = W.wave_3d()
    p = S.Problem(**c)
    # pulse + 1: no value near the FP32 subnormal range, where rounding does not scale
    # exactly by 2 (the pulse's far tail, e^-384, would be subnormal in FP32)
    D = _pulse_field(p, c) + 1.0
    s = S.ScalarWave(p, prec, S.VEL_CONSTANT, W.WAVE_VEL, (0, 0, 0), S.SOL_ZERO)
    dt = W.pulse_dt(c["n"][0])
    out = []
    for scale in (1.0, 2.0):
        s.set_state(_dev_state(p, D * scale))
        s.rk4(0.0, dt, 1)  # E4_1 on this grid is unstable (it grows ~1e8 a step): one step
        u = p.zeros()
        s.get_state(u)
        out.append(u.D)
    assert bool(_torch().isfinite(out[0]).all())
    assert _torch().equal(out[1], 2.0 * out[0])


@pytest.mark.gpu
def test_wave256_vectorised_and_per_point_stage_bitwise(monkeypatch):
    c = W.wave_3d()
    p = S.Problem(**c)
    dt = W.pulse_dt(c["n"][0])
    res = {}
    for name in ("vec", "point"):
        monkeypatch.setenv("SHOCCS_STAGE_KERNEL", name)
        s = S.ScalarWave(p, S.PREC_MIXED, S.VEL_CONSTANT, W.WAVE_VEL, (0, 0, 0),
                         S.SOL_GAUSS_PULSE, W.WAVE_PULSE)
        assert s.stage_kernel == name
        s.initialize(0.0)
        s.rk4(0.0, dt, 1)
        u = p.zeros()
        s.get_state(u)
        res[name] = u.D
        del s
    assert bool(_torch().isfinite(res["vec"]).all())
    assert _torch().equal(res["vec"], res["point"])


@pytest.mark.gpu
def test_operators512_mixed_against_fp64_and_homogeneous():
    torch = _torch()
    c = W.micro_case(512)
    p = S.Problem(**c)
    u32 = W.micro_field(p.size, torch.float32)
    u64 = u32.to(torch.float64)
    for d in range(3):
        d64 = p.zeros()
        S.Derivative(p, d, S.PREC_FP64)(_dev_state(p, u64), d64)
        d32 = p.zeros(torch.float32)
        S.Derivative(p, d, S.PREC_MIXED)(_dev_state(p, u32, torch.float32), d32)
        err = float((d32.D.double() - d64.D).abs().max() / d64.D.abs().max())
        assert err <= 2e-6, (d, err)
        if d == 2:
            d32b = p.zeros(torch.float32)
            S.Derivative(p, d, S.PREC_MIXED)(_dev_state(p, 2 * u32, torch.float32), d32b)
            assert torch.equal(d32b.D, 2 * d32.D)
        del d64, d32
    c2 = W.micro_case(512, scheme="E4_2")
    p2 = S.Problem(**c2)
    l64 = S.Laplacian(p2)(_dev_state(p2, u64), p2.zeros())
    l32 = S.Laplacian(p2, S.PREC_MIXED)(_dev_state(p2, u32, torch.float32), p2.zeros(torch.float32))
    err = float((l32.D.double() - l64.D).abs().max() / l64.D.abs().max())
    assert err <= 2e-6, err


@pytest.mark.gpu
def test_heat128_transpose_identity():
    torch = _torch()
    c = W.adjoint_case(128)
    p = S.Problem(**c)
    h = S.Heat(p, 1.0, S.PREC_FP64, S.SOL_ZERO)
    g = torch.Generator(device="cuda")
    g.manual_seed(20261209)
    x = torch.rand(p.size, dtype=torch.float64, device="cuda", generator=g) - 0.5
    y = torch.rand(p.size, dtype=torch.float64, device="cuda", generator=g) - 0.5
    h.set_state(_dev_state(p, y))
    Ay = h.rhs(0.0, p.zeros())
    ATx = h.rhs_transpose(_dev_state(p, x), p.zeros())
    lhs = float((ATx.D * y).sum())
    rhs = float((x * Ay.D).sum())
    scale = float(ATx.D.abs().sum() * y.abs().max() + x.abs().max() * Ay.D.abs().sum())
    assert abs(lhs - rhs) <= 1e-11 * scale, (lhs, rhs)


@pytest.mark.gpu
@pytest.mark.parametrize("prec", [S.PREC_FP64, S.PREC_MIXED])
def test_batch256_instances_match_single_systems(prec):
    insts = W.batch_heat_2d(256)
    probs = [S.Problem(**it["case"]) for it in insts]
    systems = [S.Heat(q, 1.0, prec, S.SOL_SINSIN, [float(it["k"])]) for q, it in zip(probs, insts)]
    for s in systems:
        s.initialize(0.0)
    dts = [it["dt"] for it in insts]
    S.Batch(systems).rk4(0.0, dts, 3)
    for i in (0, 97, 255):
        single = S.Heat(probs[i], 1.0, prec, S.SOL_SINSIN, [float(insts[i]["k"])])
        single.initialize(0.0)
        single.rk4(0.0, dts[i], 3)
        a = [np.zeros(probs[i].size)] + [np.zeros(k) for k in probs[i].nR]
        b = [np.zeros(probs[i].size)] + [np.zeros(k) for k in probs[i].nR]
        systems[i].get_state(S.ScalarField(*a))
        single.get_state(S.ScalarField(*b))
        for x, y in zip(a, b):
            assert np.array_equal(x, y), i
