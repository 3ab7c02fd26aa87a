"""Seeded workload definitions: the problem descriptions and synthetic inputs of the
benchmark configurations, shared by bench.py, the tests and users who want the same cases.

* wave_3d        3-D scalar wave, 256^3, Dirichlet sphere r = 0.3, E4_1, Gaussian pulse
* heat_2d        2-D heat, 65^2, circle, E4_2, manufactured sin(2 pi x) sin(2 pi y) e^-t
* micro_spheres  8 non-overlapping spheres for the operator microbenchmark
* micro_field    u ~ U[-1, 1] on the device
* batch_heat_2d  the independent 2-D heat instances of the batched configuration
* adjoint_gaussians  the sum-of-Gaussians initial field of the adjoint configuration

All random draws come from numpy's PCG64 generator (or torch's device generator for the
large microbenchmark field) with the fixed seeds below, so every run builds the same cases.
"""
import math

import numpy as np

SEED_MICRO_FIELD = 20261203
SEED_MICRO_SPHERES = 20261204
SEED_BATCH = 20261205
SEED_ADJOINT = 20261206
SEED_ADJOINT_DIRECTIONS = 20261207

WAVE_VEL = (1.0, 0.7, 0.4)
WAVE_PULSE = [0.2, 0.2, 0.2, 1.0, 0.7, 0.4, 0.05]  # centre, velocity, sigma


def wave_3d(n=256, radius=0.3, scheme="E4_1", alpha=(0.1, 0.7)):
    """3-D wave case: inflow faces (x, y, z min) Dirichlet, outflow faces Floating."""
    return dict(n=(n, n, n), lo=(0, 0, 0), hi=(1, 1, 1),
                spheres=[((0.5, 0.5, 0.5), radius, "dirichlet")] if radius > 0 else [],
                grid_bc=("dirichlet", "floating") * 3, scheme=scheme, alpha=alpha)


def heat_2d(n=65):
    """2-D heat case: circle (0.51, 0.49) r = 0.2, all four faces Dirichlet, E4_2."""
    return dict(n=(n, n, 1), lo=(0, 0, 0), hi=(1, 1, 0),
                spheres=[((0.51, 0.49, 0.0), 0.2, "dirichlet")],
                grid_bc=("dirichlet",) * 4 + ("floating",) * 2, scheme="E4_2")


def micro_spheres(n=512, count=8, seed=SEED_MICRO_SPHERES, gap_h=8.0, bcs=("dirichlet",)):
    """Non-overlapping spheres: centres U[0.15, 0.85]^3, radii U[0.03, 0.08], every pair at
    least gap_h grid spacings apart (rejection sampling), bc cycling through bcs."""
    rng = np.random.Generator(np.random.PCG64(seed))
    h = 1.0 / (n - 1)
    out = []
    while len(out) < count:
        c = rng.uniform(0.15, 0.85, size=3)
        r = rng.uniform(0.03, 0.08)
        if all(np.linalg.norm(c - np.array(c2)) >= r + r2 + gap_h * h for c2, r2, _ in out):
            out.append((tuple(float(v) for v in c), float(r), bcs[len(out) % len(bcs)]))
    return out


def micro_case(n=512, scheme="E4_1", bcs=("dirichlet",), alpha=(0.1, 0.7)):
    grid = ("dirichlet", "floating") * 3 if scheme.endswith("_1") else ("dirichlet",) * 6
    return dict(n=(n, n, n), lo=(0, 0, 0), hi=(1, 1, 1),
                spheres=micro_spheres(n, bcs=bcs), grid_bc=grid, scheme=scheme,
                alpha=alpha if scheme.endswith("_1") else (0.0, 0.0))


def micro_field(size, dtype=None, seed=SEED_MICRO_FIELD, device="cuda"):
    """u ~ U[-1, 1] drawn on the device from a seeded generator."""
    import torch
    dtype = dtype or torch.float64
    g = torch.Generator(device=device)
    g.manual_seed(seed)
    u = torch.rand(size, dtype=torch.float64, device=device, generator=g)
    return (2 * u - 1).to(dtype)


def batch_heat_2d(count=256, seed=SEED_BATCH, nmin=32, nmax=192):
    """Independent 2-D heat instances: N ~ U{nmin..nmax}, circle centre U[0.35, 0.65]^2,
    r ~ U[0.1, 0.25], manufactured-solution frequency k in {1, 2, 3}."""
    rng = np.random.Generator(np.random.PCG64(seed))
    out = []
    for _ in range(count):
        n = int(rng.integers(nmin, nmax + 1))
        c = rng.uniform(0.35, 0.65, size=2)
        r = float(rng.uniform(0.1, 0.25))
        k = int(rng.integers(1, 4))
        out.append(dict(case=dict(n=(n, n, 1), lo=(0, 0, 0), hi=(1, 1, 0),
                                  spheres=[((float(c[0]), float(c[1]), 0.0), r, "dirichlet")],
                                  grid_bc=("dirichlet",) * 4 + ("floating",) * 2,
                                  scheme="E4_2"),
                        k=k, dt=0.1 / (n - 1) ** 2))
    return out


def adjoint_gaussians(count=16, seed=SEED_ADJOINT, center=(0.5, 0.5, 0.5), radius=0.25):
    """Sum-of-Gaussians initial field: centres U[0.1, 0.9]^3 outside the sphere, sigma
    U[0.03, 0.1], amplitudes U[-1, 1].  Returns [(centre, sigma, amplitude)]."""
    rng = np.random.Generator(np.random.PCG64(seed))
    out = []
    while len(out) < count:
        c = rng.uniform(0.1, 0.9, size=3)
        if np.linalg.norm(c - np.array(center)) <= radius:
            continue
        out.append((tuple(float(v) for v in c), float(rng.uniform(0.03, 0.1)),
                    float(rng.uniform(-1, 1))))
    return out


def adjoint_case(n=128):
    """3-D heat, sphere (0.5, 0.5, 0.5) r = 0.25, homogeneous Dirichlet walls and sphere."""
    return dict(n=(n, n, n), lo=(0, 0, 0), hi=(1, 1, 1),
                spheres=[((0.5, 0.5, 0.5), 0.25, "dirichlet")],
                grid_bc=("dirichlet",) * 6, scheme="E4_2")


def adjoint_u0(n=128):
    """the sum-of-Gaussians initial field on the n^3 grid (flat, z fastest)"""
    x = np.linspace(0.0, 1.0, n)
    X, Y, Z = np.meshgrid(x, x, x, indexing="ij")
    return gaussian_sum(X, Y, Z, adjoint_gaussians()).ravel()


def gaussian_sum(x, y, z, gs):
    v = 0.0
    for (c, s, a) in gs:
        v = v + a * np.exp(-((x - c[0]) ** 2 + (y - c[1]) ** 2 + (z - c[2]) ** 2) / (2 * s * s))
    return v


def pulse_dt(n, cfl=0.5):
    return cfl / (n - 1)


def heat_dt(n, cfl=0.4, k=1.0):
    h = 1.0 / (n - 1)
    return cfl * h * h / (4 * k)


__all__ = [name for name in dir() if not name.startswith("_") and name not in ("math", "np")]
