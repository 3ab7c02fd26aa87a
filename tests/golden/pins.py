"""The arrays that pin the oracle to the reference's own compiled code.

Shared by tests/golden/make_golden.py (which computes them with the reference, through
oracle/_ref) and tests/test_reference_pin.py (which computes them with the oracle and
compares).  Every function takes an object with the methods of oracle.oracle.OracleProblem
(oracle.reference.RefProblem has the same ones) and returns an ordered dict of named numpy
arrays, so the two sides can be compared name by name, or by SHA-256 digest where only the
digests were kept.

TEST INFRASTRUCTURE ONLY.
"""
import hashlib
import zlib

import numpy as np

# the velocity centre and radius of the reference's radial scalar wave per case (the
# centre sits inside a sphere or outside the domain, so that |x - c| > 0 at every point)
WAVE_CASES = {
    "wave_sphere_3d": ((0.5, 0.5, 0.5), 0.22),
    "multi_sphere_e41": (None, 0.05),  # the first sphere's centre
    "micro_e41_96": (None, 0.05),
    "box_e4u": ((-0.3, -0.2, -0.1), 0.1),
    # scalar_wave.lua's system: radial wave about (-1, -1), radius 0
    "poly_scalar_wave_2d": ((-1.0, -1.0, 0.0), 0.0),
    "poly_spheres_3d": ((-0.3, -0.2, -0.1), 0.1),
    "e6u_sphere_3d": ((-0.3, -0.2, -0.1), 0.1),
    "e8u_circle_2d": ((-0.3, -0.2, 0.0), 0.1),
}
HEAT_SCHEMES = ("E2_2", "E4_2")
KAPPA = 0.7
SINSIN_K = 1.0


def digest(a):
    a = np.ascontiguousarray(a)
    a = a.astype(np.int64) if a.dtype.kind in "iub" else a.astype(np.float64)
    return hashlib.sha256(a.tobytes()).hexdigest()


def seed_of(name):
    return zlib.crc32(name.encode())


def _csr_norm(rows, u, v, w):
    """An empty matrix left by the reference's quick exit (derivative.cpp:173-175) holds no
    row-offset array; one assembled with zero rows holds a single 0.  Both are the same
    matrix."""
    if rows == 0 and len(u) == 0:
        u = np.zeros(1, dtype=np.int64)
    return u, v, w


def setup_arrays(p):
    out = {}
    out["sizes"] = np.array([p.size, *p.nR], dtype=np.int64)
    out["fluid"] = p.fluid()
    for d in range(3):
        cp = p.cut_points(d)
        for k in ("psi", "position", "normal", "ray_outside", "solid_coord", "shape_id"):
            out["R%d.%s" % (d, k)] = cp[k]
        out["lines%d" % d] = p.lines(d)
        meta, coeffs = p.block_meta(d)
        out["O%d.meta" % d] = meta
        out["O%d.coeffs" % d] = coeffs
        for which, nm in enumerate(("B", "N", "Bfx", "Bfy", "Bfz", "Brx", "Bry", "Brz")):
            rows, u, v, w = p.csr(d, which)
            u, v, w = _csr_norm(rows, u, v, w)
            out["%s%d.rows" % (nm, d)] = np.array([rows], dtype=np.int64)
            out["%s%d.u" % (nm, d)] = u
            out["%s%d.v" % (nm, d)] = v
            out["%s%d.w" % (nm, d)] = w
    return out


def _field(p, rng):
    return [rng.uniform(-1, 1, p.size)] + [rng.uniform(-1, 1, k) for k in p.nR]


def operator_arrays(p, name):
    """derivative (eq and plus_eq, with and without Neumann data), laplacian (with and
    without Neumann data) and gradient of seeded fields"""
    rng = np.random.default_rng(seed_of(name))
    u = _field(p, rng)
    nu = rng.uniform(-1, 1, p.size)
    init = _field(p, rng)
    out = {}
    for d in range(3):
        if p.n[d] < 2:
            continue
        for pe in (0, 1):
            for with_nu in (0, 1):
                du = p.derivative(d, u, [a.copy() for a in init], bool(pe),
                                  nu if with_nu else None)
                for k, a in enumerate(du):
                    out["d%d.pe%d.nu%d.%d" % (d, pe, with_nu, k)] = a
    for with_nu in (0, 1):
        du = p.laplacian(u, p.zeros(), nu if with_nu else None)
        for k, a in enumerate(du):
            out["lap.nu%d.%d" % (with_nu, k)] = a
    g = p.gradient(u)
    for d in range(3):
        for k, a in enumerate(g[d]):
            out["grad%d.%d" % (d, k)] = a
    return out


def heat_steps(case):
    return 2 if max(case["n"]) > 80 else 5


def heat_dt(case):
    """half the reference's parabolic step, p_cfl h_min^2 / (4 k) with p_cfl = 0.4
    (heat.cpp:356-361), for the grid spacing (max - min) / (n - 1) of the active axes"""
    n = list(case["n"]) + [1] * (3 - len(case["n"]))
    lo = list(case["lo"]) + [0.0] * (3 - len(case["lo"]))
    hi = list(case["hi"]) + [0.0] * (3 - len(case["hi"]))
    h = min((hi[a] - lo[a]) / (n[a] - 1) for a in range(3) if n[a] > 1)
    return 0.5 * (0.4 * h * h / (4 * KAPPA))


def wave_dt(case):
    """a tenth of the reference's hyperbolic step h_cfl h_min with h_cfl = 0.5
    (scalar_wave.cpp:357-362)"""
    n = list(case["n"]) + [1] * (3 - len(case["n"]))
    lo = list(case["lo"]) + [0.0] * (3 - len(case["lo"]))
    hi = list(case["hi"]) + [0.0] * (3 - len(case["hi"]))
    h = min((hi[a] - lo[a]) / (n[a] - 1) for a in range(3) if n[a] > 1)
    return 0.1 * (0.5 * h)


class OracleHeat:
    """the oracle's heat system behind the calls RefSystem offers (sin-sin solution)"""

    def __init__(self, p):
        self.p = p

    def initialize(self, t):
        return self.p.initialize(1, (SINSIN_K,), t)

    def rhs(self, t, u):
        return self.p.heat_rhs(KAPPA, 1, (SINSIN_K,), t, u)

    def rk4(self, t0, dt, n, u):
        return self.p.heat_rk4(KAPPA, 1, (SINSIN_K,), t0, dt, n, u)

    def stats(self, t, u):
        return self.p.stats(1, (SINSIN_K,), t, u)[:10]


class OracleWave:
    def __init__(self, p, center, radius):
        self.p, self.c, self.r = p, center, radius

    def initialize(self, t):
        return self.p.initialize(3, list(self.c) + [self.r], t)

    def rhs(self, t, u):
        return self.p.wave_rhs(1, (0.0, 0.0, 0.0), self.c, u)

    def rk4(self, t0, dt, n, u):
        return self.p.wave_rk4(1, (0.0, 0.0, 0.0), self.c, 3, list(self.c) + [self.r], t0,
                               dt, n, u)

    def stats(self, t, u):
        return self.p.stats(3, list(self.c) + [self.r], t, u)[:10]


def wave_center(case, name):
    c, r = WAVE_CASES[name]
    if c is None:
        c = tuple(case["spheres"][0][0])
    return c, r


def dirichlet_update(case, shape_ids, exact, u):
    """The Dirichlet part of the reference's update_boundary (heat.cpp:296-322,
    scalar_wave.cpp:329-355): the exact values on every Dirichlet domain face
    (for_each_grid_bc_desc, selection_desc.hpp:211-222) and at the cut points of Dirichlet
    objects.  `exact` holds the exact solution at every point, `shape_ids[d]` the object of
    every cut point along axis d."""
    n = list(case["n"]) + [1] * (3 - len(case["n"]))
    bcs = case.get("grid_bc", ("floating",) * 6)
    u = [a.copy() for a in u]
    D = u[0].reshape(n)
    E = exact[0].reshape(n)
    for a in range(3):
        for side, face in ((0, 0), (1, n[a] - 1)):
            if bcs[2 * a + side] == "dirichlet":
                sl = [slice(None)] * 3
                sl[a] = face
                D[tuple(sl)] = E[tuple(sl)]
    sphere_bc = [b for _, _, b in case.get("spheres", ())]
    for d in range(3):
        if not len(u[1 + d]):
            continue
        m = np.array([sphere_bc[i] == "dirichlet" for i in shape_ids[d]], dtype=bool)
        u[1 + d][m] = exact[1 + d][m]
    return u


def system_arrays(sys_, name, nsteps, dt, boundary=None):
    """initial state, right-hand side of a perturbed state, RK4 states and statistics.
    `boundary(t, u)` applies the system's boundary update (the reference's update_boundary)
    to the perturbed state before its right-hand side is taken; the oracle's right-hand side
    evaluates the boundary data itself."""
    out = {}
    u0 = sys_.initialize(0.0)
    for k, a in enumerate(u0):
        out["init.%d" % k] = a
    rng = np.random.default_rng(seed_of(name) + 1)
    up = [a + 0.01 * rng.uniform(-1, 1, a.shape) for a in u0]
    if boundary is not None:
        up = boundary(0.3, up)
    for k, a in enumerate(sys_.rhs(0.3, up)):
        out["rhs.%d" % k] = a
    u = sys_.rk4(0.0, dt, nsteps, u0)
    for k, a in enumerate(u):
        out["rk4.%d" % k] = a
    out["stats"] = np.asarray(sys_.stats(nsteps * dt, u))[:10]
    return out
