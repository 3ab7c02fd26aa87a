"""ctypes binding of oracle/_ref/libshoccs_ref.so: the reference's own hot-path code
(mesh and cut points, operator assembly, block and CSR matvecs, derivative, laplacian,
gradient, stencils, sphere intersection) compiled unmodified by oracle/build_ref.sh.

TEST INFRASTRUCTURE ONLY: the tests and tests/golden/make_golden.py use it to pin the
oracle restatement; it exists only where the reference tree was present at build time.
`RefProblem` has the same methods as `oracle.oracle.OracleProblem` for the parts the
reference computes, so the two can be compared array by array.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_ref", "libshoccs_ref.so")

D = ctypes.c_double
DP = ctypes.POINTER(ctypes.c_double)
IP = ctypes.POINTER(ctypes.c_int)
LP = ctypes.POINTER(ctypes.c_long)

BC = {"dirichlet": 0, "floating": 1, "neumann": 2}
SCHEME = {"E2_2": 0, "E4_2": 1, "E4_1": 2, "E4u_1": 3, "polyE2_1": 5, "E6u_1": 6, "E8u_1": 7}

_lib = None


def available():
    return os.path.exists(LIB)


def lib():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(LIB)
        _lib.ref_problem_create.restype = ctypes.c_void_p
        for n in ("ref_problem_size", "ref_lines", "ref_fluid", "ref_block", "ref_csr"):
            getattr(_lib, n).restype = ctypes.c_long
    return _lib


def _p(a):
    if a is None:
        return None
    return a.ctypes.data_as(DP) if a.dtype == np.float64 else a.ctypes.data


def _bc(b):
    return BC[b] if isinstance(b, str) else int(b)


class RefProblem:
    def __init__(self, n, lo, hi, spheres=(), grid_bc=("floating",) * 6, scheme="E4_2",
                 alpha=(0.0, 0.0)):
        L = lib()
        n = list(n) + [1] * (3 - len(n))
        lo = list(lo) + [0.0] * (3 - len(lo))
        hi = list(hi) + [0.0] * (3 - len(hi))
        spheres = list(spheres)
        cen = np.zeros(max(1, 3 * len(spheres)))
        rad = np.zeros(max(1, len(spheres)))
        sbc = np.zeros(max(1, len(spheres)), dtype=np.int32)
        for i, (c, r, b) in enumerate(spheres):
            c = list(c) + [0.0] * (3 - len(c))
            cen[3 * i:3 * i + 3] = c
            rad[i] = r
            sbc[i] = _bc(b)
        self.n = n
        self._h = ctypes.c_void_p(L.ref_problem_create(
            (ctypes.c_int * 3)(*n), (D * 3)(*lo), (D * 3)(*hi), ctypes.c_int(len(spheres)),
            _p(cen), _p(rad), sbc.ctypes.data_as(IP),
            (ctypes.c_int * 6)(*[_bc(b) for b in grid_bc]),
            ctypes.c_int(SCHEME[scheme] if isinstance(scheme, str) else scheme),
            (D * max(2, len(alpha)))(*alpha)))
        self.size = L.ref_problem_size(self._h, 0)
        self.nR = tuple(L.ref_problem_size(self._h, d + 1) for d in range(3))

    def __del__(self):
        if getattr(self, "_h", None):
            lib().ref_problem_destroy(self._h)
            self._h = None

    def cut_points(self, d):
        n = self.nR[d]
        psi, pos, nrm = np.zeros(n), np.zeros(3 * n), np.zeros(3 * n)
        ro, sc, sid = (np.zeros(n, np.int32), np.zeros(3 * n, np.int32), np.zeros(n, np.int32))
        lib().ref_cut_points(self._h, ctypes.c_int(d), _p(psi), _p(pos), _p(nrm),
                             ro.ctypes.data_as(IP), sc.ctypes.data_as(IP),
                             sid.ctypes.data_as(IP))
        return dict(psi=psi, position=pos.reshape(-1, 3), normal=nrm.reshape(-1, 3),
                    ray_outside=ro, solid_coord=sc.reshape(-1, 3), shape_id=sid)

    def lines(self, d):
        n = lib().ref_lines(self._h, ctypes.c_int(d), None)
        out = np.zeros((n, 8), dtype=np.int32)
        lib().ref_lines(self._h, ctypes.c_int(d), out.ctypes.data_as(IP))
        return out

    def fluid(self):
        n = lib().ref_fluid(self._h, None)
        out = np.zeros(n, dtype=np.int64)
        lib().ref_fluid(self._h, out.ctypes.data_as(LP))
        return out

    def block_meta(self, d):
        nc = ctypes.c_long()
        nl = lib().ref_block(self._h, ctypes.c_int(d), None, None, ctypes.byref(nc))
        meta = np.zeros((nl, 13), dtype=np.int32)
        coeffs = np.zeros(nc.value)
        lib().ref_block(self._h, ctypes.c_int(d), meta.ctypes.data_as(IP), _p(coeffs), None)
        return meta, coeffs

    def csr(self, d, which):
        """(rows, row offsets, columns, values); an empty matrix has no row offsets"""
        rows = ctypes.c_long()
        nnz = lib().ref_csr(self._h, ctypes.c_int(d), ctypes.c_int(which), ctypes.byref(rows),
                            None, None, None)
        u = np.zeros(rows.value + 1 if rows.value else 0, dtype=np.int64)
        v = np.zeros(nnz, dtype=np.int64)
        w = np.zeros(nnz)
        lib().ref_csr(self._h, ctypes.c_int(d), ctypes.c_int(which), None,
                      u.ctypes.data_as(LP), v.ctypes.data_as(LP), _p(w))
        return rows.value, u, v, w

    def zeros(self):
        return [np.zeros(self.size)] + [np.zeros(n) for n in self.nR]

    def derivative(self, d, u, du, plus_eq=False, nu=None):
        lib().ref_derivative(self._h, ctypes.c_int(d), *[_p(a) for a in u],
                             _p(nu) if nu is not None else None, *[_p(a) for a in du],
                             ctypes.c_int(1 if plus_eq else 0))
        return du

    def laplacian(self, u, du, nu=None):
        lib().ref_laplacian(self._h, *[_p(a) for a in u], _p(nu) if nu is not None else None,
                            *[_p(a) for a in du])
        return du

    def gradient(self, u):
        outs = [self.zeros() for _ in range(3)]
        ptrs = (DP * 12)(*[a.ctypes.data_as(DP) for f in outs for a in f])
        lib().ref_gradient(self._h, *[_p(a) for a in u], ptrs)
        return outs


def _problem_args(n, lo, hi, spheres, grid_bc, scheme, alpha):
    n = list(n) + [1] * (3 - len(n))
    lo = list(lo) + [0.0] * (3 - len(lo))
    hi = list(hi) + [0.0] * (3 - len(hi))
    spheres = list(spheres)
    cen = np.zeros(max(1, 3 * len(spheres)))
    rad = np.zeros(max(1, len(spheres)))
    sbc = np.zeros(max(1, len(spheres)), dtype=np.int32)
    for i, (c, r, b) in enumerate(spheres):
        c = list(c) + [0.0] * (3 - len(c))
        cen[3 * i:3 * i + 3] = c
        rad[i] = r
        sbc[i] = _bc(b)
    keep = (cen, rad, sbc)
    args = ((ctypes.c_int * 3)(*n), (D * 3)(*lo), (D * 3)(*hi), ctypes.c_int(len(spheres)),
            _p(cen), _p(rad), sbc.ctypes.data_as(IP),
            (ctypes.c_int * 6)(*[_bc(b) for b in grid_bc]),
            ctypes.c_int(SCHEME[scheme] if isinstance(scheme, str) else scheme),
            (D * max(2, len(alpha)))(*alpha))
    return n, args, keep


class RefSystem:
    """The reference's heat or scalar-wave system stepped by its RK4 integrator in the loop
    of simulation_cycle::run.  kind "heat": sol_kind 1 (sin-sin, sol=(k,)) or 4 (the
    reference's gaussian solution, sol = list of (centre, variance, amplitude, frequency));
    kind "wave": the reference's radial wave about `center` with `radius`."""

    def __init__(self, kind, n, lo, hi, spheres=(), grid_bc=("floating",) * 6, scheme="E4_2",
                 alpha=(0.0, 0.0), diffusivity=1.0, sol_kind=1, sol=(1.0,), p_cfl=0.4,
                 center=(0.0, 0.0, 0.0), radius=0.0, h_cfl=0.5):
        L = lib()
        L.ref_heat_create.restype = ctypes.c_void_p
        L.ref_wave_create.restype = ctypes.c_void_p
        L.ref_system_timestep.restype = ctypes.c_double
        self.n, args, keep = _problem_args(n, lo, hi, spheres, grid_bc, scheme, alpha)
        if kind == "heat":
            params = (D * 8)()
            terms = np.zeros(8)
            nterms = 0
            if sol_kind == 4:
                flat = []
                for c, v, a, f in sol:
                    flat += [float(x) for x in c] + [float(x) for x in v] + [float(a), float(f)]
                terms = np.array(flat)
                nterms = len(flat) // 8
            else:
                params = (D * 8)(*(list(sol) + [0.0] * (8 - len(sol))))
            h = L.ref_heat_create(*args, D(diffusivity), ctypes.c_int(sol_kind), params,
                                  ctypes.c_int(nterms), _p(terms), D(p_cfl))
        else:
            h = L.ref_wave_create(*args, (D * 3)(*center), D(radius), D(h_cfl))
        if not h:
            raise ValueError("unsupported reference system")
        self._h = ctypes.c_void_p(h)
        p = RefProblem(n, lo, hi, spheres, grid_bc, scheme, alpha)
        self.size, self.nR = p.size, p.nR

    def __del__(self):
        if getattr(self, "_h", None):
            lib().ref_system_destroy(self._h)
            self._h = None

    def zeros(self):
        return [np.zeros(self.size)] + [np.zeros(k) for k in self.nR]

    def initialize(self, t=0.0):
        u = self.zeros()
        lib().ref_system_initialize(self._h, D(t), *[_p(a) for a in u])
        return u

    def update_boundary(self, t, u):
        u = [a.copy() for a in u]
        lib().ref_system_update_boundary(self._h, D(t), *[_p(a) for a in u])
        return u

    def rhs(self, t, u):
        du = self.zeros()
        lib().ref_system_rhs(self._h, D(t), *[_p(np.ascontiguousarray(a)) for a in u],
                             *[_p(a) for a in du])
        return du

    def rk4(self, t0, dt, nsteps, u):
        u = [a.copy() for a in u]
        lib().ref_system_rk4(self._h, D(t0), D(dt), ctypes.c_int(nsteps), *[_p(a) for a in u])
        return u

    def stats(self, t, u):
        out = np.zeros(16)
        k = lib().ref_system_stats(self._h, D(t), *[_p(a) for a in u], _p(out))
        return out[:k]

    def timestep(self):
        return lib().ref_system_timestep(self._h)
