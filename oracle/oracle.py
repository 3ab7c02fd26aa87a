"""ctypes binding of the CPU oracle (oracle/shoccs_oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and bench.py's CPU
baseline leg to check and time the CUDA path; the product library never imports it.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liboracle.so")
SRC = os.path.join(HERE, "shoccs_oracle.cpp")

D = ctypes.c_double
DP = ctypes.POINTER(ctypes.c_double)
IP = ctypes.POINTER(ctypes.c_int)
LP = ctypes.POINTER(ctypes.c_long)

BC = {"dirichlet": 0, "floating": 1, "neumann": 2}
SCHEME = {"E2_2": 0, "E4_2": 1, "E4_1": 2, "E4u_1": 3, "polyE2_1": 5, "E6u_1": 6, "E8u_1": 7}


def build(force=False):
    os.makedirs(BUILD, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    subprocess.check_call(["g++", "-std=c++20", "-O2", "-fopenmp", "-ffp-contract=off",
                           "-fPIC", "-shared", SRC, "-o", LIB])
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = ctypes.CDLL(LIB)
        _lib.orc_create.restype = ctypes.c_void_p
        _lib.orc_size.restype = ctypes.c_long
        _lib.orc_lines.restype = ctypes.c_long
        _lib.orc_fluid.restype = ctypes.c_long
        _lib.orc_block.restype = ctypes.c_long
        _lib.orc_csr.restype = ctypes.c_long
        for n in ["orc_destroy", "orc_size", "orc_cut_points", "orc_lines", "orc_fluid",
                  "orc_block", "orc_csr", "orc_derivative", "orc_laplacian", "orc_gradient",
                  "orc_initialize", "orc_exact", "orc_heat_rhs", "orc_heat_rk4",
                  "orc_wave_rhs", "orc_wave_rk4", "orc_stats", "orc_error_field",
                  "orc_set_gaussian", "orc_heat_euler", "orc_wave_euler", "orc_block_layout"]:
            getattr(_lib, n).argtypes = None
    return _lib


def gaussian_terms(terms):
    """flatten Gaussian terms (centre[3], variance[3], amplitude, frequency) to 8 doubles each"""
    flat = []
    for c, v, a, f in terms:
        flat += [float(x) for x in c] + [float(x) for x in v] + [float(a), float(f)]
    return flat


def _p(a):
    if a is None:
        return None
    return a.ctypes.data_as(DP) if a.dtype == np.float64 else a.ctypes.data


def _bc(b):
    return BC[b] if isinstance(b, str) else int(b)


def set_threads(n):
    return lib().orc_num_threads(int(n))


class OracleProblem:
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
        gbc = (ctypes.c_int * 6)(*[_bc(b) for b in grid_bc])
        # E2-poly takes 13 parameters (floating, dirichlet, interpolant alpha), E6u 5, E8u 7,
        # the others 2
        al = (D * max(2, len(alpha)))(*alpha)
        self._h = ctypes.c_void_p(L.orc_create(
            (ctypes.c_int * 3)(*n), (D * 3)(*lo), (D * 3)(*hi), ctypes.c_int(len(spheres)),
            _p(cen), _p(rad), sbc.ctypes.data_as(IP), gbc,
            ctypes.c_int(SCHEME[scheme] if isinstance(scheme, str) else scheme), al))
        self.size = L.orc_size(self._h, 0)
        self.nR = tuple(L.orc_size(self._h, d + 1) for d in range(3))

    def __del__(self):
        if getattr(self, "_h", None):
            lib().orc_destroy(self._h)
            self._h = None

    def cut_points(self, d):
        n = self.nR[d]
        psi, pos, nrm = np.zeros(n), np.zeros(3 * n), np.zeros(3 * n)
        ro, sc, sid = (np.zeros(n, np.int32), np.zeros(3 * n, np.int32), np.zeros(n, np.int32))
        lib().orc_cut_points(self._h, ctypes.c_int(d), _p(psi), _p(pos), _p(nrm),
                             ro.ctypes.data_as(IP), sc.ctypes.data_as(IP),
                             sid.ctypes.data_as(IP))
        return dict(psi=psi, position=pos.reshape(-1, 3), normal=nrm.reshape(-1, 3),
                    ray_outside=ro, solid_coord=sc.reshape(-1, 3), shape_id=sid)

    def lines(self, d):
        n = lib().orc_lines(self._h, ctypes.c_int(d), None)
        out = np.zeros((n, 8), dtype=np.int32)
        lib().orc_lines(self._h, ctypes.c_int(d), out.ctypes.data_as(IP))
        return out

    def fluid(self):
        n = lib().orc_fluid(self._h, None)
        out = np.zeros(n, dtype=np.int64)
        lib().orc_fluid(self._h, out.ctypes.data_as(LP))
        return out

    def block_meta(self, d):
        nc = ctypes.c_long()
        nl = lib().orc_block(self._h, ctypes.c_int(d), None, None, ctypes.byref(nc))
        meta = np.zeros((nl, 13), dtype=np.int32)
        coeffs = np.zeros(nc.value)
        lib().orc_block(self._h, ctypes.c_int(d), meta.ctypes.data_as(IP), _p(coeffs), None)
        return meta, coeffs

    def csr(self, d, which):
        rows = ctypes.c_long()
        nnz = lib().orc_csr(self._h, ctypes.c_int(d), ctypes.c_int(which), ctypes.byref(rows),
                            None, None, None)
        u = np.zeros(rows.value + 1, dtype=np.int64)
        v = np.zeros(nnz, dtype=np.int64)
        w = np.zeros(nnz)
        lib().orc_csr(self._h, ctypes.c_int(d), ctypes.c_int(which), None,
                      u.ctypes.data_as(LP), v.ctypes.data_as(LP), _p(w))
        return rows.value, u, v, w

    def block_layout(self, lines):
        """metadata of hand-built line blocks: each line is (columns, row offset, column
        offset, stride, (left rows, left columns), interior rows, stencil width,
        (right rows, right columns))"""
        spec = np.zeros((len(lines), 10), dtype=np.int64)
        for i, (cols, ro, co, st, (lr, lc), ni, w, (rr, rc)) in enumerate(lines):
            spec[i] = (cols, ro, co, st, lr, lc, ni, w, rr, rc)
        meta = np.zeros((len(lines), 13), dtype=np.int32)
        lib().orc_block_layout(ctypes.c_int(len(lines)), spec.ctypes.data_as(LP),
                               meta.ctypes.data_as(IP))
        return meta

    # ---- operators (numpy float64 arrays) ----
    def zeros(self):
        return [np.zeros(self.size)] + [np.zeros(n) for n in self.nR]

    def derivative(self, d, u, du, plus_eq=False, nu=None):
        lib().orc_derivative(self._h, ctypes.c_int(d), *[_p(a) for a in u],
                             _p(nu) if nu is not None else None, *[_p(a) for a in du],
                             ctypes.c_int(1 if plus_eq else 0))
        return du

    def laplacian(self, u, du, nu=None):
        lib().orc_laplacian(self._h, *[_p(a) for a in u], _p(nu) if nu is not None else None,
                            *[_p(a) for a in du])
        return du

    def gradient(self, u):
        outs = [self.zeros() for _ in range(3)]
        ptrs = (DP * 12)(*[a.ctypes.data_as(DP) for f in outs for a in f])
        lib().orc_gradient(self._h, *[_p(a) for a in u], ptrs)
        return outs

    def _params(self, sol_kind, params):
        """the 8 closed-form parameters; for the Gaussian sum (kind 4) `params` is its list
        of terms (centre[3], variance[3], amplitude, frequency), set on the problem"""
        if sol_kind == 4:
            flat = gaussian_terms(params)
            arr = (D * max(len(flat), 1))(*flat)
            lib().orc_set_gaussian(self._h, ctypes.c_int(len(flat) // 8), arr)
            return (D * 8)()
        return (D * 8)(*(list(params) + [0.0] * (8 - len(params))))

    def initialize(self, sol_kind, params, t=0.0):
        u = self.zeros()
        pr = self._params(sol_kind, params)
        lib().orc_initialize(self._h, ctypes.c_int(sol_kind), pr, D(t), *[_p(a) for a in u])
        return u

    def exact(self, sol_kind, params, t):
        u = self.zeros()
        pr = self._params(sol_kind, params)
        lib().orc_exact(self._h, ctypes.c_int(sol_kind), pr, D(t), *[_p(a) for a in u])
        return u

    def heat_rhs(self, kappa, sol_kind, params, t, u):
        du = self.zeros()
        pr = self._params(sol_kind, params)
        lib().orc_heat_rhs(self._h, D(kappa), ctypes.c_int(sol_kind), pr, D(t),
                           *[_p(a) for a in u], *[_p(a) for a in du])
        return du

    def heat_rk4(self, kappa, sol_kind, params, t0, dt, nsteps, u):
        u = [a.copy() for a in u]
        pr = self._params(sol_kind, params)
        lib().orc_heat_rk4(self._h, D(kappa), ctypes.c_int(sol_kind), pr, D(t0), D(dt),
                           ctypes.c_int(nsteps), *[_p(a) for a in u])
        return u

    def heat_euler(self, kappa, sol_kind, params, t0, dt, nsteps, u):
        u = [a.copy() for a in u]
        pr = self._params(sol_kind, params)
        lib().orc_heat_euler(self._h, D(kappa), ctypes.c_int(sol_kind), pr, D(t0), D(dt),
                             ctypes.c_int(nsteps), *[_p(a) for a in u])
        return u

    def wave_euler(self, vel_kind, vel, center, sol_kind, params, t0, dt, nsteps, u):
        u = [a.copy() for a in u]
        pr = self._params(sol_kind, params)
        lib().orc_wave_euler(self._h, ctypes.c_int(vel_kind), (D * 3)(*vel), (D * 3)(*center),
                             ctypes.c_int(sol_kind), pr, D(t0), D(dt), ctypes.c_int(nsteps),
                             *[_p(a) for a in u])
        return u

    def wave_rhs(self, vel_kind, vel, center, u):
        du = self.zeros()
        lib().orc_wave_rhs(self._h, ctypes.c_int(vel_kind), (D * 3)(*vel), (D * 3)(*center),
                           *[_p(a) for a in u], *[_p(a) for a in du])
        return du

    def wave_rk4(self, vel_kind, vel, center, sol_kind, params, t0, dt, nsteps, u):
        u = [a.copy() for a in u]
        pr = self._params(sol_kind, params)
        lib().orc_wave_rk4(self._h, ctypes.c_int(vel_kind), (D * 3)(*vel), (D * 3)(*center),
                           ctypes.c_int(sol_kind), pr, D(t0), D(dt), ctypes.c_int(nsteps),
                           *[_p(a) for a in u])
        return u

    def stats(self, sol_kind, params, t, u):
        out = np.zeros(11)
        pr = self._params(sol_kind, params)
        lib().orc_stats(self._h, ctypes.c_int(sol_kind), pr, D(t), *[_p(a) for a in u],
                        _p(out))
        return out

    def error_field(self, sol_kind, params, t, u):
        """the Error field of write_scalar_error (scalar_system_utils.hpp:224-296)"""
        e = self.zeros()
        pr = self._params(sol_kind, params)
        lib().orc_error_field(self._h, ctypes.c_int(sol_kind), pr, D(t), *[_p(a) for a in u],
                              *[_p(a) for a in e])
        return e
