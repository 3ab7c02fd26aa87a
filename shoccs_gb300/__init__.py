"""shoccs_gb300 -- GB300 (sm_103a) implementation of the SHOCCS cut-cell derivative-operator
hot path: per-axis stencil sweeps with cut-cell closures, heat / scalar-wave right-hand
sides and the RK4 stage update.

The Python layer is a thin binding of the C ABI (include/shoccs_gpu.h) that keeps the
names of the reference's C++ classes:

    Problem      ccs::mesh + bcs::Grid/Object + stencil     (src/mesh/mesh.hpp, ...)
    Derivative   ccs::derivative                            (src/operators/derivative.hpp)
    Laplacian    ccs::laplacian                             (src/operators/laplacian.hpp)
    Gradient     ccs::gradient                              (src/operators/gradient.hpp)
    Heat         ccs::systems::heat                         (src/systems/heat.hpp)
    ScalarWave   ccs::systems::scalar_wave                  (src/systems/scalar_wave.hpp)
    System.rk4   ccs::integrators::rk4                      (src/temporal/rk4.hpp)

Fields are ScalarField(D, Rx, Ry, Rz) of CUDA tensors (torch is used only to hold device
memory).  All arithmetic runs in the library's CUDA kernels.
"""
import ctypes
from collections import namedtuple

from . import _capi
from ._capi import (BC_DIRICHLET, BC_FLOATING, BC_NEUMANN, PREC_FP64, PREC_MIXED,
                    SCHEME_E2_2, SCHEME_E4_1, SCHEME_E4_2, SOL_GAUSS_PULSE, SOL_GAUSSIAN,
                    SOL_RADIAL_SIN, SOL_SINSIN, SOL_ZERO, VEL_CONSTANT, VEL_RADIAL, ShoccsError)

ScalarField = namedtuple("ScalarField", ["D", "Rx", "Ry", "Rz"])

_BC = {"dirichlet": BC_DIRICHLET, "floating": BC_FLOATING, "neumann": BC_NEUMANN}
_SCHEME = {"E2_2": SCHEME_E2_2, "E4_2": SCHEME_E4_2, "E4_1": SCHEME_E4_1, "E4u_1": 3,
           "polyE2_1": 5, "E6u_1": 6, "E8u_1": 7}
# schemes whose parameters go in scheme_alpha, and how many each takes
_SCHEME_ALPHA = {5: 13, 6: 5, 7: 7}


def _bc(b):
    return _BC[b] if isinstance(b, str) else int(b)


def _ptr(t):
    if t is None:
        return None
    if hasattr(t, "data_ptr"):
        return t.data_ptr() if t.numel() else None
    return t


def _field(f):
    if f is None:
        return None
    return ctypes.byref(_capi.Field(_ptr(f.D), _ptr(f.Rx), _ptr(f.Ry), _ptr(f.Rz)))


def _stream(stream):
    if stream is None:
        return None
    return stream.cuda_stream if hasattr(stream, "cuda_stream") else stream


class Problem:
    """Mesh, boundary conditions and scheme; builds the three derivative operators.

    n, lo, hi: index_extents and domain_bounds; spheres: [(center3, radius, bc)];
    grid_bc: (xmin, xmax, ymin, ymax, zmin, zmax); scheme: "E2_2" | "E4_2" | "E4_1" | "E4u_1"
    | "polyE2_1" (type "E2-poly") | "E6u_1" | "E8u_1"; alpha: the two alpha of E4_1 / E4u_1,
    the thirteen of E2-poly (floating_alpha[6], dirichlet_alpha[3], interpolant_alpha[4], the
    reference's single-array order), the five of E6u or the seven of E8u.
    """

    def __init__(self, n, lo, hi, spheres=(), grid_bc=("floating",) * 6, scheme="E4_2",
                 alpha=(0.0, 0.0)):
        lib = _capi.lib()
        d = _capi.ProblemDesc()
        n = list(n) + [1] * (3 - len(n))
        lo = list(lo) + [0.0] * (3 - len(lo))
        hi = list(hi) + [lo[len(hi)] if len(hi) < 3 else 0.0] * (3 - len(hi))
        d.n[:] = [int(v) for v in n]
        d.lo[:] = [float(v) for v in lo]
        d.hi[:] = [float(v) for v in hi]
        spheres = list(spheres)
        d.n_spheres = len(spheres)
        self._centers = (ctypes.c_double * max(1, 3 * len(spheres)))()
        self._radii = (ctypes.c_double * max(1, len(spheres)))()
        self._sbc = (ctypes.c_int * max(1, len(spheres)))()
        for i, (c, r, b) in enumerate(spheres):
            c = list(c) + [0.0] * (3 - len(c))
            self._centers[3 * i:3 * i + 3] = [float(v) for v in c]
            self._radii[i] = float(r)
            self._sbc[i] = _bc(b)
        d.centers = ctypes.cast(self._centers, _capi.c_double_p)
        d.radii = ctypes.cast(self._radii, _capi.c_double_p)
        d.sphere_bc = ctypes.cast(self._sbc, _capi.c_int_p)
        d.grid_bc[:] = [_bc(b) for b in grid_bc]
        d.scheme = _SCHEME[scheme] if isinstance(scheme, str) else int(scheme)
        if d.scheme in _SCHEME_ALPHA:
            na = _SCHEME_ALPHA[d.scheme]
            if len(alpha) > na:
                raise ValueError("scheme takes at most %d alpha values" % na)
            d.scheme_alpha[:] = [float(v) for v in alpha] + [0.0] * (13 - len(alpha))
        else:
            d.alpha[:] = [float(alpha[0]), float(alpha[1])]
        self.desc = d
        h = ctypes.c_void_p()
        _capi.check(lib.shoccs_problem_create(ctypes.byref(d), ctypes.byref(h)))
        self._h = h
        self.n = tuple(d.n)
        s = (ctypes.c_int64 * 5)()
        _capi.check(lib.shoccs_problem_sizes(self._h, s))
        self.size = s[0]
        self.nR = (s[1], s[2], s[3])
        self.n_fluid = s[4]

    @property
    def handle(self):
        return self._h

    def __del__(self):
        if getattr(self, "_h", None):
            _capi.lib().shoccs_problem_destroy(self._h)
            self._h = None

    # --- setup introspection (host) ---
    def cut_points(self, d):
        import numpy as np
        n = self.nR[d]
        psi = np.zeros(n)
        pos = np.zeros(3 * n)
        nrm = np.zeros(3 * n)
        ro = np.zeros(n, dtype=np.int32)
        sc = np.zeros(3 * n, dtype=np.int32)
        sid = np.zeros(n, dtype=np.int32)
        P = lambda a, t: a.ctypes.data_as(t)
        _capi.check(_capi.lib().shoccs_problem_cut_points(
            self._h, d, P(psi, _capi.c_double_p), P(pos, _capi.c_double_p),
            P(nrm, _capi.c_double_p), P(ro, _capi.c_int_p), P(sc, _capi.c_int_p),
            P(sid, _capi.c_int_p)))
        return dict(psi=psi, position=pos.reshape(-1, 3), normal=nrm.reshape(-1, 3),
                    ray_outside=ro, solid_coord=sc.reshape(-1, 3), shape_id=sid)

    def block_meta(self, d):
        import numpy as np
        nl, nc = ctypes.c_int64(), ctypes.c_int64()
        lib = _capi.lib()
        _capi.check(lib.shoccs_problem_block_meta(self._h, d, None, ctypes.byref(nl), None,
                                                  ctypes.byref(nc)))
        meta = np.zeros((nl.value, 13), dtype=np.int32)
        coeffs = np.zeros(nc.value)
        _capi.check(lib.shoccs_problem_block_meta(
            self._h, d, meta.ctypes.data_as(_capi.c_int_p), None,
            coeffs.ctypes.data_as(_capi.c_double_p), None))
        return meta, coeffs

    def csr(self, d, which):
        """which: 0 B, 1 N, 2..4 Bf(r), 5..7 Br(r) -> (rows, row_offsets, cols, vals)"""
        import numpy as np
        rows, nnz = ctypes.c_int64(), ctypes.c_int64()
        lib = _capi.lib()
        _capi.check(lib.shoccs_problem_csr(self._h, d, which, ctypes.byref(rows),
                                           ctypes.byref(nnz), None, None, None))
        u = np.zeros(rows.value + 1, dtype=np.int64)
        v = np.zeros(nnz.value, dtype=np.int64)
        w = np.zeros(nnz.value)
        _capi.check(lib.shoccs_problem_csr(self._h, d, which, None, None,
                                           u.ctypes.data_as(_capi.c_int64_p),
                                           v.ctypes.data_as(_capi.c_int64_p),
                                           w.ctypes.data_as(_capi.c_double_p)))
        return rows.value, u, v, w

    def classes(self):
        import numpy as np
        out = np.zeros(self.size, dtype=np.uint8)
        _capi.check(_capi.lib().shoccs_problem_classes(self._h, out.ctypes.data))
        return out

    # --- field helpers (device) ---
    def zeros(self, dtype=None, device="cuda"):
        import torch
        dtype = dtype or torch.float64
        return ScalarField(torch.zeros(self.size, dtype=dtype, device=device),
                           *[torch.zeros(n, dtype=dtype, device=device) for n in self.nR])


class Derivative:
    """ccs::derivative: du (=|+=) D_dir u, optional Neumann data nu (FP64)."""

    def __init__(self, problem, d, prec=PREC_FP64):
        self.p, self.dir, self.prec = problem, d, prec

    def __call__(self, u, du, plus_eq=False, nu=None, stream=None):
        _capi.check(_capi.lib().shoccs_derivative_apply(
            self.p.handle, self.dir, self.prec, _field(u), _field(nu), _field(du),
            1 if plus_eq else 0, _stream(stream)))
        return du


class Laplacian:
    def __init__(self, problem, prec=PREC_FP64):
        self.p, self.prec = problem, prec

    def __call__(self, u, du, nu=None, stream=None):
        _capi.check(_capi.lib().shoccs_laplacian_apply(self.p.handle, self.prec, _field(u),
                                                       _field(nu), _field(du), _stream(stream)))
        return du


class Gradient:
    def __init__(self, problem, prec=PREC_FP64):
        self.p, self.prec = problem, prec

    def __call__(self, u, dx, dy, dz, stream=None):
        _capi.check(_capi.lib().shoccs_gradient_apply(self.p.handle, self.prec, _field(u),
                                                      _field(dx), _field(dy), _field(dz),
                                                      _stream(stream)))
        return dx, dy, dz


class System:
    """A heat or scalar-wave system with its RK4 registers on the device.

    prec: PREC_FP64, or PREC_MIXED (FP32 stage fields and interior rows).  Systems whose
    cut-point values are state (Floating or Neumann objects), with Neumann faces or the
    Gaussian solution step the whole field unfused (stage_kernel "unfused"); their state is
    FP64 in either precision, and a mixed one computes its steps with FP32 stage fields at the
    grid points and FP64 cut points."""

    def __init__(self, problem, kind, prec=PREC_FP64, diffusivity=1.0, vel_kind=VEL_CONSTANT,
                 vel=(0.0, 0.0, 0.0), center=(0.0, 0.0, 0.0), sol_kind=SOL_ZERO,
                 sol=(), max_error=100.0):
        d = _capi.SystemDesc()
        d.kind, d.prec, d.diffusivity = kind, prec, float(diffusivity)
        d.vel_kind = vel_kind
        d.vel[:] = [float(v) for v in vel]
        d.center[:] = [float(v) for v in center]
        d.sol_kind = sol_kind
        terms = None
        if sol_kind == SOL_GAUSSIAN:
            # sol: the Gaussian terms (centre[3], variance[3], amplitude, frequency)
            flat = []
            for c, v, a, f in sol:
                flat += [float(x) for x in c] + [float(x) for x in v] + [float(a), float(f)]
            terms = (ctypes.c_double * max(len(flat), 1))(*flat)
            d.sol_n_terms, d.sol_terms = len(flat) // 8, terms
            sol = ()
        sol = list(sol) + [0.0] * (8 - len(sol))
        d.sol[:] = [float(v) for v in sol]
        d.max_error = float(max_error)
        self.desc = d
        self._terms = terms  # the desc points at them
        self.p = problem
        h = ctypes.c_void_p()
        _capi.check(_capi.lib().shoccs_system_create(problem.handle, ctypes.byref(d),
                                                     ctypes.byref(h)))
        self._h = h

    @property
    def handle(self):
        return self._h

    def __del__(self):
        if getattr(self, "_h", None):
            _capi.lib().shoccs_system_destroy(self._h)
            self._h = None

    def initialize(self, t=0.0, stream=None):
        _capi.check(_capi.lib().shoccs_system_initialize(self._h, float(t), _stream(stream)))

    def set_state(self, u, stream=None):
        where = 1 if getattr(u.D, "is_cuda", False) else 0
        f = _field(u) if where == 1 else ctypes.byref(_capi.Field(*[_np_ptr(a) for a in u]))
        _capi.check(_capi.lib().shoccs_system_set_state(self._h, f, where, _stream(stream)))

    def get_state(self, u, stream=None):
        where = 1 if getattr(u.D, "is_cuda", False) else 0
        f = _field(u) if where == 1 else ctypes.byref(_capi.Field(*[_np_ptr(a) for a in u]))
        _capi.check(_capi.lib().shoccs_system_get_state(self._h, f, where, _stream(stream)))
        return u

    def error_field(self, t, err, stream=None):
        """err <- |u - exact(t)| at the fluid D points and the non-Dirichlet cut points, 0
        elsewhere (the Error field of the reference's system::write); FP64 host arrays or
        CUDA tensors"""
        where = 1 if getattr(err.D, "is_cuda", False) else 0
        f = _field(err) if where == 1 else ctypes.byref(_capi.Field(*[_np_ptr(a) for a in err]))
        _capi.check(_capi.lib().shoccs_system_error_field(self._h, float(t), f, where,
                                                          _stream(stream)))
        return err

    def rk4(self, t0, dt, nsteps, stream=None):
        _capi.check(_capi.lib().shoccs_system_rk4(self._h, float(t0), float(dt), int(nsteps),
                                                  _stream(stream)))

    def euler(self, t0, dt, nsteps, stream=None):
        """forward Euler steps (integrators::euler), FP64 systems"""
        _capi.check(_capi.lib().shoccs_system_euler(self._h, float(t0), float(dt), int(nsteps),
                                                    _stream(stream)))

    def rk4_timed(self, t0, dt, nsteps, stream=None):
        """rk4 with per-kernel CUDA-event timing: returns dict of total milliseconds."""
        ms = (ctypes.c_double * 6)()
        _capi.check(_capi.lib().shoccs_system_rk4_timed(self._h, float(t0), float(dt),
                                                        int(nsteps), _stream(stream), ms))
        return dict(aux=ms[0], stage0=ms[1], stage1=ms[2], stage2=ms[3], stage3=ms[4],
                    total=ms[5])

    def rhs(self, t, out, stream=None):
        _capi.check(_capi.lib().shoccs_system_rhs(self._h, float(t), _field(out),
                                                  _stream(stream)))
        return out

    def stats(self, t, stream=None):
        out = (ctypes.c_double * 11)()
        st = _capi.lib().shoccs_system_stats(self._h, float(t), out, _stream(stream))
        vals = list(out)
        if st not in (_capi.OK, _capi.ENONFINITE):
            _capi.check(st)
        return vals, st == _capi.OK

    STAGE_KERNELS = {0: "point", 1: "tma", 2: "col1", 3: "col2", 4: "col4", 5: "vec",
                     6: "vec3", 7: "unfused", 8: "vecx2", 9: "vecx4"}

    @property
    def stage_kernel(self):
        """name of the stage-kernel variant this system runs (see shoccs_system_path)"""
        v = ctypes.c_int()
        _capi.check(_capi.lib().shoccs_system_path(self._h, ctypes.byref(v)))
        return self.STAGE_KERNELS[v.value]

    # --- discrete adjoint (FP64 heat systems) ---
    def rhs_transpose(self, x, y, stream=None):
        """y = A^T x, A the linear part of rhs (fields of FP64 CUDA tensors)"""
        _capi.check(_capi.lib().shoccs_system_rhs_transpose(self._h, _field(x), _field(y),
                                                            _stream(stream)))
        return y

    def forward(self, t0, dt, nsteps, checkpoint_every=0, stream=None):
        """rk4 from the current state, recording a Tape for backward()"""
        h = ctypes.c_void_p()
        _capi.check(_capi.lib().shoccs_system_forward(self._h, float(t0), float(dt),
                                                      int(nsteps), int(checkpoint_every),
                                                      ctypes.byref(h), _stream(stream)))
        return Tape(h)

    def backward(self, tape, grad_uT, grad_u0, stream=None):
        """grad_u0 = (d u(T) / d u(0))^T grad_uT for the forward run recorded in tape"""
        _capi.check(_capi.lib().shoccs_system_backward(self._h, tape.handle, _field(grad_uT),
                                                       _field(grad_u0), _stream(stream)))
        return grad_u0

    def timestep(self, cfl):
        dt = ctypes.c_double()
        _capi.check(_capi.lib().shoccs_system_timestep(self._h, float(cfl), ctypes.byref(dt)))
        return dt.value


def _np_ptr(a):
    if a is None:
        return None
    if hasattr(a, "data_ptr"):
        return a.data_ptr() if a.numel() else None
    return a.ctypes.data if a.size else None


class Tape:
    """Record of a forward run (step size, step count, checkpoints every k steps)."""

    def __init__(self, h):
        self._h = h

    @property
    def handle(self):
        return self._h

    def __len__(self):
        n = ctypes.c_int()
        _capi.check(_capi.lib().shoccs_tape_checkpoint(self._h, 0, None, ctypes.byref(n), None))
        return n.value

    def checkpoint(self, i, out):
        """copy checkpoint i (D array) into the FP64 CUDA tensor out"""
        _capi.check(_capi.lib().shoccs_tape_checkpoint(self._h, int(i), _ptr(out), None, None))
        return out

    def __del__(self):
        if getattr(self, "_h", None):
            _capi.lib().shoccs_tape_destroy(self._h)
            self._h = None


class Heat(System):
    """systems::heat: u_t = k lap(u) + source of the manufactured solution."""

    def __init__(self, problem, diffusivity=1.0, prec=PREC_FP64, sol_kind=SOL_ZERO, sol=()):
        super().__init__(problem, _capi.SYS_HEAT, prec=prec, diffusivity=diffusivity,
                         sol_kind=sol_kind, sol=sol)


class ScalarWave(System):
    """systems::scalar_wave: u_t = gG . grad(u); gG = -a (constant velocity a) or the
    reference's radial -(x-c)/|x-c|."""

    def __init__(self, problem, prec=PREC_FP64, vel_kind=VEL_CONSTANT, vel=(0, 0, 0),
                 center=(0, 0, 0), sol_kind=SOL_ZERO, sol=(), max_error=100.0):
        super().__init__(problem, _capi.SYS_WAVE, prec=prec, vel_kind=vel_kind, vel=vel,
                         center=center, sol_kind=sol_kind, sol=sol, max_error=max_error)


class Batch:
    """Independent heat systems (sin-sin manufactured solution) advanced together: one launch
    per stage for the whole batch, the RK4 loop captured as a CUDA graph (see
    shoccs_batch_create in include/shoccs_gpu.h).  The systems must outlive the batch."""

    def __init__(self, systems):
        self.systems = list(systems)
        arr = (ctypes.c_void_p * len(self.systems))(*[s.handle.value for s in self.systems])
        h = ctypes.c_void_p()
        _capi.check(_capi.lib().shoccs_batch_create(arr, len(self.systems), ctypes.byref(h)))
        self._h = h

    def __del__(self):
        if getattr(self, "_h", None):
            _capi.lib().shoccs_batch_destroy(self._h)
            self._h = None

    def rk4(self, t0, dt, nsteps, stream=None):
        n = len(self.systems)
        t0 = [float(t0)] * n if not hasattr(t0, "__len__") else [float(v) for v in t0]
        dt = [float(dt)] * n if not hasattr(dt, "__len__") else [float(v) for v in dt]
        a, b = (ctypes.c_double * n)(*t0), (ctypes.c_double * n)(*dt)
        _capi.check(_capi.lib().shoccs_batch_rk4(self._h, a, b, int(nsteps), _stream(stream)))

    def info(self):
        v = (ctypes.c_int64 * 6)()
        _capi.check(_capi.lib().shoccs_batch_info(self._h, v))
        return dict(instances=v[0], tiles=v[1], cut_rows=v[2], tile_warps=v[3], grid=v[4],
                    graph_nodes=v[5])


def kernel_launches():
    return int(_capi.lib().shoccs_kernel_launches())


def rk4_solve(system, u0, t0, dt, nsteps, checkpoint_every=0):
    """torch.autograd-compatible RK4 solve: u(T) from the D array u0 (FP64 CUDA tensor);
    backward maps dL/du(T) to dL/du0 through the system's discrete adjoint."""
    import torch

    class _Solve(torch.autograd.Function):
        @staticmethod
        def forward(ctx, u):
            p = system.p
            R = [torch.zeros(n, dtype=torch.float64, device=u.device) for n in p.nR]
            system.set_state(ScalarField(u.detach().contiguous(), *R))
            ctx.tape = system.forward(t0, dt, nsteps, checkpoint_every)
            out = ScalarField(torch.empty_like(u), *R)
            system.get_state(out)
            return out.D

        @staticmethod
        def backward(ctx, g):
            p = system.p
            R = [torch.zeros(n, dtype=torch.float64, device=g.device) for n in p.nR]
            gu = torch.empty_like(g)
            system.backward(ctx.tape, ScalarField(g.contiguous(), *R), ScalarField(gu, *R))
            return gu

    return _Solve.apply(u0)


class Graph:
    """Operator applies and system right-hand sides recorded with their buffers and replayed
    as one captured CUDA graph (the reference's add_graph_nodes / build_graph /
    submit_graph; see shoccs_graph_* in include/shoccs_gpu.h).  The fields handed to the add_*
    methods must stay alive and in place while the graph exists."""

    def __init__(self):
        h = ctypes.c_void_p()
        _capi.check(_capi.lib().shoccs_graph_create(ctypes.byref(h)))
        self._h = h
        self._keep = []

    def __del__(self):
        if getattr(self, "_h", None):
            _capi.lib().shoccs_graph_destroy(self._h)
            self._h = None

    def add_derivative(self, problem, d, u, du, nu=None, plus_eq=False, prec=PREC_FP64):
        self._keep += [u, du, nu]
        _capi.check(_capi.lib().shoccs_graph_add_derivative(self._h, problem.handle, d, prec,
                                                            _field(u), _field(nu), _field(du),
                                                            1 if plus_eq else 0))
        return self

    def add_laplacian(self, problem, u, du, nu=None, prec=PREC_FP64):
        self._keep += [u, du, nu]
        _capi.check(_capi.lib().shoccs_graph_add_laplacian(self._h, problem.handle, prec,
                                                           _field(u), _field(nu), _field(du)))
        return self

    def add_gradient(self, problem, u, dx, dy, dz, prec=PREC_FP64):
        self._keep += [u, dx, dy, dz]
        _capi.check(_capi.lib().shoccs_graph_add_gradient(self._h, problem.handle, prec,
                                                          _field(u), _field(dx), _field(dy),
                                                          _field(dz)))
        return self

    def add_rhs(self, system, du):
        self._keep += [system, du]
        _capi.check(_capi.lib().shoccs_graph_add_rhs(self._h, system._h, _field(du)))
        return self

    def submit(self, t=0.0, stream=None):
        _capi.check(_capi.lib().shoccs_graph_submit(self._h, float(t), _stream(stream)))

    def info(self):
        """(recorded applies, captured graph nodes, captures so far)"""
        v = (ctypes.c_int64 * 3)()
        _capi.check(_capi.lib().shoccs_graph_info(self._h, v))
        return tuple(v)


__all__ = ["Problem", "Derivative", "Laplacian", "Gradient", "Heat", "ScalarWave", "System",
           "Batch", "Tape", "Graph", "rk4_solve", "ScalarField", "ShoccsError", "kernel_launches"]
