"""Benchmark: 3-D scalar-wave RK4 on one GB300 (the wave workload of the suite).

Workload (synthetic, generated from its parameters): u_t + a.grad u = 0 with
a = (1, 0.7, 0.4) on a 256^3 grid over [0,1]^3, a Dirichlet sphere (centre 0.5, r = 0.3),
Dirichlet inflow faces xmin/ymin/zmin and Floating outflow faces, a Gaussian pulse
(centre 0.2, sigma 0.05) as initial data and exact boundary data, E4_1 (alpha = 0.1, 0.7),
dt = 0.5 h, 1000 RK4 steps.

One benchmark "step" is one full solve of that workload (initial condition + 1000 RK4
steps).  value = RK4 DOF-updates/s = nx*ny*nz * 1000 * K / time of the mixed-precision
path (FP32 stage fields; interior and domain-wall rows in FP32 in difference form; cut-cell
rows from FP32-pair coefficients with compensated FP32 products and sums, ~44 bits; FP32
stage accumulator; compensated FP32-pair solution), with every buffer resident in HBM (the
working set, ~470 MB, is larger than the 129 MB L2).  The FP64 path is timed beside it; both report their max-norm
error against the exact solution.  e2e repeats the mixed solve through the C ABI with the
initial state copied from pinned host memory and the final state copied back inside the
timed region.

The reference's E4_1 closures are unstable under explicit RK4 on this geometry (walls are
evaluated at psi = 1, which its psi clamp turns into ~1e5/h coefficients, and small cut
cells give large ones), so the workload's solution overflows within a few dozen steps in
the reference algorithm and here alike; kernel time does not depend on the values.  The
mixed-versus-FP64 equal-accuracy criterion is therefore measured on two stable companions
on the same 256^3 grid: the same pulse and velocity with the reference's E4u_1 scheme and no
embedded sphere, 300 RK4 steps; and the heat equation around a Dirichlet sphere with E4_2
cut-cell rows (the reference's heat system), manufactured solution sin 2 pi x sin 2 pi y
sin 2 pi z e^-t, dt = 0.1 h^2, 200 RK4 steps, both precisions timed.

--impl reference times the reference algorithm's CPU path (the oracle restatement of
pbrady/shoccs, OpenMP over all host cores) on the same workload, one RK4 step per
benchmark step, bounded to about a minute in total.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

METRIC = "RK4 DOF-updates/s (3-D scalar wave, 256^3, sphere, E4_1)"
UNIT = "DOF-updates/s"
N_GRID = 256
N_STEPS = 1000
VEL = (1.0, 0.7, 0.4)
PULSE = [0.2, 0.2, 0.2, 1.0, 0.7, 0.4, 0.05]
CASE = dict(n=(N_GRID, N_GRID, N_GRID), lo=(0, 0, 0), hi=(1, 1, 1),
            spheres=[((0.5, 0.5, 0.5), 0.3, "dirichlet")],
            grid_bc=("dirichlet", "floating", "dirichlet", "floating", "dirichlet", "floating"),
            scheme="E4_1", alpha=(0.1, 0.7))
ACC_CASE = dict(n=(N_GRID, N_GRID, N_GRID), lo=(0, 0, 0), hi=(1, 1, 1), spheres=[],
                grid_bc=("dirichlet", "floating", "dirichlet", "floating", "dirichlet",
                         "floating"),
                scheme="E4u_1", alpha=(-0.7733323791884821, 0.1623961700641681))
ACC_STEPS = 300
# the cut-cell equal-accuracy companion: heat, E4_2, Dirichlet walls and sphere (off the grid
# points), sin-sin-sin e^-t, dt = 0.1 h^2
HEAT_ACC_CASE = dict(n=(N_GRID, N_GRID, N_GRID), lo=(0, 0, 0), hi=(1, 1, 1),
                     spheres=[((0.51, 0.49, 0.503), 0.3, "dirichlet")],
                     grid_bc=("dirichlet",) * 6, scheme="E4_2")
HEAT_ACC_STEPS = 200
# algorithmic HBM bytes per grid point per RK4 step (u0, accumulator, stage field each read
# and written once per stage): FP64 (8-byte everything) 8+8+8 | 24+16 | 24+16 | 24+8 = 136;
# mixed (4-byte stage field and accumulator, 8-byte compensated u0 of which stages 0-2 read
# only the 4-byte hi word)
# 4+4+4 | 12+8 | 12+8 | 16+8 = 76
BYTES_PT_STEP = {"mixed": 76, "fp64": 136}
BYTES_PT_STAGE = {"mixed": [12, 20, 20, 24], "fp64": [24, 40, 40, 32]}


def config(nsteps):
    return {"workload": "scalar_wave_3d_256cubed_sphere_E4_1", "grid": [N_GRID] * 3,
            "rk4_steps_per_solve": nsteps, "velocity": list(VEL), "sphere_radius": 0.3,
            "pulse_sigma": 0.05, "dt": "0.5*h", "l2": "working set > L2 (no flush needed)",
            "replicas": "one independent solve per GPU"}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


# ---- replicas: every rank runs its own solves; no collective touches the data path ----
def reduce_max(x, pg=None, device="cuda"):
    """the maximum of x over the ranks (x itself without a process group)"""
    if pg is None:
        return float(x)
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def reduce_sum(x, pg=None, device="cuda"):
    if pg is None:
        return float(x)
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    pg.all_reduce(t, op=pg.ReduceOp.SUM)
    return float(t.item())


def replica_rate(local_units, local_seconds, pg=None, device="cuda"):
    """whole-job rate: the units all ranks processed over the slowest rank's time"""
    return reduce_sum(local_units, pg, device) / reduce_max(local_seconds, pg, device)


def partition(count, rank, world):
    """the instances a rank owns when independent instances are spread over ranks"""
    return list(range(rank, count, world))


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons, power = [], None, set(), []
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in self.lines:
            f = [x.strip() for x in l.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
                power.append(float(f[3]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        sm.sort()
        return {"sm_mhz": sm[len(sm) // 2] if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm),
                "power_w_max": max(power) if power else None}


def measured_peak():
    p = os.path.join(HERE, "MEASURED_PEAKS.json")
    try:
        return float(json.load(open(p))["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def committed_traffic():
    p = os.path.join(HERE, "profiles", "stage_kernel_traffic.json")
    try:
        return json.load(open(p))
    except Exception:
        return None


def cpu_rate(nsteps_cap, time_budget):
    """Oracle (the reference algorithm on the host cores) on the benchmark workload."""
    from oracle import oracle as orc
    threads = orc.set_threads(os.cpu_count() or 1)
    o = orc.OracleProblem(**CASE)
    u0 = o.initialize(2, PULSE, 0.0)
    h = 1.0 / (N_GRID - 1)
    dt = 0.5 * h
    t0 = time.perf_counter()
    o.wave_rk4(0, VEL, (0, 0, 0), 2, PULSE, 0.0, dt, 0, u0)  # system setup only
    t_setup = time.perf_counter() - t0
    t0 = time.perf_counter()
    u = o.wave_rk4(0, VEL, (0, 0, 0), 2, PULSE, 0.0, dt, 1, u0)
    t1 = time.perf_counter() - t0 - t_setup
    n = max(1, min(nsteps_cap, int(time_budget / max(t1, 1e-3))))
    t0 = time.perf_counter()
    o.wave_rk4(0, VEL, (0, 0, 0), 2, PULSE, 0.0, dt, n, u0)
    tn = time.perf_counter() - t0 - t_setup
    npts = o.size
    return dict(value=npts * n / tn, unit=UNIT, cores=threads, kind="port",
                sample="%d RK4 step(s) of the 256^3 wave workload (setup excluded), "
                       "%.2f s" % (n, tn)), n, tn


def run_reference(args, rank, ws):
    if rank != 0:
        return 0
    cb, n, tn = cpu_rate(max(1, args.steps), 60.0)
    line = {"impl": "reference", "metric": METRIC, "value": cb["value"], "unit": UNIT,
            "n_gpus": args.gpus, "steps": n, "warmup": 1, "ms_per_step": 1000.0 * tn / n,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": config(1), "cpu_baseline": cb,
            "e2e": {"value": cb["value"], "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0},
            "note": "one benchmark step = one RK4 step of the 256^3 workload on the host; "
                    "the run is capped at about a minute"}
    print(json.dumps(line), flush=True)
    return 0


MICRO_N = 512


def operator_microbench(stream, peak, n=MICRO_N, reps=10):
    """The operator microbenchmark: 512^3 field u ~ U[-1, 1], 8 seeded non-overlapping
    spheres; d/dx, d/dy, d/dz (E4_1, Dirichlet spheres) and the Laplacian (E4_2, spheres
    alternately Dirichlet and Floating), each in FP64 and mixed, through the C ABI.  GB/s
    counts the algorithmic bytes: read u and write du once per point (16 B FP64, 8 B mixed)."""
    import torch
    import shoccs_gb300 as S
    from shoccs_gb300 import workloads as W
    out = {"grid": [n, n, n], "spheres": 8, "field_seed": W.SEED_MICRO_FIELD,
           "sphere_seed": W.SEED_MICRO_SPHERES,
           "bytes_per_point": {"fp64": 16, "mixed": 8}}
    for scheme, bcs, ops in (("E4_1", ("dirichlet",), ("dx", "dy", "dz")),
                             ("E4_2", ("dirichlet", "floating"), ("laplacian",))):
        p = S.Problem(**W.micro_case(n, scheme, bcs))
        N = p.size
        for pname, prec, dtype, B in (("fp64", S.PREC_FP64, torch.float64, 16),
                                      ("mixed", S.PREC_MIXED, torch.float32, 8)):
            u = S.ScalarField(W.micro_field(N, dtype),
                              *[W.micro_field(k, dtype, seed=W.SEED_MICRO_FIELD + 1 + r)
                                for r, k in enumerate(p.nR)])
            du = p.zeros(dtype)
            for op in ops:
                if op == "laplacian":
                    f = lambda: S.Laplacian(p, prec)(u, du, stream=stream)
                else:
                    d = "xyz".index(op[1])
                    f = lambda d=d: S.Derivative(p, d, prec)(u, du, stream=stream)
                for _ in range(2):
                    f()
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                torch.cuda.synchronize()
                e0.record(stream)
                for _ in range(reps):
                    f()
                e1.record(stream)
                e1.synchronize()
                ms = e0.elapsed_time(e1) / reps
                gbs = B * N / (ms / 1000) / 1e9
                out.setdefault(op, {})[pname] = {"ms": ms, "gbs": gbs, "frac": gbs / peak}
            del u, du
        del p
    return out


def batched_bench(stream, count=256, steps=200, pg=None, rank=0, world=1, looped=True,
                  precisions=("fp64", "mixed")):
    """The batched configuration: 256 independent 2-D heat instances (N ~ U{32..192}, one
    circle each, manufactured solution with k in {1, 2, 3}), 200 RK4 steps at dt = 0.1 h^2,
    in FP64 and mixed.  Timed: one run of the batch (a replay of the captured graph) against
    the same instances advanced one system after another."""
    import torch
    import shoccs_gb300 as S
    from shoccs_gb300 import workloads as W
    # over several GPUs the instances are partitioned by rank (no collective on the data)
    insts = [W.batch_heat_2d(count)[i] for i in partition(count, rank, world)]
    probs = [S.Problem(**it["case"]) for it in insts]
    dts = [it["dt"] for it in insts]
    dof = sum(p.size for p in probs) * steps
    out = {"instances": count, "rk4_steps": steps, "points": sum(p.size for p in probs),
           "seed": W.SEED_BATCH}
    for pname, prec in (("fp64", S.PREC_FP64), ("mixed", S.PREC_MIXED)):
        if pname not in precisions:
            continue
        systems = [S.Heat(p, 1.0, prec, S.SOL_SINSIN, [float(it["k"])])
                   for p, it in zip(probs, insts)]
        for s in systems:
            s.initialize(0.0, stream)
        batch = S.Batch(systems)
        batch.rk4(0.0, dts, steps, stream)  # capture + warm-up
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        reps = 3
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(reps):
            batch.rk4(0.0, dts, steps, stream)
        e1.record(stream)
        e1.synchronize()
        ms = reduce_max(e0.elapsed_time(e1) / reps, pg)
        # the same instances one system after another (no batching, no graph)
        ms_loop = float("nan")
        if looped:
            for s in systems[:4]:
                s.rk4(0.0, dts[0], 2, stream)
            torch.cuda.synchronize()
            e0.record(stream)
            for s, dt in zip(systems, dts):
                s.rk4(0.0, dt, steps, stream)
            e1.record(stream)
            e1.synchronize()
            ms_loop = reduce_max(e0.elapsed_time(e1), pg)
        errs = [s.stats(steps * dt, stream)[0][0] for s, dt in zip(systems[:16], dts[:16])]
        info = batch.info()
        dof_all = reduce_sum(dof, pg)
        out[pname] = {"ms_per_run": ms, "dof_updates_per_s": dof_all / (ms / 1000.0),
                      "looped_ms": ms_loop, "looped_dof_updates_per_s": dof_all / (ms_loop / 1000.0),
                      "speedup_vs_looped": ms_loop / ms, "max_error_first16": max(errs),
                      "tile_warps": info["tile_warps"], "graph_nodes": info["graph_nodes"]}
        del batch, systems
    return out


def unfused_bench(stream, n=128, steps=10):
    """Floating closures at scale: FP64 heat, n^3, sphere (0.5, 0.5, 0.5) r = 0.25, sin-sin
    manufactured solution.  With a Floating sphere the cut-point values are state and the
    system runs the unfused whole-field step (standalone Laplacian with its R-space rows, the
    source, whole-field axpys, the boundary update); the same grid with a Dirichlet sphere runs
    the fused FP64 stage kernels and is timed alongside.  `steps` RK4 steps after a warm-up,
    timed with CUDA events on the launching stream (10 steps: this scheme's Floating closure
    grows without bound after a few tens of steps on this geometry).  The Floating sphere is
    also timed in mixed precision (FP32 stage fields at the D points, FP64 cut points and
    state; `floating_unfused_mixed`), next to the fused mixed stages with a Dirichlet sphere."""
    import torch
    import shoccs_gb300 as S
    from shoccs_gb300 import workloads as W
    dt = W.heat_dt(n)
    res = {"grid": [n, n, n], "rk4_steps": steps, "dtype": "f64"}
    for name, bc, prec in (("floating_unfused", "floating", S.PREC_FP64),
                           ("dirichlet_fused", "dirichlet", S.PREC_FP64),
                           ("floating_unfused_mixed", "floating", S.PREC_MIXED),
                           ("dirichlet_fused_mixed", "dirichlet", S.PREC_MIXED)):
        c = dict(W.adjoint_case(n), spheres=[((0.5, 0.5, 0.5), 0.25, bc)])
        p = S.Problem(**c)
        h = S.Heat(p, 1.0, prec, S.SOL_SINSIN, [1.0])
        h.initialize(0.0, stream)
        h.rk4(0.0, dt, 2, stream)  # warm-up
        h.initialize(0.0, stream)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        n0 = S.kernel_launches()
        e0.record(stream)
        h.rk4(0.0, dt, steps, stream)
        e1.record(stream)
        e1.synchronize()
        ms = e0.elapsed_time(e1)
        st, ok = h.stats(steps * dt, stream)
        res[name] = {"ms_per_step": ms / steps, "dof_updates_per_s": (p.size + sum(p.nR)) * steps / (ms * 1e-3),
                     "stage_kernel": h.stage_kernel, "cut_points": int(sum(p.nR)), "max_error": st[0],
                     "valid": bool(ok)}
        res[name]["launches_per_step"] = (S.kernel_launches() - n0) / steps
        del h, p
    res["unfused_over_fused"] = res["floating_unfused"]["ms_per_step"] / res["dirichlet_fused"]["ms_per_step"]
    res["unfused_mixed_speedup_over_fp64"] = (res["floating_unfused"]["ms_per_step"] /
                                              res["floating_unfused_mixed"]["ms_per_step"])
    return res


def adjoint_bench(stream, n=128, steps=200, every=20, ndir=32, eps=1e-6, cg_iters=10):
    """The adjoint configuration: 3-D heat 128^3, sphere r = 0.25, homogeneous Dirichlet,
    u0 = seeded sum of 16 Gaussians, 200 RK4 steps (FP64) with a checkpoint every 20.
    J(u0) = 1/2 ||u(T) - u_obs||^2 over the fluid points, u_obs = u(T) of the true u0.
    Reports the forward and backward (gradient) times, central finite differences of J
    along 32 seeded directions against the adjoint gradient, and an initial-condition
    inversion by conjugate gradients on the normal equations started from u0 = 0."""
    import numpy as np
    import torch
    import shoccs_gb300 as S
    from shoccs_gb300 import workloads as W
    p = S.Problem(**W.adjoint_case(n))
    sys_ = S.Heat(p, 1.0, S.PREC_FP64, S.SOL_ZERO)
    dt = W.heat_dt(n)
    dev = "cuda"
    R = [torch.zeros(k, dtype=torch.float64, device=dev) for k in p.nR]
    fluid = torch.tensor((p.classes() & 0x80) != 0, dtype=torch.float64, device=dev)
    u_true = torch.tensor(W.adjoint_u0(n), dtype=torch.float64, device=dev)
    out = torch.empty_like(u_true)

    def forward(u0, ckpt=every):
        sys_.set_state(S.ScalarField(u0, *R), stream)
        tape = sys_.forward(0.0, dt, steps, ckpt, stream)
        sys_.get_state(S.ScalarField(out, *R), stream)
        return tape, out.clone()

    _, u_obs = forward(u_true)

    def loss_grad(u0, grad=True):
        tape, uT = forward(u0)
        r = (uT - u_obs) * fluid
        J = 0.5 * float(torch.dot(r, r))
        if not grad:
            return J, None
        g = torch.empty_like(u0)
        sys_.backward(tape, S.ScalarField(r, *R), S.ScalarField(g, *R), stream)
        return J, g

    # timing: forward (with checkpoints) and backward of one gradient
    u0 = 0.5 * u_true
    loss_grad(u0)
    e = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    torch.cuda.synchronize()
    e[0].record(stream)
    tape, uT = forward(u0)
    e[1].record(stream)
    r = (uT - u_obs) * fluid
    g = torch.empty_like(u0)
    sys_.backward(tape, S.ScalarField(r, *R), S.ScalarField(g, *R), stream)
    e[2].record(stream)
    e[2].synchronize()
    t_fwd, t_bwd = e[0].elapsed_time(e[1]), e[1].elapsed_time(e[2])
    # finite differences along seeded random directions
    J0, g = loss_grad(u0)
    gen = torch.Generator(device=dev)
    gen.manual_seed(W.SEED_ADJOINT_DIRECTIONS)
    rel = []
    # directions: seeded random sums of 16 Gaussian bumps (centres U[0.1, 0.9]^3, widths
    # U[0.03, 0.1], weights N(0, 1)) -- white-noise directions lie almost entirely in modes
    # that 200 heat steps damp below rounding, where neither the gradient nor a finite
    # difference carries information
    xs = torch.linspace(0.0, 1.0, n, dtype=torch.float64, device=dev)
    X, Y, Z = torch.meshgrid(xs, xs, xs, indexing="ij")
    X, Y, Z = X.reshape(-1), Y.reshape(-1), Z.reshape(-1)

    def direction():
        c = 0.1 + 0.8 * torch.rand(16, 3, dtype=torch.float64, device=dev, generator=gen)
        sg = 0.03 + 0.07 * torch.rand(16, dtype=torch.float64, device=dev, generator=gen)
        a = torch.randn(16, dtype=torch.float64, device=dev, generator=gen)
        v = torch.zeros(p.size, dtype=torch.float64, device=dev)
        for m in range(16):
            d2 = (X - c[m, 0]) ** 2 + (Y - c[m, 1]) ** 2 + (Z - c[m, 2]) ** 2
            v += a[m] * torch.exp(-d2 / (2 * sg[m] ** 2))
        return v / torch.linalg.norm(v)

    for _ in range(ndir):
        v = direction()
        # J(u0 + eps v) - J(u0 - eps v) = 1/2 (r+ - r-) . (r+ + r-) exactly; evaluated in
        # that form the difference keeps its digits (J itself is ~1e3 while the difference is
        # ~1e-8: subtracting two J values would leave rounding noise)
        _, up = forward(u0 + eps * v)
        _, um = forward(u0 - eps * v)
        rp, rm = (up - u_obs) * fluid, (um - u_obs) * fluid
        fd = 0.5 * float(torch.dot(rp - rm, rp + rm)) / (2 * eps)
        gv = float(torch.dot(g, v))
        rel.append(abs(fd - gv) / max(abs(gv), 1e-300))
    # inversion: CG on (F^T F) u0 = F^T u_obs from u0 = 0 (F: the linear solve)
    x = torch.zeros_like(u_true)
    Jx, gx = loss_grad(x)
    J_start = Jx
    rvec = -gx
    pvec = rvec.clone()
    for _ in range(cg_iters):
        # F^T F p = gradient at p of 1/2 ||F p||^2: a solve and an adjoint from the zero
        # observation, computed as the gradient difference along p
        _, gp = loss_grad(x + pvec)
        Ap = gp - gx
        alpha = float(torch.dot(rvec, rvec)) / float(torch.dot(pvec, Ap))
        x = x + alpha * pvec
        r_new = rvec - alpha * Ap
        beta = float(torch.dot(r_new, r_new)) / float(torch.dot(rvec, rvec))
        pvec = r_new + beta * pvec
        rvec = r_new
        Jx, gx = loss_grad(x)
    err0 = float(torch.linalg.norm(u_true * fluid))
    # the mixed system: FP32 stage fields forward, FP32 reverse sweep
    sysm = S.Heat(p, 1.0, S.PREC_MIXED, S.SOL_ZERO)
    sysm.set_state(S.ScalarField(u0, *R), stream)
    tm = sysm.forward(0.0, dt, steps, every, stream)
    gw = torch.empty_like(u0)  # warm-up: the first backward builds the transposed closure
    sysm.backward(tm, S.ScalarField(torch.zeros_like(u0), *R), S.ScalarField(gw, *R), stream)
    torch.cuda.synchronize()
    e[0].record(stream)
    sysm.set_state(S.ScalarField(u0, *R), stream)
    tm = sysm.forward(0.0, dt, steps, every, stream)
    e[1].record(stream)
    uTm = torch.empty_like(u0)
    sysm.get_state(S.ScalarField(uTm, *R), stream)
    rm_ = (uTm - u_obs) * fluid
    g32 = torch.empty_like(u0)
    e[1].record(stream)
    sysm.backward(tm, S.ScalarField(rm_, *R), S.ScalarField(g32, *R), stream)
    e[2].record(stream)
    e[2].synchronize()
    _, g64 = loss_grad(u0)
    mixed = {"forward_ms": e[0].elapsed_time(e[1]), "backward_ms": e[1].elapsed_time(e[2]),
             "gradient_rel_diff_vs_fp64": float(torch.linalg.norm(g32 - g64) / torch.linalg.norm(g64))}
    mixed["backward_over_forward"] = mixed["backward_ms"] / mixed["forward_ms"]
    return {"grid": [n, n, n], "rk4_steps": steps, "checkpoint_every": every,
            "dtype": "f64", "forward_ms": t_fwd, "backward_ms": t_bwd,
            "backward_over_forward": t_bwd / t_fwd, "mixed": mixed,
            "fd_check": {"directions": ndir, "eps": eps, "max_rel_error": max(rel),
                         "median_rel_error": sorted(rel)[len(rel) // 2]},
            "inversion": {"method": "conjugate gradients on the normal equations",
                          "iterations": cg_iters, "J_start": J_start, "J_end": Jx,
                          "u0_rel_error": float(torch.linalg.norm((x - u_true) * fluid)) / err0}}


def heat_sphere_accuracy(stream, steps=HEAT_ACC_STEPS):
    """Mixed against FP64 where cut cells exist: the heat equation on 256^3 around a
    Dirichlet sphere (E4_2 cut-cell rows), each precision timed over `steps` RK4 steps with
    CUDA events on the launching stream after one warm-up solve; max-norm errors against the
    exact solution at the end."""
    import torch
    import shoccs_gb300 as S
    p = S.Problem(**HEAT_ACC_CASE)
    h = 1.0 / (N_GRID - 1)
    dt = 0.1 * h * h
    out = {"case": "256^3 heat, E4_2, Dirichlet sphere r = 0.3, sin-sin-sin e^-t, "
                   "dt = 0.1 h^2, %d RK4 steps" % steps, "cut_points": int(sum(p.nR))}
    for name, prec in (("fp64", S.PREC_FP64), ("mixed", S.PREC_MIXED)):
        hs = S.Heat(p, 1.0, prec, S.SOL_SINSIN, [1.0])
        hs.initialize(0.0, stream)
        hs.rk4(0.0, dt, 4, stream)
        hs.initialize(0.0, stream)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        hs.rk4(0.0, dt, steps, stream)
        e1.record(stream)
        e1.synchronize()
        ms = e0.elapsed_time(e1)
        st, ok = hs.stats(steps * dt, stream)
        out[name] = {"max_error": st[0], "valid": bool(ok), "ms_per_step": ms / steps,
                     "dof_updates_per_s": p.size * steps / (ms * 1e-3),
                     "stage_kernel": hs.stage_kernel}
        del hs
    out["error_ratio_mixed_vs_fp64"] = out["mixed"]["max_error"] / out["fp64"]["max_error"]
    out["speedup_mixed_vs_fp64"] = out["mixed"]["dof_updates_per_s"] / out["fp64"]["dof_updates_per_s"]
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--rk4-steps", type=int, default=N_STEPS)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--only-mixed", action="store_true",
                    help="time the mixed solves only (used for short profiling runs)")
    ap.add_argument("--no-micro", action="store_true", help="skip the operator microbenchmark")
    ap.add_argument("--micro-only", action="store_true",
                    help="run the operator microbenchmark alone and print its JSON")
    ap.add_argument("--no-batched", action="store_true", help="skip the batched heat solves")
    ap.add_argument("--no-adjoint", action="store_true", help="skip the adjoint configuration")
    ap.add_argument("--no-unfused", action="store_true",
                    help="skip the Floating-sphere (unfused FP64 step) timing")
    ap.add_argument("--unfused-only", action="store_true",
                    help="only the Floating-sphere (unfused FP64 step) timing")
    ap.add_argument("--adjoint-only", action="store_true",
                    help="run the adjoint configuration alone and print its JSON")
    ap.add_argument("--batched-only", action="store_true",
                    help="run the batched heat solves alone and print their JSON")
    ap.add_argument("--batch-steps", type=int, default=200,
                    help="RK4 steps of the batched section (--batched-only)")
    ap.add_argument("--batch-no-loop", action="store_true",
                    help="skip the one-system-after-another comparison (--batched-only)")
    ap.add_argument("--batch-prec", default="fp64,mixed",
                    help="precisions of the batched section (--batched-only)")
    args = ap.parse_args()
    ws, rank, local = dist_env()
    if args.impl == "reference":
        return run_reference(args, rank, ws)

    import numpy as np
    import torch
    import shoccs_gb300 as S

    torch.cuda.set_device(local)
    pg = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
        pg = dist

    def barrier():
        if pg:
            pg.barrier()
        torch.cuda.synchronize()

    if args.micro_only or args.batched_only or args.adjoint_only or args.unfused_only:
        st = torch.cuda.Stream()
        with torch.cuda.stream(st):  # torch arithmetic and library calls on one stream
            if args.unfused_only:
                print(json.dumps(unfused_bench(st)), flush=True)
            elif args.micro_only:
                peak, _ = measured_peak()
                print(json.dumps(operator_microbench(st, peak)), flush=True)
            elif args.batched_only:
                print(json.dumps(batched_bench(st, steps=args.batch_steps, looped=not args.batch_no_loop,
                                               precisions=args.batch_prec.split(","))), flush=True)
            else:
                print(json.dumps(adjoint_bench(st)), flush=True)
        return 0

    nsteps = args.rk4_steps
    p = S.Problem(**CASE)
    N = p.size
    h = 1.0 / (N_GRID - 1)
    dt = 0.5 * h
    stream = torch.cuda.Stream()
    sysm = S.ScalarWave(p, S.PREC_MIXED, S.VEL_CONSTANT, VEL, (0, 0, 0), S.SOL_GAUSS_PULSE,
                        PULSE)
    sysd = S.ScalarWave(p, S.PREC_FP64, S.VEL_CONSTANT, VEL, (0, 0, 0), S.SOL_GAUSS_PULSE,
                        PULSE)

    def solve(sys_, timed=False):
        sys_.initialize(0.0, stream)
        if timed:
            return sys_.rk4_timed(0.0, dt, nsteps, stream)
        sys_.rk4(0.0, dt, nsteps, stream)
        return None

    # warm-up (mixed)
    for _ in range(args.warmup):
        solve(sysm)
    barrier()

    # ---- timed region: K mixed solves, CUDA events on the launching stream ----
    clocks = ClockSampler(local)
    clocks.start()
    l0 = S.kernel_launches()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier()
    ev0.record(stream)
    for _ in range(args.steps):
        solve(sysm)
    ev1.record(stream)
    barrier()
    t_ms = ev0.elapsed_time(ev1)
    launches = S.kernel_launches() - l0
    clk = clocks.stop()
    # per-kernel CUDA-event breakdown (for the roofline) from one more solve, outside the
    # timed region: its per-step event records would otherwise add their own cost to value
    kms = {"aux": 0.0, "stage0": 0.0, "stage1": 0.0, "stage2": 0.0, "stage3": 0.0}
    r = solve(sysm, timed=True)
    for k in kms:
        kms[k] = r[k] * args.steps  # scaled to the timed solves
    if pg:
        tt = torch.tensor([t_ms], device="cuda")
        pg.all_reduce(tt, op=pg.ReduceOp.MAX)
        t_ms = float(tt.item())
    t_end = nsteps * dt
    stats_m, valid_m = sysm.stats(t_end, stream)

    if args.only_mixed:
        value = N * nsteps * args.steps * ws / (t_ms / 1000.0)
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws,
                              "steps": args.steps, "warmup": args.warmup,
                              "ms_per_step": t_ms / args.steps, "higher_is_better": True,
                              "config": config(nsteps), "gpu_launches": int(launches),
                              "kernel_ms": kms, "stage_kernel": sysm.stage_kernel,
                              "note": "mixed solves only"}), flush=True)
        return 0

    # ---- FP64 path (timed beside it) ----
    for _ in range(max(1, min(args.warmup, 1))):
        solve(sysd)
    barrier()
    n64 = max(1, min(args.steps, 2))
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    kms64 = {"aux": 0.0, "stage0": 0.0, "stage1": 0.0, "stage2": 0.0, "stage3": 0.0}
    for _ in range(n64):
        r = solve(sysd, timed=True)
        for k in kms64:
            kms64[k] += r[k]
    e1.record(stream)
    barrier()
    t64_ms = e0.elapsed_time(e1)
    stats_d, valid_d = sysd.stats(t_end, stream)

    # ---- equal-accuracy companion (stable scheme, same grid and kernels) ----
    pa = S.Problem(**ACC_CASE)
    acc = {}
    for name, prec in (("fp64", S.PREC_FP64), ("mixed", S.PREC_MIXED)):
        sa_ = S.ScalarWave(pa, prec, S.VEL_CONSTANT, VEL, (0, 0, 0), S.SOL_GAUSS_PULSE, PULSE)
        sa_.initialize(0.0, stream)
        sa_.rk4(0.0, dt, ACC_STEPS, stream)
        st_, ok_ = sa_.stats(ACC_STEPS * dt, stream)
        acc[name] = {"max_error": st_[0], "valid": bool(ok_)}
        del sa_
    acc["error_ratio_mixed_vs_fp64"] = acc["mixed"]["max_error"] / acc["fp64"]["max_error"]
    acc["case"] = "256^3, E4u_1 (alpha -0.7733, 0.1624), no sphere, %d RK4 steps" % ACC_STEPS
    del pa
    acc_cc = heat_sphere_accuracy(stream)

    # ---- e2e through the C ABI with host buffers ----
    host_in = [torch.empty(N, dtype=torch.float64).pin_memory()] + \
              [torch.empty(k, dtype=torch.float64).pin_memory() for k in p.nR]
    host_out = [torch.empty(N, dtype=torch.float64).pin_memory()] + \
               [torch.empty(k, dtype=torch.float64).pin_memory() for k in p.nR]
    sysm.initialize(0.0, stream)
    sysm.get_state(S.ScalarField(*host_in), stream)  # the synthetic initial state on the host
    h2d = sum(a.numel() * 8 for a in host_in)
    d2h = sum(a.numel() * 8 for a in host_out)
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        sysm.set_state(S.ScalarField(*host_in), stream)
        sysm.rk4(0.0, dt, nsteps, stream)
        sysm.get_state(S.ScalarField(*host_out), stream)
    barrier()
    te2e = reduce_max(time.perf_counter() - t0, pg)

    value = N * nsteps * args.steps * ws / (t_ms / 1000.0)
    value64 = N * nsteps * n64 / (t64_ms / 1000.0)
    e2e = N * nsteps * args.steps * ws / te2e

    # roofline of the dominant kernels (the four fused RK4 stage kernels)
    peak, peak_kind = measured_peak()
    stage_ms = sum(kms[k] for k in ("stage0", "stage1", "stage2", "stage3"))
    n_launch = 4 * nsteps * args.steps
    bytes_step = BYTES_PT_STEP["mixed"] * N
    achieved = bytes_step * nsteps * args.steps / (stage_ms / 1000.0) / 1e9
    per_stage = {}
    for i in range(4):
        ms = kms["stage%d" % i] / (nsteps * args.steps)
        per_stage["stage%d" % i] = {"avg_ms": ms,
                                    "gbs": BYTES_PT_STAGE["mixed"][i] * N / (ms / 1000) / 1e9}
    tr = committed_traffic()
    traffic = None
    if tr and tr.get("n_points") == N:
        traffic = tr.get("bytes_per_launch_avg")
    stage64_ms = sum(kms64[k] for k in ("stage0", "stage1", "stage2", "stage3"))
    achieved64 = BYTES_PT_STEP["fp64"] * N * nsteps * n64 / (stage64_ms / 1000.0) / 1e9

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64 (mixed)",
        "data": "synthetic", "config": config(nsteps),
        "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h},
        "gpu_launches": int(launches),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic,
                     "kernel": "mixed RK4 stage kernels, %s variant (4 launches per RK4 step)"
                               % sysm.stage_kernel,
                     "algorithmic_bytes_per_launch_avg": bytes_step / 4,
                     "avg_launch_ms": stage_ms / n_launch, "peak_kind": peak_kind,
                     "per_stage": per_stage},
        "clocks": clk,
        "fp64": {"value": value64, "unit": UNIT, "solves": n64,
                 "ms_per_solve": t64_ms / n64, "roofline_achieved_gbs": achieved64,
                 "roofline_frac": achieved64 / peak, "workload_error": stats_d[0],
                 "valid": bool(valid_d)},
        "mixed": {"workload_error": stats_m[0], "valid": bool(valid_m)},
        "equal_accuracy": acc,
        "equal_accuracy_cut_cells": acc_cc,
        "speedup_mixed_vs_fp64": value / value64,
    }
    del sysm, sysd, p
    # the sections below mix torch tensor arithmetic with library calls: both run on `stream`
    with torch.cuda.stream(stream):
        if not args.no_micro:
            line["operator_microbench"] = operator_microbench(stream, peak)
        if not args.no_batched:
            line["batched"] = batched_bench(stream, pg=pg, rank=rank, world=ws)
        if not args.no_adjoint:
            line["adjoint"] = adjoint_bench(stream)
        if not args.no_unfused:
            try:
                line["floating_closures"] = unfused_bench(stream)
            except Exception as e:  # a secondary figure never costs the headline line
                line["floating_closures"] = {"error": "%s: %s" % (type(e).__name__, e)}
    if rank == 0 and not args.no_cpu_baseline:
        cb, _, _ = cpu_rate(8, 15.0)
        line["cpu_baseline"] = cb
    # the figures the metric names, repeated at the end of the line (a reader that keeps only
    # the line's tail still has them)
    summ = {"value": value, "e2e": e2e, "roofline_frac": achieved / peak,
            "fp64_value": value64, "speedup_mixed_vs_fp64": value / value64,
            "equal_accuracy_ratio_e4u_box": acc["error_ratio_mixed_vs_fp64"],
            "equal_accuracy_ratio_heat_sphere": acc_cc["error_ratio_mixed_vs_fp64"],
            "heat_sphere_speedup_mixed_vs_fp64": acc_cc["speedup_mixed_vs_fp64"]}
    if "batched" in line:
        summ["batched_mixed_dof_updates_per_s"] = line["batched"]["mixed"]["dof_updates_per_s"]
    if "adjoint" in line:
        summ["adjoint_backward_over_forward"] = line["adjoint"]["backward_over_forward"]
        summ["adjoint_mixed_backward_over_forward"] = line["adjoint"]["mixed"]["backward_over_forward"]
    line["summary"] = summ
    if rank == 0:
        print(json.dumps(line), flush=True)
    if pg:
        pg.barrier()
        pg.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
