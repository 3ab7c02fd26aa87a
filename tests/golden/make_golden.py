"""Generate the golden fixtures that pin the oracle (run in a container that has the
reference tree; the fixtures are committed and used on machines that do not).

Sources:
  * src/mesh/object_geometry.t.cpp:11-330 ("sphere intersections"): expected cut-point
    positions, solid coordinates and psi per axis, parsed from the reference test file as
    text -> object_geometry_sphere.json
  * oracle/_ref/libshoccs_ref.so: the reference's own code compiled unmodified by
    oracle/build_ref.sh -> stencils_ref.json (closure blocks, interior rows, interpolants of
    src/stencils/{E2_2,E4_2,E4_1,E4u_1}.cpp), stencils_poly_ref.json (the same of
    src/stencils/polyE2_1.cpp for two parameter sets), stencils_wide_ref.json (E6u_1, E8u_1),
    sphere_hits_ref.json (src/mesh/sphere.cpp ray /
    sphere hits) and reference_pins.json (SHA-256 digests of the arrays of
    tests/golden/pins.py -- setup, operators, heat and scalar-wave systems -- on every case
    of tests/cases.py)

Usage: python tests/golden/make_golden.py [reference_root]
(the reference root defaults to SHOCCS_REFERENCE_ROOT, else the directory `reference` beside
this repository)
"""
import ctypes
import json
import os
import re
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
REF = sys.argv[1] if len(sys.argv) > 1 else os.environ.get(
    "SHOCCS_REFERENCE_ROOT", os.path.join(os.path.dirname(REPO), "reference"))
sys.path.insert(0, REPO)


def parse_sphere_intersections():
    src = open(os.path.join(REF, "src/mesh/object_geometry.t.cpp")).read()
    start = src.index('TEST_CASE("sphere intersections")')
    end = src.index('TEST_CASE("rect_intersections")')
    body = src[start:end]
    out = {}
    sections = re.split(r'SECTION\("([XYZxyz])"\)', body)
    # sections = [pre, name1, text1, name2, text2, ...]
    for name, text in zip(sections[1::2], sections[2::2]):
        def grab(var):
            m = re.search(r"\b%s\s*=\s*\{(.*?)\};" % var, text, re.S)
            return m.group(1) if m else None
        nums = lambda s: [float(v) for v in re.findall(r"-?\d+\.?\d*(?:e-?\d+)?", s)]
        exact = nums(grab("exact"))
        sc = [int(v) for v in re.findall(r"-?\d+", grab("sc"))]
        psi = nums(grab("psi"))
        out[name.lower()] = dict(position=exact, solid_coord=sc, psi=psi)
    return dict(
        source="src/mesh/object_geometry.t.cpp:11-330",
        mesh=dict(n=[21, 22, 23], lo=[-1, -1, 0], hi=[1, 2, 2.2]),
        sphere=dict(center=[0.01, -0.01, 0.5], radius=0.25),
        tolerance=dict(position_abs=1e-14, psi_rel=1.1920929e-05 * 100),
        axes=out,
    )


def ref_fixtures():
    subprocess.check_call(["sh", os.path.join(REPO, "oracle", "build_ref.sh")],
                          env=dict(os.environ, SHOCCS_REFERENCE_ROOT=REF))
    lib = ctypes.CDLL(os.path.join(REPO, "oracle", "_ref", "libshoccs_ref.so"))
    D = ctypes.c_double
    alpha = (D * 2)(0.1, 0.7)
    alpha_u = (D * 2)(-0.7733323791884821, 0.1623961700641681)
    nbs = []
    rt = {0: {0: 4, 1: 8, 2: 8}, 1: {0: 10, 1: 15, 2: 15}, 2: {0: 28, 1: 35},
          3: {0: 10, 1: 15}}
    rng = np.random.default_rng(20261203)
    psis = [1e-12, 1e-5, 0.01, 0.25, 0.5, 0.75, 0.9, 0.999, 1.0 - 1e-12, 1.0]
    psis += list(rng.uniform(0.0, 1.0, 6))
    for scheme, bcs in rt.items():
        for bc, n in bcs.items():
            for psi in psis:
                for right in (0, 1):
                    for h in (2.0, 1.0 / 64, 0.1):
                        c, x = (D * 64)(), (D * 8)()
                        lib.ref_stencil_nbs(scheme, alpha_u if scheme == 3 else alpha, D(h),
                                            bc, D(psi), right, c, x)
                        nbs.append(dict(scheme=scheme, bc=bc, psi=float(psi), right=right,
                                        h=h, c=[float(v).hex() for v in c[:n]],
                                        x=[float(v).hex() for v in x[:3]]))
    interior = []
    for scheme in (0, 1, 2, 3):
        for h in (2.0, 1.0 / 64, 1.0 / 255):
            c = (D * 8)()
            n = lib.ref_stencil_interior(scheme, alpha_u if scheme == 3 else alpha, D(h), c)
            interior.append(dict(scheme=scheme, h=h, c=[float(v).hex() for v in c[:n]]))
    interp = []
    for scheme in (0, 1):
        for y in (-0.7, -0.3, 0.0, 0.2, 0.5, 0.9):
            c = (D * 8)()
            n = lib.ref_stencil_interp_interior(scheme, D(y), c)
            interp.append(dict(kind="interior", scheme=scheme, y=y, c=[float(v).hex() for v in c[:n]]))
            for i in (0, 1, 2):
                for psi in (0.1, 0.5, 0.95):
                    for right in (0, 1):
                        c = (D * 8)()
                        n = lib.ref_stencil_interp_wall(scheme, None, i, D(y), D(psi), right, c)
                        interp.append(dict(kind="wall", scheme=scheme, i=i, y=y, psi=psi,
                                           right=right, c=[float(v).hex() for v in c[:n]]))
    hits = []
    for _ in range(400):
        center = rng.uniform(-0.5, 1.5, 3)
        radius = float(rng.uniform(0.05, 0.6))
        axis = int(rng.integers(0, 3))
        origin = center + rng.uniform(-1.2 * radius, 1.2 * radius, 3)
        origin[axis] = center[axis] - rng.uniform(0.0, 1.5)
        direction = [0.0, 0.0, 0.0]
        direction[axis] = 1.0
        t, pos, ro, nrm = D(), (D * 3)(), ctypes.c_int(), (D * 3)()
        ok = lib.ref_sphere_hit((D * 3)(*center), D(radius), (D * 3)(*origin),
                                (D * 3)(*direction), D(0.0), D(3.0), ctypes.byref(t), pos,
                                ctypes.byref(ro), nrm)
        hits.append(dict(center=[float(v).hex() for v in center], radius=radius.hex(),
                         origin=[float(v).hex() for v in origin], axis=axis, hit=ok,
                         t=t.value.hex(), pos=[v.hex() for v in pos], ray_outside=ro.value,
                         normal=[v.hex() for v in nrm]))
    return (dict(source="src/stencils/{E2_2,E4_2,E4_1,E4u_1}.cpp via oracle/_ref",
                 alpha=[0.1, 0.7], alpha_e4u=[-0.7733323791884821, 0.1623961700641681],
                 nbs=nbs, interior=interior, interp=interp),
            dict(source="src/mesh/sphere.cpp via oracle/_ref", hits=hits))


# the reference's own input files (paths within its tree)
REFERENCE_INPUTS = ["heat.lua", "scalar_wave.lua", "scalar_wave_1d.lua", "eigenvalues.lua",
                    "lua-configs/brady_livescu_4_3_n61.lua", "lua-configs/brady_livescu_4_3.lua"]


# E2-poly (polyE2_1) parameter sets: the one of the reference's scalar_wave.lua (floating,
# dirichlet and interpolant alpha, in the single-array order of stencil.cpp:79-87) and a
# seeded random one
POLY_ALPHA = [
    [0.7039278390946743, 0.5390086175376538, -0.647109821986589, 0.2051508287133347,
     0.6062051039572746, 0.8148425279273044, -0.10739761225713096, 0.8736492896991024,
     0.40413606410467495, 0.01, -0.01, 0.01, 0.04],
    [float(v) for v in np.random.default_rng(20261206).uniform(-1.0, 1.0, 13)],
]


def poly_fixtures():
    """polyE2_1's closure blocks, interior row and interpolants from the reference's own
    src/stencils/polyE2_1.cpp (oracle/_ref) -> stencils_poly_ref.json"""
    subprocess.check_call(["sh", os.path.join(REPO, "oracle", "build_ref.sh")],
                          env=dict(os.environ, SHOCCS_REFERENCE_ROOT=REF))
    lib = ctypes.CDLL(os.path.join(REPO, "oracle", "_ref", "libshoccs_ref.so"))
    D = ctypes.c_double
    rng = np.random.default_rng(20261207)
    psis = [1e-12, 1e-5, 0.01, 0.25, 0.5, 0.75, 0.999, 1.0] + list(rng.uniform(0.0, 1.0, 4))
    out = dict(source="src/stencils/polyE2_1.cpp compiled in oracle/_ref", scheme=5,
               alpha=POLY_ALPHA, nbs=[], interior=[], interp=[])
    for ai, a in enumerate(POLY_ALPHA):
        al = (D * 13)(*a)
        for bc, n in ((0, 8), (1, 12)):
            for psi in psis:
                for right in (0, 1):
                    for h in (2.0, 1.0 / 64, 0.1):
                        c, x = (D * 64)(), (D * 8)()
                        lib.ref_stencil_nbs(5, al, D(h), bc, D(psi), right, c, x)
                        out["nbs"].append(dict(alpha=ai, bc=bc, psi=float(psi), right=right, h=h,
                                               c=[float(v).hex() for v in c[:n]]))
        for h in (2.0, 1.0 / 64, 1.0 / 255):
            c = (D * 8)()
            n = lib.ref_stencil_interior(5, al, D(h), c)
            out["interior"].append(dict(alpha=ai, h=h, c=[float(v).hex() for v in c[:n]]))
        for y in (-0.7, -0.3, 0.0, 0.2, 0.5, 0.9):
            c = (D * 8)()
            n = lib.ref_stencil_interp_interior(5, D(y), c)
            out["interp"].append(dict(alpha=ai, kind="interior", y=y,
                                      c=[float(v).hex() for v in c[:n]]))
            for i in (0, 1):
                for psi in (0.1, 0.5, 0.95, 1.0):
                    for right in (0, 1):
                        c = (D * 8)()
                        n = lib.ref_stencil_interp_wall(5, al, i, D(y), D(psi), right, c)
                        out["interp"].append(dict(alpha=ai, kind="wall", i=i, y=y, psi=psi,
                                                  right=right, c=[float(v).hex() for v in c[:n]]))
    return out


# E6u / E8u alpha: the values of the reference's own tests (src/stencils/E6u_1.t.cpp:25,
# E8u_1.t.cpp:25-31)
WIDE_ALPHA = {6: [0.1, 0.2, 0.3, 0.4, 0.5],
              7: [-0.6484343281044554, 0.1546307245964576, -0.0024361150534464,
                  -0.0767677234359209, 0.0395245547501803, -0.25779890216368, 0.0527307049447768]}


def wide_fixtures():
    """E6u_1's and E8u_1's closure blocks and interior rows from the reference's own
    src/stencils/E6u_1.cpp and E8u_1.cpp (oracle/_ref) -> stencils_wide_ref.json"""
    subprocess.check_call(["sh", os.path.join(REPO, "oracle", "build_ref.sh")],
                          env=dict(os.environ, SHOCCS_REFERENCE_ROOT=REF))
    lib = ctypes.CDLL(os.path.join(REPO, "oracle", "_ref", "libshoccs_ref.so"))
    D = ctypes.c_double
    out = dict(source="src/stencils/E6u_1.cpp, E8u_1.cpp compiled in oracle/_ref",
               alpha={str(k): v for k, v in WIDE_ALPHA.items()}, nbs=[], interior=[])
    for scheme, a in WIDE_ALPHA.items():
        al = (D * len(a))(*a)
        for bc in (0, 1):
            for right in (0, 1):
                for h in (2.0, 1.0 / 64, 0.1):
                    c, x = (D * 128)(), (D * 8)()
                    n = lib.ref_stencil_nbs(scheme, al, D(h), bc, D(1.0), right, c, x)
                    out["nbs"].append(dict(scheme=scheme, bc=bc, right=right, h=h,
                                           c=[float(v).hex() for v in c[:n]]))
        for h in (2.0, 1.0 / 64, 1.0 / 255):
            c = (D * 16)()
            n = lib.ref_stencil_interior(scheme, al, D(h), c)
            out["interior"].append(dict(scheme=scheme, h=h, c=[float(v).hex() for v in c[:n]]))
    return out


def reference_inputs():
    """The `simulation` table of each of the reference's input files as the command line's
    Lua reader evaluates it (tests/cpp/lua_eval.cpp), with the exit status of
    `shoccs --check` on the file (the template brady_livescu_4_3.lua holds unfilled markers
    and is not valid Lua)"""
    import tempfile
    sys.path.insert(0, REPO)
    from tests.reference_inputs import parse_dump
    with tempfile.TemporaryDirectory() as d:
        exe = os.path.join(d, "lua_eval")
        subprocess.check_call(["g++", "-std=c++20", "-O2", "-I" + os.path.join(REPO, "shoccs_gb300", "app"),
                               os.path.join(REPO, "tests", "cpp", "lua_eval.cpp"), "-o", exe])
        cli = os.path.join(REPO, "shoccs_gb300", "_build", "shoccs")
        out = {}
        for name in REFERENCE_INPUTS:
            path = os.path.join(REF, name)
            r = subprocess.run([exe, path, "result = simulation"], capture_output=True, text=True)
            chk = subprocess.run([cli, "--check", path], capture_output=True, text=True, cwd=d)
            def keys_to_str(t):
                return {str(k): keys_to_str(v) for k, v in t.items()} if isinstance(t, dict) else t
            out[name] = dict(check_rc=chk.returncode,
                             table=keys_to_str(parse_dump(r.stdout)) if r.returncode == 0 else None)
    return dict(source="the reference's input files, evaluated by tests/cpp/lua_eval.cpp",
                inputs=out)


def reference_pins():
    """digests (plus size and max |value|) of the arrays of tests/golden/pins.py computed by
    the reference's own code"""
    from oracle import reference as ref
    from tests.cases import cases
    from tests.golden import pins

    def summary(arrays):
        out = {}
        for k, a in arrays.items():
            v = np.asarray(a)
            out[k] = dict(sha256=pins.digest(v), n=int(v.size),
                          maxabs=float(np.abs(v.astype(np.float64)).max(initial=0.0)))
        return out

    C = cases()
    res = {}
    for name in sorted(C):
        c = C[name]
        r = ref.RefProblem(**c)
        e = dict(setup=summary(pins.setup_arrays(r)), operators=summary(pins.operator_arrays(r, name)))
        if c["scheme"] in pins.HEAT_SCHEMES:
            s = ref.RefSystem("heat", **c, diffusivity=pins.KAPPA, sol_kind=1, sol=(pins.SINSIN_K,))
            e["heat"] = summary(pins.system_arrays(s, name, pins.heat_steps(c), pins.heat_dt(c),
                                                   s.update_boundary))
        if name in pins.WAVE_CASES:
            cen, rad = pins.wave_center(c, name)
            s = ref.RefSystem("wave", **c, center=cen, radius=rad)
            e["wave"] = summary(pins.system_arrays(s, name, 3, pins.wave_dt(c), s.update_boundary))
        res[name] = e
    return dict(source="the reference's code compiled unmodified into oracle/_ref "
                       "(oracle/build_ref.sh); arrays of tests/golden/pins.py",
                kappa=pins.KAPPA, sinsin_k=pins.SINSIN_K, cases=res)


if __name__ == "__main__":
    with open(os.path.join(HERE, "object_geometry_sphere.json"), "w") as f:
        json.dump(parse_sphere_intersections(), f, indent=1)
    st, hits = ref_fixtures()
    with open(os.path.join(HERE, "stencils_ref.json"), "w") as f:
        json.dump(st, f)
    with open(os.path.join(HERE, "stencils_poly_ref.json"), "w") as f:
        json.dump(poly_fixtures(), f)
    with open(os.path.join(HERE, "stencils_wide_ref.json"), "w") as f:
        json.dump(wide_fixtures(), f)
    with open(os.path.join(HERE, "sphere_hits_ref.json"), "w") as f:
        json.dump(hits, f)
    with open(os.path.join(HERE, "reference_pins.json"), "w") as f:
        json.dump(reference_pins(), f, indent=0, sort_keys=True)
    with open(os.path.join(HERE, "reference_inputs.json"), "w") as f:
        json.dump(reference_inputs(), f, indent=1, sort_keys=True)
    print("wrote fixtures to", HERE)
