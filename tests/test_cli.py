"""The shoccs command line (shoccs_gb300/app/shoccs.cpp) and its Lua reader
(shoccs_gb300/app/lua_subset.hpp), on the host.

* The Lua subset gives the values Lua 5.4 gives for the constructs input files use
  (arithmetic and its precedence, floor division and modulo signs, comparisons, and/or,
  strings in every quote form, table constructors with all key forms, locals and scopes,
  math.*), and rejects what it does not evaluate with the line of the error.
* The command line behaves as src/app/shoccs.cpp does: usage with no arguments or --help,
  --check stops after the Lua has run (exit 0, or non-zero on a Lua error), --script runs
  after the file and takes precedence, and a section the readers reject is reported while
  the program still exits 0.  None of these cases reaches the GPU.
* A driver script's template (markers in Lua comments replaced by plain text substitution)
  gives a runnable input once filled in.
"""
import os
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
LUA = os.path.join(HERE, "lua")
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")


@pytest.fixture(scope="module")
def lua_eval(tmp_path_factory):
    d = tmp_path_factory.mktemp("lua_eval")
    exe = d / "lua_eval"
    r = subprocess.run(["g++", "-std=c++20", "-O2", "-Wall", "-Wextra",
                        "-I" + os.path.join(ROOT, "shoccs_gb300", "app"),
                        os.path.join(HERE, "cpp", "lua_eval.cpp"), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]

    def run(src, *scripts):
        f = d / "chunk.lua"
        f.write_text(src)
        r = subprocess.run([str(exe), str(f), *scripts], capture_output=True, text=True, timeout=60)
        out = {}
        for line in r.stdout.splitlines():
            k, *v = line.split("\t")
            out[k] = v
        return r.returncode, out
    return run


@pytest.fixture(scope="module")
def cli():
    exe = os.path.join(ROOT, "shoccs_gb300", "_build", "shoccs")
    if not os.path.exists(exe):
        pytest.fail("command line not built: " + exe)
    return exe


CHUNK = r'''
local a, b = 3, 4
local unused
g = 10
result = {
  arith = {1 + 2 * 3, (1 + 2) * 3, 2 ^ 3 ^ 2, -2 ^ 2, 7 // 2, -7 // 2, 7 % 3, -7 % 3, 7 % -3,
           5.5 % 2, 1 / 4, 10 - 2 - 3, 2 ^ -1, "3" + 1},
  cmp = {1 < 2, 2 <= 1, "a" < "b", 1 == 1.0, "1" == 1, nil == false, 3 ~= 4},
  logic = {nil or 5, false and 1, 1 and 2, not nil, not 0, false or nil},
  str = {"a" .. "b" .. 1 .. 2.5, #"hello", 'single', "esc\t\"q\"\65", #[[long
string]], [==[with ]] inside]==]},
  len = #{1, 2, 3, nil},
  keys = {[1] = "one", [2.5] = "real", ["k"] = "v", x = a * b, [g] = "ten"; "positional"},
  math = {math.pi, math.sqrt(2), math.floor(-2.5), math.max(1, 7, 3), math.min(4, -1),
          math.abs(-3), math.huge > 1e308, math.fmod(7, 3), math.log(8, 2), math.exp(0),
          math.atan(1, 1), math.ceil(1.2), math.tointeger(3.0)},
  fn = function(t, x) if t > 0 then return x end return 0 end,
  nested = {{1, {2, {3}}}},
  hex = 0x1F,
  expo = 1.5e3,
  unary = - -3,
}
result.assigned = g + 1
result.nested[1][2][2][2] = "deep"
do local g = 99; result.shadow = g end
result.after = g
local function helper(x) return x end
result.has_helper = helper ~= nil
'''


def _num(out, key):
    typ, v = out[key]
    assert typ == "number", (key, typ)
    return float(v)


def test_lua_subset_values(lua_eval):
    rc, out = lua_eval(CHUNK)
    assert rc == 0, out
    arith = [7, 9, 512, -4, 3, -4, 1, 2, -2, 1.5, 0.25, 5, 0.5, 4]
    assert [_num(out, "result.arith[%d]" % (i + 1)) for i in range(len(arith))] == arith
    cmp = ["true", "false", "true", "true", "false", "false", "true"]
    assert [out["result.cmp[%d]" % (i + 1)][1] for i in range(len(cmp))] == cmp
    assert _num(out, "result.logic[1]") == 5
    assert out["result.logic[2]"] == ["boolean", "false"]
    assert _num(out, "result.logic[3]") == 2
    assert out["result.logic[4]"] == ["boolean", "true"] and out["result.logic[5]"] == ["boolean", "false"]
    assert "result.logic[6]" not in out  # nil is not stored
    assert out["result.str[1]"] == ["string", "ab12.5"]
    assert _num(out, "result.str[2]") == 5
    assert out["result.str[3]"] == ["string", "single"]
    assert out["result.str[4]"] == ["string", 'esc', '"q"A']  # the tab splits the field
    assert _num(out, "result.str[5]") == 11  # the newline after [[ is not skipped here: 4+1+6
    assert out["result.str[6]"] == ["string", "with ]] inside"]
    assert _num(out, "result.len") == 3
    assert out["result.keys[1]"] == ["string", "positional"]  # positional fields win over [1]
    assert out["result.keys[2.5]"] == ["string", "real"]
    assert out["result.keys.k"] == ["string", "v"]
    assert _num(out, "result.keys.x") == 12
    assert out["result.keys[10]"] == ["string", "ten"]
    import math
    m = [math.pi, math.sqrt(2), -3, 7, -1, 3, None, 1, 3, 1, math.pi / 4, 2, 3]
    for i, want in enumerate(m):
        if want is None:
            assert out["result.math[%d]" % (i + 1)] == ["boolean", "true"]
        else:
            assert _num(out, "result.math[%d]" % (i + 1)) == want, i
    assert out["result.fn"] == ["function", "function"]
    assert _num(out, "result.nested[1][1]") == 1
    assert out["result.nested[1][2][2][2]"] == ["string", "deep"]
    assert _num(out, "result.hex") == 31 and _num(out, "result.expo") == 1500
    assert _num(out, "result.unary") == 3
    assert _num(out, "result.assigned") == 11
    assert _num(out, "result.shadow") == 99 and _num(out, "result.after") == 10
    assert out["result.has_helper"] == ["boolean", "true"]


def test_lua_subset_script_after_file(lua_eval):
    rc, out = lua_eval("result = {a = 1, b = {c = 2}}", "result.b.c = 3; result.d = result.a + 1")
    assert rc == 0
    assert _num(out, "result.a") == 1 and _num(out, "result.b.c") == 3 and _num(out, "result.d") == 2


CONTROL = r'''
result = {shapes = {}}
for i = 1, 4 do
  local r = 0.05 * i
  if i % 2 == 0 then
    result.shapes[#result.shapes + 1] = {radius = r, kind = "even"}
  elseif i == 3 then
    result.shapes[#result.shapes + 1] = {radius = r, kind = "three"}
  else
    result.shapes[#result.shapes + 1] = {radius = r, kind = "odd"}
  end
end
local n = 0
while true do
  n = n + 1
  if n >= 5 then break end
end
result.n = n
for k = 10, 1, -3 do result.last = k end
for k = 1, 0 do result.never = true end
local s = 0
for i = 1, 10 do
  if i > 3 then break end
  s = s + i
end
result.s = s
result.i_after = i
if false then result.x = 1 elseif nil then result.x = 2 else result.x = 3 end
if true then result.y = 1 end
'''


FUNCS = r'''
local function sphere(c, r, bc)
  return {type = "sphere", center = c, radius = r, boundary_condition = bc or "dirichlet"}
end
function fact(n) if n <= 1 then return 1 end return n * fact(n - 1) end
local function fib(n) if n < 2 then return n end return fib(n - 1) + fib(n - 2) end
local scale = 3
local mul = function(x) return x * scale end
result = {s = sphere({0.5, 0.5}, 0.2, "floating"), f = fact(10), g = fib(15), m = mul(7),
          none = (function() end)()}
result.shapes = {}
for i = 1, 3 do result.shapes[i] = sphere({0.2 * i, 0.5}, 0.05) end
'''


def test_lua_subset_functions(lua_eval):
    rc, out = lua_eval(FUNCS, "result.after = fact(5)")  # a function of the file, called by --script
    assert rc == 0, out
    assert out["result.s.type"] == ["string", "sphere"] and out["result.s.boundary_condition"][1] == "floating"
    assert _num(out, "result.s.radius") == 0.2 and _num(out, "result.s.center[2]") == 0.5
    assert _num(out, "result.f") == 3628800 and _num(out, "result.g") == 610 and _num(out, "result.m") == 21
    assert "result.none" not in out and _num(out, "result.after") == 120
    assert [_num(out, "result.shapes[%d].center[1]" % i) for i in (1, 2, 3)] == [0.2 * i for i in (1, 2, 3)]
    assert all(out["result.shapes[%d].boundary_condition" % i][1] == "dirichlet" for i in (1, 2, 3))


def test_lua_subset_base_functions(lua_eval):
    rc, out = lua_eval('local n = 33\n'
                       'result = {dir = string.format("io_%03d_%s_%.3f", n, "heat", 0.5), t = type(3), '
                       'ts = tostring(2.5), tn = tonumber("1e-3"), bad = tonumber("abc"), '
                       'pct = string.format("%d%%", 7), e = string.format("%.2e", 12345.678), '
                       'tt = type({}), tf = type(print)}')
    assert rc == 0, out
    assert out["result.dir"] == ["string", "io_033_heat_0.500"]
    assert out["result.t"] == ["string", "number"] and out["result.ts"] == ["string", "2.5"]
    assert _num(out, "result.tn") == 1e-3 and "result.bad" not in out
    assert out["result.pct"] == ["string", "7%"] and out["result.e"] == ["string", "1.23e+04"]
    assert out["result.tt"] == ["string", "table"] and out["result.tf"] == ["string", "function"]
    rc, out = lua_eval('x = string.format("%d")')
    assert rc == 1 and "bad argument #2 to 'format'" in out["error"][0]


def test_lua_subset_control_flow(lua_eval):
    rc, out = lua_eval(CONTROL)
    assert rc == 0, out
    kinds = [out["result.shapes[%d].kind" % i][1] for i in range(1, 5)]
    assert kinds == ["odd", "even", "three", "even"]
    assert [_num(out, "result.shapes[%d].radius" % i) for i in range(1, 5)] == [0.05 * i for i in range(1, 5)]
    assert _num(out, "result.n") == 5 and _num(out, "result.s") == 6 and _num(out, "result.last") == 1
    assert "result.never" not in out and "result.i_after" not in out  # loop variables are local
    assert _num(out, "result.x") == 3 and _num(out, "result.y") == 1


SHORT_CIRCUIT = r'''
local t = nil
calls = 0
local function bump() calls = calls + 1 return true end
local function fact(n) return n <= 1 and 1 or n * fact(n - 1) end
local guard
if t == nil then guard = "nil" elseif t.x > 0 then guard = "x" else guard = "other" end
local second
if false then second = 1 elseif true then second = 2 elseif bump() then second = 3 end
result = {a = (t ~= nil and t.x) or 3, b = t and t.y, c = false or "c", d = t and t.x.y,
          e = 1 or error_not_called(), fact = fact(6), guard = guard, second = second,
          f = (1 > 2) and bump() or "f"}
result.calls = calls
'''


def test_lua_subset_short_circuit(lua_eval):
    """`and` / `or` evaluate their right operand only when the left one does not decide, and
    the conditions after a taken branch of an if are not evaluated (Lua's semantics): nil
    guards, the recursion idiom `n <= 1 and 1 or n * f(n - 1)`, and no side effects from the
    skipped calls"""
    rc, out = lua_eval(SHORT_CIRCUIT)
    assert rc == 0, out
    assert _num(out, "result.a") == 3 and "result.b" not in out and "result.d" not in out
    assert out["result.c"] == ["string", "c"] and _num(out, "result.e") == 1
    assert _num(out, "result.fact") == 720 and out["result.guard"] == ["string", "nil"]
    assert _num(out, "result.second") == 2 and out["result.f"] == ["string", "f"]
    assert _num(out, "result.calls") == 0


def test_lua_subset_format_and_tonumber_edges(lua_eval):
    rc, out = lua_eval('result = {c = string.format("%c%c", 72, 105), '
                       'long = string.format("%s", string.format("%0700d", 1)), '
                       'ws = tonumber(" 12\\t\\n"), hex = tonumber("0x10"), inf = tonumber("inf"), '
                       'nan = tonumber("nan"), neg = tonumber("-2.5e1"), bad = tonumber("1 2")}')
    assert rc == 0, out
    assert out["result.c"] == ["string", "Hi"]
    assert len(out["result.long"][1]) == 700 and out["result.long"][1].endswith("01")
    assert _num(out, "result.ws") == 12 and _num(out, "result.hex") == 16
    assert _num(out, "result.neg") == -25
    assert "result.inf" not in out and "result.nan" not in out and "result.bad" not in out
    for src in ('x = string.format("%d", 2.5)', 'x = string.format("%d", 1e300)'):
        rc, out = lua_eval(src)
        assert rc == 1 and "number has no integer representation" in out["error"][0], out


@pytest.mark.parametrize("src,msg", [
    ("break", "break outside a loop"),
    ("for k, v in pairs({}) do end", "only numeric for loops are supported"),
    ("for i = 1, 2, 0 do end", "'for' step is zero"),
    ("if true then x = 1", "'end' expected"),
    ("x = = 1", ":1:"),
    ("\n\nrepeat x = 1 until true", ":3: unsupported statement"),
    ("function f(n) return f(n + 1) end\nx = f(1)", "stack overflow"),
    ("f = function(...) end", "varargs are not supported"),
    ("x = y.z", "attempt to index a nil value"),
    ("x = {1, 2", "'}' expected"),
    ("x = 'open", "unfinished string"),
    ("x = 1 + {}", "attempt to perform arithmetic"),
    ("x = math.sqrt('a')", "bad argument to 'math.sqrt'"),
])
def test_lua_subset_errors(lua_eval, src, msg):
    rc, out = lua_eval(src)
    assert rc == 1
    assert msg in out["error"][0], out


def _run(cli, args, cwd):
    return subprocess.run([cli] + args, cwd=str(cwd), capture_output=True, text=True, timeout=60)


def test_cli_usage_and_check(cli, tmp_path):
    for args in ([], ["--help"]):
        r = _run(cli, args, tmp_path)
        assert r.returncode == 0 and "--check" in r.stdout and "--script" in r.stdout
    for name in ("wave_radial_2d.lua", "heat_circle_2d.lua"):
        r = _run(cli, ["--check", os.path.join(LUA, name)], tmp_path)
        assert r.returncode == 0, r.stderr
    # the template is not runnable until its markers are replaced
    r = _run(cli, ["--check", os.path.join(LUA, "wave_template.lua")], tmp_path)
    assert r.returncode != 0 and "wave_template.lua:" in r.stderr
    # --script runs after the file; an error there is an error too
    r = _run(cli, ["--check", os.path.join(LUA, "wave_radial_2d.lua"), "--script", "simulation.x = ="], tmp_path)
    assert r.returncode != 0 and "script:1:" in r.stderr
    r = _run(cli, ["--check", "--script=simulation = {}"], tmp_path)
    assert r.returncode == 0
    r = _run(cli, ["--bogus"], tmp_path)
    assert r.returncode != 0
    assert not os.listdir(str(tmp_path))  # --check writes nothing


@pytest.mark.parametrize("script,msg", [
    ('simulation.scheme.type = "E2"', "scheme.order/type = 1 / E2 is not available"),
    ('simulation.scheme = {order = 3, type = "E4"}', "scheme.order/type = 3 / E4 not recognized"),
    ('simulation.scheme = nil', "simulation.scheme must be specified"),
    ('simulation.system.type = "euler"', "unrecognized system.type"),
    ('simulation.system = nil', "simulation.system must be specified"),
    ('simulation.mesh.index_extents = nil', "simulation.mesh.index_extents is required"),
    ('simulation.mesh.domain_bounds = {min = {0, 0}}', "domain_bounds.max"),
    ('simulation.domain_boundaries.xmin = "periodic"', "incorrect boundary condition"),
    ('simulation.shapes = {{type = "yz_rect"}}', "shape type 'yz_rect' is not supported"),
    ('simulation.integrator.type = "ab3"', "integrator.type must be one of: [rk4, euler]"),
    ('simulation.system.precision = "fp16"', "system.precision must be fp64 or mixed"),
    ('simulation = 3', "the global table `simulation` is required"),
])
def test_cli_rejected_sections_exit_zero(cli, tmp_path, script, msg):
    r = _run(cli, [os.path.join(LUA, "wave_radial_2d.lua"), "--script", script], tmp_path)
    assert r.returncode == 0, r.stderr
    assert msg in r.stderr, r.stderr


@pytest.mark.parametrize("scheme,msg", [
    ('{order = 1, type = "E6u", alpha = {0.1, 0.2, 0.3, 0.4, 0.5}}', "E6 uniform first scheme chosen"),
    ('{order = 1, type = "E8u", alpha = {-0.65, 0.15, 0, -0.08, 0.04, -0.26, 0.05}}',
     "E8 uniform first scheme chosen"),
])
def test_cli_reads_wide_uniform_schemes(cli, tmp_path, scheme, msg):
    """the scheme section is read and the builder goes on to the system (which needs a GPU
    here; on a machine without one the run ends at the system's creation)"""
    r = _run(cli, [os.path.join(LUA, "wave_radial_2d.lua"), "--script",
                   "simulation.scheme = " + scheme], tmp_path)
    out = r.stdout + r.stderr
    assert msg in out and "building scalar_wave system" in out, out
    assert "not available" not in out and "not recognized" not in out, out


def test_cli_heat_rejects_lua_manufactured_solutions(cli, tmp_path):
    r = _run(cli, [os.path.join(LUA, "heat_circle_2d.lua"), "--script",
                   'simulation.manufactured_solution = {type = "lua", call = function(t, x) return 0 end}'],
             tmp_path)
    assert r.returncode == 0 and "manufactured_solution.type = `lua`" in r.stderr


def fill_template(n, t_final, scheme_type, alpha):
    """The driver's substitution: three markers replaced by plain text"""
    src = open(os.path.join(LUA, "wave_template.lua")).read()
    scheme = '{ order = 1, type = "%s", alpha = {%s} }' % (scheme_type, ", ".join(repr(float(a)) for a in alpha))
    return (src.replace("--{{N}}--", str(int(n))).replace("--{{T_FINAL}}--", repr(float(t_final)))
            .replace("--{{SCHEME_TABLE}}--", scheme))


def test_template_filled_in_is_valid(cli, tmp_path):
    f = tmp_path / "filled.lua"
    f.write_text(fill_template(31, 0.1, "E4", (0.1, 0.7)))
    r = _run(cli, ["--check", str(f)], tmp_path)
    assert r.returncode == 0, r.stderr


def test_cli_geometry_log(cli, tmp_path):
    """logs/geometry.csv (src/mesh/mesh.cpp:139-151) is written from the host-side operators
    before the system is created: header, then per cut point direction, index, psi, the
    position and the solid point's indices (each triple joined by ", "), equal to the library's
    cut points.  Without a GPU the run stops at the system; only the log is checked."""
    import shoccs_gb300 as S
    _run(cli, [os.path.join(LUA, "heat_circle_2d.lua"), "--script", "simulation.step_controller.max_step = 1"],
         tmp_path)
    lines = (tmp_path / "mylogs" / "geometry.csv").read_text().splitlines()
    assert lines[0] == "Timestamp,direction,ic,psi,x,y,z,i,j,k"
    p = S.Problem(n=(65, 65, 1), lo=(0, 0, 0), hi=(1, 1, 0), spheres=[((0.51, 0.49, 0.0), 0.2, "dirichlet")],
                  grid_bc=("dirichlet",) * 4 + ("floating",) * 2, scheme="E4_2")
    want = []
    for d in range(3):
        cp = p.cut_points(d)
        for i in range(p.nR[d]):
            want.append((d, i, cp["psi"][i], tuple(cp["position"][i]), tuple(cp["solid_coord"][i])))
    rows = []
    for line in lines[1:]:
        ts, d, i, psi, rest = line.split(",", 4)
        pos_s, ijk_s = rest.split(",", 3)[:3], rest.split(",", 3)[3]
        rows.append((int(d), int(i), float(psi), tuple(float(v) for v in pos_s),
                     tuple(int(v) for v in ijk_s.split(", "))))
        assert ts[:4].isdigit() and ", " in rest
    assert rows == want
