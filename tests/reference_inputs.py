"""The reference's input files as data: the flattened `simulation` table that
tests/cpp/lua_eval.cpp prints, turned into nested Python values and back into Lua source.

Used by tests/golden/make_golden.py (which evaluates the reference's own files into
tests/golden/reference_inputs.json) and tests/test_reference_inputs.py (which writes the
tables back out as Lua input files for the command line).
"""
import re

_TOKEN = re.compile(r"\.([A-Za-z_][A-Za-z0-9_]*)|\[([^\]]+)\]")


def parse_dump(text):
    """lua_eval's "path<TAB>type<TAB>value" lines under `result` -> nested dicts (tables;
    integer keys stay integers) holding numbers, strings and booleans; functions are kept as
    the marker {"__function__": name}"""
    root = {}
    for line in text.splitlines():
        path, typ, *rest = line.split("\t")
        value = rest[0] if rest else ""
        assert path.startswith("result"), line
        keys = []
        for name, idx in _TOKEN.findall(path[len("result"):]):
            if name:
                keys.append(name)
            else:
                f = float(idx)
                keys.append(int(f) if f == int(f) else f)
        if typ == "number":
            v = float(value)
        elif typ == "boolean":
            v = value == "true"
        elif typ == "string":
            v = value
        elif typ == "function":
            v = {"__function__": value}
        else:
            continue
        node = root
        for k in keys[:-1]:
            node = node.setdefault(str(k) if isinstance(k, str) else k, {})
        node[keys[-1]] = v
    return root


def _normalise(t):
    """JSON object keys are strings: give integer keys back their type"""
    if not isinstance(t, dict) or "__function__" in t:
        return t
    out = {}
    for k, v in t.items():
        kk = int(k) if isinstance(k, str) and re.fullmatch(r"-?\d+", k) else k
        out[kk] = _normalise(v)
    return out


def to_lua(value, indent=0):
    """a Lua constructor for a nested value (numbers at full precision)"""
    value = _normalise(value)
    pad = "    " * (indent + 1)
    if isinstance(value, bool):
        return "true" if value else "false"
    if isinstance(value, (int, float)):
        return repr(float(value)) if value != int(value) or abs(value) >= 2 ** 53 else str(int(value))
    if isinstance(value, str):
        return '"' + value.replace("\\", "\\\\").replace('"', '\\"') + '"'
    if "__function__" in value:
        raise ValueError("a function value cannot be written back")
    ints = sorted(k for k in value if isinstance(k, int))
    items = []
    if ints == list(range(1, len(ints) + 1)):
        items += [to_lua(value[k], indent + 1) for k in ints]
    else:
        items += ["[%d] = %s" % (k, to_lua(value[k], indent + 1)) for k in ints]
    items += ["%s = %s" % (k, to_lua(v, indent + 1)) for k, v in sorted(
        ((k, v) for k, v in value.items() if not isinstance(k, int)), key=lambda kv: str(kv[0]))]
    if not items:
        return "{}"
    return "{\n" + "".join(pad + it + ",\n" for it in items) + "    " * indent + "}"


def lua_input(table):
    return "simulation = " + to_lua(table) + "\n"
