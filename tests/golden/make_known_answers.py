"""
Regenerates known_answers.json from the reference's own test files.

The reference (Python + Taichi) cannot be imported here -- Taichi is not
installed -- so its known answers are taken from its test sources, read as
text: the literal inputs of the test's constructor calls and the expected
values of its assertions, each with the file:line it came from.  The JSON is
committed; this script is only rerun where the reference's sources are
present (it reads them from the directory given as the first argument).

    python tests/golden/make_known_answers.py /path/to/taichimps > tests/golden/known_answers.json
"""

from __future__ import annotations

import ast
import json
import sys
from pathlib import Path


def _calls(fn: ast.FunctionDef) -> dict[str, list[tuple[int, dict]]]:
    """Literal keyword arguments of every call in a test function, by callee name."""
    out: dict[str, list[tuple[int, dict]]] = {}
    for node in ast.walk(fn):
        if not isinstance(node, ast.Call):
            continue
        f = node.func
        name = f.attr if isinstance(f, ast.Attribute) else getattr(f, "id", None)
        if name is None:
            continue
        kw = {}
        for k in node.keywords:
            try:
                kw[k.arg] = ast.literal_eval(k.value)
            except ValueError:
                pass
        out.setdefault(name, []).append((node.lineno, kw))
    return out


def _assigns(fn: ast.FunctionDef) -> dict[str, tuple[int, object]]:
    out = {}
    for node in ast.walk(fn):
        if isinstance(node, ast.Assign) and len(node.targets) == 1 and isinstance(node.targets[0], ast.Name):
            try:
                out[node.targets[0].id] = (node.lineno, ast.literal_eval(node.value))
            except ValueError:
                pass
    return out


def _subscript_sets(fn: ast.FunctionDef) -> list[tuple[int, object]]:
    """`atom.x[0] = ti.Vector([...])` assignments, in order."""
    out = []
    for node in ast.walk(fn):
        if (isinstance(node, ast.Assign) and isinstance(node.targets[0], ast.Subscript)
                and isinstance(node.value, ast.Call) and node.value.args):
            try:
                out.append((node.lineno, ast.literal_eval(node.value.args[0])))
            except ValueError:
                pass
    return sorted(out)


def _isclose_asserts(fn: ast.FunctionDef) -> list[tuple[int, int, float]]:
    """`assert np.isclose(name[k], value)`: (line, k, value)."""
    out = []
    for node in ast.walk(fn):
        if isinstance(node, ast.Assert) and isinstance(node.test, ast.Call):
            c = node.test
            if getattr(c.func, "attr", None) == "isclose" and isinstance(c.args[0], ast.Subscript):
                out.append((node.lineno, ast.literal_eval(c.args[0].slice), ast.literal_eval(c.args[1])))
    return sorted(out)


def _function(path: Path, name: str) -> ast.FunctionDef:
    tree = ast.parse(path.read_text())
    for node in ast.walk(tree):
        if isinstance(node, ast.FunctionDef) and node.name == name:
            return node
    raise KeyError(f"{name} not in {path}")


def _eval(node, names: dict):
    """Arithmetic of literals, resolved names, unary minus and np.sqrt (what the wall tests write)."""
    if isinstance(node, ast.Constant):
        return node.value
    if isinstance(node, (ast.List, ast.Tuple)):
        return [_eval(e, names) for e in node.elts]
    if isinstance(node, ast.Name):
        return names[node.id]
    if isinstance(node, ast.UnaryOp) and isinstance(node.op, ast.USub):
        return -_eval(node.operand, names)
    if isinstance(node, ast.BinOp):
        a, b = _eval(node.left, names), _eval(node.right, names)
        return {ast.Add: a + b if not isinstance(a, list) else None, ast.Sub: a - b if not isinstance(a, list) else None,
                ast.Mult: a * b if not isinstance(a, list) else None,
                ast.Div: a / b if not isinstance(a, list) else None}[type(node.op)]
    if isinstance(node, ast.Call) and getattr(node.func, "attr", None) == "sqrt":
        return _eval(node.args[0], names) ** 0.5
    raise ValueError(ast.dump(node))


def _wall_case(fn: ast.FunctionDef, ctor: str) -> dict:
    """Constructor keywords, particle 0's state, the step and the asserted values of one wall test."""
    names, arrays, fields, expected, kwargs, dt = {}, {}, {}, [], None, None
    for node in sorted((n for n in ast.walk(fn) if isinstance(n, ast.stmt)), key=lambda n: n.lineno):
        if isinstance(node, ast.Assign) and len(node.targets) == 1:
            t = node.targets[0]
            if isinstance(t, ast.Name):
                v = node.value
                if isinstance(v, ast.Call) and getattr(v.func, "attr", None) == "full":
                    arrays[t.id] = _eval(v.args[1], names)
                else:
                    try:
                        names[t.id] = _eval(v, names)
                    except (ValueError, KeyError):
                        pass
            elif isinstance(t, ast.Subscript) and isinstance(t.value, ast.Name):
                try:
                    arrays[t.value.id] = _eval(node.value, names)
                except (ValueError, KeyError):
                    pass
    for node in ast.walk(fn):
        if isinstance(node, ast.Call):
            f = node.func
            name = f.attr if isinstance(f, ast.Attribute) else getattr(f, "id", None)
            if name == ctor:
                kwargs = {k.arg: _eval(k.value, names) for k in node.keywords if k.arg != "domain"}
            elif name == "from_numpy" and isinstance(f.value, ast.Attribute):
                arg = node.args[0]
                if isinstance(arg, ast.Call) and getattr(arg.func, "attr", None) == "full":
                    fields[f.value.attr] = _eval(arg.args[1], names)
                elif isinstance(arg, ast.Name) and arg.id in arrays:
                    fields[f.value.attr] = arrays[arg.id]
            elif name == "post_force":
                dt = _eval(node.args[1], names)
        if isinstance(node, ast.Assert) and isinstance(node.test, ast.Call):
            c = node.test
            if getattr(c.func, "attr", None) == "isclose" and isinstance(c.args[0], ast.Subscript):
                expected.append({"line": node.lineno, "of": c.args[0].value.id,
                                 "k": ast.literal_eval(c.args[0].slice), "value": _eval(c.args[1], names)})
    # particle 0 of the arrays the test set by index (x_np[0] = ...), zero where it set none
    x0 = fields.get("x", [0.0, 0.0, 0.0])
    v0 = fields.get("v", [0.0, 0.0, 0.0])
    return {"fix": kwargs, "x": x0 if not isinstance(x0, float) else [x0] * 3,
            "v": v0 if not isinstance(v0, float) else [v0] * 3,
            "radius": fields["radius"], "rmass": fields["rmass"], "dt": dt,
            "expected": sorted(expected, key=lambda e: e["line"])}


def main(ref: Path) -> dict:
    rel = lambda p: str(p.relative_to(ref))
    out = {"source": "literal inputs and expected values of the reference's tests, read as text",
           "cases": {}}

    p = ref / "tests" / "test_hooke.py"
    fn = _function(p, "test_hooke_normal_contact")
    c, a = _calls(fn), _assigns(fn)
    dline, dom = c["Domain"][0]
    pline, parts = c["add_particles"][0]
    nline, nl = c["NeighborList"][0]
    gline, pair = c["GranHooke"][0]
    cline, comp = c["compute"][0]
    eline, expected = a["expected"]
    out["cases"]["hooke_normal_contact"] = {
        "cite": f"{rel(p)}:{fn.lineno}-{eline + 7}",
        "domain": dom, "particles": parts, "skin": nl["skin"], "pair": pair, "dt": comp["dt"],
        "expected_fx": [-expected, expected], "rtol": 1e-12,
        "lines": {"domain": dline, "particles": pline, "neighbor": nline, "pair": gline, "expected": eline},
    }

    p = ref / "tests" / "test_domain_neighbor.py"
    fn = _function(p, "test_domain_periodicity")
    c = _calls(fn)
    dline, dom = c["Domain"][0]
    pline, parts = c["add_particles"][0]
    out["cases"]["pbc_wrap"] = {
        "cite": f"{rel(p)}:{fn.lineno}-{fn.end_lineno}", "domain": dom, "particles": parts,
        "expected": {str(k): v for _, k, v in _isclose_asserts(fn)},
    }

    fn = _function(p, "test_neighbor_skin_displacement_check")
    c = _calls(fn)
    dline, dom = c["Domain"][0]
    pline, parts = c["add_particles"][0]
    moves = _subscript_sets(fn)
    assigns = _assigns(fn)
    out["cases"]["skin_trigger"] = {
        "cite": f"{rel(p)}:{fn.lineno}-{fn.end_lineno}", "domain": dom, "particles": parts,
        "skin": assigns["skin"][1],
        # atom 0 moved to each position in turn; the reference expects no rebuild, then a rebuild
        "moves": [m for _, m in moves], "rebuild_expected": [False, True],
    }

    fn = _function(p, "test_neighbor_list")
    c = _calls(fn)
    dline, dom = c["Domain"][0]
    pline, parts = c["add_particles"][0]
    nline, nl = c["NeighborList"][0]
    out["cases"]["neighbor_list"] = {
        "cite": f"{rel(p)}:{fn.lineno}-{fn.end_lineno}", "domain": dom, "particles": parts, "skin": nl["skin"],
        # atom 0's neighbors (reference half list: j > i): atom 1 only
        "neighbors_of_0": [1],
    }
    p = ref / "tests" / "test_wall_region.py"
    for name in ("test_fix_wall_gran_region_cylinder_in", "test_fix_wall_gran_region_cylinder_out",
                 "test_fix_wall_gran_region_friction_and_torque", "test_fix_wall_gran_region_hertz"):
        fn = _function(p, name)
        case = _wall_case(fn, "FixWallGranRegion")
        case["cite"] = f"{rel(p)}:{fn.lineno}-{fn.end_lineno}"
        out["cases"]["wall_region_" + name.split("region_", 1)[1]] = case

    p = ref / "tests" / "test_additional_models.py"
    fn = _function(p, "test_pair_granular_and_wall")
    c = _calls(fn)
    pline, parts = c["add_particles"][0]
    wline, wall = c["FixWallGran"][0]
    out["cases"]["wall_plane_sign"] = {
        "cite": f"{rel(p)}:{fn.lineno}-{wline + 5}", "particles": parts, "fix": wall,
        "dt": [kw for _, kw in c["post_force"]][0]["dt"],
        # the test asserts only that the wall pushes the particle away: f_x > 0
        "expected_sign_fx": 1,
    }
    return out


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit(__doc__)
    print(json.dumps(main(Path(sys.argv[1])), indent=1))
