"""Extract the reference's known-answer values into ``reference_goldens.json``.

Run once in a checkout that has davef96/jsolver next to it:

    python tests/golden/make_goldens.py /path/to/jsolver

It parses (as text, with ``ast``; nothing of the reference is imported or executed):

* tests/test_solver_2d.py and tests/test_solver_3d.py: for every test function, the
  problem id, the grid fixture (128^2 / 64^2 / 64x128 in 2D; 64^3 / 32^3 / 32x64x32
  in 3D), the asserted dynamic iteration count and the asserted RMSE against the
  analytic solution. For 2D test1 it also records the W/F/fixed checks.
* examples/benchmark.py:26-632: the golden dictionaries
  ``reference_{v,vskip,f,fskip,w,wskip}`` mapping (problem, resolution) to
  (iterations, rmse). NaN entries are kept as null.

The output is committed; tests read only the JSON.
"""
import ast
import json
import math
import os
import sys

FIXTURE_SHAPES = {
    "test_solver_2d.py": {"setup": [128, 128], "setup_64": [64, 64], "setup_64_128": [64, 128]},
    "test_solver_3d.py": {"setup": [64, 64, 64], "setup_32": [32, 32, 32], "setup_mixed": [32, 64, 32]},
}


def _num(node):
    v = ast.literal_eval(node) if not isinstance(node, ast.UnaryOp) else -_num(node.operand)
    return v


def _parse_tests(path, fname):
    src = open(path).read()
    tree = ast.parse(src)
    out = []
    for fn in tree.body:
        if not isinstance(fn, ast.FunctionDef) or not fn.name.startswith("test"):
            continue
        args = [a.arg for a in fn.args.args]
        fixture = next((a for a in args if a in FIXTURE_SHAPES[fname]), None)
        prob_fix = next((a for a in args if a.startswith("test") and a.endswith(("setup", "_64", "_64_128", "_32", "_mixed"))), None)
        if fixture is None or prob_fix is None:
            continue
        pid = int(prob_fix[4:].split("_")[0])
        iters, rmse, line = None, None, None
        for node in ast.walk(fn):
            if isinstance(node, ast.Assert) and isinstance(node.test, ast.Compare):
                t = node.test
                if (isinstance(t.left, ast.Name) and t.left.id == "iterations"
                        and isinstance(t.ops[0], ast.Eq) and iters is None):
                    iters = ast.literal_eval(t.comparators[0])
                    line = node.lineno
                if (isinstance(t.left, ast.Call) and getattr(t.left.func, "attr", "") == "approx"
                        and rmse is None):
                    rmse = _num(t.left.args[0])
        if iters is None:
            continue
        out.append({"file": "tests/" + fname, "line": line, "test": fn.name, "problem": pid,
                    "res": FIXTURE_SHAPES[fname][fixture], "cycle": "V", "iterations": iters, "rmse": rmse})
    return out


def _parse_bench(path):
    tree = ast.parse(open(path).read())
    out = {}
    for node in tree.body:
        if isinstance(node, ast.Assign) and isinstance(node.targets[0], ast.Name) \
                and node.targets[0].id.startswith("reference_") and isinstance(node.value, ast.Dict):
            name = node.targets[0].id
            rows = []
            for k, v in zip(node.value.keys, node.value.values):
                pid, res = ast.literal_eval(k)
                it = ast.literal_eval(v.elts[0])
                r = v.elts[1]
                try:
                    rm = _num(r)
                except ValueError:
                    rm = None  # '-np.nan'
                if isinstance(rm, float) and math.isnan(rm):
                    rm = None
                rows.append({"problem": pid, "res": res, "iterations": it, "rmse": rm, "line": k.lineno})
            out[name] = rows
    return out


def main(ref_root):
    data = {
        "source": "davef96/jsolver (tests/test_solver_2d.py, tests/test_solver_3d.py, examples/benchmark.py:26-632)",
        "tests_2d": _parse_tests(os.path.join(ref_root, "tests/test_solver_2d.py"), "test_solver_2d.py"),
        "tests_3d": _parse_tests(os.path.join(ref_root, "tests/test_solver_3d.py"), "test_solver_3d.py"),
        "benchmark_2d": _parse_bench(os.path.join(ref_root, "examples/benchmark.py")),
        # test1 extra checks on 128^2 (tests/test_solver_2d.py:177-198): F-cycle (<= 8
        # cycles), W-cycle (<= 13), fixed 13 V-cycles, fixed 13 F-cycles.
        "test1_extras_2d": {
            "fcycle": {"max_iterations": 8, "rmse": 1.010315414037897e-06, "line": 179},
            "wcycle": {"max_iterations": 13, "rmse": 1.010315424011278e-06, "line": 184},
            "fixed13": {"iterations": 13, "rmse": 1.010315424011278e-06, "line": 192},
            "fixed13_f": {"max_iterations": 13, "rmse": 1.010315424011278e-06, "line": 197},
        },
    }
    # the 3D file defines `test1_32` twice (lines 213 and 230); only the second runs
    seen = {}
    for row in data["tests_3d"]:
        seen[row["test"]] = row
    data["tests_3d_shadowed"] = [r for r in data["tests_3d"] if seen[r["test"]] is not r]
    data["tests_3d"] = list(seen.values()) + data["tests_3d_shadowed"]
    here = os.path.dirname(os.path.abspath(__file__))
    with open(os.path.join(here, "reference_goldens.json"), "w") as f:
        json.dump(data, f, indent=1)
    print("tests_2d", len(data["tests_2d"]), "tests_3d", len(data["tests_3d"]),
          {k: len(v) for k, v in data["benchmark_2d"].items()})


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_goldens.py <path of the jsolver source tree>")
    main(sys.argv[1])
