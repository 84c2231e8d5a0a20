"""Extract the reference's golden neighbour lists into a JSON fixture.

The reference (tumaer/jax-sph) cannot be imported here (it needs JAX), so this
script reads its test file as text and evaluates only the literal arrays of the
four cases in ``tests/test_neighbors.py:87-121`` (positions, box, cutoff,
mask_self flag and the expected canonical edge list). It writes
``neighbors_golden.json`` next to itself.

Usage: python tests/golden/make_golden.py path/to/jax-sph
"""

import ast
import json
import os
import sys


def _literal(node):
    """Evaluate ``jnp.array([...])`` / ``np.array([...])`` / plain literals."""
    if isinstance(node, ast.Call) and node.args:
        return ast.literal_eval(node.args[0])
    return ast.literal_eval(node)


def extract(test_file):
    tree = ast.parse(open(test_file).read())
    fn = next(n for n in ast.walk(tree)
              if isinstance(n, ast.FunctionDef) and n.name == "cases")
    cases, args = [], None
    for stmt in fn.body:
        if isinstance(stmt, ast.Assign):
            tgt = stmt.targets[0]
            if isinstance(tgt, ast.Name) and tgt.id == "args":
                args = {ast.literal_eval(k): _literal(v)
                        for k, v in zip(stmt.value.keys, stmt.value.values)}
            elif isinstance(tgt, ast.Subscript):
                key = ast.literal_eval(tgt.slice)
                args = dict(args)
                args[key] = _literal(stmt.value)
        elif isinstance(stmt, ast.Expr) and isinstance(stmt.value, ast.Call):
            call = stmt.value
            if isinstance(call.func, ast.Attribute) and call.func.attr == "body":
                cases.append(dict(args, source_line=stmt.lineno))
    return cases


def main():
    if len(sys.argv) != 2:
        sys.exit("usage: make_golden.py path/to/jax-sph (a checkout of the reference)")
    root = sys.argv[1]
    test_file = os.path.join(root, "tests", "test_neighbors.py")
    cases = extract(test_file)
    out = {
        "source": "tests/test_neighbors.py (tumaer/jax-sph), cases() :87-121",
        "comparison": "real edges sorted by idx[0] then stably by idx[1] (:77-82)",
        "cases": cases,
    }
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "neighbors_golden.json")
    with open(dst, "w") as f:
        json.dump(out, f, indent=1)
    print(f"wrote {len(cases)} cases to {dst}")


if __name__ == "__main__":
    main()
