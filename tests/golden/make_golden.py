"""Extract the reference test-suite's known-answer systems into golden fixtures.

Reads (as text, with `ast`) the literal systems that lineax's own tests solve
and assert on, and writes them to tests/golden/reference_kats.json:

* tests/test_solve.py::test_nontrivial_pytree_operator / test_mixed_dtypes —
  the 2×2 system [[1, 5], [-2, -2]] x = [3, 4], x = [-3.25, 1.25]
  (LU, QR and the default solver must all return it);
* tests/test_solve.py::test_mixed_dtypes_triangular — lower-triangular
  [[1, 0], [-2, -2]] x = [3, 4], x = [3, -5];
* tests/test_singular.py::test_gmres_stagnation_or_breakdown — the literal 4×4
  matrix and true_x on which GMRES(restart=2, rtol=atol=1e-10) must report a
  failure;
* tests/test_solve.py::test_nonfinite_input — right-hand sides containing
  inf/NaN must give RESULTS.nonfinite_input;
* tests/test_singular.py::test_nonsquare_pytree_operator1/2 — the literal
  2×3 and 3×2 systems whose QR and Normal(Cholesky()) solutions must equal the
  least-squares (minimum-norm) answer.

The JAX reference cannot run here (no JAX), so these literal cases are the
reference's own answers.  Run from the repository root:
    python tests/golden/make_golden.py [path/to/lineax-checkout]
"""

from __future__ import annotations

import ast
import json
import pathlib
import sys

HERE = pathlib.Path(__file__).resolve().parent


def _literal(node):
    """Evaluate a literal, unwrapping f32(...)/f64(...)/jnp.array(...) calls."""
    if isinstance(node, ast.Call):
        return _literal(node.args[0])
    if isinstance(node, (ast.List, ast.Tuple)):
        return [_literal(e) for e in node.elts]
    if isinstance(node, ast.UnaryOp) and isinstance(node.op, ast.USub):
        return -_literal(node.operand)
    if isinstance(node, ast.Attribute) and node.attr in ("inf", "nan"):
        return float(node.attr)
    return ast.literal_eval(node)


def _function(tree, name):
    for node in ast.walk(tree):
        if isinstance(node, ast.FunctionDef) and node.name == name:
            return node
    raise KeyError(name)


def _assigns(fn):
    out = {}
    for node in ast.walk(fn):
        if isinstance(node, ast.Assign) and len(node.targets) == 1:
            tgt = node.targets[0]
            if isinstance(tgt, ast.Name):
                out.setdefault(tgt.id, []).append(node.value)
    return out


def main(ref_root: pathlib.Path) -> dict:
    solve_src = (ref_root / "tests" / "test_solve.py").read_text()
    singular_src = (ref_root / "tests" / "test_singular.py").read_text()
    t_solve = ast.parse(solve_src)
    t_sing = ast.parse(singular_src)
    kats = {}

    a = _assigns(_function(t_solve, "test_nontrivial_pytree_operator"))
    kats["pytree_2x2"] = {
        "source": "tests/test_solve.py::test_nontrivial_pytree_operator",
        "matrix": [[float(v) for v in row] for row in _literal(a["x"][0])],
        "vector": [float(v) for v in _literal(a["y"][0])],
        "solution": [float(v) for v in _literal(a["true_out"][0])],
        "solvers": ["Auto", "LU", "QR"],
    }
    a = _assigns(_function(t_solve, "test_mixed_dtypes"))
    kats["mixed_dtypes_2x2"] = {
        "source": "tests/test_solve.py::test_mixed_dtypes",
        "matrix": [[float(v) for v in row] for row in _literal(a["x"][0])],
        "vector": [float(v) for v in _literal(a["y"][0])],
        "solution": [float(v) for v in _literal(a["true_out"][0])],
        "solvers": ["LU", "QR"],
    }
    a = _assigns(_function(t_solve, "test_mixed_dtypes_triangular"))
    kats["triangular_2x2"] = {
        "source": "tests/test_solve.py::test_mixed_dtypes_triangular",
        "matrix": [[float(v) for v in row] for row in _literal(a["x"][0])],
        "vector": [float(v) for v in _literal(a["y"][0])],
        "solution": [float(v) for v in _literal(a["true_out"][0])],
        "tags": ["lower_triangular"],
        "solvers": ["Triangular"],
    }
    fn = _function(t_sing, "test_gmres_stagnation_or_breakdown")
    a = _assigns(fn)
    kats["gmres_fails_4x4"] = {
        "source": "tests/test_singular.py::test_gmres_stagnation_or_breakdown",
        "matrix": _literal(a["matrix"][0]),
        "true_x": _literal(a["true_x"][0]),
        "solver": {"kind": "GMRES", "rtol": 1e-10, "atol": 1e-10, "restart": 2},
        "expect": "result != successful",
    }
    for name, key in (("test_nonsquare_pytree_operator1", "nonsquare_wide_2x3"),
                      ("test_nonsquare_pytree_operator2", "nonsquare_tall_3x2")):
        a = _assigns(_function(t_sing, name))
        kats[key] = {
            "source": f"tests/test_singular.py::{name}",
            "matrix": [[float(v) for v in row] for row in _literal(a["matrix"][0])],
            "vector": [float(v) for v in _literal(a["y"][0])],
            "expect": "the least-squares / minimum-norm solution (jnp.linalg.lstsq)",
            "solvers": ["Auto(well_posed=None)", "QR", "Normal(Cholesky)"],
        }
    fn = _function(t_solve, "test_nonfinite_input")
    vecs = [_literal(v) for v in _assigns(fn)["vector"]]
    kats["nonfinite_input"] = {
        "source": "tests/test_solve.py::test_nonfinite_input",
        "diagonal": [1.0, 1.0],
        "vectors": [[float(x) for x in v] for v in vecs],
        "expect": "nonfinite_input",
    }
    return kats


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <path of the lineax source tree>")
    root = pathlib.Path(sys.argv[1])
    kats = main(root)
    out = HERE / "reference_kats.json"
    out.write_text(json.dumps(kats, indent=1, allow_nan=True) + "\n")
    print(f"wrote {out}")
