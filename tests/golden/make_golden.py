"""Regenerate the golden fixtures in this folder from the reference checkout.

Run once, where the reference source tree is available:

    python tests/golden/make_golden.py /path/to/LAML

It reads the reference's unit-test *sources as text* (``ast`` on
laml_unit_tests/unit_tests_EMSolver.py and unit_tests_MLSolver.py) and pulls
out every known-answer case: the literal ``Q``, ``T``, ``msa``, ``phi``,
``nu`` and ``true_nllh`` of the likelihood tests, and the arguments of each
``__test_outllh__`` call (the reduced-tree outside identity tests); from
unit_tests_TopoSearch.py the ultrametric brute-force case with its
pre-computed optimum.  It also
copies the small data fixtures those tests load (test_EM/test1 and test4)
and the example1 inputs with the runner's outputs for them (example1/).
Nothing here imports or runs reference code.
"""
import ast
import json
import os
import shutil
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def _literal_assigns(fn):
    vals = {}
    for node in ast.walk(fn):
        if isinstance(node, ast.Assign) and len(node.targets) == 1 and \
                isinstance(node.targets[0], ast.Name):
            try:
                vals[node.targets[0].id] = ast.literal_eval(node.value)
            except Exception:
                pass
    return vals


def _solver_params(fn):
    for node in ast.walk(fn):
        if isinstance(node, ast.Call) and getattr(node.func, "id", None) in (
                "EM_solver", "ML_solver") and len(node.args) >= 4:
            try:
                return ast.literal_eval(node.args[3])
            except Exception:
                return None
    return None


def _outllh_call(fn, vals):
    for node in ast.walk(fn):
        if isinstance(node, ast.Call) and isinstance(node.func, ast.Attribute) and \
                node.func.attr == "__test_outllh__":
            names = [a.id if isinstance(a, ast.Name) else None for a in node.args]
            if names[:5] == ["T", "Q", "msa", "phi", "nu"] and all(
                    k in vals for k in ("T", "Q", "msa", "phi", "nu")):
                return {k: vals[k] for k in ("T", "Q", "msa", "phi", "nu")}
    return None


def _jsonable(v):
    if isinstance(v, dict):
        return {"__dict__": [[_jsonable(k), _jsonable(x)] for k, x in v.items()]}
    if isinstance(v, (list, tuple)):
        return [_jsonable(x) for x in v]
    return v


def extract(path, source_name):
    tree = ast.parse(open(path).read())
    llh, outside = [], []
    for cls in tree.body:
        if not isinstance(cls, ast.ClassDef):
            continue
        for fn in cls.body:
            if not isinstance(fn, ast.FunctionDef) or not fn.name.startswith("test_"):
                continue
            vals = _literal_assigns(fn)
            if "true_nllh" in vals and all(k in vals for k in ("Q", "T", "msa")):
                params = _solver_params(fn) or {}
                llh.append({"name": f"{source_name}:{fn.name}:{fn.lineno}",
                            "Q": _jsonable(vals["Q"]), "T": vals["T"],
                            "msa": _jsonable(vals["msa"]),
                            "phi": params.get("phi", 0), "nu": params.get("nu", 0),
                            "true_nllh": vals["true_nllh"]})
            oc = _outllh_call(fn, vals)
            if oc is not None:
                outside.append({"name": f"{source_name}:{fn.name}:{fn.lineno}",
                                "Q": _jsonable(oc["Q"]), "T": oc["T"],
                                "msa": _jsonable(oc["msa"]), "phi": oc["phi"],
                                "nu": oc["nu"]})
    return llh, outside


def extract_ultrametric(path, source_name):
    """The ultrametric brute-force cases of unit_tests_TopoSearch.py: tests
    whose brute-force search runs with ultra_constr=True and whose source
    keeps the pre-computed optimum in a ``nllh_bf = <value>`` comment
    (test_10: 7.0063474330891236, the best ultrametric nllh over every
    rooted topology of the four leaves)."""
    import re
    text = open(path).read()
    lines = text.splitlines()
    tree = ast.parse(text)
    out = []
    for cls in tree.body:
        if not isinstance(cls, ast.ClassDef):
            continue
        for fn in cls.body:
            if not isinstance(fn, ast.FunctionDef) or not fn.name.startswith("test_"):
                continue
            src = "\n".join(lines[fn.lineno - 1:fn.end_lineno])
            m = re.search(r"nllh_bf\s*=\s*([0-9.eE+-]+)\s*#", src)
            vals = _literal_assigns(fn)
            leaves = None
            ultra = False
            for node in ast.walk(fn):
                if isinstance(node, ast.Call) and isinstance(node.func, ast.Attribute) and \
                        node.func.attr == "__brute_force_search__" and len(node.args) >= 3:
                    try:
                        leaves = ast.literal_eval(node.args[2])
                    except Exception:
                        leaves = None
                    ultra = any(k.arg == "ultra_constr" and getattr(k.value, "value", None) is True
                                for k in node.keywords)
            if m and ultra and leaves and "Q" in vals and "msa" in vals:
                out.append({"name": f"{source_name}:{fn.name}:{fn.lineno}",
                            "Q": _jsonable(vals["Q"]), "msa": _jsonable(vals["msa"]),
                            "leaves": leaves, "nllh_bf": float(m.group(1))})
    return out


def main(ref):
    ut = os.path.join(ref, "laml_unit_tests")
    llh, outside = [], []
    for f in ("unit_tests_EMSolver.py", "unit_tests_MLSolver.py"):
        a, b = extract(os.path.join(ut, f), "laml_unit_tests/" + f)
        llh += a
        outside += b
    ultra = extract_ultrametric(os.path.join(ut, "unit_tests_TopoSearch.py"),
                                "laml_unit_tests/unit_tests_TopoSearch.py")
    with open(os.path.join(HERE, "known_answers.json"), "w") as fo:
        json.dump({"llh": llh, "outside": outside, "ultrametric": ultra}, fo, indent=1)
    td = os.path.join(ut, "test_data", "test_EM")
    for f in ("test1.tre", "test1_charMtrx.txt", "test4.tre", "test4_charMtrx.txt",
              "test4_prior.csv"):
        shutil.copyfile(os.path.join(td, f), os.path.join(HERE, f))
    # examples/example1 (inputs) and examples/out_example1 (the runner's
    # outputs for them: scaled trees, parameters, posterior annotations)
    ex = os.path.join(HERE, "example1")
    os.makedirs(ex, exist_ok=True)
    for sub, f in (("example1", "character_matrix.csv"), ("example1", "priors.csv"),
                   ("out_example1", "example1_trees.nwk"),
                   ("out_example1", "example1_params.txt"),
                   ("out_example1", "example1_annotations.txt")):
        shutil.copyfile(os.path.join(ref, "examples", sub, f), os.path.join(ex, f))
    print(f"{len(llh)} likelihood cases, {len(outside)} outside cases, "
          f"{len(ultra)} ultrametric brute-force cases")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <path of the LAML checkout>")
    main(sys.argv[1])
