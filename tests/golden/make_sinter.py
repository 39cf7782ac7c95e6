"""Writes tests/golden/sinter/classify_cases.json: the known-answer cases of sinter's
classify_discards_and_errors, read (as text, through `ast`) from the reference's own test file
glue/sample/src/sinter/_decoding/_stim_then_decode_sampler_test.py.  Nothing of sinter is imported or run.

    python tests/golden/make_sinter.py path/to/reference/root     (or set STIM_REFERENCE_TREE)
"""

import ast
import json
import os
import sys

ROOT = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("STIM_REFERENCE_TREE", "")
if not ROOT:
    sys.exit("usage: make_sinter.py path/to/reference/root (or set STIM_REFERENCE_TREE)")
SRC = os.path.join(ROOT, "glue/sample/src/sinter/_decoding/_stim_then_decode_sampler_test.py")
OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "sinter", "classify_cases.json")


def literal(node):
    """np.array([...], dtype=...) -> the list; None -> None; a name -> its identifier; else a literal."""
    if isinstance(node, ast.Call) and getattr(node.func, "attr", None) == "array":
        return ast.literal_eval(node.args[0])
    if isinstance(node, ast.Name):
        return {"name": node.id}
    return ast.literal_eval(node)


def main():
    tree = ast.parse(open(SRC).read())
    cases = []
    for node in ast.walk(tree):
        if not isinstance(node, ast.Assert) or not isinstance(node.test, ast.Compare):
            continue
        left = node.test.left
        if isinstance(left, ast.Call) and getattr(left.func, "id", None) == "classify_discards_and_errors":
            kw = {k.arg: literal(k.value) for k in left.keywords}
            kw["expected"] = list(ast.literal_eval(node.test.comparators[0]))
            cases.append(kw)
        elif isinstance(left, ast.Name) and isinstance(node.test.comparators[0], ast.Call):
            # `assert counter == collections.Counter([...])`: the combos the previous case counted.
            keys = ast.literal_eval(node.test.comparators[0].args[0])
            cases[-1]["expected_combos"] = {k: keys.count(k) for k in keys}
    for c in cases:
        c["count_combos"] = c.pop("out_count_observable_error_combos") is not None
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    with open(OUT, "w") as f:
        json.dump({"source": "glue/sample/src/sinter/_decoding/_stim_then_decode_sampler_test.py", "cases": cases},
                  f, separators=(",", ":"))
    print(f"{len(cases)} cases -> {OUT}")


if __name__ == "__main__":
    main()
