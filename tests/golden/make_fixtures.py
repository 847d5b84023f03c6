"""Generates the golden fixtures under tests/golden/.

1. reference_utils_known_answers.json: the known-answer arrays of the
   reference's only unit test (test/test_module_utils.f90:29-47, checked at
   :154-166) for get_array_union / get_array_intersection / get_array_norepeat,
   parsed from the reference source.  These are the set operations the
   interface and glob detection rely on (sorted shared-node lists).
2. oracle_small.json: iteration counts, Lanczos condition estimates, coarse
   space sizes and solution norms of the CPU oracle on small deterministic
   cases, used as regression pins of the oracle (the reference ships no
   solver goldens and cannot be built here).

Usage: python tests/golden/make_fixtures.py <path-to-reference-checkout>
"""
import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def parse_reference_utils(ref):
    src = open(os.path.join(ref, "test", "test_module_utils.f90")).read()
    out = {}
    for name in ["array1", "array2", "intersection_check", "union_check", "array3", "array3_check"]:
        m = re.search(r"::\s*" + name + r"\([^)]*\)\s*=\s*\[([^\]]*)\]", src)
        out[name] = [int(x) for x in m.group(1).split(",")]
    out["source"] = "test/test_module_utils.f90:29-47 (checked at :154-166)"
    return out


def oracle_cases():
    import numpy as np
    import oracle as orc
    from bddcml_gb300 import problems
    cases = {}
    specs = {
        "cube_4x2": lambda: problems.poisson_on_cube(4, 2),
        "cube_4x3": lambda: problems.poisson_on_cube(4, 3),
        "cube_5x4": lambda: problems.poisson_on_cube(5, 4),
        "cube_8x4": lambda: problems.poisson_on_cube(8, 4),
        "boxes_24_seed17": lambda: problems.poisson_boxes(24, problems.random_box_partition(24, 5, 10, seed=17)),
        "lognormal_16_seed3_w1": lambda: problems.poisson_on_cube(4, 4, kappa=problems.lognormal_kappa(16, 1.0, 3)),
    }
    for name, mk in specs.items():
        prob = mk()
        wt = 1 if name.endswith("_w1") else 0
        o = orc.Oracle(prob)
        o.setup(1, 1, wt)
        it, reason, cond = o.solve(1e-8, 300, 50)
        u = o.global_solution()
        cases[name] = {"weights_type": wt, "iterations": it, "reason": reason, "cond": cond,
                       "coarse": o.stats(), "solution_norm2": float(np.linalg.norm(u)),
                       "solution_max": float(np.max(u)), "relres": [float(x) for x in o.relres_history()]}
    return cases


if __name__ == "__main__":
    if len(sys.argv) != 2 or not os.path.isdir(sys.argv[1]):
        sys.exit("usage: make_fixtures.py <checkout of the reference sources>")
    with open(os.path.join(HERE, "reference_utils_known_answers.json"), "w") as f:
        json.dump(parse_reference_utils(sys.argv[1]), f, indent=1)
    with open(os.path.join(HERE, "oracle_small.json"), "w") as f:
        json.dump(oracle_cases(), f, indent=1)
