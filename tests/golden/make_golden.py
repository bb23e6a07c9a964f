"""Regenerate tests/golden/core_known_answers.json from the reference's own
test files (read as text; the reference is Julia and cannot run here).

Usage:  python tests/golden/make_golden.py /path/to/reference
        (or with the path in the environment variable BEM_REFERENCE_DIR)

Each entry records the reference file and line it was read from.  Only
numeric literals and thresholds are extracted; the closed-form identities the
reference tests use are restated in tests/test_oracle_known_answers.py.
"""
import json
import os
import re
import sys

REF = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("BEM_REFERENCE_DIR")
if not REF:
    raise SystemExit("usage: make_golden.py /path/to/reference (the reference project root), "
                     "or set BEM_REFERENCE_DIR")
OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "core_known_answers.json")


def find(path, pattern, group_names):
    lines = open(os.path.join(REF, path), encoding="utf-8").read().splitlines()
    rx = re.compile(pattern)
    for i, ln in enumerate(lines, 1):
        m = rx.search(ln)
        if m:
            vals = {g: float(m.group(g)) for g in group_names}
            return vals, f"{path}:{i}"
    raise SystemExit(f"pattern not found in {path}: {pattern}")


NUM = r"[-+]?\d+\.\d+(?:[eE][-+]?\d+)?"
g = {}
v, src = find("test/core.jl", rf"ζ0, η0 = (?P<z0>{NUM}), (?P<e0>{NUM})", ["z0", "e0"])
g["p3c_example_input"] = dict(v, source=src)
v, src = find("test/core.jl", rf"@test ζ̃ ≈ (?P<zt>{NUM}) atol=(?P<atol>\d+e-\d+)", ["zt", "atol"])
g["p3c_example_zeta_tilde"] = dict(v, source=src)
v, src = find("test/core.jl", rf"@test η̃ ≈ (?P<et>{NUM}) atol=(?P<atol>\d+e-\d+)", ["et", "atol"])
g["p3c_example_eta_tilde"] = dict(v, source=src)
v, src = find("test/core.jl", rf"a, b = (?P<a>{NUM}), (?P<b>{NUM})", ["a", "b"])
g["tangent_map_case"] = dict(v, source=src)
v, src = find("test/core.jl", rf"_tanp3ctrans\(u, w, (?P<z0>{NUM}), (?P<e0>\d+e-\d+)\)", ["z0", "e0"])
g["tanp3c_case3"] = dict(v, source=src)
v, src = find("test/laplace.jl", rf"@test rel_error\(dad\) < (?P<tol>{NUM})", ["tol"])
g["laplace_dense_rel_error_tol"] = dict(v, source=src)
v, src = find("test/laplace.jl", rf"@test maximum\(errT\[nf\]\) < (?P<tol>\d+e-\d+)", ["tol"])
g["nearfield_approach_tol"] = dict(v, source=src)
v, src = find("test/laplace.jl", rf"norm\(Float64.\(dad32.H\) - dad_ref.H\) / norm\(dad_ref.H\) < (?P<tol>\d+e-\d+)", ["tol"])
g["fp32_matrix_rel_tol"] = dict(v, source=src)
v, src = find("test/laplace.jl", rf"norm\(dad.H - dad_ref.H\) / norm\(dad_ref.H\) < (?P<tol>\d+e-\d+)", ["tol"])
g["fp64_matrix_rel_tol"] = dict(v, source=src)
v, src = find("test/elasticity.jl", rf"@test rel_error\(dad\) < (?P<tol>{NUM})", ["tol"])
g["elasticity_patch_rel_error_tol"] = dict(v, source=src)
g["_generated_by"] = "tests/golden/make_golden.py"
json.dump(g, open(OUT, "w"), indent=1, sort_keys=True)
print("wrote", OUT)
