"""Extract the reference's own golden values for the fermion hot path into
reference_goldens.json.

Run where the lehner/gpt sources are mounted, giving their root as argv[1]
or in the environment variable GPT_REFERENCE_ROOT.  Only numbers are
extracted -- no code -- from:

  tests/core/checksums.py:11-21          sha256 of a test string (vs hashlib)
  tests/random/simple.py:17-31           plaquettes of g.qcd.gauge.random
  tests/random/simple.py:66-127          normal() samples at five coordinates
  tests/random/simple.py:129-141         rng.choice() results
  tests/qcd/fermion_operators.py:338-524 Grid operator fingerprints (wilson,
                                         wilson_clover, wilson_twisted_mass,
                                         mobius, mobius_axial_mass, zmobius)
  tests/qcd/fermion_operators.py:193-218 Wilson point-source correlator
  tests/qcd/domain_wall.py:193-209       Mobius J5q correlator
  tests/qcd/domain_wall.py:248-274       Mobius point-source correlator, and
                                         the zmobius (domain_wall.py:91-112)
                                         propagator's correlator against it
"""
import ast
import json
import os
import re
import sys

root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("GPT_REFERENCE_ROOT")
if not root:
    sys.exit("usage: make_reference_goldens.py <root of the lehner/gpt sources> (or set GPT_REFERENCE_ROOT)")


def read(p):
    with open(os.path.join(root, p)) as f:
        return f.read()


def lit(src, name):
    """Evaluate the literal assigned to `name` in a reference test file."""
    tree = ast.parse(src)
    for node in ast.walk(tree):
        if isinstance(node, ast.Assign) and any(isinstance(t, ast.Name) and t.id == name for t in node.targets):
            return node.value
    raise KeyError(name)


def num(node):
    """Literal numbers and the complex expressions a + 1j * (b) of the test file."""
    if isinstance(node, ast.Constant):
        return node.value
    if isinstance(node, ast.UnaryOp) and isinstance(node.op, ast.USub):
        return -num(node.operand)
    if isinstance(node, ast.UnaryOp) and isinstance(node.op, ast.UAdd):
        return num(node.operand)
    if isinstance(node, ast.BinOp):
        a, b = num(node.left), num(node.right)
        if isinstance(node.op, ast.Add):
            return a + b
        if isinstance(node.op, ast.Sub):
            return a - b
        if isinstance(node.op, ast.Mult):
            return a * b
    if isinstance(node, ast.List):
        return [num(e) for e in node.elts]
    raise ValueError(ast.dump(node))


def cplx_list(node):
    return [[complex(ast.literal_eval(e)).real, complex(ast.literal_eval(e)).imag] for e in node.elts]


out = {"source": "lehner/gpt test files (paths relative to the project root)"}

simple = read("tests/random/simple.py")
m = re.findall(r"\(grid_\w+, ([0-9e.-]+), ([0-9e.-]+), (\d+)\)", simple)
out["plaquette"] = {
    "cite": "tests/random/simple.py:17-31",
    "seed": "block_seed_string_13",
    "cases": [
        {"grid": [8, 4, 4, 4], "tol_sq": float(m[0][0]), "plaquette": float(m[0][1]), "scale": float(m[0][2])},
        {"grid": [8, 4, 4, 4], "tol_sq": float(m[1][0]), "plaquette": float(m[1][1]), "scale": float(m[1][2]), "single": True},
        {"grid": [8, 8, 4, 8], "tol_sq": float(m[2][0]), "plaquette": float(m[2][1]), "scale": float(m[2][2])},
    ],
}
refs = re.findall(r"test_sequence_ref = np\.array\(\s*\[([^\]]*)\]", simple)
out["normal_samples"] = {
    "cite": "tests/random/simple.py:91-127",
    "seed": "block_seed_string_13",
    "grid": [8, 4, 4, 4],
    "coords": [[0, 0, 0, 0], [2, 0, 0, 0], [0, 2, 0, 0], [1, 3, 1, 3], [3, 2, 1, 0]],
    "after_0": [float(x) for x in refs[0].replace("\n", " ").split(",") if x.strip()],
    "after_1000": [float(x) for x in refs[1].replace("\n", " ").split(",") if x.strip()],
    "tol": 1e-14,
}
ch = re.search(r'assert rng\.choice\(\["A", "B", "C"\], 10\) == \[([^\]]*)\]', simple, re.S).group(1)
ch2 = re.search(r"np\.array\(\[1, 2, 3\]\), 5\) == np\.array\(\[([^\]]*)\]", simple).group(1)
out["choice"] = {
    "cite": "tests/random/simple.py:129-141",
    "abc_10": [x.strip().strip('"') for x in ch.split(",") if x.strip()],
    "123_5": [int(x) for x in ch2.split(",")],
}
cs = read("tests/core/checksums.py")
out["sha256"] = {"cite": "tests/core/checksums.py:11-21", "input": re.search(r'test = b"([^"]*)"', cs).group(1)}

fo = read("tests/qcd/fermion_operators.py")
params = {}
for pname in ["wilson_params", "wilson_clover_params", "wilson_twisted_mass_params"]:
    node = lit(fo, pname)
    params[pname] = {ast.literal_eval(k): ast.literal_eval(v) for k, v in zip(node.keys, node.values)}
mats = {}
for mname in ["wilson_matrices", "wilson_clover_matrices", "wilson_twisted_mass_matrices"]:
    node = lit(fo, mname)
    mats[mname] = {ast.literal_eval(k): cplx_list(v)[0] for k, v in zip(node.keys, node.values)}
suite = lit(fo, "test_suite")
mob = {}
for k, v in zip(suite.keys, suite.values):
    key = ast.literal_eval(k)
    if key not in ("mobius", "mobius_axial_mass", "zmobius"):
        continue
    d = {ast.literal_eval(kk): vv for kk, vv in zip(v.keys, v.values)}
    p = {ast.literal_eval(kk): num(vv) for kk, vv in zip(d["params"].keys, d["params"].values)}
    if "omega" in p:  # complex numbers as [re, im] pairs
        p["omega"] = [[complex(w).real, complex(w).imag] for w in p["omega"]]
    mm = {ast.literal_eval(kk): cplx_list(vv)[0] for kk, vv in zip(d["matrices"].keys, d["matrices"].values)}
    mob[key] = {"params": p, "matrices": mm}
out["fingerprints"] = {
    "cite": "tests/qcd/fermion_operators.py:338-524 (procedure 847-908)",
    "seed": "finger_print",
    "grid": [8, 8, 8, 16],
    "rel_tol": 1e-13,
    "wilson": {"params": params["wilson_params"], "matrices": mats["wilson_matrices"]},
    "wilson_clover": {"params": params["wilson_clover_params"], "matrices": mats["wilson_clover_matrices"]},
    "wilson_twisted_mass": {"params": params["wilson_twisted_mass_params"], "matrices": mats["wilson_twisted_mass_matrices"]},
    **mob,
}
# solve-level goldens: correlators of point-source propagators (single precision in the reference)
out["wilson_correlator"] = {
    "cite": "tests/qcd/fermion_operators.py:12-34 (gauge, parameters), 137-158 (point source, eo2_ne cg), "
            "190-218 (correlator)",
    "seed": "test", "grid": [8, 8, 8, 16], "gauge_scale": 1.0, "single": True, "kappa": 0.137,
    "boundary_phases_exp_i": [1, 2, 3, 4], "point": [1, 0, 0, 0], "cg_eps": 1e-6,
    "correlator": num(lit(fo, "correlator_ref")), "tol": 1e-5,
}
dw = read("tests/qcd/domain_wall.py")
mp = lit(dw, "mobius_params")
mp = {ast.literal_eval(k): num(v) for k, v in zip(mp.keys, mp.values)}
def call_dict(src, name):
    """The literal params dict passed to the call assigned to `name`."""
    for node in ast.walk(ast.parse(src)):
        if isinstance(node, ast.Assign) and any(isinstance(t, ast.Name) and t.id == name for t in node.targets):
            d = node.value.args[1]
            return {ast.literal_eval(k): num(v) for k, v in zip(d.keys, d.values)}
    raise KeyError(name)


zp = call_dict(dw, "qz")
zp["omega"] = [[complex(w).real, complex(w).imag] for w in zp["omega"]]
out["mobius_correlators"] = {
    "cite": "tests/qcd/domain_wall.py:15-33 (gauge, parameters), 117-127 (point source, eo2_ne cg), "
            "171-177 (bulk propagator), 193-209 (J5q), 248-274 (correlator)",
    "seed": "test", "grid": [8, 8, 8, 8], "gauge_scale": 2.0, "single": True, "params": mp,
    "point": [0, 1, 0, 0], "cg_eps": 1e-5,
    "J5q": num(lit(dw, "J5q_ref")), "J5q_tol": 1e-5,
    "correlator": num(lit(dw, "correlator_ref")), "correlator_tol": 1e-5,
    "zmobius_params": zp, "zmobius_correlator_tol": 5e-4,
}
with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_goldens.json"), "w") as f:
    json.dump(out, f, indent=1)
print("wrote reference_goldens.json")
