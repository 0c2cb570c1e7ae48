"""Generate golden fixtures from the reference itself.

Runs the reference MADAM sources compiled by oracle/ref/Makefile (the
strict-IEEE build, oracle/_ref/madam_ref_strict) on seeded synthetic rudy-style
instances and records, per instance, every evaluated node's bound, the node
count, the optimum and the optimal cut vector.  The instances are regenerated
from their seeds by madam_gb300.graphs, so the fixtures travel without the
reference.  reference_bab.json holds trees under the shipped parameter file;
reference_bab_params.json holds trees under other settings (triangles only, no
heptagons, least-fractional branching, no diff give-up, another sigma0, a fixed
triangle budget), which exercise the remaining branches of the bound and the
driver.  Run where the reference sources are present:

    python tests/golden/make_golden.py
"""
import json
import os
import re
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from madam_gb300 import graphs as G  # noqa: E402

# (name, generator, args) -- small enough for the oracle to finish in seconds
INSTANCES = [
    ("gnp40_one_s1", "gnp", (40, 0.5, "one", 1)),
    ("gnp60_int10_s14", "gnp", (60, 0.5, "int10", 14)),
    ("gnp64_pm1_s13", "gnp", (64, 0.5, "pm1", 13)),
    ("gnp70_one_s11", "gnp", (70, 0.5, "one", 11)),
    ("torus7x7_s15", "torus", (7, 7, 15)),
]

# (name, generator, args, parameter overrides of the shipped file)
VARIANTS = [
    ("gnp56_pm1_s31_tri", "gnp", (56, 0.5, "pm1", 31), dict(include_Pent=0, include_Hepta=0)),
    ("gnp56_pm1_s39_least", "gnp", (56, 0.5, "pm1", 39), dict(branchingStrategy=0)),
    ("gnp56_pm1_s49_nodiff", "gnp", (56, 0.5, "pm1", 49), dict(use_diff=0, sigma0=1.6)),
    ("gnp56_pm1_s37_nohept", "gnp", (56, 0.5, "pm1", 37), dict(include_Hepta=0)),
    ("gnp60_int10_s25_sparse", "gnp", (60, 0.2, "int10", 25), dict(TriIneq=300, adjust_TriIneq=0)),
]

SHIPPED = """sigma0 = 1
scaleSigma = 1.001
ADMM_itermax = 2000
tol0 = 5e-2
scaleTol = 0.6
minTol = 1e-3
triag_iter = 3
pent_iter = 3
hept_iter = 3
max_outer_iter = 12
extra_iter = 5
violated_TriIneq = 1e-3
TriIneq = 5000
adjust_TriIneq = 1
PentIneq = 5000
HeptaIneq = 5000
Pent_Trials = 60
Hepta_Trials = 50
include_Pent = 1
include_Hepta = 1
root = 0
use_diff = 1
branchingStrategy = 1
"""


def make_instance(kind, args):
    if kind == "gnp":
        return G.gnp(*args[:3], seed=args[3])
    return G.torus2d(args[0], args[1], seed=args[2])


def params_text(over=None):
    """The shipped parameter file with some values replaced."""
    lines = []
    for line in SHIPPED.splitlines():
        name = line.split("=")[0].strip()
        lines.append("%s = %s" % (name, over[name]) if over and name in over else line)
    return "\n".join(lines) + "\n"


def run_reference(binary, n, e, w, max_nodes=2000, over=None):
    with tempfile.TemporaryDirectory(dir=HERE) as d:
        g = os.path.join(d, "graph")
        G.write_rudy(g, n, e, w)
        p = os.path.join(d, "params")
        open(p, "w").write(params_text(over))
        out = subprocess.run([binary, g, p, str(max_nodes)], capture_output=True, text=True, cwd=d, timeout=3600)
    if out.returncode != 0:
        raise RuntimeError(out.stderr)
    txt = out.stdout
    bounds = [float(x) for x in re.findall(r"^node \d+ level \d+ n \d+ bound (\S+)", txt, re.M)]
    nodes = int(re.search(r"^Nodes = (\d+)", txt, re.M).group(1))
    opt = float(re.search(r"^Maximum value = (\S+)", txt, re.M).group(1))
    sol = [int(v) - 1 for v in re.search(r"^Solution = \( (.*)\)", txt, re.M).group(1).split()]
    return dict(bounds=bounds, nodes=nodes, opt=opt, sol=sol)


def main():
    binary = os.path.join(ROOT, "oracle", "_ref", "madam_ref_strict")
    if not os.path.exists(binary):
        sys.exit("build the reference oracle first (make -C oracle/ref)")
    fixtures = []
    for name, kind, args in INSTANCES:
        n, e, w = make_instance(kind, args)
        r = run_reference(binary, n, e, w)
        r.update(name=name, kind=kind, args=list(args), n=n, edges=len(w), params="shipped")
        fixtures.append(r)
        print(name, "nodes", r["nodes"], "opt", r["opt"], "root %.9f" % r["bounds"][0], "evaluated", len(r["bounds"]))
    json.dump({"generator": "tests/golden/make_golden.py", "reference_build": "oracle/ref/Makefile strict flavour",
               "instances": fixtures}, open(os.path.join(HERE, "reference_bab.json"), "w"), indent=1)
    variants = []
    for name, kind, args, over in VARIANTS:
        n, e, w = make_instance(kind, args)
        r = run_reference(binary, n, e, w, over=over)
        r.update(name=name, kind=kind, args=list(args), n=n, edges=len(w), params=over)
        variants.append(r)
        print(name, "nodes", r["nodes"], "opt", r["opt"], "root %.9f" % r["bounds"][0], "evaluated", len(r["bounds"]))
    json.dump({"generator": "tests/golden/make_golden.py", "reference_build": "oracle/ref/Makefile strict flavour",
               "instances": variants}, open(os.path.join(HERE, "reference_bab_params.json"), "w"), indent=1)


if __name__ == "__main__":
    main()
