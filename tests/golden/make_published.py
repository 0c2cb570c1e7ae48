"""Copy a few of the reference's published answers into a fixture.

The reference ships 90 rudy instances of order 150 with the output of its own
240-core runs (Instances/rudy/rudy_150/<dir>/<family>.<k> and the matching
.output): the parameters of the run (lines 5-27), the node count (29), the
root bound to two decimals (30), the optimum (31) and a 1-based optimal vertex
set (32).  This script copies the instances whose published trees are smallest,
one per weight family, into published_n150.json (edge list, parameters and the
published answer), so that the GPU branch-and-bound can be run to those optima
where the reference checkout is absent.  Run where the reference is present:

    python tests/golden/make_published.py
"""
import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from madam_gb300 import graphs as G  # noqa: E402
from oracle.refdir import reference_dir  # noqa: E402

# the smallest published tree of three weight families: pw01 (positive weights,
# density 0.1), pm1s (+-1, density 0.1) and w01 (integers in [-10, 10], density 0.1)
PICK = ["ro_1.6/pw01_150.5", "ro_1.6/pm1s_150.5", "ro_1.6/w01_150.2"]


def parse_output(path):
    lines = open(path).read().splitlines()
    prm = {}
    for ln in lines[4:27]:
        m = re.match(r"\s*(\w+) = (\S+)", ln)
        if m:
            v = float(m.group(2))
            prm[m.group(1)] = int(v) if v == int(v) and "." not in m.group(2) else v
    out = {}
    for ln in lines[27:34]:
        m = re.match(r"(Nodes|Root node bound|Maximum value) = (\S+)", ln)
        if m:
            out[m.group(1)] = float(m.group(2))
        m = re.match(r"Solution = \( (.*)\)", ln)
        if m:
            out["Solution"] = [int(v) for v in m.group(1).split()]
    return prm, out


def main():
    ref = reference_dir()
    if not ref:
        sys.exit("the reference checkout is not present (set MADAM_REFERENCE)")
    base = os.path.join(ref, "Instances", "rudy", "rudy_150")
    fixtures = []
    for name in PICK:
        n, e, w = G.read_rudy(os.path.join(base, name))
        prm, out = parse_output(os.path.join(base, name + ".output"))
        side = [0] * n
        for v in out["Solution"]:
            side[v - 1] = 1
        assert G.cut_value(n, e, w, side) == out["Maximum value"], name
        fixtures.append({"name": name, "n": int(n), "edges": e.tolist(), "weights": w.tolist(), "params": prm,
                         "nodes": int(out["Nodes"]), "root_bound": out["Root node bound"],
                         "opt": out["Maximum value"], "solution": out["Solution"]})
    json.dump({"generator": "tests/golden/make_published.py",
               "source": "Instances/rudy/rudy_150 of the reference, with the .output of its published runs",
               "instances": fixtures}, open(os.path.join(HERE, "published_n150.json"), "w"))
    print("wrote %d instances" % len(fixtures))


if __name__ == "__main__":
    main()
