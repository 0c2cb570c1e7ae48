"""Plain-form parity at the benchmark's full sizes, and the reference's published
optima.

(1) Node bounds of the plain FP64 form at n = 256 (G(256, 0.5), +-1 weights,
triangle + pentagonal cuts), n = 512 (G(512, 0.1), integer weights in
[-10, 10], all three cut families) and n = 400 (20 x 20 torus, +-1 weights, all
three families), several nodes per batched call, against the oracle's answers
for the same nodes (tests/golden/oracle_fullsize.json, made by
make_oracle_fullsize.py: the oracle in the counter-stream mode the GPU form
reproduces, each node bounded alone, with an incumbent that none of the nodes
improves, so the batched call shares an incumbent that never changes).
Bounds agree to 1e-6 relative and the round, ADMM-iteration and cut counts are
identical, as bounding.c:25-250 run on the same inputs would give.  The chosen
form (Newton-Schulz projection on the tensor cores, projection error ~5e-9 of
||W||) is held to the same bar on the G(n, p) nodes.  The torus nodes' ADMM runs
(1,700-5,000 iterations) converge so slowly that a projection error far below
1e-8 absolute moves their fixed point: the oracle's own answer changes by 5e-5
when only the eigenvalues below 1e-6 ||W||_F are treated as a Newton-Schulz
iteration treats them, while a 1e-9 change of the data moves it by 1e-12.  The
chosen form's torus bounds stay within 1e-3 of the oracle's (valid bounds either
way: the safe dual bound is FP64).

(2) Whole plain-form branch-and-bound runs on three of the reference's published
instances of order 150 (tests/golden/published_n150.json: the instance, the
parameters of the published run and its answer, Instances/rudy/rudy_150/
ro_1.6/*.output:5-32) reach the published optimum with a cut that attains it.
Tree sizes differ from the published ones (240 MPI workers there, batches of
open nodes here, and other random streams for the k-gonal cuts), so the
published node count is not compared; the root bound is a valid bound on the
optimum and lies within 0.5% of the published root bound.
"""
import json
import os

import numpy as np
import pytest

from madam_gb300 import graphs as G
from madam_gb300 import workload as W

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
_FULL = json.load(open(os.path.join(HERE, "golden", "oracle_fullsize.json")))
FULL, INCUMBENT = _FULL["workloads"], _FULL["incumbent"]
PUBLISHED = json.load(open(os.path.join(HERE, "golden", "published_n150.json")))["instances"]

REL = 1e-6


def _bound_nodes(M, name, recs, proj):
    wl = W.make(name)
    ctx = M.Context(M.params(**wl["params"]), wl["SL"], wl["n"], batch_max=len(recs), flags=proj)
    ctx.set_lb(INCUMBENT[name])
    b, st = ctx.bound_batch([M.node(wl["fixings"][r["node"]]) for r in recs], rank=1)
    ctx.close()
    return b, st


CASES = [(name, "fp64") for name in sorted(FULL)] + [(name, "ns") for name in sorted(FULL) if "torus" not in name]


@pytest.mark.parametrize("name,form", CASES)
def test_fullsize_node_bounds_match_oracle(gpu_lib, name, form):
    M = gpu_lib
    wl = W.make(name)
    # the plain form's torus run here is the node of 1,681 ADMM iterations (the
    # others take minutes in FP64); the chosen form's torus nodes are compared below
    recs = [r for r in FULL[name] if r["admm_iters"] <= 2000]
    proj = M.PROJ_FP64 if form == "fp64" else M.PROJ_NS_BF16
    ctx = M.Context(M.params(**wl["params"]), wl["SL"], wl["n"], batch_max=len(recs), flags=proj)
    # the incumbent no node of the list improves (so every node sees it, batched or alone)
    ctx.set_lb(INCUMBENT[name])
    b, st = ctx.bound_batch([M.node(wl["fixings"][r["node"]]) for r in recs], rank=1)
    ctx_lb = ctx.lb()[0]
    ctx.close()
    bad = []
    for r, bg, sg in zip(recs, b, st):
        got = (sg.outer_iters, sg.admm_iters, sg.ipm_iters, sg.n_tri, sg.n_pent, sg.n_hept, sg.pruned, sg.gaveup)
        want = (r["outer_iters"], r["admm_iters"], r["ipm_iters"], r["n_tri"], r["n_pent"], r["n_hept"],
                r["pruned"], r["gaveup"])
        if abs(bg - r["bound"]) > REL * abs(r["bound"]) or got != want or \
                abs(sg.basic_bound - r["basic_bound"]) > 1e-9 * abs(r["basic_bound"]):
            bad.append((r["node"], bg, r["bound"], got, want))
    assert not bad, bad
    if form == "fp64":
        assert ctx_lb == INCUMBENT[name]
    else:
        # the chosen form's own rounding heuristic (hyperplanes through X v, 1-opt on
        # the GPU) may find a better cut than the oracle's; never a worse incumbent
        assert ctx_lb >= INCUMBENT[name]


@pytest.mark.parametrize("fx", PUBLISHED, ids=lambda f: f["name"].replace("/", "_"))
def test_plain_branch_and_bound_reaches_published_optimum(gpu_lib, fx):
    M = gpu_lib
    n = fx["n"]
    e = np.asarray(fx["edges"], dtype=np.int32)
    w = np.asarray(fx["weights"])
    SL = G.extended_laplacian(n, e, w).ravel(order="F")
    ctx = M.Context(M.params(**fx["params"]), SL, n, batch_max=16, flags=M.PROJ_FP64)
    r = ctx.bab(batch=16, max_nodes=20000)
    ctx.close()
    assert not r["stopped"]
    assert r["opt"] == fx["opt"]
    side = np.zeros(n, dtype=np.int32)
    side[: n - 1] = r["sol"]
    assert G.cut_value(n, e, w, side) == fx["opt"]
    assert r["root_bound"] >= fx["opt"]
    assert abs(r["root_bound"] - fx["root_bound"]) <= 5e-3 * fx["root_bound"]


def test_chosen_form_torus_nodes_stay_close(gpu_lib):
    """The four torus nodes (1,681-5,088 ADMM iterations) in the chosen form:
    valid bounds within 1e-3 of the oracle's (their sensitivity is stated above)."""
    M = gpu_lib
    name = "torus20x20_pm1"
    recs = FULL[name]
    b, st = _bound_nodes(M, name, recs, M.PROJ_NS_BF16)
    for r, bg, sg in zip(recs, b, st):
        assert abs(bg - r["bound"]) <= 1e-3 * abs(r["bound"]), (r["node"], bg, r["bound"])
        assert bg >= INCUMBENT[name]
        assert abs(sg.admm_iters - r["admm_iters"]) <= 0.25 * r["admm_iters"]
