"""Node-bound parity: the GPU SDPbound against the CPU oracle (counter-RNG form,
canonical top-K, canonical eigenvector signs) on seeded graphs.

Tolerance: 1e-6 relative on every bound, with identical cut counts and round
counts, whenever each round's separation sees inputs that agree to rounding
(triangle cuts; one k-gonal family).  With pentagonal and heptagonal cuts
together over many rounds the simulated annealing's accept test
u < exp(-delta/t) at late (tiny) temperatures turns the 1e-13 differences
between the GPU eigensolver and LAPACK into different vertex orders of the
same k-sets, so those runs are held to the safe-bound property and 1e-3.
"""
import numpy as np
import pytest

from madam_gb300 import graphs as G

pytestmark = pytest.mark.gpu

REL = 1e-6


def _problem(n, p, wts, seed):
    nv, e, w = G.gnp(n, p, wts, seed=seed)
    return nv, G.extended_laplacian(nv, e, w).ravel(order="F")


def _run(gpu_lib, orc, n, p, wts, seed, fixed, pent, hept):
    N, SL = _problem(n, p, wts, seed)
    prm_g = gpu_lib.params(include_Pent=pent, include_Hepta=hept, use_diff=0)
    prm_o = orc.shipped_params(include_Pent=pent, include_Hepta=hept, use_diff=0)
    ctx = gpu_lib.Context(prm_g, SL, N)
    oc = orc.Ctx(prm_o, SL, N, rng=orc.RNG_COUNTER, topk=orc.TOPK_CANONICAL, canon_sign=1)
    nd = gpu_lib.node(fixed)
    ond = orc.make_node(N - 1, fixed)
    bg, sg = ctx.evaluate(nd, rank=1)
    bo, so = oc.evaluate(ond, rank=1)
    return N, ctx, oc, nd, ond, bg, sg, bo, so


@pytest.mark.parametrize("n,p,wts,seed,fixed,pent,hept", [
    (30, 0.5, "pm1", 1, {}, 1, 0),
    (40, 0.5, "one", 2, {3: 1, 11: 0}, 1, 0),
    (50, 0.3, "int10", 3, {0: 1, 5: 1, 9: 0}, 0, 1),
    (64, 0.5, "pm1", 4, {}, 0, 0),
    (64, 0.5, "pm1", 4, {}, 1, 0),
    (64, 0.5, "pm1", 4, {}, 0, 1),
    (80, 0.1, "int10", 5, {7: 1}, 0, 0),
])
def test_node_bound_matches_oracle(gpu_lib, orc, n, p, wts, seed, fixed, pent, hept):
    N, ctx, oc, nd, ond, bg, sg, bo, so = _run(gpu_lib, orc, n, p, wts, seed, fixed, pent, hept)
    assert abs(bg - bo) <= REL * abs(bo), (bg, bo)
    assert sg.outer_iters == so.outer_iters
    assert sg.admm_iters == so.admm_iters
    assert (sg.n_tri, sg.n_pent, sg.n_hept) == (so.n_tri, so.n_pent, so.n_hept)
    assert abs(sg.basic_bound - so.basic_bound) <= 1e-9 * abs(so.basic_bound)
    fg = np.ctypeslib.as_array(nd.fracsol)[: N - 1]
    fo = np.ctypeslib.as_array(ond.fracsol)[: N - 1]
    assert np.abs(fg - fo).max() <= 1e-5
    assert ctx.lb()[0] == oc.lb()[0]


def test_node_bound_all_families_long_run(gpu_lib, orc):
    N, ctx, oc, nd, ond, bg, sg, bo, so = _run(gpu_lib, orc, 64, 0.5, "pm1", 4, {}, 1, 1)
    assert abs(bg - bo) <= 1e-3 * abs(bo), (bg, bo)
    assert sg.outer_iters == so.outer_iters
    assert abs(sg.basic_bound - so.basic_bound) <= 1e-9 * abs(so.basic_bound)
    # both are safe dual bounds of the same node: neither is below the incumbent
    assert bg >= ctx.lb()[0] and bo >= oc.lb()[0]


def test_batch_is_order_independent(gpu_lib):
    """A node's bound does not depend on where it sits in a batch: random streams
    are keyed by the node, and incumbent updates are applied per round as a max."""
    N, SL = _problem(48, 0.5, "pm1", 8)
    fix = G.random_fixings(N, 6, 8, seed=3)
    prm = gpu_lib.params(include_Hepta=0, use_diff=0)
    res = []
    for order in (list(range(6)), [5, 3, 1, 0, 2, 4]):
        ctx = gpu_lib.Context(prm, SL, N, batch_max=6)
        ctx.set_lb(0.0)
        nodes = [gpu_lib.node(fix[i]) for i in order]
        b, _ = ctx.bound_batch(nodes, rank=1)
        res.append({i: b[k] for k, i in enumerate(order)})
    for i in range(6):
        assert res[0][i] == res[1][i]


def _fixtures():
    import json
    import os

    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "reference_bab.json")
    return json.load(open(path))["instances"]


@pytest.mark.parametrize("fx", _fixtures(), ids=lambda f: f["name"])
def test_plain_branch_and_bound_against_reference_trees(gpu_lib, orc, fx):
    """Whole trees of the plain FP64 form (one node per launch) on the reference's
    fixtures: the reference's optimum, the oracle's node count in counter-stream
    mode, and the reference's optimal cut wherever the oracle's counter mode finds
    that same cut.  Where the optimum has ties (the +-1 torus) the rounding
    heuristic's random stream picks among them: there the cut is checked by its value."""
    if fx["kind"] == "gnp":
        n, e, w = G.gnp(*fx["args"][:3], seed=fx["args"][3])
    else:
        n, e, w = G.torus2d(fx["args"][0], fx["args"][1], seed=fx["args"][2])
    SL = G.extended_laplacian(n, e, w).ravel(order="F")
    oc = orc.Ctx(orc.shipped_params(), SL, n, rng=orc.RNG_COUNTER, topk=orc.TOPK_CANONICAL, canon_sign=1)
    ro = oc.bab(max_nodes=2000)
    ctx = gpu_lib.Context(gpu_lib.params(), SL, n, batch_max=1, flags=gpu_lib.PROJ_FP64)
    r = ctx.bab(batch=1, max_nodes=2000)
    ctx.close()
    assert r["opt"] == fx["opt"] == ro["opt"]
    assert r["nodes"] == ro["nodes"]
    got = sorted(np.nonzero(r["sol"])[0].tolist())
    if sorted(np.nonzero(ro["sol"])[0].tolist()) == sorted(fx["sol"]):
        assert got == sorted(fx["sol"])
    side = np.zeros(n, dtype=np.int32)
    side[: n - 1] = r["sol"]
    assert G.cut_value(n, e, w, side) == fx["opt"]
