"""Several independent problems in one context, bounded in one batched pass.

The uneven batch of the benchmark is many subproblems of different orders and
densities.  Each node of a batched call belongs to its own problem: its
createSubproblem reads that problem's SP->L (evaluate.c:39-116), its heuristic
updates that problem's incumbent (heuristic.c, heap.c:185-193), and its
separation uses that problem's triangle budget (10 N under adjust_TriIneq,
process_input.c:122-123).  So every root bound of the batch equals the root
bound of its problem bounded alone, which the oracle gives: 1e-6 relative with
identical round, ADMM-iteration and cut counts, and the same incumbent.
"""
import numpy as np
import pytest

from madam_gb300 import workload as W

pytestmark = pytest.mark.gpu


def _specs(k, nmax):
    return [s for s in W.uneven_specs(400) if s[0] <= nmax][:k]


@pytest.mark.parametrize("slots", [6, 4])
def test_uneven_problems_in_one_batch_match_the_oracle_alone(gpu_lib, orc, slots):
    """All roots in one call (six slots), or in chunks of similar order (four slots)."""
    M = gpu_lib
    specs = _specs(6, 110)
    insts = [W.uneven_instance(s) for s in specs]
    order = sorted(range(len(insts)), key=lambda i: -insts[i][0])  # problem 0: the largest order
    prm = dict(include_Hepta=0, use_diff=0)
    big = insts[order[0]]
    ctx = M.Context(M.params(**prm), big[3], big[0], batch_max=slots, flags=M.PROJ_FP64)
    pid = {order[0]: 0}
    for i in order[1:]:
        pid[i] = ctx.add_problem(insts[i][3], insts[i][0])
    assert sorted(pid.values()) == list(range(len(insts)))
    nodes = [M.node({}) for _ in insts]
    b, st = ctx.bound_batch_multi(nodes, [pid[i] for i in range(len(insts))], rank=0)
    for i, (n, e, w, SL) in enumerate(insts):
        oc = orc.Ctx(orc.shipped_params(**prm), SL, n, rng=orc.RNG_COUNTER, topk=orc.TOPK_CANONICAL, canon_sign=1)
        bo, so = oc.evaluate(orc.make_node(n - 1, {}), rank=0)
        assert abs(b[i] - bo) <= 1e-6 * abs(bo), (i, n, b[i], bo)
        got = (st[i].outer_iters, st[i].admm_iters, st[i].n_tri, st[i].n_pent, st[i].n_sub)
        assert got == (so.outer_iters, so.admm_iters, so.n_tri, so.n_pent, so.n_sub), (i, got)
        assert ctx.problem_lb(pid[i])[0] == oc.lb()[0]
        oc.close()
    ctx.close()


def test_multi_batch_rejects_unknown_problems(gpu_lib):
    M = gpu_lib
    n, e, w, SL = W.uneven_instance(_specs(1, 90)[0])
    ctx = M.Context(M.params(), SL, n, batch_max=2)
    with pytest.raises(M.MCBError):
        ctx.bound_batch_multi([M.node({})], [1])
    with pytest.raises(M.MCBError):
        ctx.add_problem(np.zeros((n + 1) * (n + 1)), n + 1)  # larger than the context's slots
    ctx.close()
