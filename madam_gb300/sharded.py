"""Branch-and-bound across ranks: one process per GPU, each with its own node queue.

B&B nodes are independent bound problems, so the tree shards without moving
matrices: every rank expands the top of the tree identically (the root with
rank 0 of MADAM's Init_PQ semantics, then `depth` levels by the reference's
most-fractional rule), deals the frontier round-robin, and runs its own
best-first search.  The only exchange is the incumbent: a max-allreduce of the
lower bound after every batch (MADAM pushes NEW_VALUE to its master,
bab_functions.c:242-256), plus a sum-allreduce of queue sizes to detect global
termination.  No matrix data crosses ranks, so there is no device collective.

When a rank's queue runs dry while another holds two or more open nodes, the
ranks rebalance: every rank learns all queue sizes (an all-gather of one integer),
computes the same transfer plan from them (each empty rank takes half of the
currently largest queue), and the donors ship the fixings and bounds of their best
open nodes (an all-gather of small lists).  This plays the role of the
reference's master handing idle workers new subproblems (bab_functions.c:297-325).

`ctx` is any object with evaluate(node, rank) -> (bound, stats), set_lb(lb, sol),
lb() -> (lb, sol) and an `N` attribute; `new_node(fixed)` builds a node with
xfixed / sol / fracsol arrays (the BabNode layout).  With batch > 1 and a context
that has bound_batch(nodes, rank) -> (bounds, stats) (the GPU library's), each rank
pops up to `batch` open nodes per round and bounds them in one call, as the
library's own driver does (pop-k / push-2k around mcb_bound_batch).  The exchange
runs on whatever process group `dist` holds: gloo with host tensors, or NCCL with
tensors on the rank's current GPU (call torch.cuda.set_device first).
"""
import heapq
import itertools

import numpy as np


def _branch_var(nd, pb, strategy=1):
    best, ic = (1e9 if strategy == 1 else -1e9), -1
    for i in range(pb):
        if nd.xfixed[i]:
            continue
        v = abs(0.5 - nd.fracsol[i])
        if (strategy == 1 and v < best) or (strategy == 0 and v > best):
            best, ic = v, i
    return ic


def balance_plan(sizes):
    """Transfers [(donor, receiver, count)] that give every empty queue half of the
    currently largest non-empty one (donors are ranks that held nodes before the
    round, so every transfer comes out of a queue that exists); the same on every
    rank (a function of the sizes only)."""
    left = {d: c for d, c in enumerate(sizes) if c > 0}
    plan = []
    for r, c in enumerate(sizes):
        if c != 0:
            continue
        if not left:
            break
        d = max(left, key=lambda k: (left[k], -k))
        if left[d] < 2:
            break
        k = left[d] // 2
        plan.append((d, r, k))
        left[d] -= k
    return plan


def sharded_bab(ctx, new_node, dist=None, depth=2, max_nodes=100000, balance=True, info=None, batch=1,
                root_only=False, strategy=1):
    """Returns (optimum, solution vector, nodes evaluated on this rank, evaluated on all ranks).
    Every rank returns the same solution: the vector of the lowest rank whose own
    search found a cut of the optimum's value.  The node total counts the top of the
    tree, which every rank bounds, once.  max_nodes caps the nodes a rank bounds
    after the top of the tree; once any rank reaches it, all ranks stop in the same
    round (the decision is itself a reduction, so the collectives stay matched).
    info (a dict, optional) receives the number of rebalancing transfers and nodes moved,
    the nodes this rank bounded after the top of the tree, and the top's node count.
    root_only: bound the root and stop (the reference's `root` parameter, main.c:106,195).
    strategy: the reference's branchingStrategy (1 most fractional, 0 least fractional;
    getBranchingVariable, bab_functions.c:389-423)."""
    rank = dist.get_rank() if dist else 0
    world = dist.get_world_size() if dist else 1
    pb = ctx.N - 1

    # NCCL groups reduce device tensors (the rank's current GPU); gloo host tensors
    dev = None
    if dist and dist.get_backend() == "nccl":
        import torch

        dev = torch.device("cuda", torch.cuda.current_device())

    def allreduce(v, op):
        if not dist:
            return v
        import torch

        t = torch.tensor([v], dtype=torch.float64, device=dev)
        dist.all_reduce(t, op=op)
        return float(t[0])

    MAX = dist.ReduceOp.MAX if dist else None
    SUM = dist.ReduceOp.SUM if dist else None
    # every rank expands the top of the tree identically: the root with rank 0
    # semantics (Init_PQ), branched at once as MADAM's master does (main.c:126-158);
    # `depth` - 1 further levels are bounded redundantly on every rank
    root = new_node({})
    rb, _ = ctx.evaluate(root, 0)
    evaluated = 1
    frontier = []  # unevaluated nodes: (parent bound, fixings)

    def children(b, fx, nd):
        ic = _branch_var(nd, pb, strategy)
        out = []
        if ic >= 0 and ctx.lb()[0] + 1.0 < b:
            for v in (0, 1):
                f2 = dict(fx)
                f2[ic] = v
                out.append((b, f2))
        return out

    frontier = [] if root_only else children(rb, {}, root)
    for _ in range(depth - 1):
        nxt = []
        for b, fx in frontier:
            nd = new_node(fx)
            cb, _ = ctx.evaluate(nd, 1)
            evaluated += 1
            nxt += children(cb, fx, nd)
        frontier = nxt
    lb, sol = ctx.lb()
    sol_val = lb  # the value of this rank's own best solution `sol`
    # deal the frontier; each rank keeps a best-first heap keyed on the bound
    mine = [f for k, f in enumerate(sorted(frontier, key=lambda t: sorted(t[1].items()))) if k % world == rank]
    tie = itertools.count()
    heap = [(-b, next(tie), fx, new_node(fx)) for b, fx in mine]
    heapq.heapify(heap)
    local = 0
    transfers = moved = 0
    while True:
        g = allreduce(lb, MAX)
        if g > lb:
            lb = g
            ctx.set_lb(lb, None)
        active = allreduce(float(len(heap)), SUM)
        # every rank leaves in the same round: the cap is tested collectively
        capped = allreduce(float(local >= max_nodes), MAX)
        if active == 0 or capped > 0:
            break
        if dist and balance and world > 1:
            sizes = [None] * world
            dist.all_gather_object(sizes, len(heap))
            plan = balance_plan(sizes)
            if plan:
                out = []
                for d, r, k in plan:
                    if d == rank:
                        for _ in range(k):
                            negb, _, fx, _ = heapq.heappop(heap)
                            out.append((r, -negb, fx))
                got = [None] * world
                dist.all_gather_object(got, out)
                for lst in got:
                    for r, b, fx in lst:
                        if r == rank:
                            heapq.heappush(heap, (-b, next(tie), fx, new_node(fx)))
                transfers += len(plan)
                moved += sum(k for _, _, k in plan)
        # pop up to `batch` nodes that the incumbent does not prune (heap.c:104-168)
        take = []
        while heap and len(take) < batch:
            negb, _, fx, nd = heapq.heappop(heap)
            if lb + 1.0 < -negb:
                take.append((fx, nd))
        if take:
            if len(take) > 1 and hasattr(ctx, "bound_batch"):
                bounds, _ = ctx.bound_batch([nd for _, nd in take], 1)
            else:
                bounds = [ctx.evaluate(nd, 1)[0] for _, nd in take]
            local += len(take)
            lb2, sol2 = ctx.lb()
            if lb2 > lb:
                lb, sol, sol_val = lb2, sol2, lb2
            for (fx, nd), b in zip(take, bounds):
                if lb + 1.0 < b:
                    ic = _branch_var(nd, pb, strategy)
                    if ic < 0:  # every variable fixed: the node is a single cut, nothing to branch
                        continue
                    for v in (0, 1):
                        f2 = dict(fx)
                        f2[ic] = v
                        heapq.heappush(heap, (-b, next(tie), f2, new_node(f2)))
    best = allreduce(lb, MAX)
    # the top of the tree was bounded identically on every rank: count it once
    total = allreduce(float(local), SUM) + evaluated
    if info is not None:
        info.update(transfers=transfers, moved=moved, local=local, top=evaluated)
    own = np.asarray(sol, dtype=np.int32)[:pb] if sol is not None else None
    if dist and world > 1:
        # the lowest rank whose own solution attains the optimum hands it to all
        winner = int(allreduce(float(rank if (own is not None and sol_val == best) else world), dist.ReduceOp.MIN))
        got = [own if rank == winner else None]
        dist.broadcast_object_list(got, src=min(winner, world - 1))
        own = got[0]
    return best, own, local + evaluated, int(total)
