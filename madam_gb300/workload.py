"""Benchmark workloads: seeded synthetic stand-ins for the rudy-style instances.

The reference's published runs use rudy-generated Biq Mac families; rudy's own
random streams are not available, so each workload draws a seeded graph with the
same family semantics (size, density, weight law) and a seeded set of B&B nodes
(random fixings of a few variables), plus a fixed incumbent so that every timed
step does the same work.
"""
import numpy as np

from . import graphs as G

# configurations of the benchmark (graph, node sample, parameter overrides)
WORKLOADS = {
    # G(n=256, density 50%), weights uniform in {-1,+1}; 64 B&B nodes per batch;
    # FP64 projection; triangle + pentagonal cuts
    "gnp256_pm1_batch64": dict(n=256, p=0.5, weights="pm1", seed=1201, nodes=64, max_fixed=20,
                               params=dict(include_Hepta=0, use_diff=0)),
    # the reference's own CPU-runnable size: G(n=100, 50%), unit weights, triangles only
    "gnp100_one_tri": dict(n=100, p=0.5, weights="one", seed=1101, nodes=16, max_fixed=10,
                           params=dict(include_Pent=0, include_Hepta=0, use_diff=0)),
    # G(n=512, density 10%), integer weights in [-10,10]
    "gnp512_int10": dict(n=512, p=0.1, weights="int10", seed=1401, nodes=64, max_fixed=20,
                         params=dict(use_diff=0)),
    # 2D toroidal spin glass, 20 x 20 grid (n = 400, degree 4), weights in {-1,+1};
    # all three cut families
    "torus20x20_pm1": dict(kind="torus", rows=20, cols=20, seed=1301, nodes=64, max_fixed=20,
                           params=dict(use_diff=0)),
}


def one_opt_lb(n, edges, w, restarts=64, seed=0):
    """Best cut found by 1-flip local search from seeded random starts (a fixed,
    cheap incumbent for the benchmark; the bound path runs its own heuristic)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    A = np.zeros((n, n))
    e = np.asarray(edges, dtype=np.int64) - 1
    A[e[:, 0], e[:, 1]] = w
    A[e[:, 1], e[:, 0]] = w
    best, best_x = -np.inf, None
    for _ in range(restarts):
        x = rng.choice(np.array([-1.0, 1.0]), size=n)
        x[-1] = -1.0
        while True:
            # gain of flipping i: sum_j A_ij x_i x_j (cut changes by this)
            g = x * (A @ x)
            g[-1] = -np.inf
            i = int(np.argmax(g))
            if g[i] <= 1e-9:
                break
            x[i] = -x[i]
        val = 0.25 * float(np.sum(A * (1 - np.outer(x, x))))
        if val > best:
            best, best_x = val, x.copy()
    side = (best_x[: n - 1] != best_x[-1]).astype(np.int32)
    return G.cut_value(n, edges, w, side), side


def uneven_specs(count=2000, seed=1501):
    """Independent subproblems of uneven size, as (n, p, weights, seed) tuples:
    n uniform in [60, 400], density uniform in [0.1, 0.9], weights {-1,+1} or
    integers in [-10, 10] by a fair coin per instance.  The graphs themselves are
    drawn one at a time by uneven_instance (2000 of them hold ~0.4 GB as edge lists)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    n = rng.integers(60, 401, size=count)
    p = rng.uniform(0.1, 0.9, size=count)
    coin = rng.integers(0, 2, size=count)
    return [(int(n[i]), float(p[i]), "pm1" if coin[i] == 0 else "int10", seed * 10000 + i) for i in range(count)]


def uneven_instance(spec):
    """One subproblem of uneven_specs: (n, edges, weights, SL column-major)."""
    n, p, weights, s = spec
    n, e, w = G.gnp(n, p, weights, seed=s)
    return n, e, w, G.extended_laplacian(n, e, w).ravel(order="F")


def make(name):
    cfg = WORKLOADS[name]
    if cfg.get("kind") == "torus":
        n, e, w = G.torus2d(cfg["rows"], cfg["cols"], seed=cfg["seed"])
    else:
        n, e, w = G.gnp(cfg["n"], cfg["p"], cfg["weights"], seed=cfg["seed"])
    SL = G.extended_laplacian(n, e, w).ravel(order="F")
    fix = G.random_fixings(n, cfg["nodes"], cfg["max_fixed"], seed=cfg["seed"] + 7)
    lb, side = one_opt_lb(n, e, w, seed=cfg["seed"] + 3)
    return dict(name=name, n=n, edges=e, weights=w, SL=SL, fixings=fix, lb=lb, lb_sol=side,
                params=dict(cfg["params"]))
