"""CPU tests of the host side: graph construction, the C ABI surface of the
built library (symbols only, no device calls), parameter layout, the benchmark's
reference arm and the sharded multi-rank driver on gloo."""
import json
import os
import re
import subprocess
import sys

import numpy as np
import pytest

from madam_gb300 import graphs as G

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
from oracle.refdir import reference_dir

REF = reference_dir() or os.path.join(os.sep, "nonexistent-reference")


def test_extended_laplacian_matches_oracle(orc):
    for seed, wts in ((1, "one"), (2, "pm1"), (3, "int10")):
        n, e, w = G.gnp(30, 0.4, wts, seed=seed)
        assert np.array_equal(G.extended_laplacian(n, e, w).ravel(order="F"), orc.build_L(n, (e, w)))


def test_repeated_edges_and_self_loops_follow_the_reference(orc, tmp_path):
    """readData assigns weights edge by edge: a pair listed twice, in either
    orientation, keeps its last weight on both sides, and a self-loop cancels in
    the Laplacian.  A non-positive vertex count is an input error."""
    n = 5
    e = np.array([[1, 2], [2, 1], [3, 3], [4, 5], [4, 5], [1, 5]], dtype=np.int32)
    w = np.array([1.0, 7.0, 3.0, 2.0, -4.0, 1.0])
    L = G.extended_laplacian(n, e, w)
    assert np.array_equal(L.ravel(order="F"), orc.build_L(n, (e, w)))
    assert np.array_equal(L, L.T) and L[0, 1] == -7.0 and L[3, 3] == -4.0  # edge (4, 5): last weight -4
    rng = np.random.default_rng(3)
    for k in range(40):  # fractional weights and n > 64 too: every sum in the reference's order
        n = int(rng.integers(3, 30 if k < 20 else 140))
        m = int(rng.integers(1, 3 * n))
        e = rng.integers(1, n + 1, size=(m, 2)).astype(np.int32)
        w = rng.integers(-5, 6, size=m).astype(np.float64) if k % 2 else 3.7 * rng.standard_normal(m)
        assert np.array_equal(G.extended_laplacian(n, e, w).ravel(order="F"), orc.build_L(n, (e, w)))
    f = tmp_path / "bad.rudy"
    f.write_text("0 1\n1 1 1\n")
    with pytest.raises(ValueError):
        G.read_rudy(str(f))


@pytest.mark.skipif(not os.path.exists(os.path.join(ROOT, "oracle", "_ref", "libmadam_ref_strict.so")),
                    reason="reference build (oracle/_ref) not present")
def test_rudy_files_read_like_the_reference(tmp_path):
    """read_rudy + extended_laplacian against the reference's own readData (the
    strict build in oracle/_ref): seeded files with mixed white space, repeated
    and reversed edges, self-loops, fractional and exponent weights, and malformed
    or missing numbers (both sides reject the same files)."""
    import ctypes as C

    R = C.CDLL(os.path.join(ROOT, "oracle", "_ref", "libmadam_ref_strict.so"))
    libc = C.CDLL(None)
    libc.fopen.restype = C.c_void_p
    libc.fopen.argtypes = [C.c_char_p, C.c_char_p]
    C.c_void_p.in_dll(R, "output").value = libc.fopen(os.devnull.encode(), b"w")

    class Problem(C.Structure):  # admm.h:121-127
        _fields_ = [("L", C.POINTER(C.c_double)), ("n", C.c_int), ("NIneq", C.c_int), ("NPentIneq", C.c_int),
                    ("NHeptaIneq", C.c_int)]

    SP = C.POINTER(Problem).in_dll(R, "SP")
    rng = np.random.default_rng(29)
    weights = ["1", "-1", "7", "2.5", "-0.125", "1e1", "+3", ".5", "3.7", "x", "1.5e-2"]
    seps = [" ", "\t", "\n", "\r\n", "  "]
    for case in range(150):
        n = int(rng.integers(0, 9))
        m = int(rng.integers(-1, 8))
        toks = [str(n), str(m)]
        for _ in range(max(m, 0) + int(rng.integers(-1, 2))):
            i, j = (str(int(v)) for v in rng.integers(1, n + 2, size=2)) if n else ("1", "1")
            if rng.random() < 0.05:
                i = "1.5"
            toks += [i, j, weights[int(rng.integers(len(weights)))]]
        f = tmp_path / ("g%d.rudy" % case)
        f.write_text("".join(t + seps[int(rng.integers(len(seps)))] for t in toks))
        rc = R.readData(str(f).encode())
        try:
            nn, e, w = G.read_rudy(str(f))
            ours = G.extended_laplacian(nn, e, w).ravel(order="F")
        except ValueError:
            ours = None
        if rc != 0:
            assert ours is None, toks
        else:
            k = SP.contents.n
            ref = np.ctypeslib.as_array(SP.contents.L, shape=(k * k,)).copy()
            assert ours is not None and np.array_equal(ours, ref), toks
    libc.fflush(None)  # readData's printf output, inside the test's capture


@pytest.mark.skipif(not (os.path.isdir(os.path.join(REF, "Instances")) and
                         os.path.exists(os.path.join(ROOT, "oracle", "_ref", "libmadam_ref_strict.so"))),
                    reason="reference instances or build not present")
def test_published_instances_read_like_the_reference():
    """All 220 instance files shipped with the reference (130 rudy graphs of 60, 80
    and 100 vertices and the 90 of the rudy_150 families) give the same SP->L
    through read_rudy + extended_laplacian as through readData, bit for bit."""
    import ctypes as C
    import glob

    R = C.CDLL(os.path.join(ROOT, "oracle", "_ref", "libmadam_ref_strict.so"))
    libc = C.CDLL(None)
    libc.fopen.restype = C.c_void_p
    libc.fopen.argtypes = [C.c_char_p, C.c_char_p]
    C.c_void_p.in_dll(R, "output").value = libc.fopen(os.devnull.encode(), b"w")

    class Problem(C.Structure):  # admm.h:121-127
        _fields_ = [("L", C.POINTER(C.c_double)), ("n", C.c_int), ("NIneq", C.c_int), ("NPentIneq", C.c_int),
                    ("NHeptaIneq", C.c_int)]

    SP = C.POINTER(Problem).in_dll(R, "SP")
    files = sorted(f for f in glob.glob(os.path.join(REF, "Instances", "**", "*"), recursive=True)
                   if os.path.isfile(f) and ".output" not in f and not f.endswith((".md", ".txt", ".py")))
    assert len(files) >= 220
    for f in files:
        assert R.readData(f.encode()) == 0, f
        k = SP.contents.n
        ref = np.ctypeslib.as_array(SP.contents.L, shape=(k * k,)).copy()
        n, e, w = G.read_rudy(f)
        assert np.array_equal(G.extended_laplacian(n, e, w).ravel(order="F"), ref), f
    libc.fflush(None)


def test_rudy_roundtrip(tmp_path):
    n, e, w = G.gnp(20, 0.5, "int10", seed=4)
    f = tmp_path / "g.rudy"
    G.write_rudy(str(f), n, e, w)
    n2, e2, w2 = G.read_rudy(str(f))
    assert n2 == n and np.array_equal(e2, e) and np.array_equal(w2, w)


def test_torus_is_4_regular():
    n, e, w = G.torus2d(5, 6, seed=1)
    deg = np.bincount(np.asarray(e).ravel() - 1, minlength=n)
    assert n == 30 and np.all(deg == 4) and set(np.unique(w)) <= {-1.0, 1.0}


def test_c_abi_library_exports_every_declared_symbol():
    from madam_gb300 import build as B

    lib = B.build()
    hdr = open(os.path.join(ROOT, "include", "mcbound.h")).read()
    declared = set(re.findall(r"\b(mcb_[a-z_0-9]+)\s*\(", hdr))
    out = subprocess.run(["nm", "-D", "--defined-only", lib], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (mcb_[a-z_0-9]+)$", out, re.M))
    assert declared, "no declarations parsed"
    assert declared <= exported, declared - exported


def test_library_loads_without_a_device():
    import ctypes

    from madam_gb300 import build as B

    L = ctypes.CDLL(B.build())
    L.mcb_strerror.restype = ctypes.c_char_p
    assert L.mcb_version() >= 10000
    assert L.mcb_strerror(-5) == b"capacity exceeded"


def test_context_entry_points_accept_a_null_context():
    """Status codes, never a crash: every entry point that takes a context treats
    NULL as an argument error (setters do nothing, getters return 0)."""
    import ctypes as C

    from madam_gb300 import build as B

    L = C.CDLL(B.build())
    L.mcb_get_lb.restype = C.c_double
    L.mcb_get_diff.restype = C.c_double
    L.mcb_launch_count.restype = C.c_longlong
    L.mcb_library_launch_count.restype = C.c_longlong
    L.mcb_last_error.restype = C.c_char_p
    L.mcb_set_lb.argtypes = [C.c_void_p, C.c_double, C.c_void_p]
    L.mcb_set_diff.argtypes = [C.c_void_p, C.c_double]
    ERR_ARG = -1
    L.mcb_set_lb(None, 3.0, None)
    L.mcb_set_diff(None, 1.0)
    L.mcb_set_trials(None, 1, 2)
    L.mcb_reset_kernel_stats(None)
    L.mcb_destroy(None)
    assert L.mcb_get_lb(None, None) == 0.0 and L.mcb_get_diff(None) == 0.0
    p, h = C.c_int(7), C.c_int(7)
    L.mcb_get_trials(None, C.byref(p), C.byref(h))
    L.mcb_get_trials(None, None, None)
    assert p.value == 0 and h.value == 0
    a, b = C.c_longlong(5), C.c_longlong(5)
    L.mcb_transfer_stats(None, C.byref(a), C.byref(b))
    assert a.value == 0 and b.value == 0
    assert L.mcb_launch_count(None) == 0 and L.mcb_library_launch_count(None) == 0
    launches, ms = (C.c_longlong * 64)(), (C.c_double * 64)()
    k = L.mcb_kernel_stats(None, 64, None, launches, ms)
    assert k > 0 and all(launches[i] == 0 and ms[i] == 0.0 for i in range(k))
    work, unit = (C.c_double * 64)(), (C.c_int * 64)()
    assert L.mcb_kernel_work(None, 64, work, unit) == k
    assert L.mcb_last_error(None) == b""
    node = C.create_string_buffer(4 * 1024 * 2 + 8 * 1024 + 16)
    bound = C.c_double()
    assert L.mcb_evaluate(None, node, 1, C.byref(bound), None) == ERR_ARG
    assert L.mcb_bound_batch(None, None, 1, 1, None, None) == ERR_ARG
    assert L.mcb_bab(None, 1, 0, None, None, None, None, None, 0, None) == ERR_ARG
    assert L.mcb_set_models(None, None, None) == ERR_ARG
    assert L.mcb_log_count(None, 0) == 0 and L.mcb_log_fetch(None, 0, 0, None, None) == ERR_ARG
    assert L.mcb_autotune_table(None, 0, None, None, None, None, None) == 0
    # operator entry points check their arrays before they look for a device
    X, y = (C.c_double * 16)(), (C.c_double * 4)()
    tri = (C.c_int * 4)(2, 1, 0, 1)  # (i, j, k, type), i > j > k
    assert L.mcb_op_B(4, X, 1, None, 0, None, 0, None, y) == ERR_ARG
    assert L.mcb_op_Bt(4, X, 0, None, 1, None, 0, None, y) == ERR_ARG
    assert L.mcb_op_B(4, X, 1, tri, 0, None, 0, None, y) in (-7, 0)  # arguments fine: MCB_ERR_NODEV, or runs


def test_params_and_node_layout_match_the_reference():
    from madam_gb300 import lib as M

    names = [f[0] for f in M.PARAM_FIELDS]
    if os.path.isdir(REF):
        txt = open(os.path.join(REF, "admm.h")).read()
        ref = re.findall(r"P\((?:double|int),\s*(\w+),", txt)
        assert names == ref
    import ctypes

    assert ctypes.sizeof(M.BabNode) == 4 * 1024 * 2 + 8 * 1024 + 8 + 8
    assert M.BabNode.upper_bound.offset == 4 * 1024 * 2 + 8 * 1024 + 8


def test_workload_is_deterministic():
    from madam_gb300 import workload as W

    for name in ("gnp100_one_tri", "torus20x20_pm1"):
        a, b = W.make(name), W.make(name)
        assert np.array_equal(a["SL"], b["SL"]) and a["fixings"] == b["fixings"] and a["lb"] == b["lb"]
        assert G.cut_value(a["n"], a["edges"], a["weights"], a["lb_sol"]) == a["lb"]
    t = W.make("torus20x20_pm1")
    assert t["n"] == 400 and len(t["weights"]) == 800 and set(np.unique(t["weights"])) == {-1.0, 1.0}


def test_uneven_batch_generator():
    from madam_gb300 import workload as W

    s = W.uneven_specs()
    assert s == W.uneven_specs() and len(s) == 2000 and len({x[3] for x in s}) == 2000
    ns = np.array([x[0] for x in s])
    ps = np.array([x[1] for x in s])
    assert ns.min() >= 60 and ns.max() <= 400 and ps.min() >= 0.1 and ps.max() <= 0.9
    assert {x[2] for x in s} == {"pm1", "int10"}
    for spec in s[:3]:
        n, e, w, SL = W.uneven_instance(spec)
        n2, e2, w2, SL2 = W.uneven_instance(spec)
        assert n == spec[0] and np.array_equal(SL, SL2) and SL.size == n * n
        assert set(np.unique(w)) <= ({-1.0, 1.0} if spec[2] == "pm1" else set(range(-10, 11)))


def test_bench_reference_arm_prints_one_json_line():
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--workload",
                        "gnp100_one_tri", "--steps", "1", "--warmup", "0", "--cpu-sample", "2", "--no-compare"],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["value"] > 0 and line["unit"] == "nodes/s"
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["cpu_baseline"]["kind"] == "port"


class _BatchedOracle:
    """The oracle context with the GPU library's bound_batch entry point (one
    evaluate per node), recording the batch sizes the driver asks for."""

    def __init__(self, c):
        self.c, self.N, self.sizes = c, c.N, []

    def evaluate(self, nd, rank=1):
        return self.c.evaluate(nd, rank)

    def bound_batch(self, nodes, rank=1):
        self.sizes.append(len(nodes))
        out = [self.c.evaluate(nd, rank) for nd in nodes]
        return [b for b, _ in out], [st for _, st in out]

    def set_lb(self, lb, sol=None):
        self.c.set_lb(lb, sol)

    def lb(self):
        return self.c.lb()


def _sharded_worker(rank, world, port, q, depth=2, batch=1, max_nodes=100000):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    sys.path.insert(0, ROOT)
    from madam_gb300 import graphs as G2
    from madam_gb300.sharded import sharded_bab
    from oracle import oracle as O

    n, e, w = G2.gnp(64, 0.5, "pm1", seed=13)
    SL = O.build_L(n, (e, w))
    ctx = O.Ctx(O.shipped_params(), SL, n)
    if batch > 1:
        ctx = _BatchedOracle(ctx)
    info = {}
    best, sol, mine, total = sharded_bab(ctx, lambda fx: O.make_node(n - 1, fx), dist=dist, depth=depth, info=info,
                                         batch=batch, max_nodes=max_nodes)
    if batch > 1:
        info["batch_sizes"] = ctx.sizes
    q.put((rank, best, mine, total, None if sol is None else G2.cut_value(n, e, w, sol), info))
    dist.destroy_process_group()


@pytest.mark.parametrize("world,depth,batch", [(2, 2, 1), (3, 1, 1), (2, 2, 4)])
def test_sharded_branch_and_bound_on_gloo_ranks(orc, world, depth, batch):
    """Ranks expand the top of the tree, deal the frontier, rebalance when a queue
    runs dry, and agree on the serial optimum; with batch > 1 each rank bounds
    several open nodes per round through bound_batch."""
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + (os.getpid() + 7 * world + 13 * batch) % 1000
    ps = [ctx.Process(target=_sharded_worker, args=(r, world, port, q, depth, batch)) for r in range(world)]
    for p in ps:
        p.start()
    res = [q.get(timeout=600) for _ in ps]
    for p in ps:
        p.join(timeout=60)
    # single-process reference answer (oracle, same counter streams)
    n, e, w = G.gnp(64, 0.5, "pm1", seed=13)
    SL = orc.build_L(n, (e, w))
    c = orc.Ctx(orc.shipped_params(), SL, n)
    serial = c.bab(max_nodes=5000)
    bests = {r[1] for r in res}
    assert bests == {serial["opt"]}
    # every rank returns a solution of the optimum's value (the winner's vector)
    assert all(r[4] == serial["opt"] for r in res)
    assert len({r[3] for r in res}) == 1
    # the top of the tree, bounded identically on every rank, is counted once
    assert len({r[5]["top"] for r in res}) == 1
    assert res[0][3] == sum(r[5]["local"] for r in res) + res[0][5]["top"]
    if world == 3:  # one of three ranks starts with an empty queue (a frontier of two nodes)
        assert res[0][5]["transfers"] >= 1 and res[0][5]["moved"] >= 1
    if batch > 1:
        sizes = [k for r in res for k in r[5]["batch_sizes"]]
        assert sizes and max(sizes) <= batch and max(sizes) > 1


def test_sharded_node_cap_stops_every_rank_in_the_same_round(orc):
    """A node cap that one rank reaches before the others: all ranks leave the
    loop together (no unmatched collective), agree on the incumbent, and each
    returns a solution that attains it."""
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + (os.getpid() + 911) % 1000
    ps = [ctx.Process(target=_sharded_worker, args=(r, 2, port, q, 2, 1, 3)) for r in range(2)]
    for p in ps:
        p.start()
    res = [q.get(timeout=600) for _ in ps]
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert len({r[1] for r in res}) == 1
    assert all(r[4] == r[1] for r in res)
    assert max(r[5]["local"] for r in res) <= 3 + 1
    assert min(r[5]["local"] for r in res) < 5


def test_sharded_root_only(orc):
    """root_only bounds the root and stops, as the reference's `root` parameter."""
    from madam_gb300.sharded import sharded_bab

    n, e, w = G.gnp(40, 0.5, "pm1", seed=5)
    c = orc.Ctx(orc.shipped_params(root=1), orc.build_L(n, (e, w)), n)
    best, sol, mine, total = sharded_bab(c, lambda fx: orc.make_node(n - 1, fx), root_only=True)
    ref = orc.Ctx(orc.shipped_params(root=1), orc.build_L(n, (e, w)), n).bab()
    assert mine == total == 1 and best == ref["opt"] and ref["nodes"] == 1


def test_sharded_least_fractional_branching(orc):
    """branchingStrategy 0 through the sharded driver reaches the reference's
    optimum on the least-fractional fixture tree."""
    import json

    from madam_gb300.sharded import sharded_bab

    fx = [f for f in json.load(open(os.path.join(ROOT, "tests", "golden", "reference_bab_params.json")))["instances"]
          if f["params"].get("branchingStrategy") == 0][0]
    n, e, w = G.gnp(*fx["args"][:3], seed=fx["args"][3])
    c = orc.Ctx(orc.shipped_params(**fx["params"]), orc.build_L(n, (e, w)), n)
    best, sol, mine, total = sharded_bab(c, lambda f: orc.make_node(n - 1, f), strategy=0)
    assert best == fx["opt"] and G.cut_value(n, e, w, sol) == fx["opt"]


def test_balance_plan_properties():
    """On random queue sizes: receivers were empty, donors held nodes and keep at
    least one, nobody receives twice, nodes are conserved, and an empty rank is
    left out only when no queue could give (every remaining donor holds < 2)."""
    from madam_gb300.sharded import balance_plan

    rng = np.random.default_rng(11)
    for _ in range(2000):
        world = int(rng.integers(1, 9))
        sizes = [int(v) for v in rng.integers(0, 6, size=world) * (rng.random(world) < 0.6)]
        plan = balance_plan(sizes)
        assert plan == balance_plan(list(sizes))  # a function of the sizes only
        after = list(sizes)
        receivers = [r for _, r, _ in plan]
        assert len(receivers) == len(set(receivers))
        for d, r, k in plan:
            assert sizes[r] == 0 and sizes[d] > 0 and k >= 1
            after[d] -= k
            after[r] += k
        assert sum(after) == sum(sizes) and all(after[d] >= 1 for d, _, _ in plan)
        empty_left = [r for r in range(world) if after[r] == 0]
        if empty_left:
            assert all(after[d] < 2 for d in range(world) if sizes[d] > 0)


def test_balance_plan():
    from madam_gb300.sharded import balance_plan

    assert balance_plan([5, 0, 3]) == [(0, 1, 2)]
    assert balance_plan([0, 0, 6]) == [(2, 0, 3), (2, 1, 1)]
    assert balance_plan([0, 8, 0, 2]) == [(1, 0, 4), (1, 2, 2)]
    assert balance_plan([1, 0, 1]) == []
    assert balance_plan([4, 4]) == []


# ---- reference-format command line (madam_gb300/solve.py) ----------------------
REF_SO = os.path.join(ROOT, "oracle", "_ref", "libmadam_ref_strict.so")


@pytest.mark.skipif(not os.path.exists(REF_SO), reason="reference build (oracle/_ref) not present")
def test_parameter_files_read_like_the_reference(tmp_path):
    """read_params against the reference's own readParameters (the strict build in
    oracle/_ref) on seeded files made of well-formed, indented, tabbed, blank,
    over-long and malformed lines."""
    import ctypes as C

    from madam_gb300 import lib as M
    from madam_gb300 import solve as S

    R = C.CDLL(REF_SO)
    P = M.Params.in_dll(R, "params")
    names = [k for k, _ in M.PARAM_FIELDS]
    values = ["1.6", "7", "-2", "1e-4", "2.5e1x", ".5", "12.7", "abc", "", "0x10", "inf", " 3 ", "+4"]
    rng = np.random.default_rng(17)
    for case in range(300):
        lines = []
        for _ in range(int(rng.integers(0, 12))):
            nm = names[int(rng.integers(len(names)))] if rng.random() < 0.8 else "unknown"
            val = values[int(rng.integers(len(values)))]
            shape = int(rng.integers(0, 9))
            lines.append([nm + " = " + val, nm + "=" + val, "  " + nm + " = " + val, nm + "\t= " + val, "",
                          nm + " " + val, "= " + val, nm + " = " + val + " " * 130, nm + "^x = " + val][shape])
        f = tmp_path / ("p%d" % case)
        f.write_text("\n".join(lines) + ("\n" if rng.random() < 0.7 else ""))
        assert R.readParameters(str(f).encode(), 0) == 0
        ref = {k: getattr(P, k) for k in names}
        assert S.read_params(str(f)) == ref, (lines, S.read_params(str(f)), ref)


@pytest.mark.skipif(not os.path.exists(REF_SO), reason="reference build (oracle/_ref) not present")
def test_report_header_and_file_name_match_the_reference(tmp_path):
    """The reference's processCommandLineArguments writes the .output header
    (input file, graph size, the parameters after adjust_TriIneq) into
    INSTANCE.output, or INSTANCE.output_1, ... when taken; solve.report and
    solve.output_path give the same text and names."""
    import ctypes as C

    from madam_gb300 import lib as M
    from madam_gb300 import solve as S

    R = C.CDLL(REF_SO)
    libc = C.CDLL(None)
    libc.fclose.argtypes = [C.c_void_p]
    out = C.c_void_p.in_dll(R, "output")
    rng = np.random.default_rng(41)
    names = [k for k, _ in M.PARAM_FIELDS]
    for case in range(12):
        n, e, w = G.gnp(int(rng.integers(3, 40)), 0.4, "int10", seed=case)
        inst = str(tmp_path / ("g%d.rudy" % case))
        G.write_rudy(inst, n, e, w)
        prm = tmp_path / ("p%d" % case)
        keep = [k for k in names if rng.random() < 0.6]
        prm.write_text("".join("%s = %s\n" % (k, M.SHIPPED[k] if rng.random() < 0.7 else M.COMPILED_DEFAULTS[k])
                               for k in keep) + ("adjust_TriIneq = 0\n" if case % 3 == 0 else ""))
        for run in range(2 if case == 0 else 1):
            expect = S.output_path(inst)
            argv = (C.c_char_p * 3)(b"biqbin", inst.encode(), str(prm).encode())
            assert R.processCommandLineArguments(3, argv, 0) == 0
            libc.fclose(out.value)
            out.value = None
            assert os.path.exists(expect) and expect.endswith(".output" if run == 0 else ".output_1")
            ref = open(expect).read()
            res = dict(nodes=1, root_bound=0.0, opt=0.0, sol=[])
            ours = S.report(inst, n, len(w), S.read_params(str(prm)), res, 0.0)
            assert ours[: ours.index("\nNodes = ")] == ref, (ours, ref)
    libc.fflush(None)  # readData's printf output, inside the test's capture


def test_solve_reads_parameter_files(tmp_path):
    import re

    from madam_gb300 import lib as M
    from madam_gb300 import solve as S

    p = tmp_path / "params"
    p.write_text("sigma0 = 1.6\nscaleSigma=1.002\nTriIneq = 1500   \nminTol = 1e-3\nbogus = 4\n")
    v = S.read_params(str(p))
    assert v["sigma0"] == 1.6 and v["scaleSigma"] == 1.002 and v["TriIneq"] == 1500 and v["minTol"] == 1e-3
    # names the file leaves out keep the compiled-in defaults, not the shipped file's values
    assert all(v[k] == M.COMPILED_DEFAULTS[k] for k in M.COMPILED_DEFAULTS
               if k not in ("sigma0", "scaleSigma", "TriIneq", "minTol"))
    # an indented line keeps the previous line's name (readParameters' sscanf); numbers are C prefixes
    p.write_text("scaleSigma=1.002\n  unknown_name = 7\nTriIneq = 1e-4\nsigma0 = 1.6abc\nminTol\t= 9\n")
    v2 = S.read_params(str(p))
    assert v2["scaleSigma"] == 7.0 and v2["TriIneq"] == 1 and v2["sigma0"] == 1.6 and v2["minTol"] == 1e-4
    ref = os.path.join(REF, "params")
    if os.path.exists(ref):
        assert S.read_params(ref) == {k: type(M.SHIPPED[k])(v) for k, v in M.SHIPPED.items()}
    # the report parses like the reference's .output files
    res = dict(nodes=41, root_bound=1447.82190427, opt=1435.0, sol=[1, 0, 0, 1, 1])
    txt = S.report("g.rudy", 6, 9, v, res, 12.345)
    assert re.search(r"^Maximum value = (\S+)", txt, re.M).group(1) == "1435"
    assert re.search(r"^Root node bound = (\S+)", txt, re.M).group(1) == "1447.82"
    assert re.search(r"^Nodes = (\d+)", txt, re.M).group(1) == "41"
    assert re.search(r"^Solution = \( (.*)\)", txt, re.M).group(1).split() == ["1", "4", "5"]
    assert re.search(r"sigma0 = (\S+)", txt).group(1) == "1.600000"
    assert re.search(r"^Time = (\S+) s", txt, re.M).group(1) == "12.35"
    assert "Graph has 6 vertices and 9 edges." in txt
    assert "TIME LIMIT REACHED." not in txt and "Best value" not in txt
    # a run stopped by its node limit reads like the reference's early stop
    stop = S.report("g.rudy", 6, 9, v, dict(res, stopped=True), 1.0)
    tail = stop[stop.index("\nNodes = "):].splitlines()
    assert tail[1:5] == ["Nodes = 41", "TIME LIMIT REACHED.", "Root node bound = 1447.82", "Best value = 1435"]
    assert "Maximum value" not in stop


@pytest.mark.skipif(not os.path.isdir(REF), reason="reference headers not present")
def test_reference_shim_compiles_against_the_reference_headers():
    """The C binding a maintainer adds to MADAM (madam_gb300/shim) compiles against
    the reference's admm.h (with the oracle's single-rank mpi.h) and mcbound.h."""
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    r = subprocess.run(["gcc", "-std=gnu11", "-Wall", "-Werror", "-fsyntax-only", "-I" + REF,
                        "-I" + os.path.join(root, "oracle", "ref"), "-I" + os.path.join(root, "include"),
                        os.path.join(root, "madam_gb300", "shim", "mcb_madam_shim.c")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


@pytest.mark.skipif(not os.path.isdir(REF), reason="reference sources not present")
def test_reference_driver_links_against_the_library(tmp_path):
    """The reference's own driver, heap, input and heuristic files, linked with the
    shim in place of the bound files and with libmcbound, resolve every symbol.
    Without a device the first Evaluate ends with the shim's message and exit 1;
    with one, the run reaches the reference's optimum."""
    from madam_gb300 import build as B
    from madam_gb300 import lib as M
    from oracle import build as OB

    B.build()
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    mk = subprocess.run(["make", "-s", "-C", os.path.join(root, "oracle", "ref"), "REFDIR=" + REF,
                         "LAPACK=" + OB.find_lapack(), "../_ref/madam_drop_in"], capture_output=True, text=True)
    assert mk.returncode == 0, mk.stderr[-2000:]
    n, e, w = G.gnp(40, 0.5, "one", seed=1)  # the reference fixture gnp40_one_s1 (optimum 246)
    G.write_rudy(str(tmp_path / "g.rudy"), n, e, w)
    (tmp_path / "params").write_text("".join("%s = %s\n" % kv for kv in M.SHIPPED.items()))
    r = subprocess.run([os.path.join(root, "oracle", "_ref", "madam_drop_in"), str(tmp_path / "g.rudy"),
                        str(tmp_path / "params")], capture_output=True, text=True, timeout=300)
    assert "Graph has 40 vertices and 397 edges." in r.stdout
    if r.returncode == 0:
        assert float(re.search(r"^Maximum value = (\S+)", r.stdout, re.M).group(1)) == 246.0
    else:
        assert r.returncode == 1 and "mcb_create: no CUDA device" in r.stderr, (r.returncode, r.stderr)


def test_newton_schulz_schedule_against_a_restatement():
    """The library's step schedule (host arithmetic, no device) is the scaled
    Newton-Schulz iteration of Chen & Chow: k^2 = 3 (1 - 0.02) / (1 + l + l^2),
    p(x) = 1.5 k x - 0.5 (k x)^3, until 1 - l < 1e-7, FP32-accurate from l > 0.9,
    and at least two accurate closing steps.  Every step keeps [0, 1] inside [0, 1]."""
    from madam_gb300 import build as B
    from madam_gb300 import lib as M

    if not os.path.exists(M.LIB_PATH):
        B.build()
    for l0 in (1e-3, 1e-6, 1e-9):
        st = M.ns_schedule_for(l0)
        l, ref = l0, []
        while 1 - l > 1e-7 and len(ref) < 64:
            k2 = 3 * 0.98 / (1 + l + l * l)
            k = np.sqrt(k2) if k2 > 1 else 1.0
            ref.append((1.5 * k, -0.5 * k ** 3, int(l > 0.9)))
            p = lambda y: 1.5 * y - 0.5 * y ** 3
            l = min(p(k * l), p(k))
        while sum(r[2] for r in ref) < 2:
            ref.append((1.5, -0.5, 1))
        assert len(st) == len(ref)
        assert np.allclose([s[0] for s in st], [r[0] for r in ref], rtol=1e-6)
        assert np.allclose([s[1] for s in st], [r[1] for r in ref], rtol=1e-6)
        assert [s[2] for s in st] == [r[2] for r in ref]
        xs = np.linspace(0, 1, 4001)
        for a, b, _ in st:
            y = a * xs + b * xs ** 3
            assert y.min() >= -1e-7 and y.max() <= 1 + 1e-6
    with pytest.raises(M.MCBError):
        M.ns_schedule_for(0.6)
