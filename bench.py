#!/usr/bin/env python
"""Benchmark of the GPU node bound (MADAM's Evaluate/SDPbound) on GB300.

One step = one batched call that bounds a whole batch of branch-and-bound
nodes (IPM + cutting-plane ADMM rounds + separations + safe bound per node) of
the configured workload; the problem matrix is resident on the device.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--workload NAME] [--form F]
  python bench.py --impl reference ...   # the reference's CPU method on the host cores

Forms: "learned" (default: Newton-Schulz projection on the tensor cores plus the
shipped learned cut ranking / warm start), "mixed" (Newton-Schulz only), "fp64"
(the plain method).  Prints one JSON line (rank 0).  `value` is node bounds per
second of the chosen form over the device-timed region (CUDA events on the
library's stream); `e2e` is the same through the C ABI call with host buffers,
timed on the host; `plain_fp64` is the plain form on the same workload in the
same run, and `time_to_optimum` a full branch-and-bound of a seeded G(100, 0.5)
unit-weight instance (triangle cuts) in both forms.  `n512` compares the forms on
G(512, 0.1) with integer weights in [-10, 10] (node throughput and bound
agreement).  With --extended: `n512` adds a time-capped branch-and-bound of the
whole graph in both forms, `torus` bounds nodes of the 20 x 20 toroidal spin
glass (n = 400, all three families) against the oracle's stored answers, and
`uneven_batch` bounds the roots of 2000 seeded independent subproblems of uneven
order in one call.  Both
arms print the same `config` (the workload); the reference arm (`--impl
reference`) runs the reference's method on the host cores, one process per core
started before the timed steps.
"""
import argparse
import json
import multiprocessing as mp
import os
import statistics
import subprocess
import sys
import tempfile
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

METRIC = "node bounds/sec"
UNIT = "nodes/s"


def _args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="gnp256_pm1_batch64")
    ap.add_argument("--form", default="learned", choices=["learned", "mixed", "fp64"])
    ap.add_argument("--no-compare", action="store_true",
                    help="skip the plain-form and time-to-optimum legs (reference arm: the CPU time-to-optimum)")
    ap.add_argument("--cpu-sample", type=int, default=0, help="nodes in the CPU sample (0: one per core)")
    ap.add_argument("--cpu-only", action="store_true", help=argparse.SUPPRESS)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--extended", action="store_true",
                    help="also the time-capped n = 512 trees, the torus block and the 2000-subproblem uneven batch "
                         "(about ten more minutes)")
    return ap.parse_args()


# ---------------------------------------------------------------------------
# CPU side: the oracle (the reference's method restated in C) on host cores.
# A pool of spawned processes, one per core, is created once: every worker
# imports the oracle and builds the workload in its initializer, so process
# start-up stays outside every timed region.  Each task bounds one node of the
# workload's node list with a fresh oracle context in the reference's own mode
# (its rand() streams, top-K order and eigenvector signs) and single-threaded
# BLAS, as the reference runs one node per MPI process (setupenv.sh:6-8).
_POOL_STATE = {}


def _pool_init(wl_name):
    for v in ("OPENBLAS_NUM_THREADS", "GOTO_NUM_THREADS", "OMP_NUM_THREADS"):
        os.environ[v] = "1"
    from madam_gb300 import workload as W
    from oracle import oracle as O

    wl = W.make(wl_name)
    _POOL_STATE.update(wl=wl, O=O, prm=O.shipped_params(**wl["params"]))
    O.lib()


def _pool_bound(i):
    wl, O = _POOL_STATE["wl"], _POOL_STATE["O"]
    oc = O.Ctx(_POOL_STATE["prm"], wl["SL"], wl["n"], rng=O.RNG_GLIBC, topk=O.TOPK_REFERENCE, canon_sign=0)
    oc.set_lb(wl["lb"], wl["lb_sol"])
    nd = O.make_node(wl["n"] - 1, wl["fixings"][i])
    t0 = time.perf_counter()
    b, _ = oc.evaluate(nd, rank=1)
    dt = time.perf_counter() - t0
    oc.close()
    return i, b, dt


class CpuPool:
    """One oracle process per host core, started once, bounding nodes of one workload."""

    def __init__(self, wl_name, cores):
        self.cores = cores
        self.pool = mp.get_context("spawn").Pool(cores, initializer=_pool_init, initargs=(wl_name,))

    def run(self, idx):
        t0 = time.perf_counter()
        res = self.pool.map(_pool_bound, list(idx), chunksize=1)
        wall = time.perf_counter() - t0
        return dict(nodes=len(res), wall=wall, node_seconds=[r[2] for r in res], bounds=[r[1] for r in res])

    def close(self):
        self.pool.close()
        self.pool.join()


def cpu_sample(wl_name, nodes, cores):
    """A bounded sample on all host cores: `nodes` nodes of the workload (after one
    untimed round of one node per core that starts the workers)."""
    from madam_gb300 import workload as W

    nodes = min(nodes, W.WORKLOADS[wl_name]["nodes"])
    pool = CpuPool(wl_name, cores)
    try:
        pool.run(range(min(cores, nodes)))
        r = pool.run(range(nodes))
    finally:
        pool.close()
    return dict(nodes=r["nodes"], wall=r["wall"], cores=cores, value=r["nodes"] / r["wall"],
                node_seconds=statistics.mean(r["node_seconds"]))


def host_cores():
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


# ---------------------------------------------------------------------------
class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, index=0):
        self.f = tempfile.NamedTemporaryFile(prefix="clocks", suffix=".csv", delete=False)
        self.p = None
        self.index = index

    def start(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + q,
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None

    def stop(self):
        if self.p:
            self.p.terminate()
            try:
                self.p.wait(timeout=5)
            except Exception:
                self.p.kill()
        self.f.close()
        sm, smax, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        try:
            for line in open(self.f.name):
                parts = [x.strip() for x in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    sm.append(float(parts[1]))
                    smax = max(smax, float(parts[2]))
                except ValueError:
                    continue
                for nm, v in zip(names, parts[5:9]):
                    if v.lower() == "active":
                        reasons.add(nm)
            os.unlink(self.f.name)
        except Exception:
            pass
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax or None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    try:
        return json.load(open(os.path.join(HERE, "MEASURED_PEAKS.json")))
    except Exception:
        return {}


# ---------------------------------------------------------------------------
FORMS = {"learned": "Newton-Schulz projection (BF16 split operands, FP64 product) + learned cut ranking and warm start",
         "mixed": "Newton-Schulz projection (BF16 split operands, FP64 product)",
         "fp64": "plain FP64 tridiagonal eigensolver"}
TTO = dict(n=100, p=0.5, weights="one", seed=1101, params=dict(include_Pent=0, include_Hepta=0))


DTYPES = {"learned": "bf16 digit planes (5 x 7-bit digits, products to ~5e-10) + f64",
          "mixed": "bf16 digit planes (5 x 7-bit digits, products to ~5e-10) + f64", "fp64": "f64"}
N512 = "gnp512_int10"


def n512_block(torch, M, stream, form, nodes=16, cap_s=60.0, capped=True):
    """The n = 512 configuration (G(512, 0.1), integer weights in [-10, 10], all
    three cut families): node throughput of the chosen form and of the plain FP64
    form on the same nodes, the largest relative difference between their bounds,
    and a time-capped branch-and-bound of the whole graph in both forms.  The tree
    does not close within minutes (the root bound lies ~20% above the best cut), so
    a capped run reports the gap it closed: (root bound - largest open bound) /
    (root bound - incumbent)."""
    from madam_gb300 import workload as W

    wl = W.make(N512)
    prm = M.params(**wl["params"])
    base_trials = (prm.Pent_Trials, prm.Hepta_Trials)
    fixes = wl["fixings"][:nodes]
    out = {"workload": N512, "n": wl["n"], "nodes_per_step": len(fixes)}
    bounds = {}
    for f in (form, "fp64"):
        ctx = _context(M, prm, wl["SL"], wl["n"], len(fixes), f, stream.cuda_stream, profile=False)

        def step(ctx=ctx):
            ctx.set_trials(*base_trials)
            ctx.set_lb(wl["lb"], wl["lb_sol"])
            b, st = ctx.bound_batch([M.node(x) for x in fixes], rank=1)
            bounds[f] = b
            return st
        warm = 1 if f != "fp64" else 0
        d, w, st, _ = _time_steps(torch, ctx, step, stream, 1, warm)
        ctx.close()
        out[f] = {"value": len(fixes) / d, "unit": UNIT, "steps": 1, "warmup": warm,
                  "admm_iters": sum(s.admm_iters for s in st[0])}
    rel = [abs(x - y) / abs(y) for x, y in zip(bounds[form], bounds["fp64"])]
    out["speedup_vs_plain_fp64"] = out[form]["value"] / out["fp64"]["value"]
    out["bound_rel_diff_vs_fp64"] = {"max": max(rel), "mean": statistics.mean(rel)}
    if not capped:
        return out
    tto = {"cap_seconds": cap_s, "batch": 64}
    for f in (form, "fp64"):
        tc = _context(M, prm, wl["SL"], wl["n"], 64, f, profile=False)
        tc.set_time_limit(cap_s)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r = tc.bab(batch=64, max_nodes=0)
        sec = time.perf_counter() - t0
        tc.close()
        rec = {"seconds": sec, "nodes": r["nodes"], "incumbent": r["opt"], "root_bound": r["root_bound"],
               "closed": not r["stopped"]}
        if r["stopped"]:
            ob = r["open_bound"] if r["open_bound"] is not None else r["opt"]
            rec.update(time_to_optimum="> %.0f s" % cap_s, open_bound=ob, open_nodes=r["open_nodes"],
                       gap_closed=(r["root_bound"] - ob) / max(1e-9, r["root_bound"] - r["opt"]))
        tto[f] = rec
    out["time_capped_bab"] = tto
    return out


TORUS = "torus20x20_pm1"


def torus_block(torch, M, stream, form):
    """The 2D toroidal spin glass (20 x 20, n = 400, +-1 weights, all three cut
    families): the chosen form on the nodes whose oracle answers are stored with
    the tests (tests/golden/oracle_fullsize.json, the oracle in the mode the GPU
    reproduces), bounded together in one call with the stored incumbent; node
    throughput and each node's relative difference from the oracle's bound.  The
    plain FP64 form is left out here: one of these nodes takes minutes in it."""
    from madam_gb300 import workload as W

    fx = json.load(open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "tests", "golden",
                                     "oracle_fullsize.json")))
    recs = fx["workloads"][TORUS]
    wl = W.make(TORUS)
    prm = M.params(**wl["params"])
    ctx = _context(M, prm, wl["SL"], wl["n"], len(recs), form, stream.cuda_stream, profile=False)
    got = {}

    def step():
        ctx.set_trials(prm.Pent_Trials, prm.Hepta_Trials)
        ctx.set_lb(fx["incumbent"][TORUS])
        b, st = ctx.bound_batch([M.node(wl["fixings"][r["node"]]) for r in recs], rank=1)
        got["b"], got["st"] = b, st
        return st
    d, w, st, _ = _time_steps(torch, ctx, step, stream, 1, 0)
    ctx.close()
    rel = [abs(b - r["bound"]) / abs(r["bound"]) for b, r in zip(got["b"], recs)]
    return {"workload": TORUS, "n": wl["n"], "nodes": len(recs), "value": len(recs) / d, "unit": UNIT,
            "steps": 1, "warmup": 0, "admm_iters": [s.admm_iters for s in got["st"]],
            "oracle_admm_iters": [r["admm_iters"] for r in recs],
            "bound_rel_diff_vs_oracle": rel}


def uneven_block(torch, M, stream, form, count=2000, plain_count=128, batch=128):
    """The uneven batch: `count` seeded independent subproblems (n uniform in
    [60, 400], density in [0.1, 0.9], weights +-1 or integers in [-10, 10]), their
    root bounds in one call (mcb_bound_batch_multi; chunks of `batch` slots of
    similar order) in the chosen form, the plain FP64 form on the first
    `plain_count` of them, and the largest relative difference between the two
    forms' bounds there."""
    from madam_gb300 import workload as W

    prm = M.params()
    insts = [W.uneven_instance(sp) for sp in W.uneven_specs(count)]
    out = {"subproblems": count, "n_range": [min(x[0] for x in insts), max(x[0] for x in insts)],
           "slots": batch, "rank": 0, "params": "reference shipped params file (all three cut families)"}
    res = {}
    for f, k in ((form, count), ("fp64", plain_count)):
        idx = list(range(k))
        big = max(idx, key=lambda i: insts[i][0])  # problem 0 sizes the slots
        ctx = _context(M, prm, insts[big][3], insts[big][0], batch, f, stream.cuda_stream, profile=False)
        pid = {big: 0}
        for i in idx:
            if i != big:
                pid[i] = ctx.add_problem(insts[i][3], insts[i][0])
        nodes = [M.node({}) for _ in idx]
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        b, st = ctx.bound_batch_multi(nodes, [pid[i] for i in idx], rank=0)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        ctx.close()
        res[f] = b
        out[f] = {"value": k / dt, "unit": UNIT, "seconds": dt, "subproblems": k,
                  "admm_iters": int(sum(x.admm_iters for x in st))}
    rel = [abs(res[form][i] - res["fp64"][i]) / abs(res["fp64"][i]) for i in range(plain_count)]
    out["bound_rel_diff_vs_fp64"] = {"max": max(rel), "mean": statistics.mean(rel), "over": plain_count}
    out["speedup_vs_plain_fp64"] = out[form]["value"] / out["fp64"]["value"]
    return out


def _context(M, prm, SL, n, batch, form, stream=None, profile=True):
    flags = M.PROJ_FP64 if form == "fp64" else M.PROJ_NS_BF16
    if form == "learned":
        flags |= M.FLAG_LEARNED
    if profile:
        flags |= M.FLAG_PROFILE
    ctx = M.Context(prm, SL, n, batch_max=batch, flags=flags, stream=stream)
    if form == "learned":
        from madam_gb300 import learn as L
        from madam_gb300 import train_models as T

        ctx.set_models(*L.load(T.OUT))
    return ctx


def _time_steps(torch, ctx, step, stream, steps, warmup, dist=None, clocks=None):
    for _ in range(warmup):
        step()
    torch.cuda.synchronize()
    ctx.reset_kernel_stats()
    if dist:
        dist.barrier()
    if clocks:
        clocks.start()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    ev0.record(stream)
    stats = []
    for _ in range(steps):
        stats.append(step())
    ev1.record(stream)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    if dist:
        dist.barrier()
    clk = clocks.stop() if clocks else None
    return ev0.elapsed_time(ev1) / 1e3, wall, stats, clk


def traffic_from_profiles(workload, cls):
    """DRAM bytes (read + write) per launch of a kernel class on a workload, from the
    ncu summaries under profiles/ (a line `roofline-traffic: class=C workload=W
    bytes=B` beside the capture it was read from); (bytes, file) or None."""
    import glob
    import re

    for f in sorted(glob.glob(os.path.join(HERE, "profiles", "*.md"))):
        for m in re.finditer(r"^roofline-traffic: class=(\S+) workload=(\S+) bytes=(\S+)", open(f).read(), re.M):
            if m.group(1) == cls and m.group(2) == workload:
                return float(m.group(3)), os.path.relpath(f, HERE)
    return None


def _roofline(M, ks, kw, workload=None, tune=None):
    """Achieved rate of the dominant kernel class with counted work, against the measured peak."""
    peaks = measured_peaks()
    counted = {k: v for k, v in ks.items() if kw.get(k, (0, 0))[1] and v[1] > 0}
    if not counted:
        return None
    name, (nl, ms) = max(counted.items(), key=lambda kv: kv[1][1])
    work, unit = kw[name]
    tr = traffic_from_profiles(workload, name)
    base = {"kernel": name, "launches": nl, "ms_total": ms, "traffic": tr[0] if tr else None,
            "traffic_unit": "bytes per launch" if tr else None,
            "traffic_source": ("ncu capture summarised in " + tr[1]) if tr else None}
    if unit == 1:
        peak = M.fp64_peak_gflops() / 1e3
        ach = work / (ms / 1e3) / 1e12
        base.update(bound="fp64", achieved=ach, peak=peak, unit="TFLOP/s", frac=ach / peak,
                    peak_source="measured FP64 FMA microbenchmark (no FP64 entry in the measured peaks file)")
    elif unit == 2:
        hbm = peaks.get("hbm_gbs", 6800.0)
        ach = work / (ms / 1e3) / 1e9
        base.update(bound="hbm", achieved=ach, peak=hbm, unit="GB/s", frac=ach / hbm,
                    peak_source="measured" if "hbm_gbs" in peaks else "fallback")
    else:
        bf = peaks.get("bf16_tflops", 1900.0)
        ach = work / (ms / 1e3) / 1e12
        base.update(bound="tensor", achieved=ach, peak=bf, unit="TFLOP/s", frac=ach / bf,
                    peak_source=("measured" if "bf16_tflops" in peaks else "fallback") + " dense BF16 burst; "
                    "the work counts each digit-plane GEMM once (2 n^3), not its 19 BF16 plane products")
        if tune:
            # the autotuner's timing of the full batch: launches queued back to back
            # between two events on the library's stream (no host gaps)
            full = max(tune, key=lambda t: t["bucket"])
            us = min(full["us"])
            flops = 2.0 * full["npad"] ** 3 * full["bucket"]
            base["back_to_back"] = {"npad": full["npad"], "slots": full["bucket"], "us_per_launch": us,
                                    "achieved": flops / (us * 1e-6) / 1e12, "frac": flops / (us * 1e-6) / 1e12 / bf}
    return base


def run_ours(a):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    import torch

    from madam_gb300 import graphs as G
    from madam_gb300 import lib as M
    from madam_gb300 import workload as W

    torch.cuda.set_device(local)
    wl = W.make(a.workload)
    stream = torch.cuda.Stream()
    nodes_fix = wl["fixings"]
    batch = len(nodes_fix)
    prm = M.params(**wl["params"])
    base_trials = (prm.Pent_Trials, prm.Hepta_Trials)

    def make_step(ctx):
        def step():
            # every step starts from the same state: incumbent and the Pent/Hepta_Trials
            # that give-ups grow (bounding.c:184-187) reset
            ctx.set_trials(*base_trials)
            ctx.set_lb(wl["lb"], wl["lb_sol"])
            nodes = [M.node(f) for f in nodes_fix]
            return ctx.bound_batch(nodes, rank=1)[1]
        return step

    # timed steps run without per-class events, so the ADMM chunks replay as CUDA graphs
    ctx = _context(M, prm, wl["SL"], wl["n"], batch, a.form, stream.cuda_stream, profile=False)
    dev_s, wall, stats, clk = _time_steps(torch, ctx, make_step(ctx), stream, a.steps, a.warmup, dist, Clocks(local))
    launches = ctx.launch_count()
    lib_launches = ctx.library_launch_count()
    graphs = ctx.graph_stats()
    host = {k: round(v / a.steps, 4) for k, v in ctx.host_stats().items()}
    h2d, d2h = ctx.transfer_stats()
    tune = ctx.autotune_table() if a.form != "fp64" else []
    # one more step with per-class CUDA events: kernel shares and the roofline's kernel time
    ctx.set_profile(True)
    ctx.reset_kernel_stats()
    make_step(ctx)()
    ks = ctx.kernel_stats()
    kw = ctx.kernel_work()
    ctx.close()
    if dist:
        t = torch.tensor([dev_s, wall], device="cuda", dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        dev_s, wall = float(t[0]), float(t[1])
    total_nodes = batch * a.steps * world
    if rank != 0:
        dist.destroy_process_group()
        return
    roof = _roofline(M, ks, kw, a.workload, tune)
    tot_ms = sum(x[1] for x in ks.values())
    share = {k: round(v[1] / max(1e-9, tot_ms), 4) for k, v in ks.items() if v[1] > 0}
    plain = tto = n512 = uneven = torus = None
    if not a.no_compare and a.form != "fp64":
        # the plain FP64 form on the same workload (one warm-up, one timed step)
        pc = _context(M, prm, wl["SL"], wl["n"], batch, "fp64", stream.cuda_stream, profile=False)
        pd, pw, pst, _ = _time_steps(torch, pc, make_step(pc), stream, 1, 1)
        pc.close()
        plain = {"value": batch / pd, "unit": UNIT, "ms_per_step": pd * 1e3, "steps": 1, "warmup": 1,
                 "admm_iters_per_step": sum(s.admm_iters for s in pst[0])}
        # time to proven optimum, both forms
        n, e, w = G.gnp(TTO["n"], TTO["p"], TTO["weights"], seed=TTO["seed"])
        SLt = G.extended_laplacian(n, e, w).ravel(order="F")
        tto = {"instance": "G(%d, %.1f) %s weights seed %d, triangle cuts, batch 64" % (
            TTO["n"], TTO["p"], TTO["weights"], TTO["seed"])}
        for form in ((a.form, "mixed", "fp64") if a.form == "learned" else (a.form, "fp64")):
            tc = _context(M, M.params(**TTO["params"]), SLt, n, 64, form, profile=False)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            r = tc.bab(batch=64, max_nodes=20000)
            tto[form] = {"seconds": time.perf_counter() - t0, "optimum": r["opt"], "nodes": r["nodes"],
                         "root_bound": r["root_bound"]}
            tc.close()
        tto["speedup"] = tto["fp64"]["seconds"] / tto[a.form]["seconds"]
        tto["same_optimum"] = tto["fp64"]["optimum"] == tto[a.form]["optimum"]
        if a.workload != N512:
            n512 = n512_block(torch, M, stream, a.form, capped=a.extended)
        if a.extended:
            torus = torus_block(torch, M, stream, a.form)
            uneven = uneven_block(torch, M, stream, a.form)
    cpu = None
    if not a.no_cpu_baseline:
        cores = host_cores()
        c = cpu_sample(a.workload, a.cpu_sample or cores, cores)
        cpu = {"value": c["value"], "unit": UNIT, "cores": c["cores"], "kind": "port",
               "sample": "%d of the workload's nodes, one process per core (started before timing), the oracle "
                         "(C restatement of the reference) in the reference's mode (its rand() streams) with "
                         "single-threaded OpenBLAS; %.1f s wall, %.2f s per node" % (c["nodes"], c["wall"],
                                                                                  c["node_seconds"])}
    admm = sum(s.admm_iters for st in stats for s in st)
    out = {
        "metric": METRIC, "value": total_nodes / dev_s, "unit": UNIT, "n_gpus": world, "steps": a.steps,
        "warmup": a.warmup, "ms_per_step": dev_s * 1e3 / a.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": DTYPES[a.form],
        "data": "synthetic (seeded rudy-style G(n,p) graph and node fixings)",
        "config": workload_config(wl, world),
        "form": a.form, "projection": FORMS[a.form],
        "e2e": {"value": total_nodes / wall, "unit": UNIT, "h2d_bytes_per_step": h2d // a.steps,
                "d2h_bytes_per_step": d2h // a.steps},
        "gpu_launches": launches,
        "library_launches": lib_launches,
        "graphs": {"captured": graphs[0], "replayed": graphs[1]},
        "host_phase_seconds_per_step": host,
        "autotune": tune,
        "roofline_step": "kernel shares and roofline from one extra step with per-class CUDA events (kernels "
                         "launched one by one, not from graphs: a short kernel's time includes the host's "
                         "submission gap; roofline.back_to_back times the GEMM alone)",
        "roofline": roof,
        "kernel_time_share": share,
        "admm_iters_per_step": admm // a.steps,
        "plain_fp64": plain,
        "speedup_vs_plain_fp64": (plain["ms_per_step"] / (dev_s * 1e3 / a.steps)) if plain else None,
        "time_to_optimum": tto,
        "n512": n512,
        "torus": torus,
        "uneven_batch": uneven,
        "cpu_baseline": cpu,
        "clocks": clk,
    }
    print(json.dumps(out))
    if dist:
        dist.destroy_process_group()


def _tto_worker(rank, world, port, q):
    """One CPU rank of the reference method's branch-and-bound on the time-to-optimum
    instance (the oracle; ranks share only the incumbent and rebalance queues)."""
    for v in ("OPENBLAS_NUM_THREADS", "GOTO_NUM_THREADS", "OMP_NUM_THREADS"):
        os.environ[v] = "1"
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    # a launcher's agent store would make every rank of this private group a store client
    os.environ.pop("TORCHELASTIC_USE_AGENT_STORE", None)
    import torch.distributed as dist

    dist.init_process_group("gloo", rank=rank, world_size=world)
    from madam_gb300 import graphs as G
    from madam_gb300.sharded import sharded_bab
    from oracle import oracle as O

    n, e, w = G.gnp(TTO["n"], TTO["p"], TTO["weights"], seed=TTO["seed"])
    ctx = O.Ctx(O.shipped_params(**TTO["params"]), O.build_L(n, (e, w)), n, rng=O.RNG_GLIBC,
                topk=O.TOPK_REFERENCE, canon_sign=0)
    t0 = time.perf_counter()
    best, _, mine, total = sharded_bab(ctx, lambda fx: O.make_node(n - 1, fx), dist=dist, depth=3)
    q.put((rank, best, mine, total, time.perf_counter() - t0))
    dist.destroy_process_group()


def cpu_time_to_optimum(cores):
    """The reference method (oracle port) to proven optimum on `cores` processes."""
    import socket

    import torch.multiprocessing as tmp

    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        port = sk.getsockname()[1]
    ctx = tmp.get_context("spawn")
    q = ctx.Queue()
    t0 = time.perf_counter()
    ps = [ctx.Process(target=_tto_worker, args=(r, cores, port, q)) for r in range(cores)]
    for p in ps:
        p.start()
    res = [q.get(timeout=1800) for _ in ps]
    for p in ps:
        p.join(timeout=60)
    wall = time.perf_counter() - t0
    best = res[0][1]
    return {"instance": "G(%d, %.1f) %s weights seed %d, triangle cuts" % (TTO["n"], TTO["p"], TTO["weights"],
                                                                        TTO["seed"]),
            "seconds": max(r[4] for r in res), "wall_with_process_start": wall, "optimum": best,
            "nodes": int(res[0][3]), "cores": cores,
            "method": "oracle port of the reference in its reference mode on one process per core (gloo), "
                      "best-first per rank, shared incumbent, queue rebalancing"}


def workload_config(wl, world):
    """The `config` of both arms: the workload only (what is bounded), so that the
    two lines of one run carry the same config."""
    return {"workload": wl["name"], "n": wl["n"], "nodes_per_step": len(wl["fixings"]),
            "cuts": "tri+pent" if not wl["params"].get("include_Hepta", 1) else "tri+pent+hept",
            "params": "reference shipped params file, " + ", ".join("%s=%s" % kv for kv in wl["params"].items()),
            "incumbent": wl["lb"], "l2": "working set per step > L2 (64 nodes x 8 n^2 FP64 buffers)",
            "parallelism": "replicas" if world > 1 else "single"}


def run_reference(a):
    """The reference's method on the host cores: the oracle port in its reference
    mode, one process per core (created before the timed steps), bounding the
    workload's nodes.  A timed step bounds `--cpu-sample` nodes (default: all of the
    step's nodes when that is at most four per core, else one per core), taken in
    turn from the workload's node list so that successive steps cover all of it;
    warm-up steps bound one node per core."""
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if rank != 0:
        return
    from madam_gb300 import workload as W

    wl = W.make(a.workload)
    total = len(wl["fixings"])
    cores = host_cores()
    ns = a.cpu_sample or (total if total <= 4 * cores else cores)
    pool = CpuPool(a.workload, cores)
    per_node, walls, done = [], [], 0
    try:
        for i in range(a.warmup + a.steps):
            k = min(cores, total) if i < a.warmup else ns
            idx = [(done + j) % total for j in range(k)]
            r = pool.run(idx)
            if i >= a.warmup:
                done += k
                walls.append(r["wall"])
                per_node += r["node_seconds"]
    finally:
        pool.close()
    tot_wall = sum(walls)
    v = len(per_node) / tot_wall
    sample = ("%d of the workload's %d nodes per step (in turn through the node list), one process per core on %d "
              "cores, each node alone: the oracle (C restatement of the reference, checked bit-for-bit against it) "
              "in the reference's mode (its rand() streams) with single-threaded OpenBLAS; mean %.2f s per node"
              % (ns, total, cores, statistics.mean(per_node)))
    out = {
        "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world, "steps": a.steps, "warmup": a.warmup,
        "ms_per_step": tot_wall * 1e3 / a.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic (seeded rudy-style graph and node fixings)", "impl": "reference",
        "config": workload_config(wl, world),
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample,
                         "node_seconds_mean": statistics.mean(per_node)},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    if not a.no_compare:
        try:
            out["time_to_optimum"] = cpu_time_to_optimum(cores)
        except Exception as ex:  # a reported extra, not the arm's metric
            out["time_to_optimum"] = {"failed": str(ex)[-300:]}
    print(json.dumps(out))


def main():
    a = _args()
    if a.cpu_only:
        r = cpu_sample(a.workload, a.cpu_sample or host_cores(), host_cores())
        print(json.dumps(r))
        return
    if a.impl == "reference":
        run_reference(a)
    else:
        run_ours(a)


if __name__ == "__main__":
    main()
