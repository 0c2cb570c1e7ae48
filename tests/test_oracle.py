"""CPU checks of the oracle itself: against glibc, against fixtures produced by
the reference (compiled from its own sources), against the reference's
published outputs, and against independent numpy restatements."""
import ctypes
import glob
import json
import os
import re

import numpy as np
import pytest

from madam_gb300 import graphs as G

HERE = os.path.dirname(os.path.abspath(__file__))
from oracle.refdir import reference_dir

REF = reference_dir() or os.path.join(os.sep, "nonexistent-reference")


def test_glibc_rand_restatement_matches_libc(orc):
    libc = ctypes.CDLL("libc.so.6")
    for seed in (2020, 1, 12345):
        libc.srand(seed)
        ref = [libc.rand() for _ in range(3000)]
        assert orc.glibc_stream(seed, 3000) == ref


def _fixture_instance(f):
    if f["kind"] == "gnp":
        n, p, w, seed = f["args"]
        return G.gnp(n, p, w, seed=seed)
    return G.torus2d(f["args"][0], f["args"][1], seed=f["args"][2])


FIXTURES = json.load(open(os.path.join(HERE, "golden", "reference_bab.json")))["instances"]


@pytest.mark.parametrize("fx", FIXTURES, ids=[f["name"] for f in FIXTURES])
def test_oracle_reproduces_reference_branch_and_bound(orc, fx):
    """Whole B&B trees of the reference (strict-IEEE build), node by node."""
    n, e, w = _fixture_instance(fx)
    SL = orc.build_L(n, (e, w))
    c = orc.Ctx(orc.shipped_params(), SL, n, rng=orc.RNG_GLIBC, topk=orc.TOPK_REFERENCE, canon_sign=0)
    r = c.bab(max_nodes=2000)
    bounds = [s.bound for s in r["log"]]
    assert r["nodes"] == fx["nodes"]
    assert r["opt"] == fx["opt"]
    assert sorted(np.nonzero(r["sol"])[0].tolist()) == sorted(fx["sol"])
    assert len(bounds) == len(fx["bounds"])
    # the reference prints 12 decimals
    assert max(abs(a - b) for a, b in zip(bounds, fx["bounds"])) <= 1e-9


VARIANTS = json.load(open(os.path.join(HERE, "golden", "reference_bab_params.json")))["instances"]


@pytest.mark.parametrize("fx", VARIANTS, ids=[f["name"] for f in VARIANTS])
def test_oracle_reproduces_reference_trees_under_other_parameters(orc, fx):
    """Reference trees under non-shipped settings (triangles only, no heptagons,
    least-fractional branching, no diff give-up with sigma0 1.6, a fixed
    triangle budget), node by node."""
    n, e, w = _fixture_instance(fx)
    SL = orc.build_L(n, (e, w))
    c = orc.Ctx(orc.shipped_params(**fx["params"]), SL, n, rng=orc.RNG_GLIBC, topk=orc.TOPK_REFERENCE, canon_sign=0)
    r = c.bab(max_nodes=2000)
    bounds = [s.bound for s in r["log"]]
    assert r["nodes"] == fx["nodes"] and r["opt"] == fx["opt"]
    assert sorted(np.nonzero(r["sol"])[0].tolist()) == sorted(fx["sol"])
    assert len(bounds) == len(fx["bounds"])
    assert max(abs(a - b) for a, b in zip(bounds, fx["bounds"])) <= 1e-9


def test_oracle_stream_modes_agree_where_no_stream_is_drawn(orc):
    """The GPU form reproduces the oracle's counter-stream mode; the oracle's glibc
    mode (the reference's rand() streams, top-K order and eigenvector signs) is
    pinned bit-exact to the reference.  Where no random draw can matter -- triangle
    cuts only (no simulated annealing) and the incumbent fixed at the optimum (the
    rounding heuristic cannot change it, so pruning and give-ups see the same value)
    -- the two modes must give the same counts, and bounds equal up to rounding
    (the modes store the same cut set in different orders -- scan order against the
    reference's replacement order -- so their sums round differently; ~1e-9 here),
    which closes the chain GPU = oracle(counter) = oracle(glibc) = reference on that
    path."""
    fx = [f for f in VARIANTS if f["name"] == "gnp56_pm1_s31_tri"][0]
    n, e, w = _fixture_instance(fx)
    SL = orc.build_L(n, (e, w))
    prm = orc.shipped_params(**dict(fx["params"], use_diff=0))
    rng = np.random.default_rng(3)
    fixings = [{}] + [{int(v): int(rng.integers(0, 2)) for v in rng.choice(n - 1, size=k, replace=False)}
                      for k in (2, 5, 9)]
    ran = 0
    for fixed in fixings:
        out = []
        for mode in ((orc.RNG_COUNTER, orc.TOPK_CANONICAL, 1), (orc.RNG_GLIBC, orc.TOPK_REFERENCE, 0)):
            c = orc.Ctx(prm, SL, n, rng=mode[0], topk=mode[1], canon_sign=mode[2])
            c.set_lb(fx["opt"])
            b, st = c.evaluate(orc.make_node(n - 1, fixed), rank=1)
            out.append((b, st.admm_iters, st.outer_iters, st.n_tri))
            c.close()
        (b0, *k0), (b1, *k1) = out
        assert k0 == k1 and abs(b0 - b1) <= 1e-7 * abs(b1), (fixed, out)
        ran += k0[0] > 0
    assert ran >= 3  # the cutting-plane rounds ran on most of the nodes


def test_oracle_counter_mode_is_order_free(orc):
    """Counter streams: a node's bound does not depend on what was bounded before."""
    n, e, w = G.gnp(36, 0.5, "pm1", seed=21)
    SL = orc.build_L(n, (e, w))
    prm = orc.shipped_params(use_diff=0)
    a = orc.Ctx(prm, SL, n)
    b = orc.Ctx(prm, SL, n)
    a.set_lb(0)
    b.set_lb(0)
    a.evaluate(orc.make_node(n - 1, {4: 1}), rank=1)
    a.set_lb(0)
    ba, _ = a.evaluate(orc.make_node(n - 1, {2: 0}), rank=1)
    bb, _ = b.evaluate(orc.make_node(n - 1, {2: 0}), rank=1)
    assert ba == bb


def _published():
    out = []
    for f in sorted(glob.glob(os.path.join(REF, "Instances/rudy/rudy_150/*/*.output"))):
        txt = open(f).read()
        opt = float(re.search(r"^Maximum value = (\S+)", txt, re.M).group(1))
        root = float(re.search(r"^Root node bound = (\S+)", txt, re.M).group(1))
        sol = [int(v) for v in re.search(r"^Solution = \( (.*)\)", txt, re.M).group(1).split()]
        sigma0 = float(re.search(r"sigma0 = (\S+)", txt).group(1))
        out.append((f[: -len(".output")], opt, root, sol, sigma0))
    return out


@pytest.mark.skipif(not os.path.isdir(REF), reason="reference instances not present")
def test_published_optima_are_cut_values_of_published_solutions():
    pubs = _published()
    assert len(pubs) == 90
    for inst, opt, _, sol, _ in pubs:
        n, e, w = G.read_rudy(inst)
        side = np.zeros(n, dtype=np.int32)
        side[np.array(sol) - 1] = 1
        assert G.cut_value(n, e, w, side) == opt
        # the published optimum is also what the extended Laplacian evaluates to
        L = G.extended_laplacian(n, e, w)
        x = side[: n - 1].astype(float)
        assert abs(x @ L[: n - 1, : n - 1] @ x - opt) < 1e-6


@pytest.mark.slow
@pytest.mark.skipif(not os.path.isdir(REF), reason="reference instances not present")
def test_oracle_root_bounds_near_published(orc):
    """The published root bounds came from a -ffast-math build whose k-gonal SA
    path depends on rounding noise; the oracle lands within 0.1%."""
    for inst, opt, root, _, sigma0 in _published()[:2]:
        n, e, w = G.read_rudy(inst)
        SL = orc.build_L(n, (e, w))
        c = orc.Ctx(orc.shipped_params(sigma0=sigma0, root=1), SL, n, rng=orc.RNG_GLIBC, topk=orc.TOPK_REFERENCE,
                    canon_sign=0)
        b, _ = c.evaluate(orc.make_node(n - 1), rank=0)
        assert b >= opt
        assert abs(b - root) <= 1e-3 * root


REF_BIN = os.path.join(os.path.dirname(HERE), "oracle", "_ref", "madam_ref_strict")


@pytest.mark.skipif(not (os.path.isdir(os.path.join(REF, "Instances")) and os.path.exists(REF_BIN)),
                    reason="reference instances or build not present")
def test_oracle_root_bounds_match_the_reference_on_shipped_instances(orc, tmp_path):
    """One shipped instance of each family (g05, pm1d, pm1s, pw01, pw05, pw09, w01,
    w05, w09 at n = 60..100): the root bound of the reference's strict build and of
    the oracle in reference mode agree to 1e-12 relative.  The instance is copied
    first, since the reference writes its .output report beside its input."""
    import shutil
    import subprocess

    from madam_gb300 import lib as M

    prm = tmp_path / "params"
    prm.write_text("".join("%s = %s\n" % kv for kv in M.SHIPPED.items()))
    picks = ["g05_60.3", "pm1d_100.9", "pm1s_80.5", "pw01_100.8", "pw05_100.2", "pw09_100.1", "w01_100.4",
             "w05_100.7", "w09_100.0"]
    for name in picks:
        src = os.path.join(REF, "Instances", "rudy", name)
        inst = str(tmp_path / name)
        shutil.copyfile(src, inst)
        out = subprocess.run([REF_BIN, inst, str(prm), "1"], capture_output=True, text=True, cwd=str(tmp_path),
                             timeout=600).stdout
        ref = float(re.search(r"^node 1 level 0 n \d+ bound (\S+)", out, re.M).group(1))
        n, e, w = G.read_rudy(inst)
        c = orc.Ctx(orc.shipped_params(), orc.build_L(n, (e, w)), n, rng=orc.RNG_GLIBC, topk=orc.TOPK_REFERENCE,
                    canon_sign=0)
        got = c.bab(max_nodes=1)["log"][0].bound
        assert abs(got - ref) <= 1e-12 * abs(ref), (name, got, ref)


def test_newton_schulz_model_l0_truncation(orc, gpu_lib):
    """The chosen form's sign iteration in exact arithmetic (the oracle's projection
    model; the schedule is the library's, host arithmetic only): with l0 = 1e-6 and
    1e-5 the ADMM runs the same iterations as with the exact projection and the
    bound moves by less than 1e-8 -- the truncation costs nothing at either l0."""
    n, e, w = G.gnp(64, 0.5, "pm1", seed=4)
    SL = orc.build_L(n, (e, w))
    prm = orc.shipped_params(include_Hepta=0, use_diff=0)
    out = {}
    try:
        for l0 in (None, 1e-6, 1e-5):
            orc.set_ns_schedule(None if l0 is None else [(a, b) for a, b, _ in gpu_lib.ns_schedule_for(l0)])
            c = orc.Ctx(prm, SL, n)
            b, st = c.evaluate(orc.make_node(n - 1), rank=1)
            out[l0] = (b, st.admm_iters)
    finally:
        orc.set_ns_schedule(None)
    b0, it0 = out[None]
    assert it0 > 0
    for l0 in (1e-6, 1e-5):
        assert out[l0][1] == it0, out
        assert abs(out[l0][0] - b0) <= 1e-8 * abs(b0), out


def test_linear_solve_tolerance_slack(orc, gpu_lib):
    """Under the chosen form's projection model (l0 = 1e-6), solving (B B^T + I) t = r
    to 1e-8 instead of the chosen form's 1e-10 leaves the ADMM's iterations unchanged
    and the bound within 1e-8."""
    n, e, w = G.gnp(64, 0.5, "pm1", seed=4)
    SL = orc.build_L(n, (e, w))
    prm = orc.shipped_params(include_Hepta=0, use_diff=0)
    out = {}
    try:
        orc.set_ns_schedule([(a, b) for a, b, _ in gpu_lib.ns_schedule_for(1e-6)])
        for tol in (1e-10, 1e-8):
            orc.set_cg_tol(tol)
            b, st = orc.Ctx(prm, SL, n).evaluate(orc.make_node(n - 1), rank=1)
            out[tol] = (b, st.admm_iters)
    finally:
        orc.set_ns_schedule(None)
        orc.set_cg_tol(None)
    assert out[1e-8][1] == out[1e-10][1] > 0, out
    assert abs(out[1e-8][0] - out[1e-10][0]) <= 1e-8 * abs(out[1e-10][0]), out


@pytest.mark.parametrize("n,p,wts,seed,fixed,pent,hept", [
    (40, 0.5, "one", 2, {3: 1, 11: 0}, 1, 0),
    (64, 0.5, "pm1", 4, {}, 0, 0),
    (80, 0.1, "int10", 5, {7: 1}, 1, 1),
])
def test_cg_stand_in_matches_a_direct_factorisation(orc, n, p, wts, seed, fixed, pent, hept):
    """The oracle (and the reference build here) solve (B B^T + I) t = r by conjugate
    gradients to 1e-15 where the reference factors it with CHOLMOD (admm.c:480-487,546).
    With a dense Cholesky factor in its place the node bound runs the same rounds,
    ADMM iterations and cuts and ends within 1e-13: the stand-in does not move the
    reference's answer."""
    nv, e, w = G.gnp(n, p, wts, seed=seed)
    SL = G.extended_laplacian(nv, e, w).ravel(order="F")
    prm = orc.shipped_params(include_Pent=pent, include_Hepta=hept, use_diff=0)
    out = []
    try:
        for direct in (False, True):
            orc.set_direct_solve(direct)
            oc = orc.Ctx(prm, SL, nv, rng=orc.RNG_COUNTER, topk=orc.TOPK_CANONICAL, canon_sign=1)
            b, st = oc.evaluate(orc.make_node(nv - 1, fixed), rank=1)
            out.append((b, (st.outer_iters, st.admm_iters, st.n_tri, st.n_pent, st.n_hept)))
            oc.close()
    finally:
        orc.set_direct_solve(False)
    assert out[0][1] == out[1][1] and out[0][1][1] > 0, out
    assert abs(out[0][0] - out[1][0]) <= 1e-13 * abs(out[1][0]), out


def test_projection_dump_records_every_admm_projection(orc, tmp_path):
    """The study hook orc_set_projection_dump appends each matrix the ADMM projects:
    one record per ADMM iteration, of the subproblem's order."""
    nv, e, w = G.gnp(40, 0.5, "one", seed=2)
    SL = G.extended_laplacian(nv, e, w).ravel(order="F")
    path = str(tmp_path / "w.bin")
    try:
        orc.set_projection_dump(path)
        oc = orc.Ctx(orc.shipped_params(include_Pent=0, include_Hepta=0, use_diff=0), SL, nv)
        _, st = oc.evaluate(orc.make_node(nv - 1), rank=1)
        oc.close()
    finally:
        orc.set_projection_dump(None)
    raw = open(path, "rb").read()
    count, off, n0 = 0, 0, None
    while off < len(raw):
        n = int(np.frombuffer(raw, dtype=np.int32, count=1, offset=off)[0])
        n0 = n if n0 is None else n0
        assert n == n0
        W = np.frombuffer(raw, dtype=np.float64, count=n * n, offset=off + 4)
        assert np.isfinite(W).all()
        off += 4 + 8 * n * n
        count += 1
    assert off == len(raw) and n0 == nv and count == st.admm_iters > 0


# ---- numpy restatements of the operators ------------------------------------
def _np_op_B(X, tri, pent, hept):
    y = []
    for (i, j, k, t) in tri:
        e = {1: (1, 1, 1), 2: (1, 1, -1), 3: (1, -1, 1), 4: (-1, 1, 1)}[t]
        p = (i, j, k)
        y.append(-sum(e[a] * e[b] * X[max(p[a], p[b]), min(p[a], p[b])] for a in range(3) for b in range(a + 1, 3)))
    for c in list(pent) + list(hept):
        t, p = c[0], c[1:]
        k = len(p)
        e = [-1 if a < t - 1 else 1 for a in range(k)]
        s = {5: 0.5, 7: 1.0 / 3.0}[k]
        y.append(-s * sum(e[a] * e[b] * X[max(p[a], p[b]), min(p[a], p[b])] for a in range(k) for b in range(a + 1, k)))
    return np.array(y)


def test_oracle_operators_against_numpy(orc):
    rng = np.random.default_rng(5)
    n = 20
    X = rng.standard_normal((n, n))
    X = X + X.T
    tri = [tuple(sorted(rng.choice(n, 3, replace=False))[::-1]) + (int(rng.integers(1, 5)),) for _ in range(15)]
    pent = [(int(rng.integers(1, 4)),) + tuple(int(v) for v in rng.choice(n, 5, replace=False)) for _ in range(6)]
    hept = [(int(rng.integers(1, 5)),) + tuple(int(v) for v in rng.choice(n, 7, replace=False)) for _ in range(6)]
    assert np.allclose(orc.op_B(X, tri, pent, hept), _np_op_B(X, tri, pent, hept), atol=1e-12)
    # adjoint: <B^T t, X> = <t, B(X)> with the Frobenius product on symmetric matrices
    t = rng.standard_normal(len(tri) + len(pent) + len(hept))
    BtT = -(orc.op_Bt(np.zeros((n, n)), t, tri, pent, hept))
    Y = np.tril(X) + np.tril(X, -1).T
    assert abs(np.sum(BtT * Y) - t @ orc.op_B(Y, tri, pent, hept)) < 1e-10


def test_oracle_projection_against_numpy(orc):
    rng = np.random.default_rng(3)
    n = 40
    A = rng.standard_normal((n, n))
    W = A + A.T
    Xp, Q, Z, ev = orc.project(W, abstol=0.0)
    w, V = np.linalg.eigh(W)
    Xr = (V[:, w > 1e-8] * w[w > 1e-8]) @ V[:, w > 1e-8].T
    assert np.allclose(np.tril(Xp), np.tril(Xr), atol=1e-12)
    assert np.allclose(Z @ Z.T, Xr, atol=1e-12)
    assert np.allclose(np.tril(Q), np.tril(Xr - W), atol=1e-12)
    assert np.all(np.triu(Q, 1) == 0.0)


def test_create_subproblem_against_numpy(orc):
    n, e, w = G.gnp(25, 0.5, "int10", seed=9)
    SL = G.extended_laplacian(n, e, w)
    fixed = {3: 1, 7: 0, 10: 1}
    xf = np.zeros(n, np.int32)
    so = np.zeros(n, np.int32)
    for i, v in fixed.items():
        xf[i], so[i] = 1, v
    m, PL = orc.create_subproblem(SL.ravel(order="F"), n, xf, so)
    U = [i for i in range(n - 1) if not xf[i]]
    F1 = [i for i in range(n - 1) if xf[i] and so[i] == 1]
    Lap = SL[: n - 1, : n - 1]
    B = Lap[np.ix_(U, U)]
    fr = Lap[np.ix_(U, F1)].sum(axis=1)
    rs = B.sum(axis=1) + 2 * fr
    ref = np.zeros((m, m))
    ref[: m - 1, : m - 1] = B + np.diag(2 * fr)
    ref[m - 1, : m - 1] = rs
    ref[: m - 1, m - 1] = rs
    ref[m - 1, m - 1] = rs.sum()
    assert m == len(U) + 1
    assert np.allclose(PL, 0.25 * ref, atol=1e-12)
    fv = orc.fixed_value(SL.ravel(order="F"), n, xf, so)
    x = np.array([so[i] if xf[i] else 0 for i in range(n - 1)], float)
    assert abs(fv - x @ Lap @ x) < 1e-9


def test_mlp_restatement_gradient_against_finite_differences():
    from oracle import mlp_ref as R

    rng = np.random.default_rng(0)
    d, h1, h2 = 6, 5, 4
    P = h1 * d + h1 + h2 * h1 + 2 * h2 + 1
    p = rng.standard_normal(P) * 0.5
    X = rng.standard_normal((20, d))
    Y = rng.standard_normal(20)
    _, g = R.loss_and_grad(p, X, Y, d, h1, h2)
    eps = 1e-6
    num = np.zeros(P)
    for q in range(P):
        e = np.zeros(P)
        e[q] = eps
        num[q] = (R.loss_and_grad(p + e, X, Y, d, h1, h2)[0] - R.loss_and_grad(p - e, X, Y, d, h1, h2)[0]) / (2 * eps)
    assert np.allclose(g, num, rtol=1e-6, atol=1e-8)


def test_scaled_newton_schulz_projection_in_float64():
    """The chosen form's algorithm, restated in numpy float64: W / ||W||_F through
    the library's step schedule gives sign(W), and (W + W S) / 2 matches the
    eigendecomposition projection up to the unresolved band |lambda| < l0 ||W||_F."""
    from madam_gb300 import build as B
    from madam_gb300 import lib as M

    if not os.path.exists(M.LIB_PATH):
        B.build()
    rng = np.random.default_rng(11)
    n = 120
    A = rng.standard_normal((n, n))
    W = (A + A.T) / np.sqrt(2 * n)
    w, V = np.linalg.eigh(W)
    Xr = (V[:, w > 0] * w[w > 0]) @ V[:, w > 0].T
    for l0 in (1e-3, 1e-6):
        S = W / np.linalg.norm(W)
        for a, b, _ in M.ns_schedule_for(l0):
            S = a * S + b * (S @ S @ S)
        X = 0.5 * (W + W @ S)
        err = np.linalg.norm(X - Xr) / np.linalg.norm(W)
        # eigenvalues below l0 ||W||_F are the only ones left unresolved
        band = np.abs(w) < l0 * np.linalg.norm(W)
        bound = 0.5 * np.sqrt(np.sum(w[band] ** 2)) / np.linalg.norm(W) + 1e-9
        assert err <= max(bound, 1e-9), (l0, err, bound)
        # M = round((n + tr S) / 2) counts the positive eigenvalues, up to the unresolved band
        Mns = int(round(0.5 * (n + np.trace(S))))
        assert abs(Mns - int((w > 0).sum())) <= band.sum()
