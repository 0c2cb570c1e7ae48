"""The chosen form: Newton-Schulz PSD projection on the tensor cores.

Checks (1) the projection against an FP64 eigendecomposition (numpy.linalg.eigh)
for the default digit-plane operands (five BF16 digits, products accurate to
~5e-10) and for one-pass operands, whose rounding floor is stated; (2) node
bounds against the CPU oracle's FP64 method: the bound is the same safe dual
bound n lambda_max(L - Diag y - B^T s) + sum y + sum s, so it stays valid
whatever the projection's error, and it agrees with the FP64 method to 1e-6
relative, after the same number of ADMM iterations; (3) whole branch-and-bound
runs reach the reference's optimum and optimal cut.
"""
import json
import os

import numpy as np
import pytest

from madam_gb300 import graphs as G

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURES = json.load(open(os.path.join(HERE, "golden", "reference_bab.json")))["instances"]


def _proj_eigh(W):
    w, V = np.linalg.eigh(W)
    k = w > 1e-8
    return (V[:, k] * w[k]) @ V[:, k].T, int(k.sum())


def _spectra(n, rng):
    A = rng.standard_normal((n, n))
    gauss = (A + A.T) / np.sqrt(2 * n)
    U, _ = np.linalg.qr(rng.standard_normal((n, n)))
    r = max(2, n // 20)
    # ADMM-like: a few clearly positive eigenvalues (X / sigma), the rest negative (-Q)
    lam = np.concatenate([np.linspace(6.0, 0.3, r), -0.05 - 2.0 * np.abs(rng.standard_normal(n - r))])
    return {"gauss": gauss, "admm": (U * lam) @ U.T}


@pytest.mark.parametrize("n", [33, 130, 257, 512])
@pytest.mark.parametrize("form", ["bf16", "tf32"])
def test_ns_projection_against_eigh(gpu_lib, n, form):
    M = gpu_lib
    proj = M.PROJ_NS_BF16 if form == "bf16" else M.PROJ_NS_TF32
    rng = np.random.default_rng(n)
    for name, W in _spectra(n, rng).items():
        Xr, Mr = _proj_eigh(W)
        Xp, Q, Z, _ = M.project(W, proj)
        err = np.linalg.norm(Xp - Xr) / np.linalg.norm(W)
        # digit-plane operands: ~5e-9 of ||W|| at n = 512 (the sign iteration's own
        # resolution of the eigenvalues nearest 0)
        assert err < 3e-8, (name, err)
        assert np.array_equal(Xp, Xp.T)
        assert np.allclose(np.tril(Q), np.tril(Xp - W), atol=1e-12)
        if name == "admm":  # a spectral gap around 0: the count is exact
            assert Z.shape[1] == Mr
            assert np.isclose(np.trace(Xp), np.trace(Xr), rtol=1e-7)


def test_ns_one_pass_operands_have_a_rounding_floor(gpu_lib):
    """One pass of BF16/TF32 operands cannot resolve eigenvalues below their
    rounding (~1e-3 of ||W||): the error floor that makes the default split."""
    M = gpu_lib
    rng = np.random.default_rng(5)
    W = _spectra(256, rng)["gauss"]
    Xr, _ = _proj_eigh(W)
    Xn, _, _, _ = M.project(W, M.PROJ_NS_TF32 | M.PROJ_OPERANDS(M.NS_OPERANDS_NATIVE))
    Xs, _, _, _ = M.project(W, M.PROJ_NS_TF32 | M.PROJ_OPERANDS(M.NS_OPERANDS_SPLIT))
    en = np.linalg.norm(Xn - Xr) / np.linalg.norm(W)
    es = np.linalg.norm(Xs - Xr) / np.linalg.norm(W)
    assert 1e-5 < en < 5e-3
    assert es < en / 100


def test_ns_projection_zero_matrix(gpu_lib):
    M = gpu_lib
    Xp, Q, _, _ = M.project(np.zeros((20, 20)), M.PROJ_NS_BF16)
    assert not Xp.any() and not Q.any()


def test_ns_schedule_properties(gpu_lib):
    """Scaled Newton-Schulz steps: p(x) = a x + b x^3 keeps [0, 1] in [0, 1], raises
    the lower end of the spectrum interval from l0 to within 1e-7 of 1, and closes
    with FP32-accurate steps."""
    M = gpu_lib
    n, e, w = G.gnp(20, 0.5, "pm1", seed=1)
    ctx = M.Context(M.params(), G.extended_laplacian(n, e, w).ravel(order="F"), n, flags=M.PROJ_NS_BF16)
    for l0 in (1e-3, 1e-6):
        ctx.ns_options(M.NS_OPERANDS_SPLIT, l0)
        st = ctx.ns_schedule()
        lo, xs = l0, np.linspace(0, 1, 2001)
        for a, b, acc in st:
            assert np.all(a * xs + b * xs ** 3 <= 1 + 1e-6) and np.all(a * xs + b * xs ** 3 >= -1e-9)
            lo = min(a * lo + b * lo ** 3, a + b)
        assert lo > 1 - 1e-6
        assert st[-1][2] == 1 and st[-2][2] == 1
    with pytest.raises(M.MCBError):
        ctx.ns_options(M.NS_OPERANDS_SPLIT, 0.7)
    ctx.close()
    with pytest.raises(M.MCBError):
        M.Context(M.params(), G.extended_laplacian(n, e, w).ravel(order="F"), n).ns_options(0, 1e-6)


@pytest.mark.parametrize("n,p,wts,seed,fixed,pent", [
    (40, 0.5, "one", 2, {3: 1, 11: 0}, 1),
    (64, 0.5, "pm1", 4, {}, 0),
    (80, 0.1, "int10", 5, {7: 1}, 1),
])
def test_ns_node_bound_against_oracle(gpu_lib, orc, n, p, wts, seed, fixed, pent):
    M = gpu_lib
    nv, e, w = G.gnp(n, p, wts, seed=seed)
    SL = G.extended_laplacian(nv, e, w).ravel(order="F")
    oc = orc.Ctx(orc.shipped_params(include_Pent=pent, include_Hepta=0, use_diff=0), SL, nv,
                 rng=orc.RNG_COUNTER, topk=orc.TOPK_CANONICAL, canon_sign=1)
    bo, so = oc.evaluate(orc.make_node(nv - 1, fixed), rank=1)
    for proj in (M.PROJ_NS_BF16, M.PROJ_NS_TF32):
        ctx = M.Context(M.params(include_Pent=pent, include_Hepta=0, use_diff=0), SL, nv, flags=proj)
        bg, sg = ctx.evaluate(M.node(fixed), rank=1)
        assert abs(bg - bo) <= 1e-6 * abs(bo), (bg, bo)
        # the node's best cut (found by either heuristic) never exceeds a safe bound
        assert bg >= max(ctx.lb()[0], oc.lb()[0])
        assert sg.admm_iters == so.admm_iters and sg.outer_iters == so.outer_iters
        ctx.close()


@pytest.mark.parametrize("fx", FIXTURES, ids=lambda f: f["name"])
def test_ns_branch_and_bound_reaches_reference_optimum(gpu_lib, fx):
    M = gpu_lib
    if fx["kind"] == "gnp":
        n, e, w = G.gnp(*fx["args"][:3], seed=fx["args"][3])
    else:
        n, e, w = G.torus2d(fx["args"][0], fx["args"][1], seed=fx["args"][2])
    SL = G.extended_laplacian(n, e, w).ravel(order="F")
    ctx = M.Context(M.params(), SL, n, batch_max=4, flags=M.PROJ_NS_BF16)
    r = ctx.bab(batch=4, max_nodes=2000)
    assert r["opt"] == fx["opt"]
    side = np.zeros(n, dtype=np.int32)
    side[: n - 1] = r["sol"]
    assert G.cut_value(n, e, w, side) == fx["opt"]
    # every bound of the tree is a valid bound on the cut of its subtree; the root's on the optimum
    assert r["root_bound"] >= fx["opt"]
    ctx.close()


@pytest.mark.parametrize("npad,batch", [(128, 1), (256, 3), (512, 2)])
def test_tcgen05_split_gemm_against_float64(gpu_lib, npad, batch):
    """The tensor-core GEMM with digit-plane operands on general (non-symmetric)
    matrices, C = alpha A B^T + diag I: its FP32 output is the rounding of a
    product accurate to ~5e-10, so the error is FP32's half ulp of the largest entry."""
    rng = np.random.default_rng(npad + batch)
    A = rng.standard_normal((batch, npad, npad)).astype(np.float32)
    B = rng.standard_normal((batch, npad, npad)).astype(np.float32)
    C = gpu_lib.split_gemm(A, B, alpha=-0.75, diag=1.5)
    ref = -0.75 * np.einsum("bik,bjk->bij", A.astype(np.float64), B.astype(np.float64)) + 1.5 * np.eye(npad)
    assert np.abs(C - ref).max() <= 1e-7 * np.abs(ref).max()


def test_tcgen05_split_gemm_rejects_bad_sizes(gpu_lib):
    with pytest.raises(gpu_lib.MCBError):
        gpu_lib.split_gemm(np.zeros((1, 100, 100)), np.zeros((1, 100, 100)))


@pytest.mark.parametrize("npad", [128, 384])
def test_tcgen05_symmetric_product_is_exactly_symmetric(gpu_lib, npad):
    """sym = 1: lower tiles computed and mirrored; the result is bit-symmetric and
    FP32-exact (to the output's rounding) for a product known to be symmetric (A A^T)."""
    rng = np.random.default_rng(npad)
    A = rng.standard_normal((2, npad, npad)).astype(np.float32)
    A = A + A.transpose(0, 2, 1)
    C = gpu_lib.split_gemm(A, A, alpha=0.5, diag=-1.0, sym=True)
    ref = 0.5 * np.einsum("bik,bjk->bij", A.astype(np.float64), A.astype(np.float64)) - np.eye(npad)
    assert np.array_equal(C, C.transpose(0, 2, 1))
    assert np.abs(C - ref).max() <= 1e-7 * np.abs(ref).max()


@pytest.mark.parametrize("proj", ["fp64", "ns"])
def test_graph_replay_matches_direct_launches(gpu_lib, proj, tmp_path):
    """ADMM chunks replayed from CUDA graphs (profiling off) give bit-identical
    bounds to direct launches (profiling on); the autotuner's table round-trips."""
    M = gpu_lib
    n, e, w = G.gnp(70, 0.5, "pm1", seed=8)
    SL = G.extended_laplacian(n, e, w).ravel(order="F")
    flags = M.PROJ_FP64 if proj == "fp64" else M.PROJ_NS_BF16
    fixes = [{}, {3: 1}, {5: 0, 9: 1}, {1: 1, 2: 0}]
    out = []
    for prof in (False, True):
        ctx = M.Context(M.params(include_Hepta=0, use_diff=0), SL, n, batch_max=4,
                        flags=flags | (M.FLAG_PROFILE if prof else 0))
        b, st = ctx.bound_batch([M.node(f) for f in fixes])
        caps, reps = ctx.graph_stats()
        if prof:
            assert caps == 0 and reps == 0
        else:
            assert caps >= 1 and reps > caps
        out.append((b, [s.admm_iters for s in st]))
        if proj == "ns" and not prof:
            tab = ctx.autotune_table()
            assert tab and all(t["variant"] in (0, 1) and min(t["us"]) > 0 for t in tab)
            path = str(tmp_path / "tune.json")
            ctx.autotune_save(path)
            ctx2 = M.Context(M.params(include_Hepta=0, use_diff=0), SL, n, batch_max=4, flags=flags)
            ctx2.autotune_load(path)
            tab2 = ctx2.autotune_table()
            assert [(t["npad"], t["bucket"], t["variant"]) for t in tab2] == \
                [(t["npad"], t["bucket"], t["variant"]) for t in tab]
            assert all(abs(a - b) <= 1e-3 for t, u in zip(tab, tab2) for a, b in zip(t["us"], u["us"]))
            ctx2.close()
        ctx.close()
    assert np.array_equal(out[0][0], out[1][0]) and out[0][1] == out[1][1]


def test_solve_command_line_reaches_reference_optimum(gpu_lib, tmp_path):
    """madam_gb300.solve: rudy instance + parameter file in, the reference's
    report out, with the reference's optimum and a solution that attains it."""
    import re

    from madam_gb300 import solve as S

    fx = FIXTURES[0]
    n, e, w = G.gnp(*fx["args"][:3], seed=fx["args"][3])
    inst = tmp_path / "g.rudy"
    G.write_rudy(str(inst), n, e, w)
    prm = tmp_path / "params"
    prm.write_text("".join("%s = %s\n" % kv for kv in gpu_lib.SHIPPED.items()))
    text, r = S.solve(str(inst), str(prm), form="mixed", batch=8)
    assert r["opt"] == fx["opt"]
    assert float(re.search(r"^Maximum value = (\S+)", text, re.M).group(1)) == fx["opt"]
    sol = [int(v) - 1 for v in re.search(r"^Solution = \( (.*)\)", text, re.M).group(1).split()]
    side = np.zeros(n, dtype=np.int32)
    side[sol] = 1
    assert G.cut_value(n, e, w, side) == fx["opt"]
