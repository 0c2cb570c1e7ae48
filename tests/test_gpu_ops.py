"""GPU operator parity: every kernel of the bound path against the CPU oracle
(the reference's algorithm restated in C) on seeded inputs, through the C ABI."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _rand_psdish(n, seed, rank=None):
    rng = np.random.default_rng(seed)
    A = rng.standard_normal((n, rank or n))
    X = A @ A.T
    d = np.sqrt(np.diag(X))
    X = X / np.outer(d, d)
    return X


def _rand_sym(n, seed):
    rng = np.random.default_rng(seed)
    A = rng.standard_normal((n, n))
    return 0.5 * (A + A.T)


def _rand_cuts(n, seed, nt=40, np_=20, nh=20):
    rng = np.random.default_rng(seed)
    tri = []
    for _ in range(nt):
        i, j, k = sorted(rng.choice(n, 3, replace=False))[::-1]
        tri.append((i, j, k, int(rng.integers(1, 5))))
    pent = [(int(rng.integers(1, 4)),) + tuple(int(v) for v in rng.choice(n, 5, replace=False)) for _ in range(np_)]
    hept = [(int(rng.integers(1, 5)),) + tuple(int(v) for v in rng.choice(n, 7, replace=False)) for _ in range(nh)]
    return tri, pent, hept


@pytest.mark.parametrize("n", [7, 33, 100])
def test_op_B_bit_exact(gpu_lib, orc, n):
    X = _rand_sym(n, n)
    tri, pent, hept = _rand_cuts(n, n + 1)
    y_gpu = gpu_lib.op_B(X, tri, pent, hept)
    y_orc = orc.op_B(X, tri, pent, hept)
    assert np.array_equal(y_gpu, y_orc)


@pytest.mark.parametrize("n", [7, 33, 100])
def test_op_Bt_bit_exact(gpu_lib, orc, n):
    X = _rand_sym(n, 2 * n)
    tri, pent, hept = _rand_cuts(n, 2 * n + 1)
    t = np.random.default_rng(n).standard_normal(len(tri) + len(pent) + len(hept))
    A = gpu_lib.op_Bt(X, t, tri, pent, hept)
    B = orc.op_Bt(X, t, tri, pent, hept)
    assert np.array_equal(A, B)


@pytest.mark.parametrize("n,seed", [(1, 0), (2, 1), (3, 2), (17, 3), (64, 4), (150, 5), (257, 6)])
def test_projection_matches_eigendecomposition(gpu_lib, orc, n, seed):
    W = _rand_sym(n, seed) * 3.0
    Xp, Q, Z, ev = gpu_lib.project(W)
    w, V = np.linalg.eigh(W)
    Xref = (V[:, w > 1e-8] * w[w > 1e-8]) @ V[:, w > 1e-8].T
    scale = max(1.0, np.abs(W).max())
    # tolerance: FP64 eigensolver, relative to ||W||
    assert np.abs(Xp - Xref).max() <= 1e-10 * scale * n
    assert np.allclose(np.tril(Q), np.tril(Xp - W), atol=1e-12 * scale)
    assert len(ev) == int((w > 1e-8).sum())
    assert np.allclose(ev, w[w > 1e-8], atol=1e-11 * scale)
    Xo, Qo, Zo, evo = orc.project(W, canon_sign=1, abstol=0.0)
    assert np.abs(np.tril(Xp) - np.tril(Xo)).max() <= 1e-10 * scale * n
    # same canonical signs => same factor
    assert Z.shape == Zo.shape
    assert np.abs(Z - Zo).max() <= 1e-8 * scale


@pytest.mark.parametrize("n,seed", [(1, 0), (5, 1), (90, 2), (300, 3)])
def test_lambda_max_safe(gpu_lib, n, seed):
    A = _rand_sym(n, seed)
    lam, upper = gpu_lib.lambda_max(A)
    true = np.linalg.eigvalsh(A).max()
    assert abs(lam - true) <= 1e-12 * max(1.0, np.abs(A).max()) * n
    assert upper >= true


@pytest.mark.parametrize("n,seed", [(10, 0), (60, 1), (120, 2)])
def test_ipm_matches_oracle(gpu_lib, orc, n, seed):
    from madam_gb300 import graphs as G

    nv, e, w = G.gnp(n, 0.5, "pm1", seed=seed)
    SL = G.extended_laplacian(nv, e, w).ravel(order="F")
    _, PL = orc.create_subproblem(SL, nv, np.zeros(nv, np.int32), np.zeros(nv, np.int32))
    it_g, phi_g, Xg, yg, Zg = gpu_lib.ipm(PL)
    it_o, phi_o, Xo, yo, Zo = orc.ipm(PL)
    assert it_g == it_o
    assert abs(phi_g - phi_o) <= 1e-9 * abs(phi_o)
    assert np.abs(Xg - Xo).max() <= 1e-7


@pytest.mark.parametrize("n,seed,K", [(3, 0, 10), (40, 1, 400), (120, 2, 1200), (200, 3, 100)])
def test_triangle_separation_exact(gpu_lib, orc, n, seed, K):
    X = _rand_psdish(n, seed, rank=4)
    mx_g, cuts_g, v_g = gpu_lib.sep_triangles(X, K)
    mx_o, cuts_o, v_o = orc.sep_triangles(X, K, mode=orc.TOPK_CANONICAL)
    assert mx_g == mx_o
    assert np.array_equal(cuts_g, cuts_o)
    assert np.array_equal(v_g, v_o)


def test_triangle_separation_matches_reference_replay(gpu_lib, orc):
    # with distinct violations the canonical top-K is the reference's list as a set
    X = _rand_psdish(60, 11, rank=3)
    _, cuts_g, _ = gpu_lib.sep_triangles(X, 600)
    _, cuts_r, _ = orc.sep_triangles(X, 600, mode=orc.TOPK_REFERENCE)
    assert sorted(map(tuple, cuts_g)) == sorted(map(tuple, cuts_r))


@pytest.mark.parametrize("k,n,seed", [(5, 30, 0), (7, 45, 1), (5, 100, 2)])
def test_sa_matches_oracle_counter_streams(gpu_lib, orc, k, n, seed):
    X = _rand_psdish(n, seed, rank=3)
    key = 0x1234ABCD + seed
    trials = 6
    vals, ineq = gpu_lib.qap_sa_batch(X, k, trials, key)
    nt = 3 if k == 5 else 4
    L = orc.lib()
    for r in range(trials * nt):
        typ, trial = r % nt + 1, r // nt
        e = np.array([-1 if a < typ - 1 else 1 for a in range(k)])
        H = np.outer(e, e)
        rkey = L.orc_key2(key, trial * 8 + typ)
        v, out = orc.qap_sa(H, k, X, key=rkey, rng=orc.RNG_COUNTER)
        assert v == vals[r]
        assert list(out) == list(ineq[r])
