"""ctypes binding of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Only the tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` use this module, and only as the checker / the timed CPU baseline.
The product library never imports it.
"""
import ctypes as C

import numpy as np

from . import build as _build

NMAX = 1024
RNG_GLIBC, RNG_COUNTER = 0, 1
TOPK_REFERENCE, TOPK_CANONICAL = 0, 1

_PARAM_FIELDS = [
    ("sigma0", C.c_double), ("scaleSigma", C.c_double), ("ADMM_itermax", C.c_int),
    ("tol0", C.c_double), ("scaleTol", C.c_double), ("minTol", C.c_double),
    ("triag_iter", C.c_int), ("pent_iter", C.c_int), ("hept_iter", C.c_int),
    ("max_outer_iter", C.c_int), ("extra_iter", C.c_int), ("violated_TriIneq", C.c_double),
    ("TriIneq", C.c_int), ("adjust_TriIneq", C.c_int), ("PentIneq", C.c_int),
    ("HeptaIneq", C.c_int), ("Pent_Trials", C.c_int), ("Hepta_Trials", C.c_int),
    ("include_Pent", C.c_int), ("include_Hepta", C.c_int), ("root", C.c_int),
    ("use_diff", C.c_int), ("branchingStrategy", C.c_int),
]


class Params(C.Structure):
    _fields_ = _PARAM_FIELDS


class Node(C.Structure):
    _fields_ = [("xfixed", C.c_int * NMAX), ("sol", C.c_int * NMAX), ("fracsol", C.c_double * NMAX),
                ("level", C.c_int), ("upper_bound", C.c_double)]


class NodeStats(C.Structure):
    _fields_ = [("bound", C.c_double), ("basic_bound", C.c_double), ("n_sub", C.c_int),
                ("outer_iters", C.c_int), ("admm_iters", C.c_int), ("ipm_iters", C.c_int),
                ("n_tri", C.c_int), ("n_pent", C.c_int), ("n_hept", C.c_int),
                ("pruned", C.c_int), ("gaveup", C.c_int), ("seconds", C.c_double)]


class Glibc(C.Structure):
    _fields_ = [("r", C.c_uint32 * 34), ("pos", C.c_int)]


_lib = None

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")


def lib():
    global _lib
    if _lib is not None:
        return _lib
    path = _build.build_oracle()
    L = C.CDLL(path)
    rc = L.orc_lapack_init(_build.find_lapack().encode())
    if rc != 0:
        raise RuntimeError("oracle: LAPACK init failed (%d)" % rc)
    L.orc_glibc_seed.argtypes = [C.POINTER(Glibc), C.c_uint]
    L.orc_glibc_next.argtypes = [C.POINTER(Glibc)]
    L.orc_mix64.restype = C.c_uint64
    L.orc_mix64.argtypes = [C.c_uint64]
    L.orc_key2.restype = C.c_uint64
    L.orc_key2.argtypes = [C.c_uint64, C.c_uint64]
    L.orc_node_key.restype = C.c_uint64
    L.orc_node_key.argtypes = [_ip, _ip, C.c_int]
    L.orc_default_params.argtypes = [C.POINTER(Params)]
    L.orc_build_L.argtypes = [C.c_int, C.c_int, _ip, _ip, _dp, _dp]
    L.orc_create_subproblem.argtypes = [C.c_int, _dp, _ip, _ip, _dp]
    L.orc_fixed_value.restype = C.c_double
    L.orc_fixed_value.argtypes = [C.c_int, _dp, _ip, _ip]
    L.orc_evaluate_solution.restype = C.c_double
    L.orc_evaluate_solution.argtypes = [C.c_int, _dp, _ip]
    L.orc_op_B.argtypes = [C.c_int, _dp, C.c_int, _ip, C.c_int, _ip, C.c_int, _ip, _dp]
    L.orc_op_Bt.argtypes = [C.c_int, _dp, C.c_int, _ip, C.c_int, _ip, C.c_int, _ip, _dp]
    L.orc_project.argtypes = [C.c_int, _dp, _dp, _dp, _dp, _dp, C.c_int]
    L.orc_set_abstol.argtypes = [C.c_double]
    L.orc_set_ns_schedule.argtypes = [C.c_int, C.c_void_p, C.c_void_p]
    L.orc_set_cg_tol.argtypes = [C.c_double]
    L.orc_set_direct_solve.argtypes = [C.c_int]
    L.orc_set_projection_dump.argtypes = [C.c_char_p]
    L.orc_lambda_max.restype = C.c_double
    L.orc_lambda_max.argtypes = [C.c_int, _dp]
    L.orc_ipm.argtypes = [_dp, C.c_int, _dp, _dp, _dp, C.POINTER(C.c_double)]
    L.orc_sep_triangles.restype = C.c_double
    L.orc_sep_triangles.argtypes = [_dp, C.c_int, C.c_int, C.c_double, C.c_int, _ip, _dp,
                                    C.POINTER(C.c_int)]
    L.orc_qap_sa.restype = C.c_double
    L.orc_qap_sa.argtypes = [_ip, C.c_int, _dp, C.c_int, C.c_int, C.POINTER(Glibc), C.c_uint64, _ip]
    L.orc_create.restype = C.c_void_p
    L.orc_create.argtypes = [C.POINTER(Params), C.c_int, _dp, C.c_int, C.c_int, C.c_int]
    L.orc_destroy.argtypes = [C.c_void_p]
    L.orc_set_lb.argtypes = [C.c_void_p, C.c_double, C.c_void_p]
    L.orc_get_lb.restype = C.c_double
    L.orc_get_lb.argtypes = [C.c_void_p, C.c_void_p]
    L.orc_set_diff.argtypes = [C.c_void_p, C.c_double]
    L.orc_get_diff.restype = C.c_double
    L.orc_get_diff.argtypes = [C.c_void_p]
    L.orc_set_trials.argtypes = [C.c_void_p, C.c_int, C.c_int]
    L.orc_get_trials.argtypes = [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int)]
    L.orc_set_admm_trace.argtypes = [C.c_void_p, C.c_void_p, C.c_int]
    L.orc_evaluate.restype = C.c_double
    L.orc_evaluate.argtypes = [C.c_void_p, C.POINTER(Node), C.c_int, C.POINTER(NodeStats)]
    L.orc_bab.argtypes = [C.c_void_p, C.POINTER(C.c_double), C.c_void_p, C.POINTER(C.c_double),
                          C.c_int, C.c_void_p, C.c_int, C.POINTER(C.c_int)]
    _lib = L
    return L


def params(**over):
    p = Params()
    lib().orc_default_params(C.byref(p))
    for k, v in over.items():
        setattr(p, k, v)
    return p


def shipped_params(**over):
    """The reference's shipped parameter file (params:1-23)."""
    base = dict(sigma0=1.0, scaleSigma=1.001, ADMM_itermax=2000, tol0=5e-2, scaleTol=0.6, minTol=1e-3,
                triag_iter=3, pent_iter=3, hept_iter=3, max_outer_iter=12, extra_iter=5,
                violated_TriIneq=1e-3, TriIneq=5000, adjust_TriIneq=1, PentIneq=5000, HeptaIneq=5000,
                Pent_Trials=60, Hepta_Trials=50, include_Pent=1, include_Hepta=1, root=0, use_diff=1,
                branchingStrategy=1)
    base.update(over)
    return params(**base)


def build_L(nv, edges):
    """edges: int array (ne, 2) 1-based and weights (ne,) -> extended Laplacian (column-major)."""
    e = np.asarray(edges[0], dtype=np.int32)
    w = np.ascontiguousarray(edges[1], dtype=np.float64)
    ei = np.ascontiguousarray(e[:, 0])
    ej = np.ascontiguousarray(e[:, 1])
    L = np.zeros(nv * nv)
    lib().orc_build_L(nv, len(w), ei, ej, w, L)
    return L


def make_node(pb, fixed=None):
    nd = Node()
    if fixed:
        for i, v in fixed.items():
            nd.xfixed[i] = 1
            nd.sol[i] = int(v)
    return nd


def node_key(nd, pb):
    xf = np.ctypeslib.as_array(nd.xfixed)[:pb].astype(np.int32).copy()
    so = np.ctypeslib.as_array(nd.sol)[:pb].astype(np.int32).copy()
    return lib().orc_node_key(xf, so, pb)


class Ctx:
    """One oracle context (the reference's global state) for one problem."""

    def __init__(self, prm, SL, N, rng=RNG_COUNTER, topk=TOPK_CANONICAL, canon_sign=1):
        self.L = lib()
        self.N = N
        self.SL = np.ascontiguousarray(SL, dtype=np.float64)
        self.h = self.L.orc_create(C.byref(prm), N, self.SL, rng, topk, canon_sign)
        if not self.h:
            raise RuntimeError("orc_create failed")

    def close(self):
        if self.h:
            self.L.orc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_lb(self, lb, sol=None):
        if sol is not None:
            s = np.ascontiguousarray(sol, dtype=np.int32)
            self.L.orc_set_lb(self.h, lb, s.ctypes.data)
        else:
            self.L.orc_set_lb(self.h, lb, None)

    def lb(self):
        s = np.zeros(self.N, dtype=np.int32)
        v = self.L.orc_get_lb(self.h, s.ctypes.data)
        return v, s[: self.N - 1]

    def set_diff(self, d):
        self.L.orc_set_diff(self.h, d)

    def diff(self):
        return self.L.orc_get_diff(self.h)

    def set_trials(self, p, h):
        self.L.orc_set_trials(self.h, p, h)

    def trials(self):
        a, b = C.c_int(), C.c_int()
        self.L.orc_get_trials(self.h, C.byref(a), C.byref(b))
        return a.value, b.value

    def evaluate(self, node, rank=1):
        st = NodeStats()
        b = self.L.orc_evaluate(self.h, C.byref(node), rank, C.byref(st))
        return b, st

    def bab(self, max_nodes=0, log_cap=100000):
        opt = C.c_double()
        rb = C.c_double()
        sol = np.zeros(self.N, dtype=np.int32)
        log = (NodeStats * log_cap)()
        lc = C.c_int()
        nodes = self.L.orc_bab(self.h, C.byref(opt), sol.ctypes.data, C.byref(rb), max_nodes,
                               C.cast(log, C.c_void_p), log_cap, C.byref(lc))
        return dict(nodes=nodes, opt=opt.value, sol=sol[: self.N - 1].copy(), root_bound=rb.value,
                    log=[log[i] for i in range(lc.value)])


# ---- operator-level helpers (KATs) ----------------------------------------
def create_subproblem(SL, N, xfixed, sol):
    xf = np.ascontiguousarray(xfixed, dtype=np.int32)
    so = np.ascontiguousarray(sol, dtype=np.int32)
    PL = np.zeros(N * N)
    n = lib().orc_create_subproblem(N, np.ascontiguousarray(SL, dtype=np.float64), xf, so, PL)
    return n, PL[: n * n].reshape(n, n, order="F").copy()


def fixed_value(SL, N, xfixed, sol):
    return lib().orc_fixed_value(N, np.ascontiguousarray(SL, dtype=np.float64),
                                 np.ascontiguousarray(xfixed, dtype=np.int32),
                                 np.ascontiguousarray(sol, dtype=np.int32))


def _cuts(tri, pent, hept):
    t = np.ascontiguousarray(np.asarray(tri, dtype=np.int32).reshape(-1, 4)).ravel() if len(tri) else np.zeros(4, np.int32)
    p = np.ascontiguousarray(np.asarray(pent, dtype=np.int32).reshape(-1, 6)).ravel() if len(pent) else np.zeros(6, np.int32)
    h = np.ascontiguousarray(np.asarray(hept, dtype=np.int32).reshape(-1, 8)).ravel() if len(hept) else np.zeros(8, np.int32)
    return t, len(tri), p, len(pent), h, len(hept)


def op_B(X, tri=(), pent=(), hept=()):
    """y = B(X) (operators.c:62-150); X (n,n) read through its lower triangle."""
    n = X.shape[0]
    t, nt, p, np_, h, nh = _cuts(tri, pent, hept)
    y = np.zeros(max(nt + np_ + nh, 1))
    Xf = np.asfortranarray(X).ravel(order="F").copy()
    lib().orc_op_B(n, Xf, nt, t, np_, p, nh, h, y)
    return y[: nt + np_ + nh]


def op_Bt(X, tvec, tri=(), pent=(), hept=()):
    """X - B^T(t) (operators.c:171-513)."""
    n = X.shape[0]
    t, nt, p, np_, h, nh = _cuts(tri, pent, hept)
    Xf = np.asfortranarray(X).ravel(order="F").copy()
    tv = np.zeros(max(nt + np_ + nh, 1))
    tv[: nt + np_ + nh] = tvec
    lib().orc_op_Bt(n, Xf, nt, t, np_, p, nh, h, tv)
    return Xf.reshape(n, n, order="F")


def project(W, canon_sign=1, abstol=1e-8):
    n = W.shape[0]
    lib().orc_set_abstol(abstol)
    Wf = np.asfortranarray(W).ravel(order="F").copy()
    Xp = np.zeros(n * n)
    Q = np.zeros(n * n)
    Z = np.zeros(n * n)
    ev = np.zeros(n)
    M = lib().orc_project(n, Wf, Xp, Q, Z, ev, canon_sign)
    if M < 0:
        raise RuntimeError("dsyevr failed")
    return (Xp.reshape(n, n, order="F"), Q.reshape(n, n, order="F"),
            Z[: n * M].reshape(n, M, order="F"), ev[:M].copy())


def set_ns_schedule(steps=None):
    """Model the Newton-Schulz projection in exact arithmetic: steps = [(a, b), ...] of
    p(x) = a x + b x^3; None restores the reference projection (see orc_set_ns_schedule)."""
    if not steps:
        lib().orc_set_ns_schedule(0, None, None)
        return
    a = np.ascontiguousarray([s[0] for s in steps], dtype=np.float64)
    b = np.ascontiguousarray([s[1] for s in steps], dtype=np.float64)
    lib().orc_set_ns_schedule(len(steps), a.ctypes.data, b.ctypes.data)


def set_cg_tol(tol=None):
    """Relative residual of the ADMM's linear solve (None: the default 1e-15)."""
    lib().orc_set_cg_tol(tol if tol else 0.0)


def set_projection_dump(path=None):
    """Append every matrix W the ADMM projects to a file (int n, then n x n doubles); None closes it."""
    lib().orc_set_projection_dump(path.encode() if path else None)


def set_direct_solve(on=True):
    """The ADMM's (B B^T + I) solve by a dense Cholesky factor (the reference's CHOLMOD
    arithmetic up to ordering and rounding) instead of the conjugate-gradient stand-in."""
    lib().orc_set_direct_solve(1 if on else 0)


def lambda_max(A, abstol=1e-8):
    n = A.shape[0]
    lib().orc_set_abstol(abstol)
    return lib().orc_lambda_max(n, np.asfortranarray(A).ravel(order="F").copy())


def ipm(L):
    n = L.shape[0]
    Lf = np.asfortranarray(L).ravel(order="F").copy()
    X = np.zeros(n * n)
    y = np.zeros(n)
    Z = np.zeros(n * n)
    phi = C.c_double()
    it = lib().orc_ipm(Lf, n, X, y, Z, C.byref(phi))
    return it, phi.value, X.reshape(n, n, order="F"), y, Z.reshape(n, n, order="F")


def sep_triangles(X, K, thr=1e-3, mode=TOPK_CANONICAL):
    n = X.shape[0]
    out = np.zeros(4 * max(K, 1), dtype=np.int32)
    vals = np.zeros(max(K, 1))
    cnt = C.c_int()
    mx = lib().orc_sep_triangles(np.asfortranarray(X).ravel(order="F").copy(), n, K, thr, mode, out, vals,
                                 C.byref(cnt))
    return mx, out[: 4 * cnt.value].reshape(-1, 4), vals[: cnt.value]


def qap_sa(H, k, X, key=0, rng=RNG_COUNTER, glibc=None):
    n = X.shape[0]
    Hf = np.ascontiguousarray(np.asarray(H, dtype=np.int32).reshape(k, k).ravel(order="F"))
    out = np.zeros(k, dtype=np.int32)
    g = glibc if glibc is not None else Glibc()
    v = lib().orc_qap_sa(Hf, k, np.asfortranarray(X).ravel(order="F").copy(), n, rng, C.byref(g), key, out)
    return v, out


def glibc_stream(seed, count):
    g = Glibc()
    lib().orc_glibc_seed(C.byref(g), seed)
    return [lib().orc_glibc_next(C.byref(g)) for _ in range(count)]
