"""ctypes binding of libmcbound.so (the C ABI in include/mcbound.h).

This is the Python mirror of the reference's bound interface: ``Context.evaluate``
is MADAM's ``Evaluate(node, SP, PP, rank)`` (evaluate.c:12), ``Context.bound_batch``
bounds many nodes in one batched pass, ``Context.bab`` is the branch-and-bound
driver.  The library must be built (``madam_gb300.build.build()``); there is no
fallback: a missing library or a missing CUDA device raises.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libmcbound.so")
NMAX = 1024

OK, ERR_ARG, ERR_CUDA, ERR_NOMEM, ERR_NUMERIC, ERR_CAPACITY, ERR_ITER, ERR_NODEV = 0, -1, -2, -3, -4, -5, -6, -7
PROJ_FP64, PROJ_NS_BF16, PROJ_NS_TF32 = 0x0, 0x1, 0x2
NS_OPERANDS_NATIVE, NS_OPERANDS_SPLIT, NS_OPERANDS_FP32, NS_OPERANDS_CUBLAS_SPLIT = 0, 1, 2, 3


def PROJ_OPERANDS(op):
    """Operand choice of the Newton-Schulz forms for `project` (MCB_PROJ_OPERANDS)."""
    return (op + 1) << 4
FLAG_PROFILE, FLAG_LEARNED, FLAG_LOG = 0x100, 0x200, 0x400
CUT_FEATURES = 10
LOG_SCORER, LOG_WARM = 0, 1

PARAM_FIELDS = [
    ("sigma0", C.c_double), ("scaleSigma", C.c_double), ("ADMM_itermax", C.c_int),
    ("tol0", C.c_double), ("scaleTol", C.c_double), ("minTol", C.c_double),
    ("triag_iter", C.c_int), ("pent_iter", C.c_int), ("hept_iter", C.c_int),
    ("max_outer_iter", C.c_int), ("extra_iter", C.c_int), ("violated_TriIneq", C.c_double),
    ("TriIneq", C.c_int), ("adjust_TriIneq", C.c_int), ("PentIneq", C.c_int),
    ("HeptaIneq", C.c_int), ("Pent_Trials", C.c_int), ("Hepta_Trials", C.c_int),
    ("include_Pent", C.c_int), ("include_Hepta", C.c_int), ("root", C.c_int),
    ("use_diff", C.c_int), ("branchingStrategy", C.c_int),
]

# the reference's compiled-in defaults (PARAM_FIELDS, admm.h:59-81): what a name
# missing from a parameter file keeps
COMPILED_DEFAULTS = dict(sigma0=1.0, scaleSigma=1.001, ADMM_itermax=2000, tol0=5e-2, scaleTol=0.6, minTol=1e-4,
                         triag_iter=5, pent_iter=5, hept_iter=5, max_outer_iter=20, extra_iter=10,
                         violated_TriIneq=1e-3, TriIneq=5000, adjust_TriIneq=1, PentIneq=5000, HeptaIneq=5000,
                         Pent_Trials=60, Hepta_Trials=50, include_Pent=1, include_Hepta=1, root=0, use_diff=1,
                         branchingStrategy=1)

# defaults of the reference's shipped parameter file (params:1-23)
SHIPPED = dict(sigma0=1.0, scaleSigma=1.001, ADMM_itermax=2000, tol0=5e-2, scaleTol=0.6, minTol=1e-3,
               triag_iter=3, pent_iter=3, hept_iter=3, max_outer_iter=12, extra_iter=5,
               violated_TriIneq=1e-3, TriIneq=5000, adjust_TriIneq=1, PentIneq=5000, HeptaIneq=5000,
               Pent_Trials=60, Hepta_Trials=50, include_Pent=1, include_Hepta=1, root=0, use_diff=1,
               branchingStrategy=1)


class Params(C.Structure):
    _fields_ = PARAM_FIELDS


class BabNode(C.Structure):
    _fields_ = [("xfixed", C.c_int * NMAX), ("sol", C.c_int * NMAX), ("fracsol", C.c_double * NMAX),
                ("level", C.c_int), ("upper_bound", C.c_double)]


class NodeStats(C.Structure):
    _fields_ = [("bound", C.c_double), ("basic_bound", C.c_double), ("n_sub", C.c_int),
                ("outer_iters", C.c_int), ("admm_iters", C.c_int), ("ipm_iters", C.c_int),
                ("n_tri", C.c_int), ("n_pent", C.c_int), ("n_hept", C.c_int),
                ("pruned", C.c_int), ("gaveup", C.c_int), ("seconds", C.c_double)]


def params(**over):
    p = Params()
    d = dict(SHIPPED)
    d.update(over)
    for k, v in d.items():
        setattr(p, k, v)
    return p


def node(fixed=None):
    nd = BabNode()
    for i, v in (fixed or {}).items():
        nd.xfixed[i] = 1
        nd.sol[i] = int(v)
    return nd


class MCBError(RuntimeError):
    """A non-zero status of the library; `code` is the MCB_ERR_* value."""

    def __init__(self, msg, code=None):
        super().__init__(msg)
        self.code = code


_lib = None
_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")


def lib():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise MCBError("libmcbound.so is not built (run madam_gb300.build.build())")
    L = C.CDLL(LIB_PATH)
    L.mcb_create.restype = C.c_void_p
    L.mcb_create.argtypes = [C.POINTER(Params), C.c_int, _dp, C.c_int, C.c_int, C.c_void_p, C.POINTER(C.c_int)]
    L.mcb_destroy.argtypes = [C.c_void_p]
    L.mcb_strerror.restype = C.c_char_p
    L.mcb_strerror.argtypes = [C.c_int]
    L.mcb_last_error.restype = C.c_char_p
    L.mcb_last_error.argtypes = [C.c_void_p]
    L.mcb_set_lb.argtypes = [C.c_void_p, C.c_double, C.c_void_p]
    L.mcb_get_lb.restype = C.c_double
    L.mcb_get_lb.argtypes = [C.c_void_p, C.c_void_p]
    L.mcb_set_diff.argtypes = [C.c_void_p, C.c_double]
    L.mcb_get_diff.restype = C.c_double
    L.mcb_get_diff.argtypes = [C.c_void_p]
    L.mcb_set_trials.argtypes = [C.c_void_p, C.c_int, C.c_int]
    L.mcb_get_trials.argtypes = [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int)]
    L.mcb_evaluate.argtypes = [C.c_void_p, C.POINTER(BabNode), C.c_int, C.POINTER(C.c_double), C.POINTER(NodeStats)]
    L.mcb_bound_batch.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p]
    L.mcb_bab.argtypes = [C.c_void_p, C.c_int, C.c_int, C.POINTER(C.c_double), C.c_void_p, C.POINTER(C.c_double),
                          C.POINTER(C.c_int), C.c_void_p, C.c_int, C.POINTER(C.c_int)]
    L.mcb_set_time_limit.argtypes = [C.c_void_p, C.c_double]
    L.mcb_add_problem.argtypes = [C.c_void_p, C.c_int, _dp]
    L.mcb_problem_count.argtypes = [C.c_void_p]
    L.mcb_bound_batch_multi.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p]
    L.mcb_set_problem_lb.argtypes = [C.c_void_p, C.c_int, C.c_double, C.c_void_p]
    L.mcb_get_problem_lb.restype = C.c_double
    L.mcb_get_problem_lb.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
    L.mcb_set_cg_limit.argtypes = [C.c_void_p, C.c_int]
    L.mcb_tc_test_expiry.argtypes = [C.c_int]
    L.mcb_tc_test_expiry.restype = None
    L.mcb_bab_open_bound.restype = C.c_double
    L.mcb_bab_open_bound.argtypes = [C.c_void_p, C.POINTER(C.c_int)]
    L.mcb_op_B.argtypes = [C.c_int, _dp, C.c_int, _ip, C.c_int, _ip, C.c_int, _ip, _dp]
    L.mcb_op_Bt.argtypes = [C.c_int, _dp, C.c_int, _ip, C.c_int, _ip, C.c_int, _ip, _dp]
    L.mcb_project_psd.argtypes = [C.c_int, _dp, C.c_int, _dp, _dp, _dp, _dp, C.POINTER(C.c_int)]
    L.mcb_lambda_max.argtypes = [C.c_int, _dp, C.POINTER(C.c_double), C.POINTER(C.c_double)]
    L.mcb_ipm.argtypes = [C.c_int, _dp, _dp, _dp, _dp, C.POINTER(C.c_double), C.POINTER(C.c_int)]
    L.mcb_separate_triangles.argtypes = [C.c_int, _dp, C.c_int, C.c_double, _ip, _dp, C.POINTER(C.c_int),
                                         C.POINTER(C.c_double)]
    L.mcb_qap_sa_batch.argtypes = [C.c_int, _dp, C.c_int, C.c_int, C.c_uint64, _ip, _dp]
    L.mcb_kernel_stats.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
    L.mcb_reset_kernel_stats.argtypes = [C.c_void_p]
    L.mcb_project_psd_noalloc.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                          C.POINTER(C.c_int), C.c_void_p]
    L.mcb_kernel_work.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]
    L.mcb_transfer_stats.argtypes = [C.c_void_p, C.POINTER(C.c_longlong), C.POINTER(C.c_longlong)]
    L.mcb_measure_fp64_peak.restype = C.c_double
    L.mcb_ns_options.argtypes = [C.c_void_p, C.c_int, C.c_double]
    L.mcb_ns_schedule.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
    L.mcb_mlp_create.restype = C.c_void_p
    L.mcb_mlp_create.argtypes = [C.c_int, C.c_int, C.c_int, C.c_uint64, C.POINTER(C.c_int)]
    L.mcb_mlp_destroy.argtypes = [C.c_void_p]
    L.mcb_mlp_num_params.argtypes = [C.c_void_p]
    L.mcb_mlp_get_params.argtypes = [C.c_void_p, C.c_void_p]
    L.mcb_mlp_set_params.argtypes = [C.c_void_p, C.c_void_p]
    L.mcb_mlp_predict.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p]
    L.mcb_mlp_gradient.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]
    L.mcb_mlp_train.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_float,
                                C.c_uint64, C.c_void_p]
    L.mcb_set_models.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
    L.mcb_log_count.argtypes = [C.c_void_p, C.c_int]
    L.mcb_log_fetch.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p]
    L.mcb_log_clear.argtypes = [C.c_void_p]
    L.mcb_graph_stats.argtypes = [C.c_void_p, C.POINTER(C.c_longlong), C.POINTER(C.c_longlong)]
    L.mcb_host_stats.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]
    L.mcb_set_profile.argtypes = [C.c_void_p, C.c_int]
    L.mcb_library_launch_count.restype = C.c_longlong
    L.mcb_library_launch_count.argtypes = [C.c_void_p]
    L.mcb_ns_schedule_for.argtypes = [C.c_double, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
    L.mcb_split_gemm.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_float, C.c_float, C.c_int,
                                 C.c_int, C.c_void_p]
    L.mcb_autotune_table.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                     C.c_void_p]
    L.mcb_autotune_save.argtypes = [C.c_void_p, C.c_char_p]
    L.mcb_autotune_load.argtypes = [C.c_void_p, C.c_char_p]
    L.mcb_launch_count.restype = C.c_longlong
    L.mcb_launch_count.argtypes = [C.c_void_p]
    _lib = L
    return L


def _check(rc, ctx=None):
    if rc != OK:
        msg = lib().mcb_strerror(rc).decode()
        if ctx is not None:
            extra = lib().mcb_last_error(ctx).decode()
            if extra:
                msg += ": " + extra
        raise MCBError("mcbound error %d (%s)" % (rc, msg), rc)


class Context:
    """A device context for one problem (MADAM's SP and globals)."""

    def __init__(self, prm, SL, N, batch_max=1, flags=PROJ_FP64, stream=None):
        self.N = N
        self.SL = np.ascontiguousarray(np.asarray(SL, dtype=np.float64).reshape(-1))
        st = C.c_int()
        self.h = lib().mcb_create(C.byref(prm), N, self.SL, batch_max, flags, stream, C.byref(st))
        if not self.h:
            _check(st.value)
        self.batch_max = batch_max

    def close(self):
        if getattr(self, "h", None):
            lib().mcb_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_lb(self, lb, sol=None):
        s = None if sol is None else np.ascontiguousarray(sol, dtype=np.int32)
        lib().mcb_set_lb(self.h, lb, None if s is None else s.ctypes.data)
        self._keep = s

    def lb(self):
        s = np.zeros(self.N, dtype=np.int32)
        v = lib().mcb_get_lb(self.h, s.ctypes.data)
        return v, s[: self.N - 1]

    def set_diff(self, d):
        lib().mcb_set_diff(self.h, d)

    def diff(self):
        return lib().mcb_get_diff(self.h)

    def set_trials(self, p, h):
        lib().mcb_set_trials(self.h, p, h)

    def trials(self):
        a, b = C.c_int(), C.c_int()
        lib().mcb_get_trials(self.h, C.byref(a), C.byref(b))
        return a.value, b.value

    def evaluate(self, nd, rank=1):
        b = C.c_double()
        st = NodeStats()
        _check(lib().mcb_evaluate(self.h, C.byref(nd), rank, C.byref(b), C.byref(st)), self.h)
        return b.value, st

    def bound_batch(self, nodes, rank=1):
        arr = (C.POINTER(BabNode) * len(nodes))(*[C.pointer(nd) for nd in nodes])
        b = np.zeros(len(nodes))
        sts = (NodeStats * len(nodes))()
        _check(lib().mcb_bound_batch(self.h, C.cast(arr, C.c_void_p), len(nodes), rank, b.ctypes.data,
                                     C.cast(sts, C.c_void_p)), self.h)
        return b, [sts[i] for i in range(len(nodes))]

    def add_problem(self, SL, N):
        """Another problem (SP->L of order N <= the context's) bounded by this context; its id."""
        SLc = np.ascontiguousarray(np.asarray(SL, dtype=np.float64).reshape(-1))
        rc = lib().mcb_add_problem(self.h, N, SLc)
        if rc < 0:
            _check(rc, self.h)
        self._orders = getattr(self, "_orders", {0: self.N})
        self._orders[rc] = N
        return rc

    def bound_batch_multi(self, nodes, problems, rank=1):
        """Nodes of several problems in one batched pass (node i of problem problems[i])."""
        arr = (C.POINTER(BabNode) * len(nodes))(*[C.pointer(nd) for nd in nodes])
        pr = np.ascontiguousarray(problems, dtype=np.int32)
        b = np.zeros(len(nodes))
        sts = (NodeStats * len(nodes))()
        _check(lib().mcb_bound_batch_multi(self.h, C.cast(arr, C.c_void_p), pr.ctypes.data, len(nodes), rank,
                                           b.ctypes.data, C.cast(sts, C.c_void_p)), self.h)
        return b, [sts[i] for i in range(len(nodes))]

    def problem_lb(self, problem):
        N = getattr(self, "_orders", {0: self.N}).get(problem, self.N)
        s = np.zeros(N, dtype=np.int32)
        v = lib().mcb_get_problem_lb(self.h, problem, s.ctypes.data)
        return v, s[: N - 1]

    def set_problem_lb(self, problem, lb):
        _check(lib().mcb_set_problem_lb(self.h, problem, lb, None), self.h)

    def bab(self, batch=1, max_nodes=0, log_cap=100000):
        opt, rb = C.c_double(), C.c_double()
        nodes, lc = C.c_int(), C.c_int()
        sol = np.zeros(self.N, dtype=np.int32)
        log = (NodeStats * log_cap)()
        rc = lib().mcb_bab(self.h, batch, max_nodes, C.byref(opt), sol.ctypes.data, C.byref(rb), C.byref(nodes),
                           C.cast(log, C.c_void_p), log_cap, C.byref(lc))
        # the node or time limit ends the search early with the incumbent so far, as
        # the reference's time limit does (bab_functions.c:360-369): not an error
        stopped = rc == ERR_CAPACITY and lib().mcb_last_error(self.h) in (b"node limit reached",
                                                                           b"time limit reached")
        if not stopped:
            _check(rc, self.h)
        on = C.c_int()
        ob = lib().mcb_bab_open_bound(self.h, C.byref(on))
        return dict(nodes=nodes.value, opt=opt.value, sol=sol[: self.N - 1].copy(), root_bound=rb.value,
                    log=[log[i] for i in range(lc.value)], stopped=stopped,
                    open_bound=ob if on.value else None, open_nodes=on.value)

    def set_cg_limit(self, max_iters):
        """Iteration cap of the CG solve in every ADMM iteration (default 2000)."""
        _check(lib().mcb_set_cg_limit(self.h, int(max_iters)), self.h)

    def set_time_limit(self, seconds):
        """Wall-time limit of bab() (0: none)."""
        lib().mcb_set_time_limit(self.h, float(seconds))

    def kernel_stats(self):
        cap = 64
        names = (C.c_char * 32 * cap)()
        la = (C.c_longlong * cap)()
        ms = (C.c_double * cap)()
        k = lib().mcb_kernel_stats(self.h, cap, C.cast(names, C.c_void_p), C.cast(la, C.c_void_p),
                                   C.cast(ms, C.c_void_p))
        return {bytes(names[i]).split(b"\0")[0].decode(): (la[i], ms[i]) for i in range(k)}

    def kernel_work(self):
        cap = 64
        w = (C.c_double * cap)()
        u = (C.c_int * cap)()
        k = lib().mcb_kernel_work(self.h, cap, C.cast(w, C.c_void_p), C.cast(u, C.c_void_p))
        names = list(self.kernel_stats().keys())
        return {names[i]: (w[i], u[i]) for i in range(k)}

    def transfer_stats(self):
        a, b = C.c_longlong(), C.c_longlong()
        lib().mcb_transfer_stats(self.h, C.byref(a), C.byref(b))
        return a.value, b.value

    def set_models(self, scorer=None, warm=None):
        """Attach learned models (MLP objects; kept alive by the context)."""
        self._models = (scorer, warm)
        _check(lib().mcb_set_models(self.h, scorer.h if scorer else None, warm.h if warm else None), self.h)

    def log(self, which):
        k = lib().mcb_log_count(self.h, which)
        X = np.zeros((k, CUT_FEATURES), dtype=np.float32)
        y = np.zeros(k, dtype=np.float32)
        if k:
            lib().mcb_log_fetch(self.h, which, k, X.ctypes.data, y.ctypes.data)
        return X, y

    def clear_log(self):
        lib().mcb_log_clear(self.h)

    def ns_options(self, operands=NS_OPERANDS_SPLIT, l0=1e-6):
        _check(lib().mcb_ns_options(self.h, operands, l0), self.h)

    def ns_schedule(self):
        cap = 64
        a, b, acc = (C.c_float * cap)(), (C.c_float * cap)(), (C.c_int * cap)()
        k = lib().mcb_ns_schedule(self.h, cap, C.cast(a, C.c_void_p), C.cast(b, C.c_void_p), C.cast(acc, C.c_void_p))
        return [(a[i], b[i], acc[i]) for i in range(min(k, cap))]

    def autotune_table(self):
        cap = 256
        a, b, v = (C.c_int * cap)(), (C.c_int * cap)(), (C.c_int * cap)()
        u0, u1 = (C.c_float * cap)(), (C.c_float * cap)()
        k = lib().mcb_autotune_table(self.h, cap, *(C.cast(x, C.c_void_p) for x in (a, b, v, u0, u1)))
        return [dict(npad=a[i], bucket=b[i], variant=v[i], us=(u0[i], u1[i])) for i in range(min(k, cap))]

    def autotune_save(self, path):
        _check(lib().mcb_autotune_save(self.h, path.encode()), self.h)

    def autotune_load(self, path):
        _check(lib().mcb_autotune_load(self.h, path.encode()), self.h)

    def reset_kernel_stats(self):
        lib().mcb_reset_kernel_stats(self.h)

    def launch_count(self):
        return lib().mcb_launch_count(self.h)

    def host_stats(self):
        cap = 16
        names = (C.c_char * 32 * cap)()
        sec = (C.c_double * cap)()
        k = lib().mcb_host_stats(self.h, cap, C.cast(names, C.c_void_p), C.cast(sec, C.c_void_p))
        return {bytes(names[i]).split(b"\0")[0].decode(): sec[i] for i in range(k)}

    def graph_stats(self):
        a, b = C.c_longlong(), C.c_longlong()
        lib().mcb_graph_stats(self.h, C.byref(a), C.byref(b))
        return a.value, b.value

    def set_profile(self, on):
        lib().mcb_set_profile(self.h, int(bool(on)))

    def library_launch_count(self):
        return lib().mcb_library_launch_count(self.h)


class MLP:
    """The learned models' network, trained and evaluated by the library's own kernels."""

    def __init__(self, d_in, h1=32, h2=32, seed=0):
        st = C.c_int()
        self.d, self.h1, self.h2 = d_in, h1, h2
        self.h = lib().mcb_mlp_create(d_in, h1, h2, seed, C.byref(st))
        if not self.h:
            _check(st.value)

    def close(self):
        if getattr(self, "h", None):
            lib().mcb_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def num_params(self):
        return lib().mcb_mlp_num_params(self.h)

    def params(self):
        p = np.zeros(self.num_params(), dtype=np.float32)
        _check(lib().mcb_mlp_get_params(self.h, p.ctypes.data))
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        assert p.size == self.num_params()
        _check(lib().mcb_mlp_set_params(self.h, p.ctypes.data))

    def predict(self, X):
        X = np.ascontiguousarray(X, dtype=np.float32)
        out = np.zeros(len(X), dtype=np.float32)
        _check(lib().mcb_mlp_predict(self.h, X.ctypes.data, len(X), out.ctypes.data))
        return out

    def gradient(self, X, Y):
        X = np.ascontiguousarray(X, dtype=np.float32)
        Y = np.ascontiguousarray(Y, dtype=np.float32)
        g = np.zeros(self.num_params(), dtype=np.float32)
        loss = C.c_float()
        _check(lib().mcb_mlp_gradient(self.h, X.ctypes.data, Y.ctypes.data, len(X), g.ctypes.data, C.byref(loss)))
        return float(loss.value), g

    def train(self, X, Y, epochs=50, batch=256, lr=3e-3, seed=0):
        X = np.ascontiguousarray(X, dtype=np.float32)
        Y = np.ascontiguousarray(Y, dtype=np.float32)
        loss = C.c_float()
        _check(lib().mcb_mlp_train(self.h, X.ctypes.data, Y.ctypes.data, len(X), epochs, batch, lr, seed,
                                   C.byref(loss)))
        return float(loss.value)


def tc_test_expiry(on):
    """Switch the tensor-core kernel's wait-expiry test on or off (process-wide)."""
    lib().mcb_tc_test_expiry(1 if on else 0)


def fp64_peak_gflops():
    return lib().mcb_measure_fp64_peak()


# ---- operator-level entry points ---------------------------------------------
def _cuts(tri, pent, hept):
    t = np.ascontiguousarray(np.asarray(tri, dtype=np.int32).reshape(-1)) if len(tri) else np.zeros(4, np.int32)
    p = np.ascontiguousarray(np.asarray(pent, dtype=np.int32).reshape(-1)) if len(pent) else np.zeros(6, np.int32)
    h = np.ascontiguousarray(np.asarray(hept, dtype=np.int32).reshape(-1)) if len(hept) else np.zeros(8, np.int32)
    return t, len(tri), p, len(pent), h, len(hept)


def _fcol(A):
    return np.ascontiguousarray(np.asarray(A, dtype=np.float64).ravel(order="F"))


def op_B(X, tri=(), pent=(), hept=()):
    n = X.shape[0]
    t, nt, p, np_, h, nh = _cuts(tri, pent, hept)
    y = np.zeros(max(nt + np_ + nh, 1))
    _check(lib().mcb_op_B(n, _fcol(X), nt, t, np_, p, nh, h, y))
    return y[: nt + np_ + nh]


def op_Bt(X, tvec, tri=(), pent=(), hept=()):
    n = X.shape[0]
    t, nt, p, np_, h, nh = _cuts(tri, pent, hept)
    Xf = _fcol(X)
    tv = np.zeros(max(nt + np_ + nh, 1))
    tv[: nt + np_ + nh] = tvec
    _check(lib().mcb_op_Bt(n, Xf, nt, t, np_, p, nh, h, tv))
    return Xf.reshape(n, n, order="F")


def project(W, proj=PROJ_FP64):
    n = W.shape[0]
    Xp, Q, Z, ev = np.zeros(n * n), np.zeros(n * n), np.zeros(n * n), np.zeros(n)
    M = C.c_int()
    _check(lib().mcb_project_psd(n, _fcol(W), proj, Xp, Q, Z, ev, C.byref(M)))
    m = M.value
    return (Xp.reshape(n, n, order="F"), Q.reshape(n, n, order="F"), Z[: n * m].reshape(n, m, order="F"),
            ev[:m].copy())


def project_noalloc(n, W_dev, Xp_dev, Q_dev, Z_dev, evals_dev, stream=None):
    """Allocation-free projection on caller-owned device buffers (pointers as ints)."""
    M = C.c_int()
    _check(lib().mcb_project_psd_noalloc(n, C.c_void_p(W_dev), C.c_void_p(Xp_dev), C.c_void_p(Q_dev),
                                         C.c_void_p(Z_dev), C.c_void_p(evals_dev), C.byref(M),
                                         None if stream is None else C.c_void_p(stream)))
    return M.value


def ns_schedule_for(l0=1e-6):
    """The Newton-Schulz step schedule (a, b, closing step) for l0; needs no device."""
    cap = 64
    a, b, acc = (C.c_float * cap)(), (C.c_float * cap)(), (C.c_int * cap)()
    k = lib().mcb_ns_schedule_for(l0, cap, C.cast(a, C.c_void_p), C.cast(b, C.c_void_p), C.cast(acc, C.c_void_p))
    if k < 0:
        _check(k)
    return [(a[i], b[i], acc[i]) for i in range(min(k, cap))]


def split_gemm(A, B, alpha=1.0, diag=0.0, sym=False, variant=0):
    """alpha A[k] B[k]^T + diag I for a batch of square FP32 matrices (tcgen05, split BF16 operands);
    sym: the product is known to be symmetric (lower tiles computed and mirrored)."""
    A = np.ascontiguousarray(A, dtype=np.float32)
    B = np.ascontiguousarray(B, dtype=np.float32)
    if A.ndim == 2:
        A, B = A[None], B[None]
    C = np.zeros_like(A)
    _check(lib().mcb_split_gemm(A.shape[1], A.shape[0], A.ctypes.data, B.ctypes.data, alpha, diag, int(sym),
                                variant, C.ctypes.data))
    return C


def lambda_max(A):
    n = A.shape[0]
    a, b = C.c_double(), C.c_double()
    _check(lib().mcb_lambda_max(n, _fcol(A), C.byref(a), C.byref(b)))
    return a.value, b.value


def ipm(L):
    n = L.shape[0]
    X, y, Z = np.zeros(n * n), np.zeros(n), np.zeros(n * n)
    phi, it = C.c_double(), C.c_int()
    _check(lib().mcb_ipm(n, _fcol(L), X, y, Z, C.byref(phi), C.byref(it)))
    return it.value, phi.value, X.reshape(n, n, order="F"), y, Z.reshape(n, n, order="F")


def sep_triangles(X, K, thr=1e-3):
    n = X.shape[0]
    out = np.zeros(4 * K, dtype=np.int32)
    vals = np.zeros(K)
    cnt, mv = C.c_int(), C.c_double()
    _check(lib().mcb_separate_triangles(n, _fcol(X), K, thr, out, vals, C.byref(cnt), C.byref(mv)))
    return mv.value, out[: 4 * cnt.value].reshape(-1, 4), vals[: cnt.value]


def qap_sa_batch(X, k, trials, key):
    n = X.shape[0]
    nt = 3 if k == 5 else 4
    ineq = np.zeros(trials * nt * k, dtype=np.int32)
    vals = np.zeros(trials * nt)
    _check(lib().mcb_qap_sa_batch(n, _fcol(X), k, trials, C.c_uint64(key), ineq, vals))
    return vals, ineq.reshape(-1, k)
