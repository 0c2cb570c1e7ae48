"""Failure paths of the GPU bound, driven without faulting the GPU.

The reference exits the process on a failed factorisation or LAPACK call
(ipm_mc_pk.c:124-134,161-165,218-222; admm.c:749-752).  Here every such
failure is a status code that the host reads after a normal kernel exit, and
the device stays usable for the next call:

- non-finite input (NaN, or values whose sums overflow) ends the IPM with
  MCB_ERR_NUMERIC, through mcb_ipm and through a whole node bound;
- a CG iteration cap that a solve reaches before its tolerance ends the node's
  ADMM with MCB_ERR_ITER; the same context bounds normally once the cap is
  raised again;
- the tensor-core kernel's bounded mbarrier waits: with the expiry test on, the
  kernel issues no TMA loads (nothing is in flight) and its first wait runs out;
  the call reports MCB_ERR_ITER, and the next call, with the test off, gives the
  normal result.
"""
import numpy as np
import pytest

from madam_gb300 import graphs as G

pytestmark = pytest.mark.gpu

ERR_NUMERIC, ERR_ITER = -4, -6


def _problem(n=30, seed=1):
    nv, e, w = G.gnp(n, 0.5, "pm1", seed=seed)
    return nv, G.extended_laplacian(nv, e, w).ravel(order="F")


def test_ipm_reports_non_finite_input(gpu_lib):
    M = gpu_lib
    n, SL = _problem()
    L = SL.reshape(n, n, order="F").copy()
    for bad in (L * 1e308, np.where(np.eye(n, k=1) > 0, np.nan, L)):
        with pytest.raises(M.MCBError) as ex:
            M.ipm(bad)
        assert ex.value.code == ERR_NUMERIC
    # the device is still usable: a finite input solves
    it, phi, X, y, Z = M.ipm(L)
    assert np.isfinite(phi) and it > 0


def test_node_bound_reports_non_finite_problem(gpu_lib):
    M = gpu_lib
    n, SL = _problem()
    bad = SL.copy()
    bad[5 + 3 * n] = bad[3 + 5 * n] = np.nan
    ctx = M.Context(M.params(use_diff=0), bad, n)
    with pytest.raises(M.MCBError) as ex:
        ctx.evaluate(M.node({}), rank=1)
    assert ex.value.code == ERR_NUMERIC
    ctx.close()
    ok = M.Context(M.params(use_diff=0), SL, n)
    b, st = ok.evaluate(M.node({}), rank=1)
    assert np.isfinite(b) and st.admm_iters > 0


@pytest.mark.parametrize("proj", ["fp64", "ns"])
def test_cg_cap_reports_iteration_limit(gpu_lib, proj):
    M = gpu_lib
    n, SL = _problem(40, 3)
    flags = M.PROJ_FP64 if proj == "fp64" else M.PROJ_NS_BF16
    prm = M.params(include_Hepta=0, use_diff=0)
    ref = M.Context(prm, SL, n, flags=flags)
    b_ref, st_ref = ref.evaluate(M.node({}), rank=1)
    ref.close()
    assert st_ref.admm_iters > 0
    ctx = M.Context(prm, SL, n, flags=flags)
    ctx.set_cg_limit(1)
    with pytest.raises(M.MCBError) as ex:
        ctx.evaluate(M.node({}), rank=1)
    assert ex.value.code == ERR_ITER
    ctx.set_cg_limit(2000)
    ctx.set_lb(0.0)
    b, st = ctx.evaluate(M.node({}), rank=1)
    assert abs(b - b_ref) <= 1e-9 * abs(b_ref) and st.admm_iters == st_ref.admm_iters
    with pytest.raises(M.MCBError):
        ctx.set_cg_limit(0)
    ctx.close()


def test_tcgen05_wait_expiry_is_reported_and_recovered(gpu_lib):
    M = gpu_lib
    rng = np.random.default_rng(7)
    A = rng.standard_normal((2, 128, 128)).astype(np.float32)
    B = rng.standard_normal((2, 128, 128)).astype(np.float32)
    ref = np.einsum("bik,bjk->bij", A.astype(np.float64), B.astype(np.float64))
    M.tc_test_expiry(True)
    try:
        for variant in (0, 1):
            with pytest.raises(M.MCBError) as ex:
                M.split_gemm(A, B, variant=variant)
            assert ex.value.code == ERR_ITER
    finally:
        M.tc_test_expiry(False)
    for variant in (0, 1):
        C = M.split_gemm(A, B, variant=variant)
        assert np.abs(C - ref).max() <= 1e-5 * np.abs(ref).max()
    # through a context of the Newton-Schulz form: the bound reports the expiry,
    # and the same context bounds normally afterwards
    n, SL = _problem(40, 4)
    prm = M.params(include_Hepta=0, use_diff=0)
    fresh = M.Context(prm, SL, n, flags=M.PROJ_NS_BF16)
    b_ref, _ = fresh.evaluate(M.node({}), rank=1)
    fresh.close()
    ctx = M.Context(prm, SL, n, flags=M.PROJ_NS_BF16)
    M.tc_test_expiry(True)
    try:
        with pytest.raises(M.MCBError) as ex:
            ctx.evaluate(M.node({}), rank=1)
        assert ex.value.code == ERR_ITER
    finally:
        M.tc_test_expiry(False)
    ctx.set_lb(0.0)
    b, _ = ctx.evaluate(M.node({}), rank=1)
    assert abs(b - b_ref) <= 1e-9 * abs(b_ref)
    ctx.close()
