"""Ablation of the learned cut ranking and dual warm start.

Both models are trained on the GPU from the plain solver's logs of seeded
G(90, 0.5) unit-weight instances, then the branch-and-bound runs with and
without them on held-out G(100, 0.5) instances.  The learned form must reach the
same optimum (its bounds are the same safe dual bounds) and, summed over the
instances, evaluate fewer ADMM iterations than the plain form."""
import numpy as np
import pytest

from madam_gb300 import learn as L

pytestmark = pytest.mark.gpu

PRM = dict(include_Pent=0, include_Hepta=0)


@pytest.fixture(scope="module")
def models(gpu_lib):
    inst = [L.instance("gnp", 90, 0.5, "one", seed=s) for s in (31, 32)]
    Xs, ys, Xw, yw = L.collect(inst, proj=gpu_lib.PROJ_FP64, batch=8, max_nodes=120, params=PRM)
    assert len(ys) > 1000 and len(yw) > 1000
    assert np.all(ys >= 0) and np.all(yw >= 0)
    scorer, ls = L.train(Xs, ys, epochs=40, seed=1)
    warm, lw = L.train(Xw, yw, epochs=40, seed=2)
    # better than predicting the mean
    assert ls < 0.9 * ys.var() and lw < 0.9 * yw.var()
    return scorer, warm


def _bab(M, n, SL, models=None):
    flags = M.PROJ_NS_BF16 | (M.FLAG_LEARNED if models else 0)
    ctx = M.Context(M.params(**PRM), SL, n, batch_max=8, flags=flags)
    if models:
        ctx.set_models(*models)
    r = ctx.bab(batch=8, max_nodes=3000)
    ctx.close()
    return r["opt"], sum(s.admm_iters for s in r["log"]), len(r["log"])


def test_learned_form_gains_over_plain(gpu_lib, models):
    tot_plain = tot_learned = 0
    for seed in (42, 43):
        n, SL = L.instance("gnp", 100, 0.5, "one", seed=seed)
        op, ap, _ = _bab(gpu_lib, n, SL)
        ol, al, _ = _bab(gpu_lib, n, SL, models)
        assert ol == op
        tot_plain += ap
        tot_learned += al
    assert tot_learned < tot_plain, (tot_learned, tot_plain)


def test_models_save_and_load(gpu_lib, models, tmp_path):
    p = tmp_path / "m.npz"
    L.save(str(p), *models)
    s2, w2 = L.load(str(p))
    X = np.random.default_rng(0).standard_normal((50, gpu_lib.CUT_FEATURES)).astype(np.float32)
    assert np.array_equal(s2.predict(X), models[0].predict(X))
    assert np.array_equal(w2.predict(X), models[1].predict(X))


def test_shipped_models_load(gpu_lib):
    import os
    from madam_gb300 import train_models as T

    if not os.path.exists(T.OUT):
        pytest.skip("no trained models shipped")
    s, w = L.load(T.OUT)
    assert s.num_params() == w.num_params() > 0
