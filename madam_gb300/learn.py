"""Learned cut ranking and dual warm start: data collection, training, storage.

Training data comes from the plain solver's own runs: `collect` runs the
branch-and-bound with logging on (MCB_FLAG_LOG, cold starts, violation-ranked
separation) and returns two sets of (features, log(1 + dual)) pairs:
  * cut scorer: a separated triangle's features at separation time -> its dual
    after the next ADMM call (cutting_planes.c:132-214 purges cuts whose dual is
    below 1e-5, so the dual measures whether the cut was worth adding);
  * warm start: a parent's final cut (features at the parent's final X, with
    its dual) -> the same cut's dual at the end of the child's bound (0 when the
    child's own cutting-plane loop does not end with it).
`train` fits one MLP per set with the library's own GPU kernels
(madam_gb300/csrc/mlp.cu); `save` / `load` keep the parameters in an .npz.
"""
import numpy as np

from . import graphs as G
from . import lib as M

HIDDEN = (32, 32)


def instance(kind, *args, seed):
    if kind == "gnp":
        n, e, w = G.gnp(*args, seed=seed)
    else:
        n, e, w = G.torus2d(*args, seed=seed)
    return n, G.extended_laplacian(n, e, w).ravel(order="F")


def collect(instances, proj=M.PROJ_FP64, batch=8, max_nodes=400, params=None):
    """Run the plain method with logging on each (n, SL); return (Xs, ys, Xw, yw)."""
    xs, ys, xw, yw = [], [], [], []
    for n, SL in instances:
        ctx = M.Context(M.params(**(params or {})), SL, n, batch_max=batch, flags=proj | M.FLAG_LOG)
        try:
            ctx.bab(batch=batch, max_nodes=max_nodes)
        except M.MCBError:
            pass  # a failed run keeps what was logged (a node limit returns normally)
        a, b = ctx.log(M.LOG_SCORER)
        c, d = ctx.log(M.LOG_WARM)
        xs.append(a); ys.append(b); xw.append(c); yw.append(d)
        ctx.close()
    return np.concatenate(xs), np.concatenate(ys), np.concatenate(xw), np.concatenate(yw)


def train(X, y, epochs=60, batch=256, lr=3e-3, seed=0):
    net = M.MLP(M.CUT_FEATURES, *HIDDEN, seed=seed)
    loss = net.train(X, y, epochs=epochs, batch=batch, lr=lr, seed=seed)
    return net, loss


def save(path, scorer, warm):
    np.savez(path, scorer=scorer.params(), warm=warm.params(), hidden=np.array(HIDDEN),
             features=np.array(M.CUT_FEATURES))


def load(path):
    z = np.load(path)
    h1, h2 = (int(v) for v in z["hidden"])
    nets = []
    for key in ("scorer", "warm"):
        net = M.MLP(int(z["features"]), h1, h2)
        net.set_params(z[key])
        nets.append(net)
    return nets
