"""Train the learned cut scorer and warm-start models from the plain solver's logs.

The training data are the plain method's own branch-and-bound runs (logging on,
cold starts, violation-ranked separation) on seeded instances of the two
smaller benchmark families: G(n, 0.5) with unit weights and triangle cuts, and
G(n, 0.5) with weights in {-1, +1} and triangle + pentagonal cuts.  Both models
are trained on the GPU by the library's kernels and written to
madam_gb300/models/cut_models.npz.

    python -m madam_gb300.train_models [output.npz]
"""
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

from madam_gb300 import learn as L  # noqa: E402
from madam_gb300 import lib as M  # noqa: E402

OUT = os.path.join(HERE, "models", "cut_models.npz")

# (family args, seeds, parameter overrides, node cap per run)
SOURCES = [
    (("gnp", 90, 0.5, "one"), (31, 32, 33), dict(include_Pent=0, include_Hepta=0), 150),
    (("gnp", 80, 0.5, "pm1"), (34, 35), dict(include_Hepta=0), 100),
]


def main(out=OUT, epochs=60):
    import numpy as np

    t0 = time.time()
    parts = []
    for (kind, *args), seeds, over, cap in SOURCES:
        inst = [L.instance(kind, *args, seed=s) for s in seeds]
        parts.append(L.collect(inst, proj=M.PROJ_FP64, batch=8, max_nodes=cap, params=over))
    Xs = np.concatenate([p[0] for p in parts]); ys = np.concatenate([p[1] for p in parts])
    Xw = np.concatenate([p[2] for p in parts]); yw = np.concatenate([p[3] for p in parts])
    scorer, ls = L.train(Xs, ys, epochs=epochs, seed=1)
    warm, lw = L.train(Xw, yw, epochs=epochs, seed=2)
    os.makedirs(os.path.dirname(out), exist_ok=True)
    L.save(out, scorer, warm)
    print("scorer: %d pairs, loss %.5f (target variance %.5f); warm: %d pairs, loss %.5f (variance %.5f); %.1f s"
          % (len(ys), ls, ys.var(), len(yw), lw, yw.var(), time.time() - t0))


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else OUT)
