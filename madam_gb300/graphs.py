"""Graph inputs for the Max-Cut bound: rudy edge lists and seeded generators.

The rudy format is the reference's input (process_input.c:182-225): a header
line ``n m`` followed by ``m`` lines ``i j w`` with 1-based vertices.  The
extended objective matrix built from it (process_input.c:255-299) is

    SP->L = [Lap, Lap e; (Lap e)^T, e^T Lap e]

where Lap = Diag(A e) - A restricted to the first n-1 vertices (the last vertex
is fixed to the 0 side of the cut) and A is the weighted adjacency matrix.

The generators produce rudy-style families with seeded streams: G(n, p) with
unit, +-1 or uniform-integer weights, and 2D toroidal grids (spin glasses).
They follow the families' semantics (density, weight law), not rudy's own
random streams, which are not available.
"""
import numpy as np


def read_rudy(path):
    """Return (n, edges[m,2] 1-based int32, weights[m] float64), reading the file as
    readData does (process_input.c:182-224): fscanf "%d %d" for the header, then
    "%d %d %lf" per edge over one stream of white-space separated numbers.  A
    failed conversion, a vertex count below 1 or a vertex out of range raises
    ValueError; a negative edge count reads no edges; text after the edges is
    ignored."""
    from . import cformat as C

    with open(path, "rb") as f:
        text = f.read().decode("latin-1")
    n, pos = C.scan_int(text, 0)
    m, pos = C.scan_int(text, pos) if n is not None else (None, pos)
    if n is None or m is None:
        raise ValueError("problem reading number of vertices and edges")
    if n <= 0:  # process_input.c:199
        raise ValueError("number of vertices has to be positive")
    e = np.zeros((max(m, 0), 2), dtype=np.int32)
    w = np.zeros(max(m, 0))
    for k in range(max(m, 0)):
        i, pos = C.scan_int(text, pos)
        j, pos = C.scan_int(text, pos) if i is not None else (None, pos)
        x, pos = C.scan_double(text, pos) if j is not None else (None, pos)
        if x is None:
            raise ValueError("problem reading edges of the graph")
        if not (1 <= i <= n and 1 <= j <= n):
            raise ValueError("problem with edge: vertex not in range")
        e[k] = (i, j)
        w[k] = x
    return n, e, w


def write_rudy(path, n, edges, w):
    with open(path, "w") as f:
        f.write("%d %d\n" % (n, len(w)))
        for (i, j), x in zip(edges, w):
            f.write("%d %d %g\n" % (i, j, x))


def extended_laplacian(n, edges, w):
    """SP->L of process_input.c:255-299 as an (n, n) array (symmetric)."""
    A = np.zeros((n, n))
    e = np.asarray(edges, dtype=np.int64).reshape(-1, 2) - 1
    w = np.asarray(w, dtype=np.float64)
    if len(w):
        # readData assigns edge by edge (process_input.c:215-224): a pair listed
        # twice, in either orientation, keeps its last weight on both sides
        lo, hi = np.minimum(e[:, 0], e[:, 1]), np.maximum(e[:, 0], e[:, 1])
        _, last = np.unique((lo * n + hi)[::-1], return_index=True)
        keep = len(w) - 1 - last
        A[lo[keep], hi[keep]] = w[keep]
        A[hi[keep], lo[keep]] = w[keep]
    # every sum in the reference's order (process_input.c:255-299), left to right;
    # np.cumsum accumulates strictly in sequence, unlike np.sum's pairwise tree
    deg = np.cumsum(A, axis=0)[-1]
    m = n - 1
    L = np.zeros((n, n))
    Lap = np.diag(deg[:m]) - A[:m, :m]
    L[:m, :m] = Lap
    if m > 0:
        rs = np.cumsum(Lap, axis=0)[-1]  # column sums of Lap, top to bottom
        L[:m, m] = rs
        L[m, :m] = rs
        L[m, m] = np.cumsum(rs)[-1]
    return L


def gnp(n, p, weights="one", seed=0):
    """Seeded G(n, p); weights: 'one', 'pm1' (uniform {-1,+1}) or 'int10' (uniform integers in [-10, 10],
    zero weights kept as edges)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    iu, ju = np.triu_indices(n, k=1)
    keep = rng.random(iu.size) < p
    i, j = iu[keep] + 1, ju[keep] + 1
    if weights == "one":
        w = np.ones(i.size)
    elif weights == "pm1":
        w = rng.choice(np.array([-1.0, 1.0]), size=i.size)
    elif weights == "int10":
        w = rng.integers(-10, 11, size=i.size).astype(np.float64)
    else:
        raise ValueError(weights)
    return n, np.stack([i, j], axis=1).astype(np.int32), w


def torus2d(rows, cols, seed=0):
    """2D toroidal grid with uniform {-1,+1} couplings (n = rows*cols, degree 4)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    ed = []
    for r in range(rows):
        for c in range(cols):
            v = r * cols + c
            ed.append((v, r * cols + (c + 1) % cols))
            ed.append((v, ((r + 1) % rows) * cols + c))
    ed = np.array(ed, dtype=np.int64)
    lo = np.minimum(ed[:, 0], ed[:, 1]) + 1
    hi = np.maximum(ed[:, 0], ed[:, 1]) + 1
    w = rng.choice(np.array([-1.0, 1.0]), size=len(ed))
    return rows * cols, np.stack([lo, hi], axis=1).astype(np.int32), w


def cut_value(n, edges, w, side):
    """Weight of the cut given a 0/1 side vector over the first n-1 vertices (last vertex on side 0)."""
    s = np.zeros(n, dtype=np.int64)
    s[: n - 1] = side[: n - 1]
    e = np.asarray(edges, dtype=np.int64) - 1
    return float(np.sum(np.asarray(w)[s[e[:, 0]] != s[e[:, 1]]]))


def random_fixings(n, count, max_fixed, seed=0):
    """`count` node fixings over the first n-1 vertices: 0..max_fixed fixed variables each."""
    rng = np.random.Generator(np.random.PCG64(seed))
    out = []
    for _ in range(count):
        k = int(rng.integers(0, max_fixed + 1))
        idx = rng.choice(n - 1, size=k, replace=False) if k else np.zeros(0, dtype=np.int64)
        val = rng.integers(0, 2, size=k)
        out.append({int(i): int(v) for i, v in zip(idx, val)})
    return out
