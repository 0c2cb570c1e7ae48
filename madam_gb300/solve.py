"""Command-line branch-and-bound in the reference's formats.

Reads a rudy-format instance and a parameter file the way process_input.c does
(readParameters, process_input.c:141-178, with its line semantics restated in
read_params; readData, :182-312) and writes the report of bab_functions.c
(printFinalOutput / printSolution, :337-373), so a run can be diffed against the
reference's .output files.  The branch-and-bound is the library's batched driver
(mcb_bab) on the GPU.

    python -m madam_gb300.solve INSTANCE PARAMS [--form learned|mixed|fp64] [--batch 64] [--max-nodes K] [--out FILE]
"""
import argparse
import os
import re
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
if os.path.dirname(HERE) not in sys.path:
    sys.path.insert(0, os.path.dirname(HERE))

from madam_gb300 import cformat as C  # noqa: E402
from madam_gb300 import graphs as G  # noqa: E402
from madam_gb300 import lib as M  # noqa: E402

# value formats of the reference's PARAM_FIELDS (admm.h), in its order
_FLOAT = {"sigma0", "scaleSigma", "tol0", "scaleTol", "minTol", "violated_TriIneq"}
PARAM_ORDER = [name for name, _ in M.PARAM_FIELDS]


_NAME = re.compile(r"[^=^ ]+")


def _pieces(text):
    """What fgets(s, 120, f) returns, one call at a time: at most 119 characters,
    ending after a newline; C sees each up to its first NUL."""
    for line in re.findall(r"[^\n]*\n|[^\n]+$", text):
        for k in range(0, len(line), 119):
            yield line[k:k + 119].split("\0")[0]


def read_params(path):
    """Parameter file -> dict over every field, as readParameters reads it
    (process_input.c:141-178).  Names missing from the file keep the compiled-in
    defaults (admm.h:59-81).  Per fgets piece: the name is the longest prefix of
    characters other than '=', '^' and ' '; a piece that starts with one of those
    keeps the previous piece's name.  If that name is a parameter, the value is the
    number (C's %d or %lf) after the first '=', which needs at least one character
    before it; a piece without one changes nothing."""
    vals = dict(M.COMPILED_DEFAULTS)
    with open(path, "rb") as f:
        text = f.read().decode("latin-1")
    name = None
    for piece in _pieces(text):
        m = _NAME.match(piece)
        if m:
            name = m.group(0)
        if name not in vals:
            continue
        eq = piece.find("=")
        if eq < 1:
            continue
        v, _ = (C.scan_double if name in _FLOAT else C.scan_int)(piece, eq + 1)
        if v is not None:
            vals[name] = v
    return vals


def format_params(vals):
    lines = ["Parameters:"]
    for name in PARAM_ORDER:
        v = vals[name]
        lines.append("%20s = %s" % (name, ("%f" % v) if name in _FLOAT else ("%d" % v)))
    return "\n".join(lines)


def report(instance, n, n_edges, vals, result, seconds):
    """The reference's output file text for one run (printFinalOutput,
    bab_functions.c:353-373; a run stopped by its node limit is reported as the
    reference reports one stopped by its time limit)."""
    sol = " ".join(str(i + 1) for i, x in enumerate(result["sol"]) if x == 1)
    shown = dict(vals)
    if shown["adjust_TriIneq"]:  # the block is printed after the adjustment (process_input.c:119-132)
        shown["TriIneq"] = n * 10
    return "".join([
        "Input file: %s\n" % instance,
        "\nGraph has %d vertices and %d edges.\n" % (n, n_edges),
        format_params(shown) + "\n",
        "\nNodes = %d\n" % result["nodes"],
        "TIME LIMIT REACHED.\n" if result.get("stopped") else "",
        "Root node bound = %.2f\n" % result["root_bound"],
        ("Best value = %.0f\n" if result.get("stopped") else "Maximum value = %.0f\n") % result["opt"],
        "Solution = ( %s%s)\n" % (sol, " " if sol else ""),
        "Time = %.2f s\n\n" % seconds,
    ])


def solve(instance, params_path, form="mixed", batch=64, max_nodes=0):
    n, e, w = G.read_rudy(instance)
    vals = read_params(params_path)
    SL = G.extended_laplacian(n, e, w).ravel(order="F")
    flags = M.PROJ_FP64 if form == "fp64" else M.PROJ_NS_BF16
    if form == "learned":
        flags |= M.FLAG_LEARNED
    ctx = M.Context(M.params(**vals), SL, n, batch_max=batch, flags=flags)
    if form == "learned":
        from madam_gb300 import learn as L
        from madam_gb300 import train_models as T

        ctx.set_models(*L.load(T.OUT))
    t0 = time.perf_counter()
    r = ctx.bab(batch=batch, max_nodes=max_nodes)
    secs = time.perf_counter() - t0
    ctx.close()
    return report(instance, n, len(w), vals, r, secs), r


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("instance")
    ap.add_argument("params")
    ap.add_argument("--form", default="mixed", choices=["learned", "mixed", "fp64"])
    ap.add_argument("--batch", type=int, default=64)
    ap.add_argument("--max-nodes", type=int, default=0, help="stop after this many node bounds (0: none)")
    ap.add_argument("--out", default=None, help="report file (default: INSTANCE.output, never overwritten)")
    a = ap.parse_args(argv)
    text, _ = solve(a.instance, a.params, a.form, a.batch, a.max_nodes)
    sys.stdout.write(text)
    with open(a.out or output_path(a.instance), "w") as f:
        f.write(text)


def output_path(instance):
    """INSTANCE.output, or INSTANCE.output_1, _2, ... if taken (process_input.c:52-60)."""
    path, k = instance + ".output", 1
    while os.path.exists(path):
        path, k = "%s.output_%d" % (instance, k), k + 1
    return path


if __name__ == "__main__":
    main()
