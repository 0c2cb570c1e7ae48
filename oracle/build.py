"""Build recipe for the CPU oracle (test infrastructure only).

``build_oracle()`` compiles the C restatement in this folder into
``oracle/libmcb_oracle.so`` with gcc.  ``find_lapack()`` locates an LP64
BLAS/LAPACK shared library (the OpenBLAS copy shipped inside SciPy or NumPy)
that the oracle dlopens at run time.
"""
import glob
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "libmcb_oracle.so")
SOURCES = ["orc_core.c", "orc_cuts.c", "orc_bab.c", "orc_gram.c"]


def find_lapack():
    """Return the path of an LP64 LAPACK library (SciPy's OpenBLAS)."""
    cands = []
    try:
        import scipy  # noqa: F401

        base = os.path.dirname(os.path.dirname(scipy.__file__))
        cands += sorted(glob.glob(os.path.join(base, "scipy.libs", "libscipy_openblas*.so*")))
    except ImportError:
        pass
    try:
        import numpy

        base = os.path.dirname(os.path.dirname(numpy.__file__))
        cands += sorted(glob.glob(os.path.join(base, "numpy.libs", "libscipy_openblas*.so*")))
    except ImportError:
        pass
    # LP64 builds only: the ILP64 copy NumPy ships uses the "64_" symbol suffix and 64-bit ints
    cands = [c for c in cands if "openblas64" not in os.path.basename(c)]
    for extra in ("/usr/lib/x86_64-linux-gnu/liblapack.so.3", "/usr/lib/aarch64-linux-gnu/liblapack.so.3"):
        if os.path.exists(extra):
            cands.append(extra)
    if not cands:
        raise RuntimeError("no LP64 LAPACK library found for the oracle")
    return cands[0]


def build_oracle(force=False, quiet=True):
    srcs = [os.path.join(HERE, s) for s in SOURCES]
    hdrs = glob.glob(os.path.join(HERE, "*.h"))
    if not force and os.path.exists(ORACLE_SO):
        t = os.path.getmtime(ORACLE_SO)
        if all(os.path.getmtime(s) < t for s in srcs + hdrs):
            return ORACLE_SO
    # -ffp-contract=off keeps a*b+c unfused on every host, so x86 and Arm agree bit for bit
    cmd = ["gcc", "-O2", "-std=gnu11", "-fPIC", "-shared", "-ffp-contract=off", "-Wall",
           "-Wno-unused-function", "-o", ORACLE_SO] + srcs + ["-ldl", "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        sys.stderr.write(r.stdout + r.stderr)
        raise RuntimeError("oracle build failed")
    if not quiet and r.stderr:
        sys.stderr.write(r.stderr)
    return ORACLE_SO


if __name__ == "__main__":
    print(build_oracle(force=True, quiet=False))
    print(find_lapack())
