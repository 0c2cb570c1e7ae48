"""Where the reference's own sources are read from (test infrastructure only).

The environment variable MADAM_REFERENCE names a checkout of HrgaT/MADAM.  Without
it, the default of the recipe that compiles the reference (`DEFAULT_REFDIR` in
oracle/ref/Makefile) is used.  Either way the directory must exist; otherwise
there is no reference here (the GPU machine has none), and the callers skip what
needs it.
"""
import os
import re

MAKEFILE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "ref", "Makefile")


def reference_dir():
    """The reference checkout, or None when it is absent."""
    d = os.environ.get("MADAM_REFERENCE")
    if not d:
        try:
            m = re.search(r"^DEFAULT_REFDIR := (\S+)", open(MAKEFILE).read(), re.M)
            d = m.group(1) if m else None
        except OSError:
            d = None
    return d if d and os.path.isdir(d) else None
