"""TEST INFRASTRUCTURE ONLY: compile the C restatement in ``oracle/spline.c``.

The result is ``oracle/_build/libodtspline.so`` (git-ignored).  Called by
``__graft_entry__.build()`` and lazily by ``oracle.odt_oracle``.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "spline.c")
OUTDIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUTDIR, "libodtspline.so")


def build(force=False, verbose=False):
    """Compile the oracle library if it is missing or older than its source."""
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= os.path.getmtime(SRC)):
        return LIB
    os.makedirs(OUTDIR, exist_ok=True)
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = ["gcc", "-O2", "-fPIC", "-shared", "-fopenmp",
           "-ffp-contract=off", "-std=c99", SRC, "-o", tmp, "-lm"]
    if verbose:
        print(" ".join(cmd), file=sys.stderr)
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
