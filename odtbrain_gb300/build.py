"""Build the in-tree CUDA library ``odtbrain_gb300/_lib/libodtbrain_gb300.so``.

nvcc compiles the sources in ``odtbrain_gb300/csrc`` for sm_103a only
(``-gencode arch=compute_103a,code=sm_103a``), one process per translation
unit, then links them into a shared library with a plain C ABI
(``include/odtbrain_gb300.h``).  No PyTorch headers are involved.
"""
import concurrent.futures
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "_lib")
OBJDIR = os.path.join(LIBDIR, "obj")
LIBNAME = "libodtbrain_gb300.so"
LIB = os.path.join(LIBDIR, LIBNAME)
SOURCES = ["capi.cu", "stages.cu", "rotate.cu", "adjoint.cu", "mlp.cu", "translate.cu",
           "unwrap.cu", "apple.cu"]
HEADERS = ["odt_fft.cuh", "odt_internal.cuh", "odt_stage_util.cuh"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
           "--expt-relaxed-constexpr"]


def _nvcc():
    cand = shutil.which("nvcc")
    if cand:
        return cand
    for root in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if root and os.path.exists(os.path.join(root, "bin", "nvcc")):
            return os.path.join(root, "bin", "nvcc")
    raise RuntimeError("nvcc not found: cannot build the odtbrain_gb300 CUDA "
                       "library")


def _inputs():
    files = [os.path.join(CSRC, s) for s in SOURCES + HEADERS]
    files.append(os.path.join(HERE, os.pardir, "include", "odtbrain_gb300.h"))
    files.append(os.path.abspath(__file__))
    return files


def is_stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    return any(os.path.getmtime(f) > t for f in _inputs())


def build(force=False, verbose=False, extra_flags=()):
    """Compile and link the library if it is missing or stale; returns its
    path."""
    if not force and not is_stale():
        return LIB
    nvcc = _nvcc()
    os.makedirs(OBJDIR, exist_ok=True)

    def compile_one(src):
        obj = os.path.join(OBJDIR, src.replace(".cu", ".o"))
        cmd = [nvcc, *ARCH, *NVFLAGS, *extra_flags, "-c",
               os.path.join(CSRC, src), "-o", obj]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s" % (src, res.stderr))
        return obj

    with concurrent.futures.ThreadPoolExecutor(len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = [nvcc, *ARCH, "-shared", "-o", tmp, *objs]
    if verbose:
        print(" ".join(cmd), file=sys.stderr)
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("nvcc link failed:\n%s" % res.stderr)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
