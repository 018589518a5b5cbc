"""Build recipe for the native library (libtmrg.so, sm_103a).

Each CUDA translation unit is compiled in parallel with nvcc for
``compute_103a``/``sm_103a`` and linked into ``tmr_gb300/_build/libtmrg.so``.
Floating-point contraction is disabled (``--fmad=false``) so that every
FP64 expression rounds in source order, like the reference's x86-64 build.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libtmrg.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

SOURCES = [
    "tmrg_conn.cu",
    "tmrg_forest.cu",
    "tmrg_nodes.cu",
    "tmrg_interp.cu",
    "tmrg_filter.cu",
    "tmrg_helmholtz.cu",
    "tmrg_stl.cu",
    "tmrg_quad.cu",
    "tmrg_capi.cu",
    "tmrg_tune.cu",
]

NVCC_FLAGS = [
    "-gencode", "arch=compute_103a,code=sm_103a",
    "-O3", "-lineinfo", "-std=c++17", "--fmad=false",
    "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
    "--expt-relaxed-constexpr", "--extended-lambda",
]


def nvcc():
    cand = os.environ.get("NVCC") or "/usr/local/cuda/bin/nvcc"
    return cand if os.path.exists(cand) else "nvcc"


def _compile(src, verbose=False):
    obj = os.path.join(OUT, os.path.basename(src).replace(".cu", ".o"))
    cmd = [nvcc(), *NVCC_FLAGS, "-I", INCLUDE, "-c", os.path.join(SRC, src), "-o", obj]
    if verbose:
        cmd += ["-Xptxas", "-v"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s%s" % (src, r.stdout, r.stderr))
    return obj, r.stderr


def _stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(SRC, f) for f in os.listdir(SRC)] + [os.path.join(INCLUDE, "tmrg.h")]
    return any(os.path.getmtime(d) > t for d in deps)


def build(force=False, verbose=False):
    """Compile the library if any source is newer than it; returns its path."""
    if not force and not _stale():
        return LIB
    os.makedirs(OUT, exist_ok=True)
    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        results = list(ex.map(lambda s: _compile(s, verbose), SOURCES))
    objs = [o for o, _ in results]
    if verbose:
        for _, log in results:
            sys.stderr.write(log)
    tmp = LIB + ".tmp"
    cmd = [nvcc(), "-shared", "-gencode", "arch=compute_103a,code=sm_103a",
           "-Xcompiler", "-fPIC", *objs, "-o", tmp, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s%s" % (r.stdout, r.stderr))
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
