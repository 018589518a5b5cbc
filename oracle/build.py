"""Build recipe for the CPU checkers (test infrastructure).

* ``oracle/_build/libtmr_oracle.so`` — the C restatement (tmr_oracle.c),
  built wherever the repository is built.
* ``oracle/_ref/libtmrref.so`` — the reference's own TMROctant.cpp,
  TMROctForest.cpp, TMRBase.cpp, TMR_STLTools.cpp and the quadtree core
  (TMRQuadrant.cpp, TMRQuadForest.cpp) compiled in place with the
  single-rank shims in ``oracle/ref_shim``, on whatever machine builds the
  repository (x86-64 or aarch64).

Where the reference's ``src`` directory is found, in this order:

1. ``TMR_REFERENCE_SRC`` (environment), the reference tree's ``src``;
2. ``baseline/_ref/src`` in this repository: a staged copy of just the
   files above and the headers they include, made by
   ``python oracle/build.py --stage <reference>/src``.  The folder is
   git-ignored (no reference source enters the history) but is carried
   with the working tree, so a machine without the reference tree still
   builds the reference checker from it.

With neither, ``build_ref`` returns None and the reference checker is
absent (the tests that need it skip; ``bench.py --impl reference`` falls
back to the C restatement and says so).
"""
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
ORACLE_SO = os.path.join(HERE, "_build", "libtmr_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libtmrref.so")
STAGED_SRC = os.path.join(ROOT, "baseline", "_ref", "src")
REF_SOURCES = ("TMROctant.cpp", "TMROctForest.cpp", "TMRBase.cpp", "TMR_STLTools.cpp",
               "TMRQuadrant.cpp", "TMRQuadForest.cpp")

CFLAGS = ["-O2", "-fPIC", "-shared", "-ffp-contract=off"]


def ref_src():
    """The reference ``src`` directory to compile, or None."""
    env = os.environ.get("TMR_REFERENCE_SRC")
    if env:
        if not all(os.path.exists(os.path.join(env, f)) for f in REF_SOURCES):
            raise FileNotFoundError("TMR_REFERENCE_SRC=%s does not hold %s"
                                    % (env, ", ".join(REF_SOURCES)))
        return env
    if all(os.path.exists(os.path.join(STAGED_SRC, f)) for f in REF_SOURCES):
        return STAGED_SRC
    return None


def stage(src):
    """Copy the reference files the checker compiles (REF_SOURCES and every
    header of the reference's src directory) into baseline/_ref/src."""
    missing = [f for f in REF_SOURCES if not os.path.exists(os.path.join(src, f))]
    if missing:
        raise FileNotFoundError("%s lacks %s" % (src, ", ".join(missing)))
    os.makedirs(STAGED_SRC, exist_ok=True)
    files = [os.path.join(src, f) for f in REF_SOURCES] + sorted(glob.glob(os.path.join(src, "*.h")))
    for f in files:
        shutil.copy2(f, os.path.join(STAGED_SRC, os.path.basename(f)))
    return STAGED_SRC


def _newer(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build_oracle(force=False):
    src = os.path.join(HERE, "tmr_oracle.c")
    hdr = os.path.join(HERE, "tmr_oracle.h")
    if force or _newer(ORACLE_SO, [src, hdr]):
        os.makedirs(os.path.dirname(ORACLE_SO), exist_ok=True)
        subprocess.run(["gcc", *CFLAGS, "-o", ORACLE_SO, src, "-lm"], check=True)
    return ORACLE_SO


def build_ref(force=False):
    """Compile the reference octree core for one rank, if its sources exist."""
    src_dir = ref_src()
    if src_dir is None:
        return None
    srcs = [os.path.join(src_dir, f) for f in REF_SOURCES]
    shim = os.path.join(HERE, "ref_shim")
    deps = srcs + [os.path.join(shim, f) for f in os.listdir(shim)]
    if force or _newer(REF_SO, deps):
        os.makedirs(os.path.dirname(REF_SO), exist_ok=True)
        # math.h is force-included because TMROctForest.cpp calls cos()
        # without including it
        tmp = REF_SO + ".tmp"
        subprocess.run(["g++", *CFLAGS, "-w", "-include", "math.h", "-I", shim,
                        "-I", src_dir, *srcs, os.path.join(shim, "ref_capi.cpp"),
                        os.path.join(shim, "ref_quad.cpp"),
                        "-o", tmp], check=True)
        os.replace(tmp, REF_SO)
    return REF_SO


def build(force=False):
    build_oracle(force)
    return build_ref(force)


if __name__ == "__main__":
    if len(sys.argv) == 3 and sys.argv[1] == "--stage":
        print(stage(sys.argv[2]))
    else:
        print(build_oracle(True), build_ref(True))
