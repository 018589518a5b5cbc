"""Build recipe for the CPU checkers (test infrastructure).

* ``oracle/_build/libtmr_oracle.so`` — the C restatement (tmr_oracle.c),
  built wherever the repository is built.
* ``oracle/_ref/libtmrref.so`` — the reference's own TMROctant.cpp,
  TMROctForest.cpp, TMRBase.cpp, TMR_STLTools.cpp and the quadtree core
  (TMRQuadrant.cpp, TMRQuadForest.cpp) compiled in place from the reference
  source tree with the single-rank shims in ``oracle/ref_shim``; built only
  when that tree is present (``TMR_REFERENCE_SRC`` or the default path).
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "libtmr_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libtmrref.so")
REF_SRC = os.environ.get("TMR_REFERENCE_SRC", "/root/reference/src")

CFLAGS = ["-O2", "-fPIC", "-shared", "-ffp-contract=off"]


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
    srcs = [os.path.join(REF_SRC, f) for f in
            ("TMROctant.cpp", "TMROctForest.cpp", "TMRBase.cpp", "TMR_STLTools.cpp",
             "TMRQuadrant.cpp", "TMRQuadForest.cpp")]
    if not all(os.path.exists(s) for s in srcs):
        return None
    shim = os.path.join(HERE, "ref_shim")
    deps = srcs + [os.path.join(shim, f) for f in os.listdir(shim)]
    if force or _newer(REF_SO, deps):
        os.makedirs(os.path.dirname(REF_SO), exist_ok=True)
        # math.h is force-included because TMROctForest.cpp calls cos()
        # without including it
        subprocess.run(["g++", *CFLAGS, "-w", "-include", "math.h", "-I", shim,
                        "-I", REF_SRC, *srcs, os.path.join(shim, "ref_capi.cpp"),
                        os.path.join(shim, "ref_quad.cpp"),
                        "-o", REF_SO], check=True)
    return REF_SO


def build(force=False):
    build_oracle(force)
    return build_ref(force)


if __name__ == "__main__":
    print(build_oracle(True), build_ref(True))
