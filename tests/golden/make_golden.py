"""Generate the golden fixtures of the octree path from the reference itself.

Runs the reference's own TMROctant.cpp/TMROctForest.cpp/TMRBase.cpp,
compiled for one rank by oracle/build.py (oracle/_ref/libtmrref.so), on the
parity cases of tests/pipeline.py and stores every product as compressed
numpy arrays: tests/golden/<case>.npz.  Run it where the reference sources
are present:

    python tests/golden/make_golden.py
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import build as ob  # noqa: E402
from tests import pipeline  # noqa: E402

CASES = ["c1_small", "brick_o2", "brick_o3", "rot_o2", "rot_o3", "rot_o4", "nocorner",
         "uniform_o3"]


def case_meta(case):
    meta = {k: v for k, v in case.items() if k != "conn"}
    return json.dumps(meta, sort_keys=True)


def main():
    if ob.build_ref() is None:
        sys.exit("reference sources not found; set TMR_REFERENCE_SRC")
    allc = pipeline.cases()
    for name in CASES:
        case = allc[name]
        r = pipeline.run_cpu(case, "ref")
        arrs = {
            "meta": np.array(case_meta(case)),
            "block_conn": case["conn"],
            "octants": r["oct"],
            "sizes": np.array([r["sizes"][k] for k in
                               ("num_local", "num_owned", "num_dep", "ext_pre",
                                "num_elements", "dep_nnz")], np.int64),
            "conn": r["conn"],
            "node_numbers": r["nn"],
            "dep_ptr": r["dep"][0], "dep_conn": r["dep"][1], "dep_w": r["dep"][2],
        }
        for k, lv in enumerate(r["levels"]):
            arrs["L%d_octants" % k] = lv["oct"]
            arrs["L%d_conn" % k] = lv["conn"]
            arrs["L%d_P_rowptr" % k] = lv["P"][0]
            arrs["L%d_P_cols" % k] = lv["P"][1]
            arrs["L%d_P_vals" % k] = lv["P"][2]
        out = os.path.join(HERE, name + ".npz")
        np.savez_compressed(out, **arrs)
        print(name, len(r["oct"]), "octants ->", out, os.path.getsize(out), "bytes")


if __name__ == "__main__":
    main()
