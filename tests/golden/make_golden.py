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
         "uniform_o3", "mixed_o2", "gap_o2", "gap_o3", "pcoarse_o3", "pcoarse_o4",
         "coarse_o4", "bern_o3", "bern_p3", "bern_o4", "bern_o5", "deep_o2", "deep_o3",
         "deep_l29", "deep_l30"]


def case_meta(case):
    meta = {k: v for k, v in case.items() if k != "conn"}
    return json.dumps(meta, sort_keys=True)


def main(names=None):
    if ob.build_ref() is None:
        sys.exit("reference sources not found; set TMR_REFERENCE_SRC")
    allc = pipeline.cases()
    for name in names or CASES:
        case = allc[name]
        r = pipeline.run_cpu(case, "ref")
        if r.get("octants_only"):
            out = os.path.join(HERE, name + ".npz")
            np.savez_compressed(out, meta=np.array(case_meta(case)), block_conn=case["conn"],
                                octants=r["oct"])
            print(name, len(r["oct"]), "octants ->", out, os.path.getsize(out), "bytes")
            continue
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


def make_digest_golden():
    """tests/golden/digest_<case>.npz: checksums, samples and moments of the
    reference's products on the configuration-size cases (pipeline.py
    digest_cases), which are too large to store whole."""
    for name, case in pipeline.digest_cases().items():
        r = pipeline.run_cpu(case, "ref")
        d = pipeline.digest(r)
        d["meta"] = np.array(case_meta(case))
        d["block_conn"] = case["conn"]
        out = os.path.join(HERE, "digest_" + name + ".npz")
        np.savez_compressed(out, **d)
        print("digest", name, len(r["oct"]), "octants ->", os.path.getsize(out), "bytes")


def make_api_golden():
    """tests/golden/api.npz: evalInterp tables, block connectivity getters,
    findEnclosing and transformNode results of the reference."""
    import ctypes
    from oracle.oracle import RefForest, _lib
    from tmr_gb300 import workloads as W
    L = _lib("ref").lib
    vp = ctypes.c_void_p
    L.tmrref_forest_create.restype = vp
    P = lambda a: a.ctypes.data_as(vp)
    arrs = {}
    # evalInterp: orders 2-4, uniform / GLL / Bernstein, five points
    pts = np.array([[0.0, 0.0, 0.0], [0.3, -0.7, 0.9], [-1.0, 1.0, 0.25],
                    [0.123456789, 0.5, -0.333], [0.99, -0.01, 0.6]])
    for order in (2, 3, 4):
        for it in (0, 1, 2):
            f = L.tmrref_forest_create(order, it)
            kn = np.zeros(16)
            L.tmrref_get_knots(vp(f), P(kn))
            arrs["ev_o%d_t%d_knots" % (order, it)] = kn[:order]
            n = order ** 3
            for ip_, pt in enumerate(pts):
                pt = np.ascontiguousarray(pt)
                N = np.zeros(n)
                L.tmrref_eval_interp(vp(f), P(pt), P(N), None, None, None)
                d1 = [np.zeros(n) for _ in range(4)]
                L.tmrref_eval_interp(vp(f), P(pt), *[P(a) for a in d1])
                d2 = [np.zeros(n) for _ in range(10)] + [np.full(n, -7.0)]
                L.tmrref_eval_interp2(vp(f), P(pt), *[P(a) for a in d2])
                key = "ev_o%d_t%d_p%d" % (order, it, ip_)
                arrs[key + "_N"] = N
                arrs[key + "_d1"] = np.stack(d1)
                arrs[key + "_d2"] = np.stack(d2)
            L.tmrref_forest_destroy(vp(f))
    arrs["ev_points"] = pts
    # connectivity of randomly rotated blocks
    conn = W.rotate_blocks(W.brick(3, 2, 2), 2)
    ref = RefForest(2, 1)
    ref.setConnectivity(conn)
    sizes = np.zeros(4, np.int32)
    L.tmrref_get_connectivity(vp(ref.h), P(sizes), None, None, None, None)
    nb, nf, ne, nn = (int(v) for v in sizes)
    bc, bf, be, fi = (np.zeros(nb * w, np.int32) for w in (8, 6, 12, 6))
    L.tmrref_get_connectivity(vp(ref.h), P(sizes), P(bc), P(bf), P(be), P(fi))
    ncn, ncp = np.zeros(8 * nb, np.int32), np.zeros(nn + 1, np.int32)
    ecn, ecp = np.zeros(12 * nb, np.int32), np.zeros(ne + 1, np.int32)
    fcn, fcp = np.zeros(6 * nb, np.int32), np.zeros(nf + 1, np.int32)
    L.tmrref_get_inverse_connectivity(vp(ref.h), P(ncn), P(ncp), P(ecn), P(ecp), P(fcn), P(fcp))
    arrs.update({"cn_block_conn_in": conn, "cn_sizes": sizes, "cn_block_conn": bc,
                 "cn_block_face": bf, "cn_block_edge": be, "cn_face_ids": fi,
                 "cn_node_conn": ncn, "cn_node_ptr": ncp, "cn_edge_conn": ecn,
                 "cn_edge_ptr": ecp, "cn_face_conn": fcn, "cn_face_ptr": fcp})
    # transformNode on nodes at block corners, edges, faces and interiors
    rng = np.random.default_rng(3)
    hmax = 1 << 30
    m = 3000
    nodes = np.zeros((m, 7), np.int32)
    nodes[:, 0] = rng.integers(0, nb, m)
    for c in (1, 2, 3):
        pick = rng.integers(0, 3, m)
        val = rng.integers(0, 1 << 10, m) << 20
        nodes[:, c] = np.where(pick == 0, 0, np.where(pick == 1, hmax, val))
    for ed in (-1, 0, 1, 2):
        out = nodes.copy()
        rev, fid = np.zeros(m, np.int32), np.zeros(m, np.int32)
        L.tmrref_transform_nodes(vp(ref.h), m, P(out), ed, P(rev), P(fid))
        arrs["tn_out_e%d" % (ed + 1)] = out
        arrs["tn_rev_e%d" % (ed + 1)] = rev
        arrs["tn_fid_e%d" % (ed + 1)] = fid
    arrs["tn_nodes"] = nodes
    # findEnclosing: every local node of a small refined order-3 forest
    # searched in its coarsened forest
    case = dict(pipeline.cases()["rot_o3"])
    case["passes"] = 2
    fine = RefForest(3, 1)
    fine.setConnectivity(case["conn"])
    fine.createTrees(case["L0"])
    for p in range(case["passes"]):
        o = fine.getOctants()
        fine.refine(pipeline.indicator(o, case, p), 0, case["max_level"])
        fine.balance(1)
    coarse = fine.coarsen()
    coarse.balance(1)
    fo = fine.getOctants()
    q = np.repeat(fo, 27, axis=0)
    q[:, 6] = np.tile(np.arange(27), len(fo))
    idx = np.zeros(len(q), np.int64)
    L.tmrref_find_enclosing(vp(coarse.h), 3, P(_ref_knots(fine)), len(q),
                            P(np.ascontiguousarray(q)), P(idx))
    arrs.update({"fe_conn": case["conn"], "fe_case": np.array(json.dumps(
        {k: v for k, v in case.items() if k != "conn"}, sort_keys=True)),
        "fe_nodes": q, "fe_index": idx, "fe_coarse_octants": coarse.getOctants()})
    # design -> analysis weights: analysis forest = a refined forest, filter
    # forest = its coarsened forest (orders 2 and 3)
    L.tmrref_topo_weights.restype = ctypes.c_long
    for name in ("brick_o2", "rot_o3", "bern_o3", "coarse_o4"):
        case = dict(pipeline.cases()[name])
        case["passes"] = 2
        ana = RefForest(case["order"], case.get("interp", 1))
        ana.setConnectivity(case["conn"])
        ana.createTrees(case["L0"])
        for p in range(case["passes"]):
            o = ana.getOctants()
            ana.refine(pipeline.indicator(o, case, p), 0, case["max_level"])
            ana.balance(1)
        filt = ana.coarsen()
        filt.balance(1)
        filt.createNodes()
        n = len(ana.getOctants())
        rp = np.zeros(n + 1, np.int32)
        nnz = L.tmrref_topo_weights(vp(filt.h), vp(ana.h), P(rp), None, None)
        cols, w = np.zeros(max(nnz, 1), np.int32), np.zeros(max(nnz, 1))
        L.tmrref_topo_weights(vp(filt.h), vp(ana.h), P(rp), P(cols), P(w))
        arrs.update({"tw_%s_case" % name: np.array(json.dumps(
            {k: v for k, v in case.items() if k != "conn"}, sort_keys=True)),
            "tw_%s_conn" % name: case["conn"], "tw_%s_rowptr" % name: rp,
            "tw_%s_cols" % name: cols[:nnz], "tw_%s_w" % name: w[:nnz]})
    out = os.path.join(HERE, "api.npz")
    np.savez_compressed(out, **arrs)
    print("api ->", out, os.path.getsize(out), "bytes")


def _ref_knots(f):
    import ctypes
    from oracle.oracle import _lib
    k = np.zeros(16)
    _lib("ref").lib.tmrref_get_knots(ctypes.c_void_p(f.h), k.ctypes.data_as(ctypes.c_void_p))
    return k


def make_stl_golden():
    """tests/golden/api_stl.npz: the reference's own TMR_GenerateSTLTriangles
    output (oracle/_ref) on parity forests with block boxes and a seeded
    field (tests/pipeline.py STL_CASES)."""
    from oracle.oracle import RefForest
    arrs = {}
    for name, sc in pipeline.STL_CASES.items():
        case = pipeline.cases()[name]
        o = case["order"]
        f = RefForest(o, case.get("interp", 1))
        f.setConnectivity(case["conn"])
        f.createTrees(case["L0"])
        for p in range(case["passes"]):
            oc = f.getOctants()
            f.refine(pipeline.indicator(oc, case, p), 0, case["max_level"])
            f.balance(case.get("corner", 1))
        f.createNodes()
        s = f.nodeSizes()
        knots = [-1.0, 1.0] if o == 2 else ([-1.0, -np.cos(np.pi / 2), 1.0]
                                            if case.get("interp", 1) == 1 else [-1.0, 0.0, 1.0])
        boxes = pipeline.brick_boxes(*sc["grid"])
        X = pipeline.node_points(f.getOctants(), f.getMeshConn(o), s["num_dep"], s["num_local"],
                                 o, knots, boxes)
        x = pipeline.stl_field(X[s["num_dep"]:], sc["vpn"])
        tris = f.stlTriangles(X, x, sc["vpn"], sc["offset"], sc["cutoff"])
        arrs[name + "_tris"] = tris
        arrs[name + "_octants"] = f.getOctants()
        print(name, len(tris), "reference triangles")
    out = os.path.join(HERE, "api_stl.npz")
    np.savez_compressed(out, **arrs)
    print("->", out, os.path.getsize(out), "bytes")


def make_quad_golden():
    """tests/golden/quad_<case>.npz: the reference's own TMRQuadForest
    (oracle/_ref) on the quadtree parity cases (tests/pipeline.py
    quad_cases)."""
    for name, case in pipeline.quad_cases().items():
        r = pipeline.run_quad_ref(case)
        arrs = {"meta": np.array(case_meta(case)), "face_conn": case["conn"],
                "quads": r["quads"], "conn": r["conn"], "dep_ptr": r["dep"][0],
                "dep_conn": r["dep"][1], "dep_w": r["dep"][2]}
        for k, lv in enumerate(r["levels"]):
            arrs["L%d_quads" % k] = lv["quads"]
            arrs["L%d_conn" % k] = lv["conn"]
            arrs["L%d_dep_ptr" % k], arrs["L%d_dep_conn" % k], arrs["L%d_dep_w" % k] = lv["dep"]
            arrs["L%d_P_rowptr" % k], arrs["L%d_P_cols" % k], arrs["L%d_P_vals" % k] = lv["P"]
        out = os.path.join(HERE, "quad_" + name + ".npz")
        np.savez_compressed(out, **arrs)
        print("quad", name, len(r["quads"]), "quadrants ->", os.path.getsize(out), "bytes")


if __name__ == "__main__":
    if len(sys.argv) > 1:  # only the named octree cases (or "digest")
        if sys.argv[1:] == ["digest"]:
            make_digest_golden()
        else:
            main(sys.argv[1:])
        sys.exit(0)
    main()
    make_digest_golden()
    make_api_golden()
    make_stl_golden()
    make_quad_golden()
