"""The rest of TMROctForest's public surface on the GPU library, against
the reference's own results (tests/golden/api.npz, from the reference build)
or restatements in this file: getConnectivity / getInverseConnectivity,
setFullConnectivity, createRandomTrees, findEnclosing, transformNode,
getLocalNodeNumber, getPoints, evalInterp through a forest."""
import json
import os

import numpy as np
import pytest

from tests import pipeline
from tmr_gb300 import workloads as W

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


def _golden():
    return np.load(os.path.join(HERE, "golden", "api.npz"))


def test_connectivity_getters_match_reference(gpu_lib):
    from tmr_gb300 import TMR
    z = _golden()
    f = TMR.OctForest(order=2)
    f.setConnectivity(z["cn_block_conn_in"])
    bc, bf, be, fi, nn, ne, nf = f.getConnectivity()
    nb = bc.shape[0]
    assert [nb, nf, ne, nn] == list(z["cn_sizes"])
    np.testing.assert_array_equal(bc.ravel(), z["cn_block_conn"])
    np.testing.assert_array_equal(bf.ravel(), z["cn_block_face"])
    np.testing.assert_array_equal(be.ravel(), z["cn_block_edge"])
    np.testing.assert_array_equal(fi.ravel(), z["cn_face_ids"])
    inv = f.getInverseConnectivity()
    np.testing.assert_array_equal(inv["node"][0], z["cn_node_ptr"])
    np.testing.assert_array_equal(inv["node"][1], z["cn_node_conn"])
    np.testing.assert_array_equal(inv["edge"][0], z["cn_edge_ptr"])
    np.testing.assert_array_equal(inv["edge"][1], z["cn_edge_conn"])
    np.testing.assert_array_equal(inv["face"][0], z["cn_face_ptr"])
    np.testing.assert_array_equal(inv["face"][1], z["cn_face_conn"])


def test_full_connectivity_gives_the_same_forest(gpu_lib):
    from tmr_gb300 import TMR
    z = _golden()
    conn = z["cn_block_conn_in"]
    nb = conn.shape[0]
    ref = pipeline.run_gpu(dict(conn=conn, order=3, L0=1, passes=2, max_level=4, prob=0.4,
                                seed=9, coarse_levels=1))
    f = TMR.OctForest(order=3)
    f.setFullConnectivity(conn, z["cn_block_edge"].reshape(nb, 12),
                          z["cn_block_face"].reshape(nb, 6))
    bc, bf, be, fi, nn, ne, nf = f.getConnectivity()
    np.testing.assert_array_equal(fi.ravel(), z["cn_face_ids"])
    f.createTrees(1)
    case = dict(conn=conn, order=3, L0=1, passes=2, max_level=4, prob=0.4, seed=9)
    for p in range(2):
        o = f.getOctantsArray()
        f.refine(pipeline.indicator(o, case, p), 0, 4)
        f.balance(1)
    f.createNodes()
    np.testing.assert_array_equal(f.getOctantsArray(), ref["oct"])
    np.testing.assert_array_equal(f.getMeshConn(), ref["conn"])
    with pytest.raises(TMR._lib.TMRGError):
        bad = z["cn_block_edge"].reshape(nb, 12).copy()
        bad[0, 0] = ne + 5
        f.setFullConnectivity(conn, bad, z["cn_block_face"].reshape(nb, 6), num_edges=ne)


def _morton_key(o):
    """Sort key of TMROctant::compare: block, then the x-most-significant
    interleave of the coordinates, then the level."""
    b, x, y, z, lev = (int(v) for v in o)
    m = 0
    for bit in range(29, -1, -1):
        m = (m << 3) | (((x >> bit) & 1) << 2) | (((y >> bit) & 1) << 1) | ((z >> bit) & 1)
    return (b, m, lev)


def test_random_trees_match_restatement(gpu_lib):
    from tmr_gb300 import TMR
    conn = W.brick(2, 2, 1)
    nrand, lo, hi, seed = 40, 1, 5, 17
    f = TMR.OctForest(order=2)
    f.setConnectivity(conn)
    f.createRandomTrees(nrand, lo, hi, seed)
    got = f.getOctantsArray()
    # restatement: U(seed, block, 4i + k) draws, sort, keep the finest per position
    cand = []
    for b in range(conn.shape[0]):
        u = W.uniform(seed, b, 4 * nrand)
        for i in range(nrand):
            lev = min(lo + int(u[4 * i] * (hi - lo + 1)), hi)
            h = 1 << (30 - lev)
            xyz = [h * min(int(u[4 * i + 1 + k] * (1 << lev)), (1 << lev) - 1) for k in range(3)]
            cand.append((b, *xyz, lev))
    cand.sort(key=_morton_key)
    keep = [c for i, c in enumerate(cand)
            if i + 1 == len(cand) or _morton_key(cand[i + 1])[:2] != _morton_key(c)[:2]]
    exp = np.array([[c[0], c[1], c[2], c[3], i, c[4], 0] for i, c in enumerate(keep)], np.intc)
    np.testing.assert_array_equal(got, exp)


def test_transform_nodes_match_reference(gpu_lib):
    from tmr_gb300 import TMR
    z = _golden()
    f = TMR.OctForest(order=2)
    f.setConnectivity(z["cn_block_conn_in"])
    nodes = z["tn_nodes"]
    for ed in (-1, 0, 1, 2):
        out, rev, fid = f.transformNodes(nodes, edge_dir=ed)
        exp = z["tn_out_e%d" % (ed + 1)]
        for j, name in enumerate(("block", "x", "y", "z")):
            np.testing.assert_array_equal(out[name], exp[:, j])
        np.testing.assert_array_equal(rev, z["tn_rev_e%d" % (ed + 1)])
        np.testing.assert_array_equal(fid, z["tn_fid_e%d" % (ed + 1)])


def test_find_enclosing_matches_reference(gpu_lib):
    from tmr_gb300 import TMR
    z = _golden()
    case = json.loads(str(z["fe_case"]))
    case["conn"] = z["fe_conn"]
    fine = TMR.OctForest(order=3)
    fine.setConnectivity(case["conn"])
    fine.createTrees(case["L0"])
    for p in range(case["passes"]):
        o = fine.getOctantsArray()
        fine.refine(pipeline.indicator(o, case, p), 0, case["max_level"])
        fine.balance(1)
    coarse = fine.coarsen()
    coarse.balance(1)
    np.testing.assert_array_equal(coarse.getOctantsArray(), z["fe_coarse_octants"])
    idx = coarse.findEnclosing(3, fine.getInterpKnots(), z["fe_nodes"])
    np.testing.assert_array_equal(idx, z["fe_index"])


def test_local_node_numbers_and_points(gpu_lib):
    from tmr_gb300 import TMR
    conn = W.brick(2, 1, 1)
    f = TMR.OctForest(order=3)
    f.setConnectivity(conn)
    f.createTrees(1)
    n = f.getNumOctants()
    f.refine(W.random_indicator(n, 4, 0, 0.5), 0, 3)
    f.balance(1)
    f.createNodes()
    nn = f.getNodeNumbers()
    for k in (0, len(nn) // 2, len(nn) - 1):
        assert f.getLocalNodeNumber(int(nn[k])) == k
    assert f.getLocalNodeNumber(int(nn[-1]) + 1) == -1
    # no geometry: every point is 0, as the reference without a topology
    assert not f.getPoints().any()
    boxes = np.array([[0.0, 0.0, 0.0, 1.0, 2.0, 0.5], [1.0, 0.0, 0.0, 1.0, 2.0, 0.5]])
    f.setBlockBoxes(boxes)
    X = f.getPoints()
    # restatement: the first (element, local index) using each node places it
    octs = f.getOctantsArray()
    mc = f.getMeshConn()
    kn = f.getInterpKnots()
    exp = np.full((len(nn), 3), np.nan)
    num_dep = int(f._sizes()[2])
    s = 1.0 / (1 << 30)
    for e in range(len(octs)):
        b, x, y, zc, _, lev, _ = octs[e]
        d = (1 << (30 - lev)) * s
        for l in range(27):
            li = int(mc[e, l]) + num_dep
            if not np.isnan(exp[li, 0]):
                continue
            ijk = (l % 3, (l // 3) % 3, l // 9)
            for a, c in enumerate((x, y, zc)):
                u = c * s + 0.5 * d * (1.0 + kn[ijk[a]])
                exp[li, a] = boxes[b, a] + boxes[b, 3 + a] * u
    np.testing.assert_array_equal(X, exp)


def test_forest_eval_interp_matches_reference(gpu_lib):
    from tmr_gb300 import TMR
    z = _golden()
    for order in (2, 3):
        for itype in (0, 1):
            f = TMR.OctForest(order=order, interp=itype)
            np.testing.assert_array_equal(f.getInterpKnots(), z["ev_o%d_t%d_knots" % (order, itype)])
            for ip, pt in enumerate(z["ev_points"]):
                key = "ev_o%d_t%d_p%d" % (order, itype, ip)
                np.testing.assert_array_equal(f.evalInterp(pt), z[key + "_N"])
                np.testing.assert_array_equal(np.stack(f.evalInterp(pt, 1)), z[key + "_d1"])
                d2 = np.stack(f.evalInterp(pt, 2))
                np.testing.assert_array_equal(d2[:10], z[key + "_d2"][:10])


@pytest.mark.parametrize("name", ["brick_o2", "rot_o3", "bern_o3", "coarse_o4"])
def test_topo_weights_match_reference(gpu_lib, name):
    """Design -> analysis weights of every element against the reference's
    computeWeights steps run on the reference forests (Lagrange filters of
    orders 2-4 and a Bernstein filter)."""
    from tmr_gb300 import TMR
    z = _golden()
    case = json.loads(str(z["tw_%s_case" % name]))
    case["conn"] = z["tw_%s_conn" % name]
    ana = TMR.OctForest(order=case["order"], interp=case.get("interp", 1))
    ana.setConnectivity(case["conn"])
    ana.createTrees(case["L0"])
    for p in range(case["passes"]):
        o = ana.getOctantsArray()
        ana.refine(pipeline.indicator(o, case, p), 0, case["max_level"])
        ana.balance(1)
    filt = ana.coarsen()
    filt.balance(1)
    filt.createNodes()
    W_ = TMR.createTopoWeights(filt, ana)
    rp, ci, w = W_.getCSR()
    np.testing.assert_array_equal(rp, z["tw_%s_rowptr" % name])
    np.testing.assert_array_equal(ci, z["tw_%s_cols" % name])
    np.testing.assert_allclose(w, z["tw_%s_w" % name], rtol=1e-13, atol=1e-13)
    # the element values of a constant design field are that constant
    rows, cols, _ = W_.sizes()
    y = np.zeros(rows)
    W_.mult(np.full(cols, 0.7), y)
    np.testing.assert_allclose(y, 0.7, rtol=1e-13)


def test_interpolate_design_vec_keeps_constants(gpu_lib):
    from tmr_gb300 import TMR
    case = dict(pipeline.cases()["brick_o2"])
    f = TMR.OctForest(order=2)
    f.setConnectivity(case["conn"])
    f.createTrees(1)
    f.refine(W.random_indicator(f.getNumOctants(), 3, 0, 0.5), 0, 4)
    f.balance(1)
    f.createNodes()
    g = f.duplicate()
    g.refine(W.random_indicator(g.getNumOctants(), 3, 1, 0.3), 0, 5)
    g.balance(1)
    g.createNodes()
    nf, ng = f.getNodeRange()[1], g.getNodeRange()[1]
    x = np.tile([1.5, -2.0], nf)
    y = np.zeros(2 * ng)
    TMR.interpolateDesignVec(f, x, g, y)
    np.testing.assert_allclose(y.reshape(-1, 2), np.tile([1.5, -2.0], (ng, 1)), rtol=1e-12)


def test_write_forest_to_vtk(gpu_lib, tmp_path):
    """writeForestToVTK: eight corner points per octant (x fastest) through
    the block boxes, the reference's corner order in CELLS, the block index
    as entity_index; nothing is written without block boxes (the
    reference's behaviour without a topology)."""
    from tmr_gb300 import TMR
    case = pipeline.cases()["brick_o2"]
    f = TMR.OctForest(order=2)
    f.setConnectivity(case["conn"])
    f.createTrees(1)
    f.refine(W.random_indicator(f.getNumOctants(), 5, 0, 0.4), 0, 3)
    f.balance(1)
    fn = tmp_path / "forest.vtk"
    f.writeForestToVTK(str(fn))
    assert not fn.exists()
    boxes = pipeline.brick_boxes(3, 2, 2, ext=(2.0, 1.0, 0.5))
    f.setBlockBoxes(boxes)
    f.writeForestToVTK(str(fn))
    lines = fn.read_text().split("\n")
    o = f.getOctantsArray()
    n = len(o)
    i = lines.index("POINTS %d float" % (8 * n))
    pts = np.array([[float(v) for v in ln.split()] for ln in lines[i + 1:i + 1 + 8 * n]])
    h = (1 << (30 - o[:, 5].astype(np.int64))) / 2.0 ** 30
    for k in (0, n // 2, n - 1):
        b = boxes[o[k, 0]]
        for c in range(8):
            u = o[k, 1:4] / 2.0 ** 30 + h[k] * np.array([c & 1, (c >> 1) & 1, c >> 2])
            np.testing.assert_allclose(pts[8 * k + c], b[:3] + b[3:] * u, rtol=1e-6)
    j = lines.index("CELLS %d %d" % (n, 9 * n))
    assert lines[j + 1] == "8 0 1 3 2 4 5 7 6"
    e = lines.index("SCALARS entity_index float 1")
    ent = np.array([float(v) for v in lines[e + 2:e + 2 + n]])
    np.testing.assert_array_equal(ent, o[:, 0])


def test_write_to_tecplot(gpu_lib, tmp_path):
    """writeToTecplot: the block mesh, each connectivity node at its owner
    block's corner (lowest-numbered block touching it) through the block
    boxes, the block index cell-centred, corners in the reference's
    (0 1 3 2 4 5 7 6) order counted from 1; nothing without block boxes."""
    from tmr_gb300 import TMR
    conn = W.rotate_blocks(W.brick(3, 2, 2), 8)
    f = TMR.OctForest(order=2)
    f.setConnectivity(conn)
    fn = tmp_path / "blocks.dat"
    f.writeToTecplot(str(fn))
    assert not fn.exists()
    boxes = pipeline.brick_boxes(3, 2, 2, ext=(2.0, 1.0, 0.5))
    f.setBlockBoxes(boxes)
    f.writeToTecplot(str(fn))
    lines = fn.read_text().split("\n")
    nb, nn = conn.shape[0], int(conn.max()) + 1
    assert lines[0] == "Variables = X,Y,Z,block"
    assert lines[1] == "Zone N = %d E = %d DATAPACKING=BLOCK, ZONETYPE=FEBRICK" % (nn, nb)
    assert lines[2] == "VARLOCATION = ([4]=CELLCENTERED)"
    vals = np.array([float(v) for v in lines[3:3 + 3 * nn + nb]])
    X = vals[:3 * nn].reshape(3, nn).T
    for k in range(nn):
        b = min(np.argwhere(conn == k)[:, 0])
        c = int(np.argwhere(conn[b] == k)[0, 0])
        uvw = np.array([c & 1, (c >> 1) & 1, c >> 2], np.float64)
        np.testing.assert_allclose(X[k], boxes[b, :3] + boxes[b, 3:] * uvw, rtol=1e-6)
    np.testing.assert_array_equal(vals[3 * nn:], np.arange(nb))
    cells = np.array([[int(v) for v in ln.split()] for ln in lines[3 + 3 * nn + nb:3 + 3 * nn + 2 * nb]])
    np.testing.assert_array_equal(cells, conn[:, [0, 1, 3, 2, 4, 5, 7, 6]] + 1)



def test_write_to_vtk_blocks(gpu_lib, tmp_path):
    """writeToVTK: the block mesh (as the reference writes it): each
    connectivity node at its owner block's corner through the block boxes,
    hexahedra in the (0 1 3 2 4 5 7 6) corner order, the block index as
    entity_index; nothing without block boxes."""
    from tmr_gb300 import TMR
    conn = W.rotate_blocks(W.brick(3, 2, 2), 8)
    f = TMR.OctForest(order=2)
    f.setConnectivity(conn)
    fn = tmp_path / "blocks.vtk"
    f.writeToVTK(str(fn))
    assert not fn.exists()
    boxes = pipeline.brick_boxes(3, 2, 2, ext=(2.0, 1.0, 0.5))
    f.setBlockBoxes(boxes)
    f.writeToVTK(str(fn))
    lines = fn.read_text().split("\n")
    nb, nn = conn.shape[0], int(conn.max()) + 1
    i = lines.index("POINTS %d float" % nn)
    pts = np.array([[float(v) for v in ln.split()] for ln in lines[i + 1:i + 1 + nn]])
    for k in range(nn):
        b = min(np.argwhere(conn == k)[:, 0])
        c = int(np.argwhere(conn[b] == k)[0, 0])
        uvw = np.array([c & 1, (c >> 1) & 1, c >> 2], np.float64)
        np.testing.assert_allclose(pts[k], boxes[b, :3] + boxes[b, 3:] * uvw, rtol=1e-6)
    j = lines.index("CELLS %d %d" % (nb, 9 * nb))
    cells = np.array([[int(v) for v in ln.split()] for ln in lines[j + 1:j + 1 + nb]])
    np.testing.assert_array_equal(cells[:, 1:], conn[:, [0, 1, 3, 2, 4, 5, 7, 6]])
