"""Batched forests: independent forests held as one forest over the
disjoint union of their blocks give, forest by forest, the octants, node
connectivity and prolongation that each forest gives alone."""
import numpy as np
import pytest

from tmr_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _alone(TMR, conn, seed, k, prob, target, max_level):
    f = TMR.OctForest(order=2)
    f.setConnectivity(conn)
    f.createTrees(1)
    for p in range(8):
        n = f.getNumOctants()
        if n >= target:
            break
        f.refine(TMR.random_refinement(n, seed, k * 1024 + p, prob), 0, max_level)
        f.balance(1)
    f.createNodes()
    c = f.coarsen()
    c.balance(1)
    c.createNodes()
    I = TMR.VecInterp()
    f.createInterpolation(c, I)
    return f, c, I


def _renumber(conn, own_lo, dep_lo):
    out = conn.copy()
    pos = conn >= 0
    out[pos] -= own_lo
    out[~pos] = -((-conn[~pos] - 1) - dep_lo) - 1
    return out


def _offsets(conn):
    pos = conn[conn >= 0]
    neg = -conn[conn < 0] - 1
    return int(pos.min()), (int(neg.min()) if neg.size else 0)


def test_batch_equals_forests_alone(gpu_lib):
    from tmr_gb300 import TMR
    from tmr_gb300.batch import ForestBatch
    conns = [W.brick(1, 1, 1), W.brick(2, 2, 2), W.rotate_blocks(W.brick(2, 1, 2), 3),
             W.brick(3, 1, 1), W.brick(1, 1, 1)]
    probs = [0.5, 0.3, 0.4, 0.2, 0.45]
    targets = [300, 4000, 2500, 900, 50]
    seed, max_level = 21, 6
    B = ForestBatch(conns, order=2)
    f = B.forest
    f.createTrees(1)
    for p in range(8):
        starts = B.octant_starts()
        active = np.diff(starts) < np.array(targets)
        if not active.any():
            break
        f.refine(B.random_refinement(seed, p, probs, active), 0, max_level)
        f.balance(1)
    f.createNodes()
    c = f.coarsen()
    c.balance(1)
    c.createNodes()
    I = TMR.VecInterp()
    f.createInterpolation(c, I)
    fo, fs = f.getOctantsArray(), B.octant_starts()
    co, cs = c.getOctantsArray(), B.octant_starts(c)
    fconn, cconn = f.getMeshConn(), c.getMeshConn()
    rp, ci, w = I.getCSR()
    per_f, per_c = B.split_octants(fo, fs), B.split_octants(co, cs)
    for k, conn in enumerate(conns):
        fa, ca, Ia = _alone(TMR, conn, seed, k, probs[k], targets[k], max_level)
        np.testing.assert_array_equal(per_f[k], fa.getOctantsArray())
        np.testing.assert_array_equal(per_c[k], ca.getOctantsArray())
        sub = fconn[fs[k]:fs[k + 1]]
        own_f, dep_f = _offsets(sub)
        np.testing.assert_array_equal(_renumber(sub, own_f, dep_f), fa.getMeshConn())
        csub = cconn[cs[k]:cs[k + 1]]
        own_c, dep_c = _offsets(csub)
        np.testing.assert_array_equal(_renumber(csub, own_c, dep_c), ca.getMeshConn())
        # P of the forest = rows own_f.., columns shifted by own_c
        ra, ca_, wa = Ia.getCSR()
        rows = len(ra) - 1
        lo, hi = rp[own_f], rp[own_f + rows]
        np.testing.assert_array_equal(rp[own_f:own_f + rows + 1] - lo, ra)
        np.testing.assert_array_equal(ci[lo:hi] - own_c, ca_)
        np.testing.assert_array_equal(w[lo:hi], wa)


def test_batch_matches_oracle(gpu_lib):
    """Each forest of a batch against the CPU oracle run on that forest
    alone with the same refinement draws: octants, connectivity (rebased)
    and P (rebased) bit-exact / within 1e-13."""
    from oracle.oracle import OracleForest, interp_to_csr
    from tmr_gb300 import TMR
    from tmr_gb300.batch import ForestBatch
    conns = [W.brick(2, 1, 1), W.rotate_blocks(W.brick(2, 2, 1), 7), W.brick(1, 1, 1)]
    probs = [0.35, 0.3, 0.5]
    seed, max_level, passes = 9, 5, 3
    B = ForestBatch(conns, order=2)
    f = B.forest
    f.createTrees(1)
    for p in range(passes):
        f.refine(B.random_refinement(seed, p, probs, np.ones(len(conns), bool)), 0, max_level)
        f.balance(1)
    f.createNodes()
    c = f.coarsen()
    c.balance(1)
    c.createNodes()
    I = TMR.VecInterp()
    f.createInterpolation(c, I)
    fo, fs = f.getOctantsArray(), B.octant_starts()
    cs = B.octant_starts(c)
    fconn, cconn = f.getMeshConn(), c.getMeshConn()
    rp, ci, w = I.getCSR()
    per_f = B.split_octants(fo, fs)
    for k, conn in enumerate(conns):
        o = OracleForest(2, 1)
        o.setConnectivity(conn)
        o.createTrees(1)
        for p in range(passes):
            n = len(o.getOctants())
            o.refine(W.random_indicator(n, seed, k * 1024 + p, probs[k]), 0, max_level)
            o.balance(1)
        o.createNodes()
        oc = o.coarsen()
        oc.balance(1)
        oc.createNodes()
        orows, optr, ocols, ow = o.createInterpolation(oc)
        orp, oci, ov = interp_to_csr(orows, optr, ocols, ow, o.nodeSizes()["num_owned"])
        ref = o.getOctants().copy()
        got = per_f[k].copy()
        np.testing.assert_array_equal(got, ref)
        sub = fconn[fs[k]:fs[k + 1]]
        own_f, dep_f = _offsets(sub)
        np.testing.assert_array_equal(_renumber(sub, own_f, dep_f), o.getMeshConn(2))
        csub = cconn[cs[k]:cs[k + 1]]
        own_c, _ = _offsets(csub)
        rows = len(orp) - 1
        lo, hi = rp[own_f], rp[own_f + rows]
        np.testing.assert_array_equal(rp[own_f:own_f + rows + 1] - lo, orp)
        np.testing.assert_array_equal(ci[lo:hi] - own_c, oci)
        np.testing.assert_allclose(w[lo:hi], ov, rtol=1e-13, atol=1e-13)
