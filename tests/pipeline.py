"""Runs one adaptation pipeline (createTrees -> refine/balance passes ->
createNodes -> coarsen/balance/createNodes/createInterpolation per level)
on the GPU library or on a CPU checker, and returns every product as
numpy arrays so the two can be compared."""
import json
import os

import numpy as np

from tmr_gb300 import workloads as W

RTOL = 1e-13  # FP64 tolerance for weights and applies (relative)


def indicator(octs, case, p):
    if case.get("indicator", "random") == "sphere":
        return W.sphere_indicator(octs)
    if case.get("indicator") == "point":
        return W.point_indicator(octs, case["point"])
    if case.get("indicator") == "qpoint":
        return W.quad_point_indicator(octs, case["point"])
    if case.get("indicator") == "mixed":
        return W.mixed_indicator(len(octs), case.get("seed", 0), p, case.get("prob", 0.3),
                                 case.get("coarsen_prob", 0.3))
    return W.random_indicator(len(octs), case.get("seed", 0), p, case.get("prob", 0.3))


def _csr_from_records(rows, ptr, cols, w, nrows):
    from oracle.oracle import interp_to_csr
    return interp_to_csr(rows, ptr, cols, w, nrows)


def hierarchy_steps(case):
    """The coarse levels of a case: "h" = coarsen + balance (the geometric
    step), "p" = duplicate + setMeshOrder(order - 1) on the same octants
    (the order step createTopoProblem takes while the order is above its
    lowest, TopOptUtils.py:80-88)."""
    return case.get("hier") or ["h"] * case.get("coarse_levels", 1)


def coarser(f, case, step="h", order=None):
    """The next coarse forest.  "h": coarsen + balance, `coarse_steps` times
    (two or more give fine elements several levels below their coarse
    element).  "p": duplicate + setMeshOrder(order - 1), same octants and
    knot family, not re-balanced (as TopOptUtils.py:82-85 does)."""
    if step == "p":
        c = f.duplicate()
        c.setMeshOrder(order - 1, case.get("interp", 1))
        return c
    c = f
    for _ in range(case.get("coarse_steps", 1)):
        c = c.coarsen()
        c.balance(case.get("corner", 1))
    return c


def run_gpu(case):
    from tmr_gb300 import TMR
    order = case["order"]
    f = TMR.OctForest(order=order, interp=case.get("interp", TMR.GAUSS_LOBATTO_POINTS))
    f.setConnectivity(case["conn"])
    f.createTrees(case["L0"])
    for p in range(case["passes"]):
        o = f.getOctantsArray()
        f.refine(indicator(o, case, p), 0, case["max_level"])
        f.balance(case.get("corner", 1))
    if case.get("octants_only"):
        return dict(oct=f.getOctantsArray(), octants_only=True, forests=[f])
    f.createNodes()
    out = dict(oct=f.getOctantsArray(), conn=f.getMeshConn(),
               nn=f.getNodeNumbers(), dep=f.getDepNodeConn(),
               sizes=_gpu_sizes(f), levels=[])
    c = f
    forests = [f]
    for step in hierarchy_steps(case):
        cc = coarser(c, case, step, c.getMeshOrder())
        cc.createNodes()
        I = TMR.VecInterp()
        c.createInterpolation(cc, I)
        out["levels"].append(dict(oct=cc.getOctantsArray(), conn=cc.getMeshConn(),
                                  P=I.getCSR(), I=I))
        forests.append(cc)
        c = cc
    out["forests"] = forests
    return out


def _gpu_sizes(f):
    s = f._sizes()
    return dict(num_local=int(s[0]), num_owned=int(s[1]), num_dep=int(s[2]),
                ext_pre=int(s[3]), num_elements=int(s[4]), dep_nnz=int(s[5]))


def run_cpu(case, kind="oracle"):
    from oracle.oracle import OracleForest, RefForest
    cls = OracleForest if kind == "oracle" else RefForest
    order = case["order"]
    f = cls(order, case.get("interp", 1))
    f.setConnectivity(case["conn"])
    f.createTrees(case["L0"])
    for p in range(case["passes"]):
        o = f.getOctants()
        f.refine(indicator(o, case, p), 0, case["max_level"])
        f.balance(case.get("corner", 1))
    if case.get("octants_only"):
        return dict(oct=f.getOctants(), octants_only=True)
    f.createNodes()
    out = dict(oct=f.getOctants(), conn=f.getMeshConn(order), nn=f.getNodeNumbers(),
               dep=f.getDepNodeConn(), sizes=f.nodeSizes(), levels=[])
    c = f
    for step in hierarchy_steps(case):
        cc = coarser(c, case, step, order)
        if step == "p":
            order -= 1
        cc.createNodes()
        rows, ptr, cols, w = c.createInterpolation(cc)
        P = _csr_from_records(rows, ptr, cols, w, c.nodeSizes()["num_owned"])
        out["levels"].append(dict(oct=cc.getOctants(), conn=cc.getMeshConn(order), P=P))
        c = cc
    return out


def compare(a, b):
    """List of mismatch descriptions (empty when a and b agree: integers
    exactly, floating point within RTOL)."""
    bad = []

    def ints(name, x, y):
        x, y = np.asarray(x), np.asarray(y)
        if x.shape != y.shape:
            bad.append("%s: shape %s vs %s" % (name, x.shape, y.shape))
        elif not np.array_equal(x, y):
            i = np.argwhere(x != y)[0]
            bad.append("%s: first difference at %s: %s vs %s" % (
                name, tuple(i), x[tuple(i)], y[tuple(i)]))

    def fps(name, x, y):
        x, y = np.asarray(x), np.asarray(y)
        if x.shape != y.shape:
            bad.append("%s: shape %s vs %s" % (name, x.shape, y.shape))
        elif x.size and not np.allclose(x, y, rtol=RTOL, atol=RTOL * max(1.0, np.abs(y).max())):
            bad.append("%s: max abs diff %g" % (name, np.abs(x - y).max()))

    ints("octants", a["oct"], b["oct"])
    if a.get("octants_only") or b.get("octants_only"):
        return bad
    if a["sizes"] != b["sizes"]:
        bad.append("sizes %s vs %s" % (a["sizes"], b["sizes"]))
    ints("conn", a["conn"], b["conn"])
    ints("node_numbers", a["nn"], b["nn"])
    ints("dep_ptr", a["dep"][0], b["dep"][0])
    ints("dep_conn", a["dep"][1], b["dep"][1])
    fps("dep_weights", a["dep"][2], b["dep"][2])
    for k, (la, lb) in enumerate(zip(a["levels"], b["levels"])):
        ints("L%d octants" % k, la["oct"], lb["oct"])
        ints("L%d conn" % k, la["conn"], lb["conn"])
        ints("L%d P rowptr" % k, la["P"][0], lb["P"][0])
        ints("L%d P cols" % k, la["P"][1], lb["P"][1])
        fps("L%d P vals" % k, la["P"][2], lb["P"][2])
    return bad


GOLDEN_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def golden_cases():
    """Names of the pipeline fixtures in tests/golden (api*.npz hold the
    single-call getters and the STL output, digest_*.npz the checksummed
    configuration-size cases; each is read by its own tests)."""
    return sorted(f[:-4] for f in os.listdir(GOLDEN_DIR)
                  if f.endswith(".npz") and not f.startswith(("api", "quad_", "digest_")))


# ---------------------------------------------------------------------------
# Configuration-size cases: too large to store whole, so their fixtures hold
# a digest of every product (tests/golden/digest_<case>.npz).
def digest_cases():
    return {
        # the one-tree configuration exactly as specified: createTrees(4),
        # 3 passes refining the octants whose centre lies within 0.3 of the
        # cube centre (max level 7) + balance(1), order 2 GLL, one coarsened
        # level and its P (about 237k octants)
        "c1": dict(conn=W.brick(1, 1, 1), order=2, L0=4, passes=3, max_level=7,
                   indicator="sphere", coarse_levels=1),
    }


def product_arrays(r):
    """Every product of a pipeline result by name, integers as int64 and
    weights as float64 (so GPU and CPU results hash alike)."""
    s = r["sizes"]
    out = {"octants": r["oct"], "conn": r["conn"], "node_numbers": r["nn"],
           "dep_ptr": r["dep"][0], "dep_conn": r["dep"][1], "dep_w": r["dep"][2],
           "sizes": [s[k] for k in ("num_local", "num_owned", "num_dep", "ext_pre",
                                    "num_elements", "dep_nnz")]}
    for k, lv in enumerate(r["levels"]):
        out["L%d_octants" % k] = lv["oct"]
        out["L%d_conn" % k] = lv["conn"]
        out["L%d_P_rowptr" % k], out["L%d_P_cols" % k], out["L%d_P_vals" % k] = lv["P"]
    norm = {}
    for k, a in out.items():
        a = np.asarray(a)
        if hasattr(a, "dtype") and a.dtype.names:  # structured octants
            a = np.stack([a[n] for n in a.dtype.names], 1)
        a = np.ascontiguousarray(a, np.float64 if a.dtype.kind == "f" else np.int64)
        norm[k] = a
    return norm


DIGEST_SAMPLES = 4096


def _sample_index(n):
    return np.unique(np.linspace(0, max(n - 1, 0), min(n, DIGEST_SAMPLES)).astype(np.int64))


def digest(r):
    """The fixture of a configuration-size case: per integer product its
    shape, the SHA-256 of its bytes and an evenly spaced sample of its
    entries (to locate a difference); weights are stored whole (they take
    few distinct values and compress to a few KB)."""
    import hashlib
    d = {}
    for k, a in product_arrays(r).items():
        d[k + "__shape"] = np.array(a.shape, np.int64)
        if a.dtype.kind == "f":
            d[k + "__full"] = a
            continue
        d[k + "__sha"] = np.array(hashlib.sha256(a.tobytes()).hexdigest())
        flat = a.reshape(a.shape[0], -1) if a.ndim > 1 else a
        d[k + "__sample"] = flat[_sample_index(flat.shape[0])]
    return d


def compare_digest(r, z):
    """Mismatches between a pipeline result and a digest fixture (empty when
    they agree): integer products bit for bit (by hash), weights entry by
    entry within RTOL."""
    import hashlib
    bad = []
    arrs = product_arrays(r)
    names = sorted({k.split("__")[0] for k in z.files if "__" in k})
    if sorted(arrs) != names:
        bad.append("products %s vs fixture %s" % (sorted(arrs), names))
    for k in names:
        if k not in arrs:
            continue
        a = arrs[k]
        if tuple(a.shape) != tuple(z[k + "__shape"]):
            bad.append("%s: shape %s vs %s" % (k, a.shape, tuple(z[k + "__shape"])))
        elif a.dtype.kind == "f":
            ref = z[k + "__full"]
            if a.size and not np.allclose(a, ref, rtol=RTOL,
                                          atol=RTOL * max(1.0, np.abs(ref).max())):
                bad.append("%s: max abs diff %g" % (k, np.abs(a - ref).max()))
        elif hashlib.sha256(a.tobytes()).hexdigest() != str(z[k + "__sha"]):
            flat = a.reshape(a.shape[0], -1) if a.ndim > 1 else a
            smp, ref = flat[_sample_index(flat.shape[0])], z[k + "__sample"]
            diff = np.argwhere(smp != ref)
            bad.append("%s: hash differs%s" % (k, "" if not len(diff) else
                                                " (sample entry %s: %s vs %s)" % (
                                                    tuple(diff[0]), smp[tuple(diff[0])],
                                                    ref[tuple(diff[0])])))
    return bad


def load_golden(name):
    """Products of the reference itself for parity case `name`
    (tests/golden/<name>.npz, written by tests/golden/make_golden.py), in
    the format run_gpu/run_cpu return."""
    z = np.load(os.path.join(GOLDEN_DIR, name + ".npz"))
    if "sizes" not in z:
        return dict(oct=z["octants"], octants_only=True)
    s = z["sizes"]
    out = dict(oct=z["octants"], conn=z["conn"], nn=z["node_numbers"],
               dep=(z["dep_ptr"], z["dep_conn"], z["dep_w"]),
               sizes=dict(num_local=int(s[0]), num_owned=int(s[1]), num_dep=int(s[2]),
                          ext_pre=int(s[3]), num_elements=int(s[4]), dep_nnz=int(s[5])),
                   levels=[])
    k = 0
    while "L%d_octants" % k in z:
        out["levels"].append(dict(oct=z["L%d_octants" % k], conn=z["L%d_conn" % k],
                                  P=(z["L%d_P_rowptr" % k], z["L%d_P_cols" % k],
                                     z["L%d_P_vals" % k])))
        k += 1
    return out


def golden_case(name):
    """The parity case as stored with its fixture (block connectivity
    included), so the fixture alone defines the input."""
    z = np.load(os.path.join(GOLDEN_DIR, name + ".npz"))
    case = json.loads(str(z["meta"]))
    case["conn"] = z["block_conn"]
    return case


# Parity cases, small enough for the checker to finish in seconds.
def cases():
    return {
        "c1_small": dict(conn=W.brick(1, 1, 1), order=2, L0=3, passes=3, max_level=6,
                         indicator="sphere"),
        "brick_o2": dict(conn=W.brick(3, 2, 2), order=2, L0=1, passes=3, max_level=6,
                         prob=0.3, seed=7, coarse_levels=2),
        "brick_o3": dict(conn=W.brick(3, 2, 2), order=3, L0=1, passes=3, max_level=5,
                         prob=0.3, seed=7, coarse_levels=2),
        "rot_o2": dict(conn=W.rotate_blocks(W.brick(3, 3, 2), 1), order=2, L0=1, passes=3,
                       max_level=5, prob=0.3, seed=3),
        "rot_o3": dict(conn=W.rotate_blocks(W.brick(2, 2, 2), 2), order=3, L0=1, passes=3,
                       max_level=5, prob=0.3, seed=4, coarse_levels=2),
        "rot_o4": dict(conn=W.rotate_blocks(W.brick(2, 2, 1), 5), order=4, L0=1, passes=2,
                       max_level=4, prob=0.3, seed=5, coarse_levels=0),
        "nocorner": dict(conn=W.rotate_blocks(W.brick(2, 2, 2), 6), order=2, L0=1, passes=3,
                         max_level=5, prob=0.3, seed=6, corner=0),
        "uniform_o3": dict(conn=W.brick(2, 1, 1), order=3, L0=2, passes=1, max_level=3,
                           prob=1.0, seed=1, interp=0),
        # P across two or three levels (fine elements up to three levels
        # below their coarse element)
        "gap_o2": dict(conn=W.rotate_blocks(W.brick(2, 2, 1), 9), order=2, L0=1, passes=3,
                       max_level=5, prob=0.4, seed=21, coarse_levels=1, coarse_steps=3),
        "gap_o3": dict(conn=W.brick(2, 1, 1), order=3, L0=1, passes=3, max_level=5,
                       prob=0.4, seed=22, coarse_levels=2, coarse_steps=2),
        # the hierarchy createTopoProblem builds from an order-3 forest:
        # 3 -> 2 on the same octants, then geometric coarsening at order 2
        "pcoarse_o3": dict(conn=W.rotate_blocks(W.brick(3, 2, 2), 11), order=3, L0=1,
                           passes=3, max_level=5, prob=0.3, seed=17, hier=["p", "h", "h"]),
        # order 4: 4 -> 3 -> 2 on the same octants, then one geometric step
        "pcoarse_o4": dict(conn=W.brick(2, 2, 1), order=4, L0=1, passes=2, max_level=4,
                           prob=0.3, seed=18, hier=["p", "p", "h"]),
        # geometric coarsening at order 4 (coarse elements of order 4)
        "coarse_o4": dict(conn=W.rotate_blocks(W.brick(2, 1, 1), 13), order=4, L0=1,
                          passes=2, max_level=3, prob=0.3, seed=19, coarse_levels=2),
        # forests deeper than 64-bit keys hold (octant keys of bb + 3W + 5
        # bits, node keys of bb + 3(W + 1) + label bits): refinement paths
        # toward one block-local point, the coarse levels crossing back
        # to 64-bit keys
        "deep_o2": dict(conn=W.brick(1, 1, 1), order=2, L0=1, passes=22, max_level=23,
                        indicator="point", point=[0.3, 0.6, 0.45], coarse_levels=2),
        "deep_o3": dict(conn=W.rotate_blocks(W.brick(2, 1, 1), 27), order=3, L0=1, passes=20,
                        max_level=21, indicator="point", point=[1.0 - 2.0 ** -25, 0.37, 0.61],
                        coarse_levels=3),
        "deep_l29": dict(conn=W.brick(1, 1, 1), order=2, L0=0, passes=29, max_level=29,
                         indicator="point", point=[0.7, 0.2, 0.55], coarse_levels=1),
        # refine + balance down to level 30 (side 1); octants only: the
        # reference's element connectivity takes a half side of
        # 1 << (TMR_MAX_LEVEL - level - 1) (TMROctForest.cpp:4693), a negative
        # shift at level 30, so its nodes there have no defined value
        "deep_l30": dict(conn=W.rotate_blocks(W.brick(2, 1, 1), 31), order=2, L0=0, passes=30,
                         max_level=30, indicator="point", point=[0.999, 0.2, 0.55],
                         octants_only=True),
        # Bernstein elements (interp 2): dependent rows from the subdivision
        # weights, P from the Bernstein basis (same order) or the degree
        # elevation table (order one lower)
        "bern_o3": dict(conn=W.rotate_blocks(W.brick(2, 2, 1), 14), order=3, L0=1, passes=3,
                        max_level=4, prob=0.3, seed=23, interp=2, coarse_levels=2),
        "bern_p3": dict(conn=W.brick(3, 2, 1), order=3, L0=1, passes=3, max_level=5,
                        prob=0.3, seed=24, interp=2, hier=["p", "h"]),
        "bern_o4": dict(conn=W.rotate_blocks(W.brick(2, 1, 1), 15), order=4, L0=1, passes=2,
                        max_level=4, prob=0.3, seed=25, interp=2, hier=["h", "p", "h"]),
        "bern_o5": dict(conn=W.brick(1, 1, 1), order=5, L0=1, passes=2, max_level=3,
                        prob=0.3, seed=26, interp=2, hier=["p", "h"]),
        # refinement arrays with -1 entries: coarsening inside refine
        "mixed_o2": dict(conn=W.rotate_blocks(W.brick(3, 2, 2), 8), order=2, L0=2, passes=3,
                         max_level=4, indicator="mixed", prob=0.35, coarsen_prob=0.3, seed=12,
                         coarse_levels=2),
    }


# ---------------------------------------------------------------------------
# Iso-surface (STL) cases: the parity forests with unit-cube block boxes,
# node points by the box map, and a smooth seeded design field.
STL_CASES = {
    "brick_o2": dict(cutoff=0.1, vpn=2, offset=0, grid=(3, 2, 2)),
    "uniform_o3": dict(cutoff=0.05, vpn=2, offset=1, grid=(2, 1, 1)),
}


def brick_boxes(nx, ny, nz, ext=(1.0, 1.0, 1.0)):
    """Block boxes (origin xyz, extent xyz) of W.brick(nx, ny, nz)."""
    return np.array([[i * ext[0], j * ext[1], k * ext[2], *ext] for k in range(nz)
                     for j in range(ny) for i in range(nx)], np.float64)


def node_points(octs, conn, num_dep, num_local, order, knots, boxes):
    """getPoints with block boxes: each node placed by the first (element,
    local index) that uses it (local index of node g: g + num_dep)."""
    X = np.full((num_local, 3), np.nan)
    s = 1.0 / (1 << 30)
    for e in range(len(octs)):
        b, x, y, z, _, lev, _ = (int(v) for v in octs[e])
        d = (1 << (30 - lev)) * s
        for l in range(order ** 3):
            li = int(conn[e, l]) + num_dep
            if not np.isnan(X[li, 0]):
                continue
            ijk = (l % order, (l // order) % order, l // (order * order))
            for a, c in enumerate((x, y, z)):
                u = c * s + 0.5 * d * (1.0 + knots[ijk[a]])
                X[li, a] = boxes[b, a] + boxes[b, 3 + a] * u
    return X


def stl_field(P, vpn):
    """Design values at the independent nodes' points P: component 0 is
    sin(2x) cos(1.5y) + 0.3z, component 1 its negative plus 0.2."""
    f = np.sin(2.0 * P[:, 0]) * np.cos(1.5 * P[:, 1]) + 0.3 * P[:, 2]
    comps = [f, 0.2 - f][:vpn]
    return np.stack(comps, 1).ravel()


# ---------------------------------------------------------------------------
# Quadtree (2-D twin) parity cases.
def quad_cases():
    return {
        "brick_o2": dict(conn=W.brick2d(4, 3), order=2, L0=1, passes=4, max_level=8,
                         prob=0.3, seed=7, coarse_levels=2),
        "brick_o3": dict(conn=W.brick2d(3, 2), order=3, L0=1, passes=4, max_level=7,
                         prob=0.3, seed=8, coarse_levels=2),
        "rot_o2": dict(conn=W.rotate_faces(W.brick2d(4, 4), 3), order=2, L0=1, passes=4,
                       max_level=7, prob=0.3, seed=9, coarse_levels=1),
        "rot_o3": dict(conn=W.rotate_faces(W.brick2d(3, 3), 4), order=3, L0=1, passes=3,
                       max_level=6, prob=0.35, seed=10, coarse_levels=2),
        "nocorner_o2": dict(conn=W.rotate_faces(W.brick2d(3, 3), 5), order=2, L0=1,
                            passes=4, max_level=7, prob=0.3, seed=11, corner=0,
                            coarse_levels=1),
        "uniform_o3": dict(conn=W.brick2d(2, 2), order=3, L0=2, passes=3, max_level=6,
                           prob=0.3, seed=12, interp=0, coarse_levels=1),
        "mixed_o2": dict(conn=W.rotate_faces(W.brick2d(4, 3), 6), order=2, L0=2, passes=3,
                         max_level=6, indicator="mixed", prob=0.35, coarsen_prob=0.3, seed=13,
                         coarse_levels=2),
        # deeper than 64-bit keys hold (quadrant keys of face bits + 2W + 5
        # bits, node keys of face bits + 2(W + 1)): refinement paths toward
        # one face-local point, the coarse levels crossing back to 64-bit keys
        "deep_o2": dict(conn=W.rotate_faces(W.brick2d(8, 4), 14), order=2, L0=0, passes=29,
                        max_level=29, indicator="qpoint", point=[0.999, 0.31], coarse_levels=2),
        "deep_o3": dict(conn=W.brick2d(8, 4), order=3, L0=0, passes=28, max_level=28,
                        indicator="qpoint", point=[0.42, 0.0001], coarse_levels=2),
    }


def _quad_run(f, case, make_interp):
    for p in range(case["passes"]):
        q = f.getQuadrantsArray() if hasattr(f, "getQuadrantsArray") else f.getQuadrants()
        f.refine(indicator(q, case, p), 0, case["max_level"])
        f.balance(case.get("corner", 1))
    f.createNodes()
    out = dict(quads=_quads(f), conn=f.getMeshConn(), dep=f.getDepNodeConn(), levels=[])
    c = f
    for _ in range(case.get("coarse_levels", 1)):
        cc = c.coarsen()
        cc.balance(case.get("corner", 1))
        cc.createNodes()
        out["levels"].append(dict(quads=_quads(cc), conn=cc.getMeshConn(),
                                  dep=cc.getDepNodeConn(), P=make_interp(c, cc)))
        c = cc
    return out


def _quads(f):
    q = f.getQuadrantsArray() if hasattr(f, "getQuadrantsArray") else f.getQuadrants()
    q = np.array(q, np.int32).copy()
    q[:, 3] = 0  # the tag column is bookkeeping (element index on the GPU)
    return q


def run_quad_gpu(case):
    from tmr_gb300 import TMR
    f = TMR.QuadForest(order=case["order"], interp=case.get("interp", 1))
    f.setConnectivity(case["conn"])
    f.createTrees(case["L0"])

    def interp(fine, coarse):
        I = TMR.VecInterp()
        fine.createInterpolation(coarse, I)
        return I.getCSR()
    return _quad_run(f, case, interp)


def run_quad_ref(case):
    from oracle.oracle import RefQuadForest
    f = RefQuadForest(case["order"], case.get("interp", 1))
    f.setConnectivity(case["conn"])
    f.createTrees(case["L0"])

    def interp(fine, coarse):
        rows, ptr, cols, w = fine.createInterpolation(coarse)
        return _csr_from_records(rows, ptr, cols, w, fine.nodeSizes()["num_owned"])
    return _quad_run(f, case, interp)


def load_quad_golden(name):
    z = np.load(os.path.join(GOLDEN_DIR, "quad_" + name + ".npz"))
    out = dict(quads=z["quads"], conn=z["conn"], dep=(z["dep_ptr"], z["dep_conn"], z["dep_w"]),
               levels=[])
    k = 0
    while "L%d_quads" % k in z:
        out["levels"].append(dict(quads=z["L%d_quads" % k], conn=z["L%d_conn" % k],
                                  dep=(z["L%d_dep_ptr" % k], z["L%d_dep_conn" % k],
                                       z["L%d_dep_w" % k]),
                                  P=(z["L%d_P_rowptr" % k], z["L%d_P_cols" % k],
                                     z["L%d_P_vals" % k])))
        k += 1
    return out


def compare_quad(a, b):
    """Differences between two quadtree pipeline results (empty = equal):
    integers bit-exact, weights within 1e-13 relative (observed equal)."""
    bad = []

    def arr(name, x, y, tol=None):
        x, y = np.asarray(x), np.asarray(y)
        if x.shape != y.shape:
            bad.append("%s shape %s != %s" % (name, x.shape, y.shape))
        elif tol is None:
            if not np.array_equal(x, y):
                bad.append("%s differs at %d entries" % (name, int((x != y).sum())))
        elif x.size and np.abs(x - y).max() > tol * max(1.0, np.abs(y).max()):
            bad.append("%s max diff %g" % (name, np.abs(x - y).max()))

    def level(pfx, A, B):
        arr(pfx + "quads", A["quads"], B["quads"])
        arr(pfx + "conn", A["conn"], B["conn"])
        for j, nm in enumerate(("dep_ptr", "dep_conn")):
            arr(pfx + nm, A["dep"][j], B["dep"][j])
        arr(pfx + "dep_w", A["dep"][2], B["dep"][2], 1e-13)
    level("", a, b)
    if len(a["levels"]) != len(b["levels"]):
        bad.append("levels %d != %d" % (len(a["levels"]), len(b["levels"])))
    for k, (A, B) in enumerate(zip(a["levels"], b["levels"])):
        level("L%d_" % k, A, B)
        arr("L%d_P_rowptr" % k, A["P"][0], B["P"][0])
        arr("L%d_P_cols" % k, A["P"][1], B["P"][1])
        arr("L%d_P_vals" % k, A["P"][2], B["P"][2], 1e-13)
    return bad


def quad_golden_case(name):
    """The quadtree parity case as stored with its fixture."""
    z = np.load(os.path.join(GOLDEN_DIR, "quad_" + name + ".npz"))
    case = json.loads(str(z["meta"]))
    case["conn"] = z["face_conn"]
    return case


def quad_golden_names():
    return sorted(f[5:-4] for f in os.listdir(GOLDEN_DIR)
                  if f.startswith("quad_") and f.endswith(".npz"))
