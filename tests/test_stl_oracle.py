"""The CPU restatement of the iso-surface triangles (oracle/stl.py) against
the reference's own TMR_GenerateSTLTriangles: its output on parity forests
(tests/golden/api_stl.npz, written from oracle/_ref) and, where the
reference build is present, every one of the 256 marching-cubes cases and
its ASCII converter.  Crossing points are compared bit for bit; per cell,
the loops (vertex sets, triangle counts and vector areas, which do not
depend on how a loop is split into triangles) are compared."""
import os

import numpy as np
import pytest

from oracle import oracle as O
from oracle import stl as S
from tests import pipeline

HERE = os.path.dirname(os.path.abspath(__file__))


def _varea(T):
    T = np.asarray(T).reshape(-1, 3, 3)
    if not len(T):
        return np.zeros(3)
    return 0.5 * np.cross(T[:, 1] - T[:, 0], T[:, 2] - T[:, 0]).sum(0)


def same_loops(ref, ours, where):
    """Per cell of `where` (the cell of each of our triangles): equal
    triangle counts, vertex sets and vector areas; returns the number of
    differing cells."""
    assert ref.shape == ours.shape
    keys = [tuple(w) for w in where]
    bounds = [0] + [i for i in range(1, len(keys)) if keys[i] != keys[i - 1]] + [len(keys)]
    bad = 0
    for a, b in zip(bounds[:-1], bounds[1:]):
        R, U = ref[a:b], ours[a:b]
        va, vb = _varea(R), _varea(U)
        # tolerance relative to the cell's total triangle area (a closed
        # loop set can have a near-zero vector area)
        scale = 0.5 * np.linalg.norm(np.cross(R[:, 1] - R[:, 0], R[:, 2] - R[:, 0]), axis=1).sum()
        if (set(map(tuple, R.reshape(-1, 3))) != set(map(tuple, U.reshape(-1, 3))) or
                np.abs(va - vb).max() > 1e-12 * max(scale, 1e-300)):
            bad += 1
    return bad


def stl_inputs(name, forest_cls):
    sc = pipeline.STL_CASES[name]
    case = pipeline.cases()[name]
    o = case["order"]
    f = forest_cls(o, case.get("interp", 1))
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
    X = pipeline.node_points(f.getOctants(), f.getMeshConn(o), s["num_dep"], s["num_local"], o,
                             knots, boxes)
    x = pipeline.stl_field(X[s["num_dep"]:], sc["vpn"])
    return sc, case, f, X, x


def _bface_brick(nx, ny, nz):
    """Boundary flags of the brick's block faces, from its geometry."""
    out = []
    for k in range(nz):
        for j in range(ny):
            for i in range(nx):
                out.append([i == 0, i == nx - 1, j == 0, j == ny - 1, k == 0, k == nz - 1])
    return np.array(out, bool)


@pytest.mark.parametrize("name", sorted(pipeline.STL_CASES))
def test_oracle_matches_reference_fixture(name):
    z = np.load(os.path.join(HERE, "golden", "api_stl.npz"))
    sc, case, f, X, x = stl_inputs(name, O.OracleForest)
    np.testing.assert_array_equal(f.getOctants(), z[name + "_octants"])
    tris, where = S.triangles(f.getOctants(), f.getMeshConn(case["order"]), f.getDepNodeConn(), X,
                              x, sc["vpn"], sc["offset"], sc["cutoff"], case["order"],
                              _bface_brick(*sc["grid"]), cells=True)
    ref = z[name + "_tris"]
    assert len(tris) == len(ref) > 100
    assert same_loops(ref, tris, where) == 0


def test_case_tables():
    vt, ft = S.volume_table(), S.face_table()
    assert vt[0] == [] and vt[255] == []
    assert max(len(t) for t in vt) <= 12
    # complementary cases cross the same edges; the loops of case c are
    # closed (every crossing used by an even number of triangle sides)
    for c in range(256):
        crossed = {e for e, (a, b) in enumerate(S.EDGE) if ((c >> a) & 1) != ((c >> b) & 1)}
        used = {e for t in vt[c] for e in t}
        assert used == crossed
    assert ft[0] == [(0, 1, 2), (0, 2, 3)] and ft[15] == []


@pytest.mark.skipif(not O.ref_available(), reason="reference build not present")
def test_every_cube_case_matches_reference():
    from tmr_gb300 import workloads as W
    f = O.RefForest(2, 1)
    f.setConnectivity(W.brick(1, 1, 1))
    f.createTrees(0)
    f.createNodes()
    mc = f.getMeshConn(2)
    X = np.zeros((8, 3))
    for t in range(8):
        X[mc[0, t]] = (t & 1, (t >> 1) & 1, (t >> 2) & 1)
    bface = np.ones((1, 6), bool)
    rng = np.random.default_rng(0)
    for c in range(256):
        vals = np.zeros(8)
        for m, (ii, jj, kk) in enumerate(S.CORNER):
            vals[mc[0, ii + 2 * jj + 4 * kk]] = (0.2 if (c >> m) & 1 else 0.8) + \
                0.05 * rng.uniform()
        ref = f.stlTriangles(X, vals, 1, 0, 0.5)
        ours, where = S.triangles(f.getOctants(), mc, f.getDepNodeConn(), X, vals, 1, 0, 0.5, 2,
                                  bface, cells=True)
        assert len(ref) == len(ours)
        if len(ours):
            assert same_loops(ref, ours, where) == 0, c


@pytest.mark.skipif(not O.ref_available(), reason="reference build not present")
def test_ascii_writer_matches_reference_converter(tmp_path):
    sc, case, f, X, x = stl_inputs("brick_o2", O.OracleForest)
    tris = S.triangles(f.getOctants(), f.getMeshConn(2), f.getDepNodeConn(), X, x, sc["vpn"],
                       sc["offset"], sc["cutoff"], 2, _bface_brick(*sc["grid"]))
    b = str(tmp_path / "t.bin")
    t = str(tmp_path / "t.stl")
    S.write_bin(b, tris[:300])
    L = O._lib("ref").lib
    import ctypes
    L.tmrref_convert_bin_to_stl.argtypes = [ctypes.c_char_p, ctypes.c_char_p]
    assert L.tmrref_convert_bin_to_stl(b.encode(), t.encode()) == 0
    with open(t) as fp:
        assert fp.read() == S.stl_ascii(tris[:300])
