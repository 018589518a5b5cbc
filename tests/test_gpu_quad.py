"""The quadtree twin on the GPU against the reference's own TMRQuadForest
results (tests/golden/quad_*.npz): quadrants, element connectivity and
dependent rows bit-exact, dependent weights and P within 1e-13 relative;
then the applies of P on device vectors."""
import numpy as np
import pytest

from tests import pipeline

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", pipeline.quad_golden_names())
def test_quad_pipeline_matches_reference(gpu_lib, name):
    g = pipeline.run_quad_gpu(pipeline.quad_golden_case(name))
    bad = pipeline.compare_quad(g, pipeline.load_quad_golden(name))
    assert bad == [], "; ".join(bad)


def test_quad_applies_and_api(gpu_lib):
    import torch
    from tmr_gb300 import TMR
    case = pipeline.quad_golden_case("brick_o3")
    f = TMR.QuadForest(order=3)
    f.setConnectivity(case["conn"])
    f.createTrees(2)
    f.refine(np.ones(f.getNumQuadrants(), np.intc), 0, 5)
    f.balance(1)
    f.createNodes()
    c = f.coarsen()
    c.balance(1)
    c.createNodes()
    I = TMR.VecInterp()
    f.createInterpolation(c, I)
    rows, cols, nnz = I.sizes()
    one = torch.ones(cols * 2, dtype=torch.float64, device="cuda")
    y = torch.empty(rows * 2, dtype=torch.float64, device="cuda")
    I.mult(one, y)
    np.testing.assert_allclose(y.cpu().numpy(), 1.0, rtol=1e-12)
    x = torch.rand(rows, dtype=torch.float64, device="cuda")
    z = torch.rand(cols, dtype=torch.float64, device="cuda")
    px = torch.empty(rows, dtype=torch.float64, device="cuda")
    ptz = torch.empty(cols, dtype=torch.float64, device="cuda")
    I.mult(z, px)
    I.multTranspose(x, ptz)
    assert float(x @ px) == pytest.approx(float(z @ ptz), rel=1e-12)
    # connectivity getters, evalInterp, points
    fc, fe, nn, ne = f.getConnectivity()
    np.testing.assert_array_equal(fc, case["conn"])
    assert ne == 17 and nn == 12
    N = f.evalInterp([0.3, -0.2])
    assert N.shape == (9,) and abs(N.sum() - 1.0) < 1e-14
    boxes = np.array([[i, j, 1.0, 1.0] for j in range(2) for i in range(3)], float)
    f.setFaceBoxes(boxes)
    X = f.getPoints()
    assert X.shape == (f._sizes()[0], 3) and X[:, 2].max() == 0.0
    assert 0.0 <= X[:, 0].min() and X[:, 0].max() <= 3.0


def _morton2_key(q):
    """Sort key of TMRQuadrant::compare: face, then the x-most-significant
    interleave of the coordinates, then the level."""
    f, x, y, lev = (int(v) for v in q)
    m = 0
    for bit in range(29, -1, -1):
        m = (m << 2) | (((x >> bit) & 1) << 1) | ((y >> bit) & 1)
    return (f, m, lev)


@pytest.mark.gpu
def test_quad_random_trees_match_restatement(gpu_lib):
    from tmr_gb300 import TMR
    from tmr_gb300 import workloads as W
    conn = W.brick2d(3, 2)
    nrand, lo, hi, seed = 60, 1, 7, 23
    f = TMR.QuadForest(order=2)
    f.setConnectivity(conn)
    f.createRandomTrees(nrand, lo, hi, seed)
    got = f.getQuadrantsArray()
    # restatement: U(seed, face, 3i + k) draws, sort, keep the finest per position
    cand = []
    for face in range(conn.shape[0]):
        u = W.uniform(seed, face, 3 * nrand)
        for i in range(nrand):
            lev = min(lo + int(u[3 * i] * (hi - lo + 1)), hi)
            h = 1 << (30 - lev)
            xy = [h * min(int(u[3 * i + 1 + k] * (1 << lev)), (1 << lev) - 1) for k in range(2)]
            cand.append((face, *xy, lev))
    cand.sort(key=_morton2_key)
    keep = [c for i, c in enumerate(cand)
            if i + 1 == len(cand) or _morton2_key(cand[i + 1])[:2] != _morton2_key(c)[:2]]
    exp = np.array([[c[0], c[1], c[2], i, c[3], 0] for i, c in enumerate(keep)], np.intc)
    np.testing.assert_array_equal(got, exp)


@pytest.mark.gpu
def test_quad_vtk_writers(gpu_lib, tmp_path):
    """writeToVTK: the face mesh, nodes at their owner face's corner through
    the face boxes, cells in the reference's (0 1 3 2) corner order;
    writeForestToVTK: four corners per quadrant (x fastest); both write
    nothing without face boxes."""
    from tmr_gb300 import TMR
    from tmr_gb300 import workloads as W
    conn = W.rotate_faces(W.brick2d(3, 2), 4)
    f = TMR.QuadForest(order=2)
    f.setConnectivity(conn)
    f.createTrees(2)
    fa, fq = tmp_path / "faces.vtk", tmp_path / "quads.vtk"
    f.writeToVTK(str(fa))
    f.writeForestToVTK(str(fq))
    assert not fa.exists() and not fq.exists()
    boxes = np.array([[i % 3, i // 3, 1.0, 1.0] for i in range(6)], np.float64)
    f.setFaceBoxes(boxes)
    f.writeToVTK(str(fa))
    f.writeForestToVTK(str(fq))
    lines = fa.read_text().split("\n")
    nn = int(conn.max()) + 1
    i = lines.index("POINTS %d float" % nn)
    pts = np.array([[float(v) for v in ln.split()] for ln in lines[i + 1:i + 1 + nn]])
    for k in range(nn):
        face = min(np.argwhere(conn == k)[:, 0])
        c = int(np.argwhere(conn[face] == k)[0, 0])
        np.testing.assert_allclose(pts[k, :2], boxes[face, :2] + boxes[face, 2:] *
                                   np.array([c & 1, c >> 1]), rtol=1e-6)
    j = lines.index("CELLS 6 30")
    cells = np.array([[int(v) for v in ln.split()] for ln in lines[j + 1:j + 7]])
    np.testing.assert_array_equal(cells[:, 1:], conn[:, [0, 1, 3, 2]])
    q = f.getQuadrantsArray()
    n = len(q)
    lines = fq.read_text().split("\n")
    i = lines.index("POINTS %d float" % (4 * n))
    pts = np.array([[float(v) for v in ln.split()] for ln in lines[i + 1:i + 1 + 4 * n]])
    h = (1 << (30 - q[:, 4].astype(np.int64))) / 2.0 ** 30
    for k in (0, n // 2, n - 1):
        b = boxes[q[k, 0]]
        for c in range(4):
            u = q[k, 1:3] / 2.0 ** 30 + h[k] * np.array([c & 1, c >> 1])
            np.testing.assert_allclose(pts[4 * k + c, :2], b[:2] + b[2:] * u, rtol=1e-6)
    e = lines.index("SCALARS entity_index float 1")
    np.testing.assert_array_equal(np.array([float(v) for v in lines[e + 2:e + 2 + n]]), q[:, 0])
