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
