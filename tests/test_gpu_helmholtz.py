"""Helmholtz PDE filter on the GPU against the CPU restatement
(oracle/helmholtz.py: restated element integrals, assembled sparse K and M,
direct solve) on the reference's own forests (tests/golden fixtures).

Tolerances: the operators K x and M x agree to 1e-12 relative (FP64
sums in a different order); the filtered fields to 1e-9 relative (the
GPU solve stops at a residual of 1e-12 |b|, as the reference's GMRES
does, and the error is at most cond(K) times that)."""
import numpy as np
import pytest

from oracle import helmholtz as HO
from tests import pipeline

pytestmark = pytest.mark.gpu

EXT = (1.0, 0.75, 0.5)


def brick_boxes(nx, ny, nz, ext=EXT):
    """Block boxes of W.brick(nx, ny, nz): block (i, j, k), x fastest."""
    boxes = []
    for k in range(nz):
        for j in range(ny):
            for i in range(nx):
                boxes.append([i * ext[0], j * ext[1], k * ext[2], *ext])
    return np.array(boxes)


_cache = {}


def _setup(name, r):
    key = (name, r)
    if key in _cache:
        return _cache[key]
    from tmr_gb300 import TMR
    case = pipeline.golden_case(name)
    gold = pipeline.load_golden(name)
    out = pipeline.run_gpu(case)
    np.testing.assert_array_equal(out["oct"], gold["oct"])
    np.testing.assert_array_equal(out["conn"], gold["conn"])
    forests = out["forests"]
    boxes = brick_boxes(3, 2, 2)
    for f in forests:
        f.setBlockBoxes(boxes)
    Hf = TMR.HelmholtzFilter(r, None, forests)
    n = gold["sizes"]["num_owned"]
    dp, dc, dw = gold["dep"]
    K, M = HO.assemble(gold["oct"], gold["conn"], dp, dc, dw, n, case["order"],
                       forests[0].getInterpKnots(), boxes, r)
    _cache[key] = (forests, Hf, K, M, n)
    return _cache[key]


def _rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


@pytest.mark.parametrize("name", ["brick_o2", "brick_o3"])
def test_operators_match_oracle(gpu_lib, name):
    import torch
    forests, Hf, K, M, n = _setup(name, 0.15)
    x = np.random.default_rng(3).standard_normal(n)
    xd = torch.tensor(x, device="cuda")
    y = torch.empty_like(xd)
    Hf.mult(0, 0, xd, y)
    assert _rel(y.cpu().numpy(), K @ x) <= 1e-12
    Hf.mult(0, 1, xd, y)
    assert _rel(y.cpu().numpy(), M @ x) <= 1e-12
    # K 1 = M 1 on every level
    for lev, (nn, _, _, _) in enumerate(Hf.sizes()):
        one = torch.ones(int(nn), dtype=torch.float64, device="cuda")
        a = torch.empty_like(one)
        b = torch.empty_like(one)
        Hf.mult(lev, 0, one, a)
        Hf.mult(lev, 1, one, b)
        assert (a - b).abs().max().item() <= 1e-13 * b.abs().max().item()


@pytest.mark.parametrize("name", ["brick_o2", "brick_o3"])
@pytest.mark.parametrize("r", [0.05, 0.3])
def test_filter_matches_direct_solve(gpu_lib, name, r):
    forests, Hf, K, M, n = _setup(name, r)
    x = np.random.default_rng(5).uniform(0.0, 1.0, n)
    y = np.zeros(n)
    Hf.applyFilter(x, y)
    exp = HO.apply_filter(K, M, x)
    assert _rel(y, exp) <= 1e-9
    it, res = Hf.lastSolve()
    assert 1 <= it <= 60
    assert res[0] <= 1e-12 * np.linalg.norm(M @ x)
    yt = np.zeros(n)
    Hf.applyTranspose(x, yt)
    assert _rel(yt, HO.apply_transpose(K, M, x)) <= 1e-9


def test_constants_adjoint_and_components(gpu_lib):
    import torch
    forests, Hf, K, M, n = _setup("brick_o2", 0.3)
    one = np.ones(n)
    y = np.zeros(n)
    Hf.applyFilter(one, y)
    np.testing.assert_allclose(y, 1.0, rtol=1e-10)
    rng = np.random.default_rng(11)
    x, w = rng.standard_normal(n), rng.standard_normal(n)
    fx, ftw = np.zeros(n), np.zeros(n)
    Hf.applyFilter(x, fx)
    Hf.applyTranspose(w, ftw)
    assert w @ fx == pytest.approx(ftw @ x, rel=1e-10)
    # three interleaved components solved together = one at a time (device)
    X = rng.standard_normal((n, 3))
    Y = torch.empty(n * 3, dtype=torch.float64, device="cuda")
    Hf.applyFilter(torch.tensor(X.ravel(), device="cuda"), Y, vpn=3)
    Y = Y.cpu().numpy().reshape(n, 3)
    for c in range(3):
        yc = np.zeros(n)
        Hf.applyFilter(np.ascontiguousarray(X[:, c]), yc)
        assert _rel(Y[:, c], yc) <= 1e-10
    # setDesignVars: the finest level is the filtered field
    lv = Hf.setDesignVars(x)
    assert len(lv) == len(forests)
    assert _rel(lv[0], fx) <= 1e-12


def test_single_level_dense_solve(gpu_lib):
    from tmr_gb300 import TMR
    forests, _, _, _, _ = _setup("brick_o2", 0.3)
    coarse = forests[-1]
    Hf = TMR.HelmholtzFilter(0.3, None, [coarse])
    n = int(Hf.sizes()[0][0])
    assert n <= 2048
    x = np.random.default_rng(2).standard_normal(n)
    y = np.zeros(n)
    Hf.applyFilter(x, y)
    it, _ = Hf.lastSolve()
    assert it <= 2


def test_no_geometry_is_an_error(gpu_lib):
    from tmr_gb300 import TMR
    f = TMR.OctForest(order=2)
    from tmr_gb300 import workloads as W
    f.setConnectivity(W.brick(2, 1, 1))
    f.createTrees(1)
    f.createNodes()
    with pytest.raises(TMR._lib.TMRGError, match="geometry"):
        TMR.HelmholtzFilter(0.1, None, [f])


def _quad_forests(name):
    """The quadtree forests of a quad fixture case (finest first), checked
    against the fixture's mesh."""
    from tmr_gb300 import TMR
    case = pipeline.quad_golden_case(name)
    gold = pipeline.load_quad_golden(name)
    f = TMR.QuadForest(order=case["order"], interp=case.get("interp", 1))
    f.setConnectivity(case["conn"])
    f.createTrees(case["L0"])
    for p in range(case["passes"]):
        f.refine(pipeline.indicator(f.getQuadrantsArray(), case, p), 0, case["max_level"])
        f.balance(case.get("corner", 1))
    f.createNodes()
    np.testing.assert_array_equal(f.getMeshConn(), gold["conn"])
    forests = [f]
    for _ in range(case.get("coarse_levels", 1)):
        c = forests[-1].coarsen()
        c.balance(case.get("corner", 1))
        c.createNodes()
        forests.append(c)
    return case, gold, forests


# faces per row / column of the brick2d grids of the quad fixtures
QUAD_GRID = {"brick_o2": (4, 3), "brick_o3": (3, 2)}


@pytest.mark.parametrize("name", ["brick_o2", "brick_o3"])
@pytest.mark.parametrize("r", [0.02, 0.1])
def test_quad_filter_matches_direct_solve(gpu_lib, name, r):
    """The 2-D filter on the reference's quadtree forests: K x, M x and
    the filtered field against the assembled direct solve."""
    import torch
    from tmr_gb300 import TMR
    case, gold, forests = _quad_forests(name)
    nx, ny = QUAD_GRID[name]
    boxes = np.array([[i * 1.0, j * 0.6, 1.0, 0.6] for j in range(ny) for i in range(nx)])
    for g in forests:
        g.setFaceBoxes(boxes)
    Hf = TMR.HelmholtzFilter(r, None, forests)
    sizes = Hf.sizes()
    assert len(sizes) == len(forests)
    n = int(sizes[0][0])
    dp, dc, dw = gold["dep"]
    K, M = HO.assemble2d(gold["quads"], gold["conn"], dp, dc, dw, n, case["order"],
                         forests[0].getInterpKnots(), boxes, r)
    rng = np.random.default_rng(4)
    x = rng.standard_normal(n)
    xd = torch.tensor(x, device="cuda")
    y = torch.empty_like(xd)
    Hf.mult(0, 0, xd, y)
    assert _rel(y.cpu().numpy(), K @ x) <= 1e-12
    Hf.mult(0, 1, xd, y)
    assert _rel(y.cpu().numpy(), M @ x) <= 1e-12
    u = rng.uniform(0.0, 1.0, n)
    out = np.zeros(n)
    Hf.applyFilter(u, out)
    assert _rel(out, HO.apply_filter(K, M, u)) <= 1e-9
    it, res = Hf.lastSolve()
    assert 1 <= it <= 60
    Hf.applyTranspose(u, out)
    assert _rel(out, HO.apply_transpose(K, M, u)) <= 1e-9
    Hf.applyFilter(np.ones(n), out)
    np.testing.assert_allclose(out, 1.0, rtol=1e-10)
