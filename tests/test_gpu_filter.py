"""Matrix density filter on the GPU vs the CPU restatement, plus the
identities the reference documents (F 1 = 1, TMRMatrixFilter.h:48-49) and
the exactness of the hand-written adjoint."""
import ctypes

import numpy as np
import pytest

from tests import pipeline

R_FILTER = 0.08
N_TERMS = 10


def _oracle_filter(case):
    from oracle.oracle import OracleForest, _lib
    L = _lib("oracle").lib
    L.oo_filter_create.restype = ctypes.c_void_p
    L.oo_filter_create.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_double, ctypes.c_int]
    f = OracleForest(case["order"], 1)
    f.setConnectivity(case["conn"])
    f.createTrees(case["L0"])
    for p in range(case["passes"]):
        o = f.getOctants()
        f.refine(pipeline.indicator(o, case, p), 0, case["max_level"])
        f.balance(1)
    f.createNodes()
    F = L.oo_filter_create(ctypes.c_void_p(f.h), 1.0, R_FILTER, N_TERMS)
    return f, F, L


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["brick_o2", "rot_o2", "c1_small", "brick_o3", "rot_o4"])
def test_filter_matches_oracle(gpu_lib, name):
    # orders 3 and 4 use the quadratic / cubic Bernstein element mass and a
    # different (blocked) summation order on the GPU: M agrees to rounding
    import torch

    from tmr_gb300 import TMR
    case = pipeline.cases()[name]
    g = pipeline.run_gpu(dict(case, coarse_levels=0))
    F = TMR.MatrixFilter(R_FILTER, N_TERMS, None, [g["forests"][0]])
    of, OF, L = _oracle_filter(case)
    s = np.zeros(2, np.intc)
    L.oo_filter_sizes(ctypes.c_void_p(OF), _p(s))
    n, nnz = F.size()
    assert (n, nnz) == (s[0], s[1])
    rp, cols, vals, A, B, T = F.getMatrix()
    orp = np.zeros(n + 1, np.intc)
    oc = np.zeros(nnz, np.intc)
    ov = np.zeros(nnz)
    oA, oB, oT = np.zeros(n), np.zeros(n), np.zeros(n)
    L.oo_filter_get_matrix(ctypes.c_void_p(OF), _p(orp), _p(oc), _p(ov), _p(oA), _p(oB), _p(oT))
    np.testing.assert_array_equal(rp, orp)
    np.testing.assert_array_equal(cols, oc)
    np.testing.assert_allclose(vals, ov, rtol=1e-13, atol=1e-14 * np.abs(ov).max())
    np.testing.assert_allclose(A, oA, rtol=1e-13)
    np.testing.assert_allclose(B, oB, rtol=1e-13)
    np.testing.assert_allclose(T, oT, rtol=1e-13)
    # forward and adjoint on 3 interleaved components
    vpn = 3
    rng = np.random.default_rng(3)
    x = rng.random(n * vpn)
    y = np.zeros(n * vpn)
    F.applyFilter(x, y, vpn)
    yo = np.zeros(n * vpn)
    L.oo_filter_apply(ctypes.c_void_p(OF), vpn, _p(x), _p(yo))
    np.testing.assert_allclose(y, yo, rtol=1e-13, atol=1e-15)
    yt = np.zeros(n * vpn)
    F.applyTranspose(x, yt, vpn)
    yto = np.zeros(n * vpn)
    L.oo_filter_apply_t(ctypes.c_void_p(OF), vpn, _p(x), _p(yto))
    np.testing.assert_allclose(yt, yto, rtol=1e-13, atol=1e-15)
    # F 1 = 1 and <F x, z> = <x, F^T z>
    one = np.ones(n)
    f1 = np.zeros(n)
    F.applyFilter(one, f1, 1)
    np.testing.assert_allclose(f1, 1.0, rtol=1e-12)
    z = rng.standard_normal(n * vpn)
    fz = np.zeros(n * vpn)
    F.applyTranspose(z, fz, vpn)
    assert abs(np.dot(y, z) - np.dot(x, fz)) <= 1e-11 * np.abs(np.dot(y, z))
    # FP32 variant against FP64 (error stated, not a parity claim)
    xd = torch.tensor(x, dtype=torch.float32, device="cuda")
    yd = torch.empty_like(xd)
    F.applyFilter(xd, yd, vpn)
    err32 = np.abs(yd.cpu().numpy() - y).max() / np.abs(y).max()
    assert err32 < 1e-5, err32
    L.oo_filter_destroy(ctypes.c_void_p(OF))


@pytest.mark.gpu
def test_filter_interp_autograd_matches_fd(gpu_lib):
    import torch

    from tmr_gb300 import TMR
    from tmr_gb300.autograd import filter_interp
    case = pipeline.cases()["brick_o2"]
    g = pipeline.run_gpu(dict(case, coarse_levels=1))
    fine, coarse = g["forests"][0], g["forests"][1]
    F = TMR.MatrixFilter(R_FILTER, N_TERMS, None, [coarse])
    I = g["levels"][0]["I"]
    n, _ = F.size()
    rows, cols, _ = I.sizes()
    assert cols == n
    vpn = 1
    gen = torch.Generator(device="cpu").manual_seed(5)
    x = torch.rand(n * vpn, generator=gen, dtype=torch.float64).cuda().requires_grad_(True)
    w = torch.rand(rows * vpn, generator=gen, dtype=torch.float64).cuda()

    def obj(v):
        rho = filter_interp(v, F, I, vpn)
        return (w * rho ** 3).sum()

    J = obj(x)
    J.backward()
    gx = x.grad.detach()
    h = 1e-6
    for k in range(20):
        d = torch.randn(n * vpn, generator=gen, dtype=torch.float64).cuda()
        with torch.no_grad():
            fd = (obj(x + h * d) - obj(x - h * d)) / (2 * h)
        an = torch.dot(gx, d)
        assert abs(fd.item() - an.item()) <= 1e-6 * max(1.0, abs(an.item())), (k, fd.item(), an.item())


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["brick_o2", "nocorner_o2"])
def test_quad_filter_matches_restatement(gpu_lib, name):
    """The matrix filter on a quadtree forest (TMRMatrixFilter's
    TMRQuadForest constructor): M against the 2-D assembly of the Helmholtz
    oracle (bilinear mass through the dependent weights), Ainv and B by the
    reference's 2-D formulas (TMRMatrixFilter.cpp:133-137), and the apply
    against its Horner recurrence (:191-211)."""
    import scipy.sparse as sp

    from oracle import helmholtz as HO
    from tmr_gb300 import TMR
    case = pipeline.quad_golden_case(name)
    gold = pipeline.load_quad_golden(name)
    f = TMR.QuadForest(order=2, interp=case.get("interp", 1))
    f.setConnectivity(case["conn"])
    f.createTrees(case["L0"])
    for p in range(case["passes"]):
        f.refine(pipeline.indicator(f.getQuadrantsArray(), case, p), 0, case["max_level"])
        f.balance(case.get("corner", 1))
    f.createNodes()
    np.testing.assert_array_equal(f.getMeshConn(), gold["conn"])
    c = f.coarsen()
    c.balance(case.get("corner", 1))
    c.createNodes()
    F = TMR.MatrixFilter(R_FILTER, N_TERMS, None, [f, c])
    n, nnz = F.size()
    rp, cols, vals, A, B, T = F.getMatrix()
    M = sp.csr_matrix((vals, cols, rp), shape=(n, n))
    # square faces of side 1 (block_len): the box of face q is its own
    # unit square, in its own frame
    boxes = np.array([[0.0, 0.0, 1.0, 1.0]] * case["conn"].shape[0])
    dp, dc, dw = gold["dep"]
    _, Mo = HO.assemble2d(gold["quads"], gold["conn"], dp, dc, dw, n, 2,
                          np.array([-1.0, 1.0]), boxes, 0.0)
    assert abs(M - Mo).max() <= 1e-13 * abs(Mo).max()
    D = np.asarray(Mo.sum(axis=1)).ravel()
    r2 = R_FILTER * R_FILTER
    Ao = 1.0 / (1.0 + r2 / D)
    Bo = Ao * R_FILTER * R_FILTER / (D * D)
    np.testing.assert_allclose(A, Ao, rtol=1e-13)
    np.testing.assert_allclose(B, Bo, rtol=1e-13)

    def horner(x, Tinv):
        t1 = Ao * x
        out = t1.copy()
        for _ in range(N_TERMS):
            out = Bo * (Mo @ out) + t1
        return Tinv * out

    To = 1.0 / horner(np.ones(n), np.ones(n))
    np.testing.assert_allclose(T, To, rtol=1e-12)
    x = np.random.default_rng(2).uniform(0.0, 1.0, n)
    y = np.zeros(n)
    F.applyFilter(x, y)
    np.testing.assert_allclose(y, horner(x, To), rtol=1e-12)
    F.applyFilter(np.ones(n), y)
    np.testing.assert_allclose(y, 1.0, rtol=1e-12)
    w = np.random.default_rng(3).standard_normal(n)
    yt = np.zeros(n)
    F.applyTranspose(w, yt)
    assert w @ horner(x, To) == pytest.approx(yt @ x, rel=1e-11)


@pytest.mark.gpu
def test_filter_chain_c3_shape_fd_1000_directions(gpu_lib):
    """The differentiable filter -> prolongation chain on a reduced copy of
    the 16x8x8-brick, 16-bump configuration (vpn 3, r = 2 h_min, N = 10):
    the gradient of sum w rho^3 against central differences (h = 1e-6) in
    1000 seeded directions, and the backward pass (P^T then F^T) against
    the oracle's CSR transpose followed by the reference's applyTranspose
    recurrence restated in numpy on the library's M, Ainv, B, Tinv (M
    itself is checked against the oracle in test_filter_matches_oracle)."""
    import torch

    import bench
    from oracle.oracle import _lib
    from tmr_gb300 import TMR
    from tmr_gb300.autograd import filter_interp
    FW = dict(bench.FILTER_WORKLOAD, target=400_000, max_level=8)
    fine, coarse, I, F, r = bench.build_filter_chain(TMR, FW)
    vpn = FW["vpn"]
    n, _ = F.size()
    rows, cols, _ = I.sizes()
    assert cols == n and rows > 100_000
    gen = torch.Generator(device="cpu").manual_seed(11)
    x = torch.rand(n * vpn, generator=gen, dtype=torch.float64).cuda().requires_grad_(True)
    w = torch.rand(rows * vpn, generator=gen, dtype=torch.float64).cuda()

    def obj(v):
        return (w * filter_interp(v, F, I, vpn) ** 3).sum()

    J = obj(x)
    J.backward()
    gx = x.grad.detach()
    h = 1e-6
    # the central difference carries the roundoff of two sums of
    # rows * vpn terms: about eps * sum |w rho^3| / h, on top of the
    # O(h^2) truncation of the cubic objective
    with torch.no_grad():
        S = (w * filter_interp(x.detach(), F, I, vpn).abs() ** 3).sum().item()
    fd_noise = 4.0 * 2.2e-16 * S / h
    worst = 0.0
    with torch.no_grad():
        for k in range(1000):
            d = torch.randn(n * vpn, generator=gen, dtype=torch.float64).cuda()
            fd = ((obj(x + h * d) - obj(x - h * d)) / (2 * h)).item()
            an = torch.dot(gx, d).item()
            worst = max(worst, abs(fd - an) / (1e-7 * abs(an) + fd_noise))
    assert worst <= 1.0, worst
    # backward pass against the oracle: g = F^T (P^T gy)
    L = _lib("oracle").lib
    P_ = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    rp, pc, pv = I.getCSR()
    gy = (3.0 * w * filter_interp(x.detach(), F, I, vpn) ** 2).cpu().numpy()
    gp = np.zeros(cols * vpn)
    L.oo_csr_mult_t(rows, cols, P_(rp), P_(pc), P_(pv), vpn, P_(gy), P_(gp))
    frp, fc, fv, fA, fB, fT = F.getMatrix()
    gx_ref = _horner_t(frp, fc, fv, fA, fB, fT, N_TERMS, gp, vpn)
    np.testing.assert_allclose(gx.cpu().numpy(), gx_ref, rtol=1e-13,
                               atol=1e-13 * np.abs(gx_ref).max())


def _horner_t(rp, cols, vals, A, B, T, N, x, vpn):
    """TMRMatrixFilter::applyTranspose (TMRMatrixFilter.cpp:216-235) on the
    given matrices: t1 = T x, out = M (B out) + t1 N times, then A out."""
    import scipy.sparse as sp
    n = len(A)
    M = sp.csr_matrix((vals, cols, rp), shape=(n, n))
    X = x.reshape(n, vpn)
    t1 = T[:, None] * X
    out = t1.copy()
    for _ in range(N):
        out = M @ (B[:, None] * out) + t1
    return (A[:, None] * out).ravel()
