"""GPU path vs the CPU oracle on the same seeded forests: octants, conn,
node numbering and the dependent CSR bit-exact; dependent weights and P
within 1e-13 relative."""
import numpy as np
import pytest

from tests import pipeline

CASES = pipeline.cases()


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(CASES))
def test_pipeline_matches_oracle(gpu_lib, name):
    case = CASES[name]
    g = pipeline.run_gpu(case)
    o = pipeline.run_cpu(case, "oracle")
    bad = pipeline.compare(g, o)
    assert not bad, "\n".join(bad)


@pytest.mark.gpu
def test_interp_applies_match_oracle(gpu_lib):
    import torch

    from oracle.oracle import _lib
    case = CASES["brick_o3"]
    g = pipeline.run_gpu(case)
    L = _lib("oracle").lib
    for lev in g["levels"]:
        rp, cols, vals = lev["P"]
        I = lev["I"]
        rows, ncols, nnz = I.sizes()
        # the applies use the entries with |w| >= 2^-49 (a separate copy
        # when at least 1/8 of P is below that: for Gauss-Lobatto order 3
        # the rounding residue of the middle knot, about half of P); the
        # products below still agree with the full P to 1e-13
        kept = int((np.abs(vals) >= 2.0 ** -49).sum())
        assert I.applyNnz() == (kept if (nnz - kept) * 8 >= nnz else nnz)
        assert kept < 0.6 * nnz
        assert np.abs(vals[np.abs(vals) < 2.0 ** -49]).max(initial=0.0) < 1e-15
        k = 16
        rng = np.random.default_rng(7)
        x = rng.standard_normal(ncols * k)
        xf = rng.standard_normal(rows * k)
        import ctypes
        P = lambda a: a.ctypes.data_as(ctypes.c_void_p)
        y_ref = np.zeros(rows * k)
        L.oo_csr_mult(rows, P(rp), P(cols), P(vals), k, P(x), P(y_ref))
        yt_ref = np.zeros(ncols * k)
        L.oo_csr_mult_t(rows, ncols, P(rp), P(cols), P(vals), k, P(xf), P(yt_ref))
        yw_ref = np.zeros(ncols * k)
        L.oo_csr_mult_wt(rows, ncols, P(rp), P(cols), P(vals), k, P(xf), P(yw_ref))
        # host-buffer path
        y = np.zeros(rows * k)
        I.mult(x, y)
        np.testing.assert_allclose(y, y_ref, rtol=1e-13, atol=1e-13)
        yt = np.zeros(ncols * k)
        I.multTranspose(xf, yt)
        np.testing.assert_allclose(yt, yt_ref, rtol=1e-13, atol=1e-13)
        yw = np.zeros(ncols * k)
        I.multWeightTranspose(xf, yw)
        np.testing.assert_allclose(yw, yw_ref, rtol=1e-13, atol=1e-13)
        # device-pointer path, one vector
        xd = torch.tensor(x[:ncols], device="cuda")
        yd = torch.empty(rows, dtype=torch.float64, device="cuda")
        I.mult(xd, yd)
        y1 = np.zeros(rows)
        L.oo_csr_mult(rows, P(rp), P(cols), P(vals), 1, P(np.ascontiguousarray(x[:ncols])), P(y1))
        np.testing.assert_allclose(yd.cpu().numpy(), y1, rtol=1e-13, atol=1e-13)
        # properties: P 1 = 1 (Lagrange prolongation), <Px, y> = <x, P^T y>
        ones = np.ones(ncols)
        p1 = np.zeros(rows)
        I.mult(ones, p1)
        np.testing.assert_allclose(p1, 1.0, rtol=1e-12)
        a = np.dot(y_ref, xf)
        b = np.dot(x, yt_ref)
        assert abs(a - b) <= 1e-10 * max(1.0, abs(a))


@pytest.mark.gpu
def test_bench_sample_matches_oracle(gpu_lib):
    # the multi-tree order-3 bench workload's CPU sample (its first 2 of 5
    # refinement passes, 4-level hierarchy, ~140k octants), the case the
    # CPU baseline times: GPU and oracle agree bit for bit on octants,
    # conn, node numbers and the dependent CSR, P within 1e-13
    import bench
    case = bench.cpu_sample_case()
    g = pipeline.run_gpu(case)
    o = pipeline.run_cpu(case, "oracle")
    assert len(g["oct"]) > 50000
    bad = pipeline.compare(g, o)
    assert not bad, "\n".join(bad)


@pytest.mark.gpu
def test_device_refinement_draws_match_host(gpu_lib):
    # the bench's resident arm draws its refinement flags on the device, the
    # host-buffer arm and every CPU checker on the host: the same bits
    from tmr_gb300 import TMR
    from tmr_gb300 import workloads as W
    for n, seed, stream, prob in [(1, 7, 0, 0.3), (1000003, 7, 4, 0.3), (65536, 3, 1, 0.5),
                                  (12345, 21, 2, 0.0), (777, 9, 3, 1.0)]:
        d = TMR.random_refinement(n, seed, stream, prob).cpu().numpy()
        np.testing.assert_array_equal(d, W.random_indicator(n, seed, stream, prob))


@pytest.mark.gpu
def test_host_buffer_applies_in_pieces(gpu_lib):
    # the host-buffer prolongation computed in row pieces whose copies back
    # overlap the next piece (P with more than 16 x 4096 rows), and the
    # restriction whose input arrives in pieces: the same values as the
    # device-pointer applies (same kernel and shape) and the oracle's CSR
    import ctypes

    import bench
    import torch

    from oracle.oracle import _lib
    case = bench.cpu_sample_case()
    g = pipeline.run_gpu(dict(case, coarse_levels=1))
    I = g["levels"][0]["I"]
    rows, ncols, _ = I.sizes()
    assert rows > 16 * 4096
    k = 16
    rng = np.random.default_rng(12)
    x = rng.standard_normal(ncols * k)
    xd = torch.tensor(x, device="cuda")
    yd = torch.empty(rows * k, dtype=torch.float64, device="cuda")
    I.mult(xd, yd)  # the device apply (tunes the shape of this size class)
    yh = torch.empty(rows * k, dtype=torch.float64, pin_memory=True).numpy()
    I.mult(x, yh)
    np.testing.assert_array_equal(yh, yd.cpu().numpy())
    y_pageable = np.zeros(rows * k)
    I.mult(x, y_pageable)
    np.testing.assert_array_equal(y_pageable, yh)
    rp, cols, vals = I.getCSR()
    L = _lib("oracle").lib
    P_ = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    y_ref = np.zeros(rows * k)
    L.oo_csr_mult(rows, P_(rp), P_(cols), P_(vals), k, P_(x), P_(y_ref))
    np.testing.assert_allclose(yh, y_ref, rtol=1e-13, atol=1e-13)
    xf = rng.standard_normal(rows * k)
    yt_ref = np.zeros(ncols * k)
    L.oo_csr_mult_t(rows, ncols, P_(rp), P_(cols), P_(vals), k, P_(xf), P_(yt_ref))
    yt = np.zeros(ncols * k)
    I.multTranspose(xf, yt)
    np.testing.assert_allclose(yt, yt_ref, rtol=1e-13, atol=1e-13)


@pytest.mark.gpu
def test_every_apply_shape_matches_oracle(gpu_lib):
    # each launch shape the autotuner may pick, forced on the P and P^T
    # applies (device pointers and the host-buffer pieces): the oracle's CSR
    # products to 1e-13, and the TMA-staged shape (6) the same bits as the
    # shape whose entry order it follows (4: 2 lanes x 4 pairs)
    import ctypes

    import bench
    import torch

    from oracle.oracle import _lib
    from tmr_gb300 import TMR
    case = bench.cpu_sample_case()
    g = pipeline.run_gpu(dict(case, coarse_levels=1))
    I = g["levels"][0]["I"]
    rows, ncols, _ = I.sizes()
    k = 16
    rng = np.random.default_rng(31)
    x = rng.standard_normal(ncols * k)
    xf = rng.standard_normal(rows * k)
    rp, cols, vals = I.getCSR()
    L = _lib("oracle").lib
    P_ = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    y_ref = np.zeros(rows * k)
    L.oo_csr_mult(rows, P_(rp), P_(cols), P_(vals), k, P_(x), P_(y_ref))
    yt_ref = np.zeros(ncols * k)
    L.oo_csr_mult_t(rows, ncols, P_(rp), P_(cols), P_(vals), k, P_(xf), P_(yt_ref))
    lib = TMR.lib()
    xd = torch.tensor(x, device="cuda")
    xfd = torch.tensor(xf, device="cuda")
    out = {}
    try:
        for shape in range(7):
            assert lib.tmrg_tune_force(1, shape) == 0 and lib.tmrg_tune_force(2, shape) == 0
            yd = torch.empty(rows * k, dtype=torch.float64, device="cuda")
            I.mult(xd, yd)
            ytd = torch.empty(ncols * k, dtype=torch.float64, device="cuda")
            I.multTranspose(xfd, ytd)
            yh = np.zeros(rows * k)
            I.mult(x, yh)  # pieces with copies back
            yth = np.zeros(ncols * k)
            I.multTranspose(xf, yth)  # input in pieces
            y, yt = yd.cpu().numpy(), ytd.cpu().numpy()
            np.testing.assert_allclose(y, y_ref, rtol=1e-13, atol=1e-13, err_msg="P %d" % shape)
            np.testing.assert_allclose(yt, yt_ref, rtol=1e-13, atol=1e-13,
                                       err_msg="PT %d" % shape)
            np.testing.assert_array_equal(yh, y)
            np.testing.assert_allclose(yth, yt_ref, rtol=1e-13, atol=1e-13)
            out[shape] = (y, yt)
    finally:
        lib.tmrg_tune_force(1, -1)
        lib.tmrg_tune_force(2, -1)
    np.testing.assert_array_equal(out[6][0], out[4][0])
    np.testing.assert_array_equal(out[6][1], out[4][1])


@pytest.mark.gpu
def test_applies_outside_double_float_window(gpu_lib):
    # inputs the double-float pairs cannot hold (|x| < 2^-40 or >= 2^60) send
    # the applies to FP64: device and host-buffer P and P^T still match the
    # oracle's CSR within 1e-13, including the host-buffer paths that split
    # their input in pieces (a piece with such a value switches the rows
    # computed after it)
    import ctypes

    import bench
    import torch

    from oracle.oracle import _lib
    case = bench.cpu_sample_case()
    g = pipeline.run_gpu(dict(case, coarse_levels=1))
    I = g["levels"][0]["I"]
    rows, ncols, _ = I.sizes()
    assert rows > 16 * 4096
    k = 16
    rp, cols, vals = I.getCSR()
    L = _lib("oracle").lib
    P_ = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    rng = np.random.default_rng(31)
    for scale, tiny in ((1.0, True), (1e30, False)):
        x = rng.standard_normal(ncols * k) * scale
        xf = rng.standard_normal(rows * k) * scale
        if tiny:
            # a few values below the window in the last input pieces
            x[-5 * k::k] = 1e-20
            xf[-7 * k::k] = -3e-19
        y_ref = np.zeros(rows * k)
        L.oo_csr_mult(rows, P_(rp), P_(cols), P_(vals), k, P_(x), P_(y_ref))
        yt_ref = np.zeros(ncols * k)
        L.oo_csr_mult_t(rows, ncols, P_(rp), P_(cols), P_(vals), k, P_(xf), P_(yt_ref))
        yd = torch.empty(rows * k, dtype=torch.float64, device="cuda")
        I.mult(torch.tensor(x, device="cuda"), yd)
        ytd = torch.empty(ncols * k, dtype=torch.float64, device="cuda")
        I.multTranspose(torch.tensor(xf, device="cuda"), ytd)
        yh = torch.empty(rows * k, dtype=torch.float64, pin_memory=True).numpy()
        I.mult(x, yh)
        yth = np.zeros(ncols * k)
        I.multTranspose(xf, yth)
        for got, ref, what in ((yd.cpu().numpy(), y_ref, "P device"), (yh, y_ref, "P host"),
                               (ytd.cpu().numpy(), yt_ref, "PT device"),
                               (yth, yt_ref, "PT host")):
            np.testing.assert_allclose(got / scale, ref / scale, rtol=1e-13, atol=1e-13,
                                       err_msg="%s, scale %g" % (what, scale))
