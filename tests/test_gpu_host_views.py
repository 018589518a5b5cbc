"""Borrowed host views (getOctants, getMeshConn(copy=False),
getDepNodeConn(copy=False)): page-locked copies owned by the forest that
match the copying getters and follow the forest through changes."""
import numpy as np
import pytest

from tmr_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _forest(TMR, order=3, passes=2):
    f = TMR.OctForest(order=order)
    f.setConnectivity(W.brick(2, 2, 1))
    f.createTrees(1)
    for p in range(passes):
        n = f.getNumOctants()
        f.refine(W.random_indicator(n, 11, p, 0.4), 0, 6)
        f.balance(1)
    return f


def test_views_match_copies(gpu_lib):
    from tmr_gb300 import TMR
    f = _forest(TMR)
    f.createNodes()
    v = f.getOctants()
    assert v.array.dtype.itemsize == 24
    np.testing.assert_array_equal(v.asArray7(), f.getOctantsArray())
    np.testing.assert_array_equal(f.getMeshConn(copy=False), f.getMeshConn())
    for a, b in zip(f.getDepNodeConn(copy=False), f.getDepNodeConn()):
        np.testing.assert_array_equal(a, b)
    with pytest.raises(ValueError):
        v[0] = v[1]


def test_views_follow_changes(gpu_lib):
    from tmr_gb300 import TMR
    f = _forest(TMR, passes=1)
    n0 = len(f.getOctants())
    f.refine(np.ones(n0, np.intc), 0, 6)  # child-0 seeds; balance adds siblings
    f.balance(1)
    v = f.getOctants()
    assert len(v) == f.getNumOctants() > n0
    np.testing.assert_array_equal(v.asArray7(), f.getOctantsArray())
    f.createNodes()
    c1 = np.array(f.getMeshConn(copy=False))
    f.setMeshOrder(2)
    f.createNodes()
    c2 = f.getMeshConn(copy=False)
    assert c2.shape == (f.getNumOctants(), 8) and c1.shape[1] == 27
    np.testing.assert_array_equal(c2, f.getMeshConn())


def test_pool_reuse_across_forests(gpu_lib):
    from tmr_gb300 import TMR
    sums = []
    for _ in range(3):
        f = _forest(TMR)
        f.createNodes()
        sums.append(int(f.getMeshConn(copy=False).astype(np.int64).sum()))
        del f
    assert sums[0] == sums[1] == sums[2]
    TMR.lib().tmrg_host_pool_trim()


def test_apply_into_page_locked_output(gpu_lib):
    """Host-buffer applies give the same values whether the output is
    pageable (copied back after the kernel) or page-locked (written by the
    kernel over the host link)."""
    import torch
    from tmr_gb300 import TMR
    f = _forest(TMR)
    f.createNodes()
    c = f.coarsen()
    c.balance(1)
    c.createNodes()
    I = TMR.VecInterp()
    f.createInterpolation(c, I)
    rows, cols, _ = I.sizes()
    nv = 4
    x = np.random.default_rng(5).standard_normal(cols * nv)
    xt = np.random.default_rng(6).standard_normal(rows * nv)
    y_page = np.zeros(rows * nv)
    y_pin = torch.zeros(rows * nv, dtype=torch.float64, pin_memory=True).numpy()
    I.mult(x, y_page)
    I.mult(x, y_pin)
    np.testing.assert_array_equal(y_page, y_pin)
    z_page = np.zeros(cols * nv)
    z_pin = torch.zeros(cols * nv, dtype=torch.float64, pin_memory=True).numpy()
    I.multTranspose(xt, z_page)
    I.multTranspose(xt, z_pin)
    np.testing.assert_array_equal(z_page, z_pin)


def test_staged_transpose_matches_device_apply(gpu_lib):
    """Host-input restriction (input copied in pieces overlapped with the
    rows they complete) equals the device-resident apply bit for bit."""
    import torch
    from tmr_gb300 import TMR
    f = _forest(TMR, passes=3)
    f.createNodes()
    c = f.coarsen()
    c.balance(1)
    c.createNodes()
    I = TMR.VecInterp()
    f.createInterpolation(c, I)
    rows, cols, _ = I.sizes()
    nv = 16
    x = np.random.default_rng(8).standard_normal(rows * nv)
    xd = torch.tensor(x, device="cuda")
    for name in ("multTranspose", "multWeightTranspose"):
        yd = torch.zeros(cols * nv, dtype=torch.float64, device="cuda")
        getattr(I, name)(xd, yd)
        y_page = np.zeros(cols * nv)
        getattr(I, name)(x, y_page)
        y_pin = torch.zeros(cols * nv, dtype=torch.float64, pin_memory=True).numpy()
        getattr(I, name)(x, y_pin)
        np.testing.assert_array_equal(y_page, yd.cpu().numpy())
        np.testing.assert_array_equal(y_pin, yd.cpu().numpy())
