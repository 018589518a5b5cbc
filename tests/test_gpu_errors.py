"""Error behaviour of the C ABI: every failure is a status code with a
message (the reference prints to stderr and returns, TMROctForest.cpp:
2919-2922, 4066-4069); the forest stays usable afterwards."""
import numpy as np
import pytest

from tmr_gb300 import workloads as W


@pytest.mark.gpu
def test_error_statuses_and_recovery(gpu_lib):
    from tmr_gb300 import TMR
    from tmr_gb300._lib import TMRGError

    f = TMR.OctForest(order=2)
    with pytest.raises(TMRGError) as e:
        f.createTrees(1)  # no connectivity yet
    assert e.value.status == 2
    f.setConnectivity(W.brick(2, 1, 1))
    with pytest.raises(TMRGError) as e:
        f.balance(1)  # no octants yet
    assert e.value.status == 2 and "balance" in str(e.value)
    f.createTrees(2)
    n = f.getNumOctants()
    with pytest.raises(TMRGError) as e:
        f.refine(np.ones(n + 1, np.intc))  # wrong length
    assert e.value.status == 1
    # unchanged after the failed refine
    assert f.getNumOctants() == n
    with pytest.raises(ValueError):
        f.setConnectivity(np.zeros((2, 7), np.intc))
    with pytest.raises(TMRGError):
        f.setConnectivity(np.array([[0, 1, 2, 3, 4, 5, 6, 99]], np.intc) - 100)
    # still usable
    f.refine(np.ones(n, np.intc), 0, 4)
    f.balance(1)
    f.createNodes()
    assert f.getMeshConn().shape == (f.getNumOctants(), 8)
    with pytest.raises(ValueError):
        f.createInterpolation(f, TMR.VecInterp())
    # Bernstein elements of order 6: the reference tabulates dependent
    # weights for orders 2-5 only (eval_bernstein_weights)
    b = TMR.OctForest(order=6, interp=TMR.BERNSTEIN_POINTS)
    b.setConnectivity(W.brick(1, 1, 1))
    b.createTrees(1)
    with pytest.raises(TMRGError) as e:
        b.createNodes()
    assert e.value.status == 6
    # Bernstein meshes two orders apart (the reference's degree-elevation
    # table covers one order)
    b4 = TMR.OctForest(order=4, interp=TMR.BERNSTEIN_POINTS)
    b4.setConnectivity(W.brick(1, 1, 1))
    b4.createTrees(1)
    b4.createNodes()
    b2 = b4.duplicate()
    b2.setMeshOrder(2, TMR.BERNSTEIN_POINTS)
    b2.createNodes()
    with pytest.raises(TMRGError) as e:
        b4.createInterpolation(b2, TMR.VecInterp())
    assert e.value.status == 6
    # matrix filter on an order-5 forest (no element basis in the reference)
    f5 = TMR.OctForest(order=5)
    f5.setConnectivity(W.brick(1, 1, 1))
    f5.createTrees(1)
    with pytest.raises(TMRGError) as e:
        TMR.MatrixFilter(0.1, 10, None, [f5])
    assert e.value.status == 6


@pytest.mark.gpu
def test_empty_and_edge_inputs(gpu_lib):
    from tmr_gb300 import TMR
    f = TMR.OctForest(order=2)
    f.setConnectivity(W.brick(1, 1, 1))
    f.createTrees(0)  # one level-0 octant
    f.balance(1)
    assert f.getNumOctants() == 1
    f.createNodes()
    assert f.getMeshConn().shape == (1, 8)
    ptr, conn, w = f.getDepNodeConn()
    assert len(ptr) == 1 and len(conn) == 0
    # refine nothing / coarsen everything at level 0 are no-ops
    f.refine(np.zeros(1, np.intc))
    assert f.getNumOctants() == 1
    f.refine(-np.ones(1, np.intc))
    assert f.getNumOctants() == 1
    c = f.coarsen()
    assert c.getNumOctants() == 1
    # refine with no array refines everything by one level
    f.refine(None)
    f.balance(0)
    assert f.getNumOctants() == 8
    # maximum refinement level clamps
    f.refine(np.full(8, 40, np.intc), 0, 2)
    o = f.getOctantsArray()
    assert o[:, 5].max() == 2


@pytest.mark.gpu
def test_device_octant_views_match_host_copy(gpu_lib):
    from tmr_gb300 import TMR
    f = TMR.OctForest(order=2)
    f.setConnectivity(W.brick(2, 2, 1))
    f.createTrees(2)
    f.refine(TMR.random_refinement(f.getNumOctants(), 5, 0, 0.4), 0, 5)
    f.balance(1)
    d = f.getOctantsDevice()
    h = f.getOctantsArray()
    for k, col in (("block", 0), ("x", 1), ("y", 2), ("z", 3), ("level", 5), ("info", 6)):
        assert np.array_equal(d[k].cpu().numpy().astype(np.int64), h[:, col].astype(np.int64)), k
