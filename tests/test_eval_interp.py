"""evalInterp (TMROctForest.cpp:1510-1631): the library's host evaluation
of the tensor-product bases and their derivatives against the reference's
own values (tests/golden/api.npz, written from the reference build by
tests/golden/make_golden.py), bit for bit, for orders 2-4 and uniform,
Gauss-Lobatto and Bernstein points.  Runs on the CPU: no GPU call."""
import ctypes
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def _lib():
    from tmr_gb300 import build
    build.build()
    from tmr_gb300 import _lib as L
    return L


def _P(a):
    return a.ctypes.data_as(ctypes.c_void_p)


@pytest.mark.parametrize("order", [2, 3, 4])
@pytest.mark.parametrize("itype", [0, 1, 2])
def test_eval_interp_matches_reference(order, itype):
    L = _lib()
    z = np.load(os.path.join(HERE, "golden", "api.npz"))
    kn = np.ascontiguousarray(z["ev_o%d_t%d_knots" % (order, itype)])
    n = order ** 3
    for ip, pt in enumerate(z["ev_points"]):
        pt = np.ascontiguousarray(pt)
        key = "ev_o%d_t%d_p%d" % (order, itype, ip)
        N = np.zeros(n)
        L.call("tmrg_eval_interp", order, itype, _P(kn), _P(pt), _P(N), None, None, None)
        np.testing.assert_array_equal(N, z[key + "_N"])
        d1 = [np.zeros(n) for _ in range(4)]
        L.call("tmrg_eval_interp", order, itype, _P(kn), _P(pt), *[_P(a) for a in d1])
        np.testing.assert_array_equal(np.stack(d1), z[key + "_d1"])
        d2 = [np.zeros(n) for _ in range(10)] + [np.full(n, -7.0)]
        L.call("tmrg_eval_interp2", order, itype, _P(kn), _P(pt), *[_P(a) for a in d2])
        np.testing.assert_array_equal(np.stack(d2), z[key + "_d2"])


def test_eval_interp_rejects_bad_order():
    L = _lib()
    pt = np.zeros(3)
    N = np.zeros(8)
    with pytest.raises(L.TMRGError):
        L.call("tmrg_eval_interp", 1, 1, _P(np.zeros(2)), _P(pt), _P(N), None, None, None)
