"""The CPU restatement of the Helmholtz filter (oracle/helmholtz.py) against
known answers: closed-form element matrices of the trilinear cube, the
quadratic Bernstein mass matrix, and the exact properties of the assembled
operators on a reference fixture (tests/golden/brick_o2.npz)."""
import os

import numpy as np
import pytest

from oracle import helmholtz as H

HERE = os.path.dirname(os.path.abspath(__file__))


def _cube(order, h):
    X = np.zeros((order ** 3, 3))
    t = np.linspace(0.0, h, order)
    for k in range(order):
        for j in range(order):
            for i in range(order):
                X[i + order * j + order * order * k] = (t[i], t[j], t[k])
    return X


def test_trilinear_cube_matrices_closed_form():
    h, r = 0.5, 0.3
    Ke, Me = H.element_matrices(_cube(2, h), 2, r)
    for a in range(8):
        for b in range(8):
            nd = bin(a ^ b).count("1")
            # mass: h^3 / 27 / 2^nd
            assert Me[a, b] == pytest.approx(h ** 3 / 27.0 / 2 ** nd, rel=1e-14)
            # Laplacian of the trilinear cube: h/3 on the diagonal, 0 across a
            # face diagonal... the 1-D factors are K1 = [1,-1;-1,1]/h and
            # M1 = h [2,1;1,2]/6, summed over the three directions
            lap = 0.0
            for d in range(3):
                f = 1.0
                for c in range(3):
                    same = ((a >> c) & 1) == ((b >> c) & 1)
                    if c == d:
                        f *= (1.0 if same else -1.0) / h
                    else:
                        f *= h * (2.0 if same else 1.0) / 6.0
                lap += f
            assert Ke[a, b] == pytest.approx(r * r * lap + h ** 3 / 27.0 / 2 ** nd, rel=1e-13,
                                             abs=1e-16)


def test_bernstein_mass_closed_form():
    # int_{-1}^{1} B_a B_b = 2 C(2,a) C(2,b) / (5 C(4,a+b)) for the quadratic
    # Bernstein basis; the element of side 2 has Jacobian 1
    from math import comb
    _, Me = H.element_matrices(_cube(3, 2.0), 3, 0.0)
    m1 = np.array([[2.0 * comb(2, a) * comb(2, b) / (5.0 * comb(4, a + b)) for b in range(3)]
                   for a in range(3)])
    exp = np.einsum("ad,be,cf->cbafed", m1, m1, m1).reshape(27, 27)
    np.testing.assert_allclose(Me, exp, rtol=1e-13)


def test_assembled_operators_properties():
    z = np.load(os.path.join(HERE, "golden", "brick_o2.npz"))
    nb = z["block_conn"].shape[0]
    boxes = np.zeros((nb, 6))
    boxes[:, 3:] = (1.0, 0.75, 0.5)
    n = int(z["sizes"][1])
    K, M = H.assemble(z["octants"], z["conn"], z["dep_ptr"], z["dep_conn"], z["dep_w"], n, 2,
                      [-1.0, 1.0], boxes, 0.2)
    one = np.ones(n)
    np.testing.assert_allclose(K @ one, M @ one, rtol=1e-12, atol=1e-16)
    assert abs(K - K.T).max() <= 1e-15 * abs(K).max()
    assert abs(M - M.T).max() <= 1e-15 * abs(M).max()
    # total mass = volume of the blocks
    assert one @ (M @ one) == pytest.approx(nb * 1.0 * 0.75 * 0.5, rel=1e-12)
    # the filter keeps constants and is adjoint to its transpose
    x = np.random.default_rng(0).standard_normal(n)
    y = np.random.default_rng(1).standard_normal(n)
    np.testing.assert_allclose(H.apply_filter(K, M, one), one, rtol=1e-10)
    a = y @ H.apply_filter(K, M, x)
    b = H.apply_transpose(K, M, y) @ x
    assert a == pytest.approx(b, rel=1e-10)


def test_quad_element_matrices_closed_form():
    """Bilinear square of side h: M = h^2/36 [4 2 2 1; ...], K 1 = M 1."""
    X = np.array([[0, 0], [0.5, 0], [0, 0.5], [0.5, 0.5]], float)
    Ke, Me = H.element_matrices2d(X, 2, 0.3)
    exp = np.array([[4, 2, 2, 1], [2, 4, 1, 2], [2, 1, 4, 2], [1, 2, 2, 4]]) * 0.25 / 36
    np.testing.assert_allclose(Me, exp, rtol=1e-14)
    np.testing.assert_allclose(Ke.sum(1), Me.sum(1), atol=1e-16)
    # stiffness part: r^2 times the Laplacian of a square (scale-free in 2-D)
    L = (Ke - Me) / 0.09
    exp_l = np.array([[4, -1, -1, -2], [-1, 4, -2, -1], [-1, -2, 4, -1], [-2, -1, -1, 4]]) / 6
    np.testing.assert_allclose(L, exp_l, rtol=1e-13, atol=1e-15)
    # quadratic Bernstein: partition of unity, mass sums to the area of the
    # level-1 element of a 2 x 1 face (1 x 0.5)
    X3 = H.element_points2d(np.array([0, 0, 0, 0, 1, 0]), 3, np.array([-1.0, 0.0, 1.0]),
                             np.array([[0.0, 0.0, 2.0, 1.0]]))
    K3, M3 = H.element_matrices2d(X3, 3, 0.1)
    assert M3.sum() == pytest.approx(0.5, rel=1e-13)
    np.testing.assert_allclose(K3.sum(1), M3.sum(1), atol=1e-15)
