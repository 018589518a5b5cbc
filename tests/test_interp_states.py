"""The direction states of the P-row table (tmr_gb300/csrc/tmrg_interp.cu,
dir_state / k_uvw_table): for fine orders 2 and 3 and a fine element at most
one level below its coarse element, the coarse coordinate u that the
per-row kernel computes in double,

    t = x + 0.5 h (1 + k_i)          (x: fine element origin, h its side)
    u = -1 + (t - ox) * (2 / hc)     (ox, hc: coarse element origin, side)

(the reference's computeElemInterp, TMROctForest.cpp:6497-6548) is one of
seven values, and the state rule names it without floating point.  This
checks the rule against that double sequence bit for bit, signed zeros
included, for Gauss-Lobatto (middle knot -cos(pi/2)) and uniform knots."""
import math

import numpy as np

ML = 30  # levels of the octant coordinate


def knots(order, gll):
    if order == 2:
        return [-1.0, 1.0]
    return [-1.0, -math.cos(math.pi / 2) if gll else 0.0, 1.0]


def u_double(x, lf, k, ox, lc):
    half = 2.0 ** (ML - 1 - lf)
    two_ihc = 2.0 ** (lc + 1 - ML)
    t = float(x) + half * (1.0 + k)
    return -1.0 + (t - float(ox)) * two_ihc


def state(x, lf, i, ox, lc, fk1, odd):
    """dir_state without the face-hit case; -1 where the table does not
    apply (the host then takes the general kernel)."""
    if lf - lc > 1 or (lf < lc and odd):
        return -1
    if odd and x == 0 and lf == lc:
        return 6
    h, hc = 1 << (ML - lf), 1 << (ML - lc)
    num = 2 * (x - ox) + h * int(round(fk1)) - hc
    lm = max(lf, lc)
    m = num >> (ML - lm)
    assert (m << (ML - lm)) == num
    return m * (1 << (1 - (lm - lc))) + 2


def state_u(s, fk1):
    if s == 6:  # the double sequence at x = ox = 0, lf = lc
        return -1.0 + ((0.0 + 2.0 ** 19 * fk1) - 0.0) * 2.0 ** -19
    return -1.0 + 0.5 * s


def same(a, b):
    return a == b and math.copysign(1.0, a) == math.copysign(1.0, b)


def test_states_reproduce_the_double_coordinate():
    rng = np.random.default_rng(11)
    seen = set()
    checked = 0
    for order in (2, 3):
        for gll in (True, False):
            kn = knots(order, gll)
            fk1 = [1.0 + k for k in kn]
            odd = [v != round(v) for v in fk1]
            # 1 + k is within 2^-53 of 0, 1 or 2, at most one inexact
            assert all(abs(v - round(v)) <= 2.0 ** -53 for v in fk1)
            assert sum(odd) <= 1
            for _ in range(20000):
                lc = int(rng.integers(0, 14))
                lf = lc + int(rng.integers(-1, 2))
                if not 0 <= lf <= 28:
                    continue
                h, hc = 1 << (ML - lf), 1 << (ML - lc)
                ox = 0 if rng.random() < 0.3 else int(rng.integers(0, (1 << ML) // hc)) * hc
                if lf >= lc:
                    x = ox + (0 if rng.random() < 0.3 else int(rng.integers(0, hc // h)) * h)
                else:
                    x = (ox // h) * h
                i = int(rng.integers(0, order))
                pos2 = 2 * x + h * int(round(fk1[i]))
                if not 2 * ox <= pos2 <= 2 * (ox + hc):
                    continue  # the node is not in the coarse element
                s = state(x, lf, i, ox, lc, fk1[i], odd[i])
                if s < 0:
                    continue
                assert 0 <= s <= 6
                assert same(state_u(s, fk1[i]), u_double(x, lf, kn[i], ox, lc)), \
                    (order, gll, x, lf, i, ox, lc, s)
                seen.add((s, odd[i]))
                checked += 1
    assert checked > 50000
    # every interior state and the middle-knot origin state occur
    assert {0, 1, 2, 3, 4, 6} <= {s for s, _ in seen}


def test_middle_knot_one_level_down_rounds_to_minus_half():
    # the tie -1 + (1/2 - 2^-54) rounds to even: -1/2 (state 1), which the
    # host checks before it takes the table
    fk1 = 1.0 - math.cos(math.pi / 2)
    assert fk1 != 1.0
    t = 2.0 ** 18 * fk1  # x = 0 at level 11
    assert -1.0 + t * 2.0 ** -19 == -0.5  # coarse level 10
    assert u_double(0, 11, -math.cos(math.pi / 2), 0, 10) == -0.5
