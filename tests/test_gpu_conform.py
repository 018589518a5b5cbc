"""ConformFilter / LagrangeFilter (TMRConformFilter.cpp:144-156,
TMRLagrangeFilter.cpp:130-139): the design variables restricted down the
filter forests with the weight-normalised P^T, against the reference's own
P matrices (tests/golden) applied on the CPU."""
import numpy as np
import pytest

from tests import pipeline

pytestmark = pytest.mark.gpu


def _forests(TMR, case):
    f = TMR.OctForest(order=case["order"])
    f.setConnectivity(case["conn"])
    f.createTrees(case["L0"])
    for p in range(case["passes"]):
        o = f.getOctantsArray()
        f.refine(pipeline.indicator(o, case, p), 0, case["max_level"])
        f.balance(case.get("corner", 1))
    f.createNodes()
    out = [f]
    for _ in range(case["coarse_levels"]):
        c = out[-1].coarsen()
        c.balance(case.get("corner", 1))
        c.createNodes()
        out.append(c)
    return out


def _weighted_t(rp, ci, w, x, ncols, vpn):
    rows = len(rp) - 1
    r = np.repeat(np.arange(rows), np.diff(rp))
    num = np.zeros((ncols, vpn))
    np.add.at(num, ci, w[:, None] * x.reshape(rows, vpn)[r])
    den = np.zeros(ncols)
    np.add.at(den, ci, w)
    out = np.where(den[:, None] != 0, num / np.where(den == 0, 1, den)[:, None], 0.0)
    return out.ravel()


@pytest.mark.parametrize("cls", ["ConformFilter", "LagrangeFilter"])
def test_restriction_chain_matches_reference_P(gpu_lib, cls):
    from tmr_gb300 import TMR
    case = pipeline.golden_case("brick_o2")
    gold = pipeline.load_golden("brick_o2")
    forests = _forests(TMR, case)
    vpn = 2
    F = getattr(TMR, cls)(None, forests, vpn=vpn)
    assert F.getNumLevels() == len(forests)
    x = np.random.default_rng(1).standard_normal(F.interps[0].sizes()[0] * vpn)
    levels = F.setDesignVars(x)
    np.testing.assert_array_equal(F.getDesignVars(), x)
    ref = x
    for k, lv in enumerate(gold["levels"]):
        rp, ci, w = lv["P"]
        ncols = F.interps[k].sizes()[1]
        ref = _weighted_t(np.asarray(rp), np.asarray(ci), np.asarray(w), ref, ncols, vpn)
        np.testing.assert_allclose(levels[k + 1], ref, rtol=1e-13, atol=1e-13)
