"""Quadtree fixtures (tests/golden/quad_*.npz, written from the reference's
own TMRQuadForest in oracle/_ref): re-running the reference reproduces
them, and their products satisfy the identities of the path (P 1 = 1,
dependent weights sum to 1, every element node numbered)."""
import numpy as np
import pytest

from oracle import oracle as O
from tests import pipeline


@pytest.mark.parametrize("name", pipeline.quad_golden_names())
def test_quad_fixture_identities(name):
    g = pipeline.load_quad_golden(name)
    ptr, conn, w = g["dep"]
    order = pipeline.quad_golden_case(name)["order"]
    assert np.all(np.diff(ptr) == order)
    if len(w):
        np.testing.assert_allclose(np.add.reduceat(w, ptr[:-1]), 1.0, rtol=1e-13)
    assert g["conn"].min() >= -(len(ptr) - 1)
    for lv in g["levels"]:
        rp, cols, vals = lv["P"]
        sums = np.add.reduceat(vals, rp[:-1]) if len(vals) else np.zeros(0)
        np.testing.assert_allclose(sums, 1.0, rtol=1e-12)


@pytest.mark.skipif(not O.ref_available(), reason="reference build not present")
@pytest.mark.parametrize("name", pipeline.quad_golden_names())
def test_reference_reproduces_quad_fixture(name):
    r = pipeline.run_quad_ref(pipeline.quad_golden_case(name))
    assert pipeline.compare_quad(r, pipeline.load_quad_golden(name)) == []
