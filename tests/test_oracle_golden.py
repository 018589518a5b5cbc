"""The CPU oracle (oracle/tmr_oracle.c) pinned against the golden vectors
the reference itself produced (tests/golden/*.npz): octants, element
connectivity, node numbering and dependent-node CSR bit-exact, weights and
P within 1e-13."""
import os

import numpy as np
import pytest

from tests import pipeline

CASES = pipeline.golden_cases()


@pytest.mark.parametrize("name", CASES)
def test_oracle_matches_reference_golden(name):
    case = pipeline.golden_case(name)
    g = pipeline.load_golden(name)
    o = pipeline.run_cpu(case, "oracle")
    bad = pipeline.compare(o, g)
    assert not bad, "\n".join(bad)


def test_golden_cases_are_the_parity_cases():
    # the fixture inputs are exactly the seeded parity cases
    allc = pipeline.cases()
    for name in CASES:
        c = pipeline.golden_case(name)
        np.testing.assert_array_equal(c["conn"], allc[name]["conn"])
        for k, v in allc[name].items():
            if k != "conn":
                assert c[k] == v, (name, k)
    for name, case in pipeline.digest_cases().items():
        c = pipeline.golden_case("digest_" + name)
        np.testing.assert_array_equal(c["conn"], case["conn"])
        assert {k: v for k, v in c.items() if k != "conn"} == \
            {k: v for k, v in case.items() if k != "conn"}


@pytest.mark.parametrize("name", sorted(pipeline.digest_cases()))
def test_oracle_matches_reference_digest(name):
    # the configuration-size case (C1 as specified) against the digest of
    # the reference's own products
    case = pipeline.golden_case("digest_" + name)
    o = pipeline.run_cpu(case, "oracle")
    z = np.load(os.path.join(pipeline.GOLDEN_DIR, "digest_%s.npz" % name))
    bad = pipeline.compare_digest(o, z)
    assert not bad, "\n".join(bad)


def test_digest_check_catches_planted_mistakes():
    # a wrong weight (1e-9 off) and a wrong connectivity entry planted in the
    # oracle's products are both reported
    case = pipeline.golden_case("digest_c1")
    o = pipeline.run_cpu(case, "oracle")
    z = np.load(os.path.join(pipeline.GOLDEN_DIR, "digest_c1.npz"))
    o["levels"][0]["P"][2][1234] += 1e-9
    o["conn"][77, 3] += 1
    bad = pipeline.compare_digest(o, z)
    assert any("L0_P_vals" in b for b in bad) and any(b.startswith("conn") for b in bad)


def test_golden_properties():
    # size-independent identities of the reference's own output
    for name in CASES:
        g = pipeline.load_golden(name)
        o = g["oct"]
        assert np.array_equal(o[:, 4], np.arange(len(o)))  # tags are indices
        if g.get("octants_only"):
            # octants-only fixture: levels within the 2^30 grid
            assert o[:, 5].min() >= 0 and o[:, 5].max() <= 30
            continue
        s = g["sizes"]
        nn = g["nn"]
        assert np.array_equal(nn, np.concatenate([np.arange(-s["num_dep"], 0),
                                                   np.arange(s["num_owned"])]))
        assert g["conn"].min() >= -s["num_dep"] and g["conn"].max() < s["num_owned"]
        # dependent weights interpolate constants exactly
        ptr, _, w = g["dep"]
        sums = np.add.reduceat(w, ptr[:-1]) if len(w) else np.zeros(0)
        np.testing.assert_allclose(sums, 1.0, rtol=1e-13)
        for lv in g["levels"]:
            rp, cols, vals = lv["P"]
            rs = np.add.reduceat(vals, rp[:-1])
            np.testing.assert_allclose(rs, 1.0, rtol=1e-12)  # P 1 = 1


@pytest.mark.skipif(not __import__("oracle.oracle", fromlist=["x"]).ref_available(),
                    reason="reference sources not built here")
@pytest.mark.parametrize("name", sorted(pipeline.cases()))
def test_oracle_matches_live_reference(name):
    case = pipeline.cases()[name]
    a = pipeline.run_cpu(case, "oracle")
    b = pipeline.run_cpu(case, "ref")
    bad = pipeline.compare(a, b)
    assert not bad, "\n".join(bad)
