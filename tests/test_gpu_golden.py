"""GPU path vs the golden vectors the reference itself produced
(tests/golden/*.npz, made by tests/golden/make_golden.py from the
reference's own TMROctant.cpp/TMROctForest.cpp/TMRBase.cpp): bit-exact
integers, 1e-13 relative FP64, no CPU code in the loop."""
import os

import pytest

from tests import pipeline

CASES = pipeline.golden_cases()


@pytest.mark.gpu
@pytest.mark.parametrize("name", CASES)
def test_gpu_matches_reference_golden(gpu_lib, name):
    case = pipeline.golden_case(name)
    g = pipeline.run_gpu(case)
    ref = pipeline.load_golden(name)
    bad = pipeline.compare(g, ref)
    assert not bad, "\n".join(bad)


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(pipeline.digest_cases()))
def test_gpu_matches_reference_digest(gpu_lib, name):
    # the configuration-size case (C1 exactly as specified, ~237k octants)
    # against the digest of the reference's own products
    import numpy as np
    case = pipeline.golden_case("digest_" + name)
    g = pipeline.run_gpu(case)
    z = np.load(os.path.join(pipeline.GOLDEN_DIR, "digest_%s.npz" % name))
    bad = pipeline.compare_digest(g, z)
    assert not bad, "\n".join(bad)


@pytest.mark.gpu
@pytest.mark.parametrize("cand", range(3))
def test_every_radix_candidate_matches_reference(gpu_lib, cand):
    # every radix-scatter shape the autotuner may pick gives the reference's
    # products: the one-tree configuration at full size (hundreds of tiles
    # per sort), a rotated multi-block forest and a level-29 forest (128-bit
    # keys, sorted as two 64-bit stages)
    import numpy as np
    from tmr_gb300 import TMR
    lib = TMR.lib()
    assert lib.tmrg_tune_force(5, cand) == 0
    try:
        case = pipeline.golden_case("digest_c1")
        z = np.load(os.path.join(pipeline.GOLDEN_DIR, "digest_c1.npz"))
        bad = pipeline.compare_digest(pipeline.run_gpu(case), z)
        assert not bad, "\n".join(bad)
        for name in ("rot_o3", "deep_l29"):
            g = pipeline.run_gpu(pipeline.golden_case(name))
            bad = pipeline.compare(g, pipeline.load_golden(name))
            assert not bad, name + "\n" + "\n".join(bad)
    finally:
        lib.tmrg_tune_force(5, -1)
