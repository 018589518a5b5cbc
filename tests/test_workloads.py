"""Seeded inputs: the numpy generator equals the C generator shared with
the GPU (oo_uniform / k_random_refinement), and the synthetic block
connectivities are valid hexahedral meshes."""
import numpy as np

from tmr_gb300 import workloads as W


def test_uniform_matches_c_generator():
    from oracle.oracle import uniform as cu
    for seed, stream in [(7, 0), (7, 4), (3, 99), (0, 0)]:
        np.testing.assert_array_equal(W.uniform(seed, stream, 2000), cu(seed, stream, 2000))


def test_uniform_is_uniform():
    u = W.uniform(11, 2, 200000)
    assert 0.0 <= u.min() and u.max() < 1.0
    assert abs(u.mean() - 0.5) < 0.005
    assert abs((u < 0.3).mean() - 0.3) < 0.005


def test_brick_connectivity():
    c = W.brick(8, 4, 4)
    assert c.shape == (128, 8)
    assert c.max() + 1 == 9 * 5 * 5
    # corners x fastest
    assert list(c[0]) == [0, 1, 9, 10, 45, 46, 54, 55]


def test_rotated_blocks_keep_shared_faces():
    from oracle.oracle import OracleForest
    c = W.rotate_blocks(W.brick(3, 2, 2), 5)
    assert sorted(map(tuple, np.sort(c, 1))) == sorted(map(tuple, np.sort(W.brick(3, 2, 2), 1)))
    f = OracleForest(2, 1)
    f.setConnectivity(c)
    f.createTrees(1)
    f.balance(1)
    assert len(f.getOctants()) == 12 * 8
