"""Iso-surface triangles on the GPU (tmrg_stl_triangles) against the CPU
restatement (oracle/stl.py), triangle for triangle and bit for bit, and
against the reference's own output (tests/golden/api_stl.npz) cell by
cell; the binary and ASCII STL writers against the restatement's bytes."""
import os

import numpy as np
import pytest

from oracle import stl as S
from tests import pipeline
from tests.test_stl_oracle import _bface_brick, same_loops

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


def _gpu_case(name):
    from tmr_gb300 import TMR
    sc = pipeline.STL_CASES[name]
    case = pipeline.cases()[name]
    g = pipeline.run_gpu(case)
    f = g["forests"][0]
    boxes = pipeline.brick_boxes(*sc["grid"])
    f.setBlockBoxes(boxes)
    s = g["sizes"]
    X = f.getPoints()
    Xr = pipeline.node_points(g["oct"], g["conn"], s["num_dep"], s["num_local"], case["order"],
                              f.getInterpKnots(), boxes)
    np.testing.assert_array_equal(X, Xr)
    x = pipeline.stl_field(X[s["num_dep"]:], sc["vpn"])
    return sc, case, g, f, X, x, TMR


@pytest.mark.parametrize("name", sorted(pipeline.STL_CASES))
def test_triangles_match_oracle_and_reference(gpu_lib, name):
    sc, case, g, f, X, x, TMR = _gpu_case(name)
    pts = TMR.getSTLTriangles(f, x, offset=sc["offset"], cutoff=sc["cutoff"], vpn=sc["vpn"])
    tris = pts.reshape(-1, 3, 3)
    exp, where = S.triangles(g["oct"], g["conn"], g["dep"], X, x, sc["vpn"], sc["offset"],
                             sc["cutoff"], case["order"], _bface_brick(*sc["grid"]), cells=True)
    np.testing.assert_array_equal(tris, exp)
    ref = np.load(os.path.join(HERE, "golden", "api_stl.npz"))[name + "_tris"]
    assert same_loops(ref, tris, where) == 0
    # device values in, device triangles out
    import torch
    xd = torch.tensor(x, device="cuda")
    np.testing.assert_array_equal(
        TMR.getSTLTriangles(f, xd, offset=sc["offset"], cutoff=sc["cutoff"], vpn=sc["vpn"]), pts)


def test_stl_files_and_empty_level_set(gpu_lib, tmp_path):
    sc, case, g, f, X, x, TMR = _gpu_case("brick_o2")
    b = str(tmp_path / "a.bin")
    t = str(tmp_path / "a.stl")
    TMR.writeSTLToBin(b, f, x, index=sc["offset"], cutoff=sc["cutoff"], vpn=sc["vpn"])
    tris = TMR.getSTLTriangles(f, x, offset=sc["offset"], cutoff=sc["cutoff"], vpn=sc["vpn"])
    e = str(tmp_path / "e.bin")
    S.write_bin(e, tris.reshape(-1, 3, 3))
    with open(b, "rb") as fa, open(e, "rb") as fb:
        assert fa.read() == fb.read()
    TMR.convertBinToSTL(b, t)
    with open(t) as fp:
        assert fp.read() == S.stl_ascii(tris.reshape(-1, 3, 3))
    # everything below the cutoff: no iso-surface and no solid boundary face
    none = TMR.getSTLTriangles(f, x, offset=0, cutoff=1e9, vpn=sc["vpn"])
    assert none.shape == (1, 0)
    # a filter writes its finest-level design variables
    F = TMR.ConformFilter(None, g["forests"], vpn=sc["vpn"])
    F.setDesignVars(x)
    F.writeSTLFile(sc["offset"], sc["cutoff"], str(tmp_path / "c.bin"))
    with open(str(tmp_path / "c.bin"), "rb") as fa, open(b, "rb") as fb:
        assert fa.read() == fb.read()
    with pytest.raises(ValueError):
        TMR.getSTLTriangles(f, x[:-1], vpn=sc["vpn"])
