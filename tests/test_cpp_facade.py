"""The C++ TMROctForest facade (include/tmrg_octforest.hpp) over the C ABI:
compiles and links against libtmrg.so here; on a GPU its pipeline output
equals the Python binding's on the same input."""
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "facade_pipeline.cpp")
SRC_QUAD = os.path.join(ROOT, "tests", "cpp", "facade_quad.cpp")


def _build(tmp_path, src=SRC):
    from tmr_gb300 import build
    lib = build.build()
    exe = str(tmp_path / os.path.basename(src)[:-4])
    cuda_inc = "/usr/local/cuda/include"
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"),
                    "-I", cuda_inc, src, "-o", exe, "-L", os.path.dirname(lib), "-ltmrg",
                    "-Wl,-rpath," + os.path.dirname(lib)], check=True)
    return exe


def test_facade_compiles_and_links(tmp_path):
    assert os.path.exists(_build(tmp_path))
    assert os.path.exists(_build(tmp_path, SRC_QUAD))


@pytest.mark.gpu
def test_facade_matches_python_binding(gpu_lib, tmp_path):
    exe = _build(tmp_path)
    vtk, tec, bvtk = (str(tmp_path / "cpp.vtk"), str(tmp_path / "cpp.dat"),
                      str(tmp_path / "cpp_blocks.vtk"))
    out = subprocess.run([exe, vtk, tec, bvtk], check=True, capture_output=True,
                         text=True).stdout.split()
    vals = dict(zip(out[0::2], out[1::2]))
    from tmr_gb300 import TMR
    from tmr_gb300 import workloads as W
    f = TMR.OctForest(order=3)
    f.setConnectivity(W.brick(3, 2, 2))
    f.createTrees(1)
    for p in range(3):
        o = f.getOctantsArray()
        ref = (((o[:, 1] >> 20) + (o[:, 2] >> 21) + o[:, 0] + p) % 3 == 0).astype(np.intc)
        f.refine(ref, 0, 5)
        f.balance(1)
    f.createNodes()
    c = f.coarsen()
    c.balance(1)
    c.createNodes()
    I = TMR.VecInterp()
    f.createInterpolation(c, I)
    rows, cols, nnz = I.sizes()
    y = np.zeros(rows)
    I.mult(np.ones(cols), y)
    conn = f.getMeshConn()
    assert int(vals["elements"]) == conn.shape[0]
    assert int(vals["conn_sum"]) == int(conn.astype(np.int64).sum())
    assert int(vals["P_rows"]) == rows and int(vals["P_nnz"]) == nnz
    assert float(vals["P1_sum"]) == pytest.approx(y.sum(), rel=1e-12)
    bc, bf, be, fi, nn, ne, nf = f.getConnectivity()
    assert int(vals["blocks"]) == bc.shape[0] and int(vals["nodes"]) == nn
    assert int(vals["edges"]) == ne and int(vals["faces"]) == nf
    assert int(vals["node_refs"]) == 8 * bc.shape[0]
    assert int(vals["local_ok"]) == 1
    assert float(vals["pu"]) == pytest.approx(1.0, abs=1e-14)
    assert float(vals["du"]) == pytest.approx(0.0, abs=1e-13)
    assert int(vals["enclosed_self"]) == 1
    assert int(vals["corner_block"]) == 0
    # the same files from the Python binding with the same block boxes
    nb = bc.shape[0]
    boxes = np.zeros((nb, 6))
    boxes[:, 0] = np.arange(nb)
    boxes[:, 3:] = 1.0
    f.setBlockBoxes(boxes)
    f.writeForestToVTK(str(tmp_path / "py.vtk"))
    f.writeToTecplot(str(tmp_path / "py.dat"))
    f.writeToVTK(str(tmp_path / "py_blocks.vtk"))
    assert open(tec).read() == (tmp_path / "py.dat").read_text()
    assert open(vtk).read() == (tmp_path / "py.vtk").read_text()
    assert open(bvtk).read() == (tmp_path / "py_blocks.vtk").read_text()


@pytest.mark.gpu
def test_quad_facade_matches_python_binding(gpu_lib, tmp_path):
    exe = _build(tmp_path, SRC_QUAD)
    fvtk, qvtk, tec = (str(tmp_path / "cpp_faces.vtk"), str(tmp_path / "cpp_quads.vtk"),
                       str(tmp_path / "cpp_faces.dat"))
    out = subprocess.run([exe, fvtk, qvtk, tec], check=True, capture_output=True,
                         text=True).stdout.split()
    vals = dict(zip(out[0::2], out[1::2]))
    from tmr_gb300 import TMR
    from tmr_gb300 import workloads as W
    f = TMR.QuadForest(order=3)
    f.setConnectivity(W.brick2d(3, 2))
    f.createTrees(1)
    for p in range(3):
        q = f.getQuadrantsArray()
        ref = (((q[:, 1] >> 20) + (q[:, 2] >> 21) + q[:, 0] + p) % 3 == 0).astype(np.intc)
        f.refine(ref, 0, 6)
        f.balance(1)
    f.createNodes()
    c = f.coarsen()
    c.balance(1)
    c.createNodes()
    I = TMR.VecInterp()
    f.createInterpolation(c, I)
    rows, cols, nnz = I.sizes()
    y = np.zeros(rows)
    I.mult(np.ones(cols), y)
    conn = f.getMeshConn()
    assert int(vals["elements"]) == conn.shape[0]
    assert int(vals["conn_sum"]) == int(conn.astype(np.int64).sum())
    assert int(vals["dep"]) == len(f.getDepNodeConn()[0]) - 1
    assert int(vals["P_rows"]) == rows and int(vals["P_nnz"]) == nnz
    assert float(vals["P1_sum"]) == pytest.approx(y.sum(), rel=1e-12)
    assert (int(vals["faces"]), int(vals["edges"]), int(vals["nodes"])) == (6, 17, 12)
    # the VTK writers through the same face boxes, and seeded random trees
    boxes = np.zeros((6, 4))
    boxes[:, 0] = np.arange(6)
    boxes[:, 2:] = 1.0
    f.setFaceBoxes(boxes)
    f.writeToVTK(str(tmp_path / "py_faces.vtk"))
    f.writeForestToVTK(str(tmp_path / "py_quads.vtk"))
    assert open(fvtk).read() == (tmp_path / "py_faces.vtk").read_text()
    assert open(qvtk).read() == (tmp_path / "py_quads.vtk").read_text()
    f.writeToTecplot(str(tmp_path / "py_faces.dat"))
    assert open(tec).read() == (tmp_path / "py_faces.dat").read_text()
    nums = f.getNodeNumbers()
    assert int(vals["node_numbers"]) == len(nums) and int(vals["first"]) == int(nums[0])
    assert int(vals["local_of_first"]) == f.getLocalNodeNumber(int(nums[0])) == 0
    assert int(vals["ext_pre"]) == f.getExtPreOffset()
    r = TMR.QuadForest(order=2)
    r.setConnectivity(W.brick2d(3, 2))
    r.createRandomTrees(25, 1, 6, 5)
    r.repartition()
    rq = r.getQuadrantsArray().astype(np.int64)
    assert int(vals["rand_quads"]) == len(rq)
    assert int(vals["rand_sum"]) == int((rq[:, 1] + 3 * rq[:, 2] + rq[:, 4]).sum())
    # STL tools through the facade = the Python binding
    o = TMR.OctForest(order=2)
    o.setConnectivity(np.arange(8, dtype=np.intc).reshape(1, 8))
    o.createTrees(2)
    o.createNodes()
    no = o.getNodeRange()[1]
    xv = (np.arange(no) % 3) * 0.5
    pts = TMR.getSTLTriangles(o, xv, offset=0, cutoff=0.4, vpn=1)
    assert int(vals["stl_tris"]) == len(pts) // 3 > 0
    assert float(vals["stl_sum"]) == pytest.approx(float(pts.sum()), rel=1e-13)
    # the matrix filter facade on an order-2 quadtree forest = the binding
    q2 = TMR.QuadForest(order=2)
    q2.setConnectivity(W.brick2d(3, 2))
    q2.createTrees(3)
    q2.createNodes()
    mf = TMR.MatrixFilter(0.1, 10, None, [q2])
    n2 = mf.size()[0]
    fx = (np.arange(n2) % 5) * 0.25
    fy = np.zeros(n2)
    mf.applyFilter(fx, fy)
    assert int(vals["filter_nodes"]) == n2
    assert float(vals["filter_sum"]) == pytest.approx(fy.sum(), rel=1e-12)
