"""ctypes bindings for the CPU checkers (test infrastructure only).

Two interchangeable forest classes:

* ``OracleForest`` — the C restatement in ``tmr_oracle.c`` (built into
  ``oracle/_build/libtmr_oracle.so``), which exists wherever the repository
  is built.
* ``RefForest`` — the reference's own ``TMROctant.cpp``/``TMROctForest.cpp``/
  ``TMRBase.cpp`` compiled for one rank (``oracle/_ref/libtmrref.so``); it
  exists only where the reference sources were available at build time.

Only tests, the smoke check and the benchmark's CPU-baseline leg use this.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "libtmr_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libtmrref.so")

_V = ctypes.c_void_p


def _p(a):
    return a.ctypes.data_as(_V)


class _Lib:
    def __init__(self, path, prefix):
        self.lib = ctypes.CDLL(path)
        self.prefix = prefix
        for name in ("forest_create", "coarsen", "duplicate", "create_interp"):
            getattr(self.lib, prefix + name).restype = _V

    def __getattr__(self, name):
        return getattr(self.lib, self.prefix + name)


_libs = {}


def _lib(kind):
    if kind not in _libs:
        if kind == "oracle":
            _libs[kind] = _Lib(ORACLE_SO, "oo_")
        else:
            _libs[kind] = _Lib(REF_SO, "tmrref_")
    return _libs[kind]


def ref_available():
    return os.path.exists(REF_SO)


class _Forest:
    kind = None

    def __init__(self, order=2, interp=1, _handle=None, _conn=None):
        self.L = _lib(self.kind)
        self.h = _handle if _handle is not None else self.L.forest_create(order, interp)
        self.conn = _conn

    def __del__(self):
        try:
            self.L.forest_destroy(_V(self.h))
        except Exception:
            pass

    def setConnectivity(self, conn):
        conn = np.ascontiguousarray(conn, dtype=np.int32)
        self.conn = conn
        self.L.set_connectivity(_V(self.h), int(conn.max()) + 1, _p(conn), conn.shape[0])

    def setMeshOrder(self, order, interp=1):
        self.L.set_mesh_order(_V(self.h), order, interp)

    def createTrees(self, level):
        self.L.create_trees(_V(self.h), level)

    def refine(self, refine=None, min_lev=0, max_lev=30):
        if refine is None:
            self.L.refine(_V(self.h), None, min_lev, max_lev)
        else:
            r = np.ascontiguousarray(refine, dtype=np.int32)
            self.L.refine(_V(self.h), _p(r), min_lev, max_lev)

    def balance(self, corner=1):
        self.L.balance(_V(self.h), corner)

    def coarsen(self):
        return type(self)(_handle=self.L.coarsen(_V(self.h)), _conn=self.conn)

    def duplicate(self):
        return type(self)(_handle=self.L.duplicate(_V(self.h)), _conn=self.conn)

    def createNodes(self):
        self.L.create_nodes(_V(self.h))

    def getOctants(self):
        """(n, 7) int32 array of {block, x, y, z, tag, level, info}."""
        n = self.L.num_octants(_V(self.h))
        out = np.zeros((n, 7), np.int32)
        if n:
            self.L.get_octants(_V(self.h), _p(out))
        return out

    def nodeSizes(self):
        s = np.zeros(6, np.int32)
        self.L.node_sizes(_V(self.h), _p(s))
        return dict(num_local=int(s[0]), num_owned=int(s[1]), num_dep=int(s[2]),
                    ext_pre=int(s[3]), num_elements=int(s[4]), dep_nnz=int(s[5]))

    def getMeshConn(self, order):
        s = self.nodeSizes()
        out = np.zeros(s["num_elements"] * order ** 3, np.int32)
        if out.size:
            self.L.get_conn(_V(self.h), _p(out))
        return out.reshape(s["num_elements"], order ** 3)

    def getNodeNumbers(self):
        s = self.nodeSizes()
        out = np.zeros(s["num_local"], np.int32)
        if out.size:
            self.L.get_node_numbers(_V(self.h), _p(out))
        return out

    def getDepNodeConn(self):
        s = self.nodeSizes()
        ptr = np.zeros(s["num_dep"] + 1, np.int32)
        conn = np.zeros(max(s["dep_nnz"], 1), np.int32)
        w = np.zeros(max(s["dep_nnz"], 1), np.float64)
        self.L.get_dep(_V(self.h), _p(ptr), _p(conn), _p(w))
        return ptr, conn[: s["dep_nnz"]], w[: s["dep_nnz"]]

    def createInterpolation(self, coarse):
        """Returns (rows, ptr, cols, weights): one record per addInterp call,
        in call order; ptr has len(rows)+1 entries."""
        h = self.L.create_interp(_V(self.h), _V(coarse.h))
        s = np.zeros(2, np.int32)
        self.L.interp_sizes(_V(h), _p(s))
        rows = np.zeros(max(s[0], 1), np.int32)
        end = np.zeros(max(s[0], 1), np.int32)
        cols = np.zeros(max(s[1], 1), np.int32)
        w = np.zeros(max(s[1], 1), np.float64)
        self.L.interp_get(_V(h), _p(rows), _p(end), _p(cols), _p(w))
        self.L.interp_destroy(_V(h))
        ptr = np.concatenate([[0], end[: s[0]]]).astype(np.int32)
        return rows[: s[0]], ptr, cols[: s[1]], w[: s[1]]


class OracleForest(_Forest):
    kind = "oracle"


class RefForest(_Forest):
    kind = "ref"

    def stlTriangles(self, X, x, vpn, offset, cutoff):
        """The reference's TMR_GenerateSTLTriangles with node points X
        (num_local x 3) and design values x (vpn per independent node):
        (ntris, 3, 3)."""
        X = np.ascontiguousarray(X, np.float64)
        x = np.ascontiguousarray(x, np.float64)
        self.L.stl_triangles.argtypes = [_V, _V, _V, ctypes.c_int, ctypes.c_int,
                                         ctypes.c_double]
        n = self.L.stl_triangles(_V(self.h), _p(X), _p(x), vpn, offset, cutoff)
        out = np.zeros(max(n, 1) * 9, np.float64)
        if n:
            self.L.stl_get(_p(out))
        return out[: 9 * n].reshape(-1, 3, 3)

    def stlFiles(self, X, x, vpn, offset, cutoff, binfile, stlfile):
        """TMR_GenerateBinFile then TMR_ConvertBinToSTL; returns fail."""
        X = np.ascontiguousarray(X, np.float64)
        x = np.ascontiguousarray(x, np.float64)
        self.L.stl_files.argtypes = [_V, _V, _V, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                     ctypes.c_char_p, ctypes.c_char_p]
        return self.L.stl_files(_V(self.h), _p(X), _p(x), vpn, offset, cutoff,
                                binfile.encode(), stlfile.encode() if stlfile else None)

    def getConnectivityTables(self):
        """(block_face (nb x 6), face_ptr) from getConnectivity /
        getInverseConnectivity."""
        nb = len(self.conn)
        sizes = np.zeros(4, np.int32)
        bc = np.zeros(8 * nb, np.int32)
        bf = np.zeros(6 * nb, np.int32)
        be = np.zeros(12 * nb, np.int32)
        fi = np.zeros(6 * nb, np.int32)
        self.L.get_connectivity(_V(self.h), _p(sizes), _p(bc), _p(bf), _p(be), _p(fi))
        nf, ne, nn = int(sizes[1]), int(sizes[2]), int(sizes[3])
        ncon, nptr = np.zeros(8 * nb, np.int32), np.zeros(nn + 1, np.int32)
        econ, eptr = np.zeros(12 * nb, np.int32), np.zeros(ne + 1, np.int32)
        fcon, fptr = np.zeros(6 * nb, np.int32), np.zeros(nf + 1, np.int32)
        self.L.get_inverse_connectivity(_V(self.h), _p(ncon), _p(nptr), _p(econ), _p(eptr),
                                        _p(fcon), _p(fptr))
        return bf.reshape(nb, 6), fptr


def interp_to_csr(rows, ptr, cols, w, n_rows):
    """Sort the addInterp records by row into CSR (rowptr, cols, vals)."""
    order = np.argsort(rows, kind="stable")
    lens = np.diff(ptr)
    rowptr = np.zeros(n_rows + 1, np.int64)
    rowptr[rows + 1] = lens
    rowptr = np.cumsum(rowptr)
    out_c = np.zeros(len(cols), np.int32)
    out_w = np.zeros(len(cols), np.float64)
    for r in order:
        a, b = ptr[r], ptr[r + 1]
        d = rowptr[rows[r]]
        out_c[d:d + b - a] = cols[a:b]
        out_w[d:d + b - a] = w[a:b]
    return rowptr.astype(np.int32), out_c, out_w


def uniform(seed, stream, n):
    """Vector of oo_uniform(seed, stream, i) for i < n (the seeded input
    generator shared with the GPU path)."""
    L = _lib("oracle").lib
    L.oo_uniform.restype = ctypes.c_double
    L.oo_uniform.argtypes = [ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64]
    return np.array([L.oo_uniform(seed, stream, i) for i in range(n)])


class RefQuadForest:
    """The reference's own TMRQuadForest (oracle/_ref/libtmrref.so), the
    checker of the quadtree twin."""

    def __init__(self, order=2, interp=1, _handle=None, _conn=None):
        self.L = _lib("ref")
        for name in ("qforest_create", "qcoarsen", "qduplicate", "qcreate_interp"):
            getattr(self.L.lib, "tmrref_" + name).restype = _V
        self.h = _handle if _handle is not None else self.L.qforest_create(order, interp)
        self.conn = _conn
        self.order = order

    def __del__(self):
        try:
            self.L.qforest_destroy(_V(self.h))
        except Exception:
            pass

    def setConnectivity(self, conn):
        conn = np.ascontiguousarray(conn, dtype=np.int32)
        self.conn = conn
        self.L.qset_connectivity(_V(self.h), int(conn.max()) + 1, _p(conn), conn.shape[0])

    def createTrees(self, level):
        self.L.qcreate_trees(_V(self.h), level)

    def refine(self, refine=None, min_lev=0, max_lev=30):
        if refine is None:
            self.L.qrefine(_V(self.h), None, min_lev, max_lev)
        else:
            r = np.ascontiguousarray(refine, dtype=np.int32)
            self.L.qrefine(_V(self.h), _p(r), min_lev, max_lev)

    def balance(self, corner=1):
        self.L.qbalance(_V(self.h), corner)

    def coarsen(self):
        return RefQuadForest(self.order, _handle=self.L.qcoarsen(_V(self.h)), _conn=self.conn)

    def duplicate(self):
        return RefQuadForest(self.order, _handle=self.L.qduplicate(_V(self.h)), _conn=self.conn)

    def setMeshOrder(self, order, interp=1):
        self.order = order
        self.L.qset_mesh_order(_V(self.h), order, interp)

    def createNodes(self):
        self.L.qcreate_nodes(_V(self.h))

    def getQuadrants(self):
        """(n, 6) int32 array of {face, x, y, tag, level, info}."""
        n = self.L.qnum_quads(_V(self.h))
        out = np.zeros((n, 6), np.int32)
        if n:
            self.L.qget_quads(_V(self.h), _p(out))
        return out

    def nodeSizes(self):
        s = np.zeros(6, np.int32)
        self.L.qnode_sizes(_V(self.h), _p(s))
        return dict(num_local=int(s[0]), num_owned=int(s[1]), num_dep=int(s[2]),
                    ext_pre=int(s[3]), num_elements=int(s[4]), dep_nnz=int(s[5]))

    def getMeshConn(self):
        s = self.nodeSizes()
        out = np.zeros(s["num_elements"] * self.order ** 2, np.int32)
        if out.size:
            self.L.qget_conn(_V(self.h), _p(out))
        return out.reshape(s["num_elements"], self.order ** 2)

    def getNodeNumbers(self):
        s = self.nodeSizes()
        out = np.zeros(s["num_local"], np.int32)
        if out.size:
            self.L.qget_node_numbers(_V(self.h), _p(out))
        return out

    def getDepNodeConn(self):
        s = self.nodeSizes()
        ptr = np.zeros(s["num_dep"] + 1, np.int32)
        conn = np.zeros(max(s["dep_nnz"], 1), np.int32)
        w = np.zeros(max(s["dep_nnz"], 1), np.float64)
        self.L.qget_dep(_V(self.h), _p(ptr), _p(conn), _p(w))
        return ptr, conn[: s["dep_nnz"]], w[: s["dep_nnz"]]

    def getConnectivity(self):
        nf = len(self.conn)
        sizes = np.zeros(3, np.int32)
        fc = np.zeros(4 * nf, np.int32)
        fe = np.zeros(4 * nf, np.int32)
        self.L.qget_connectivity(_V(self.h), _p(sizes), _p(fc), _p(fe))
        return sizes, fc.reshape(nf, 4), fe.reshape(nf, 4)

    def createInterpolation(self, coarse):
        """(rows, ptr, cols, weights) records of the addInterp calls."""
        h = self.L.qcreate_interp(_V(self.h), _V(coarse.h))
        s = np.zeros(2, np.int32)
        self.L.interp_sizes(_V(h), _p(s))
        rows = np.zeros(max(s[0], 1), np.int32)
        end = np.zeros(max(s[0], 1), np.int32)
        cols = np.zeros(max(s[1], 1), np.int32)
        w = np.zeros(max(s[1], 1), np.float64)
        self.L.interp_get(_V(h), _p(rows), _p(end), _p(cols), _p(w))
        self.L.interp_destroy(_V(h))
        ptr = np.concatenate([[0], end[: s[0]]]).astype(np.int32)
        return rows[: s[0]], ptr, cols[: s[1]], w[: s[1]]
