"""Drop-in for the octree part of the ``tmr.TMR`` Cython module.

Same class and method names as TMR.pyx (OctForest :3393-3790, Octant and
OctantArray :3270-3392, VecInterp, MatrixFilter :4660-5039), backed by the
GPU library through its C ABI.  ``comm`` is accepted and ignored: one GPU
holds the whole forest (the reference's single-rank behaviour).

Vectors passed to VecInterp / MatrixFilter may be numpy arrays (host
buffers, copied in and out) or CUDA torch tensors (used in place).
"""
import ctypes

import numpy as np

from . import _lib
from ._lib import call, lib

UNIFORM_POINTS = 0
GAUSS_LOBATTO_POINTS = 1
BERNSTEIN_POINTS = 2
MAX_LEVEL = 30

_vp = ctypes.c_void_p


def _ptr(a):
    return a.ctypes.data_as(_vp)


def _host_view(addr, n, dtype):
    """Read-only numpy view of n items at a host address owned by the
    library (empty when n == 0)."""
    dt = np.dtype(dtype)
    if n <= 0 or not addr:
        return np.zeros(0, dt)
    buf = (ctypes.c_char * (n * dt.itemsize)).from_address(addr)
    a = np.frombuffer(buf, dtype=dt, count=n)
    a.flags.writeable = False
    return a


def _octant_struct(nodes):
    """Contiguous OCTANT_DTYPE array from an OctantArray, an (n, 7) int
    array or a structured octant array."""
    if isinstance(nodes, OctantArray):
        nodes = nodes.array
    a = np.asarray(nodes)
    if a.dtype.names:
        return np.ascontiguousarray(a.astype(OCTANT_DTYPE))
    a = a.reshape(-1, 7)
    out = np.zeros(a.shape[0], OCTANT_DTYPE)
    for j, name in enumerate(OCTANT_DTYPE.names):
        out[name] = a[:, j]
    return out


def _is_torch(a):
    return type(a).__module__.startswith("torch")


def _check_vectors(what, x, y, nin, nout, dtypes):
    """Validate an (x -> y) vector pair before its pointers reach the C ABI
    and return the number of vectors per node.

    x must hold nin * nvec values and y nout * nvec (nvec >= 1), both of one
    dtype from `dtypes` (numpy dtype names), both contiguous, and both on
    the same side: CUDA tensors for the device entry points, host arrays
    otherwise.  A wrong size would make a kernel read or write past the end
    of a buffer, so every mismatch raises ValueError instead."""
    if nin <= 0 or nout <= 0:
        raise ValueError("%s: empty operator (%d inputs, %d outputs)" % (what, nin, nout))
    tx, ty = _is_torch(x), _is_torch(y)
    if tx or ty:
        if not (tx and ty and x.is_cuda and y.is_cuda):
            raise ValueError("%s: x and y must both be CUDA tensors (or both host arrays)"
                             % what)
        if x.device != y.device:
            raise ValueError("%s: x on %s, y on %s" % (what, x.device, y.device))
        if x.dtype != y.dtype:
            raise ValueError("%s: x is %s, y is %s" % (what, x.dtype, y.dtype))
        name = str(x.dtype).replace("torch.", "")
        if name not in dtypes:
            raise ValueError("%s: dtype %s not supported (%s)" % (what, name, "/".join(dtypes)))
        if not (x.is_contiguous() and y.is_contiguous()):
            raise ValueError("%s: x and y must be contiguous" % what)
        nx, ny = x.numel(), y.numel()
    else:
        nx, ny = np.size(x), np.size(y)
    if nx == 0 or nx % nin != 0:
        raise ValueError("%s: x holds %d values, not a multiple of %d" % (what, nx, nin))
    nvec = nx // nin
    if ny != nout * nvec:
        raise ValueError("%s: y holds %d values, expected %d (%d x %d)"
                         % (what, ny, nout * nvec, nout, nvec))
    return nvec


class _DeviceArray:
    """Exposes a borrowed device pointer through __cuda_array_interface__."""

    def __init__(self, ptr, n, typestr):
        self.__cuda_array_interface__ = {
            "shape": (n,), "typestr": typestr, "data": (ptr, False), "version": 3,
            "strides": None}


class Octant:
    """TMROctant value (TMROctant.h:36-54)."""

    __slots__ = ("block", "x", "y", "z", "tag", "level", "info")

    def __init__(self, block=0, x=0, y=0, z=0, tag=0, level=0, info=0):
        self.block, self.x, self.y, self.z = block, x, y, z
        self.tag, self.level, self.info = tag, level, info

    def __repr__(self):
        return "Octant(block=%d, x=%d, y=%d, z=%d, tag=%d, level=%d, info=%d)" % (
            self.block, self.x, self.y, self.z, self.tag, self.level, self.info)


# TMROctant layout (TMROctant.h:47-52): five int32 then two int16, 24 bytes
OCTANT_DTYPE = np.dtype([("block", "<i4"), ("x", "<i4"), ("y", "<i4"), ("z", "<i4"),
                         ("tag", "<i4"), ("level", "<i2"), ("info", "<i2")])


class OctantArray:
    """A forest's octants (TMR.pyx:3270-3330).  Built over an (n, 7) int32
    array {block, x, y, z, tag, level, info} or over a structured
    OCTANT_DTYPE array; OctForest.getOctants() returns the latter as a
    borrowed view of the forest's host octants (valid until the forest
    changes, like the reference's OctantArray that does not own its
    array)."""

    def __init__(self, arr, owner=None):
        self.array = arr
        self._owner = owner  # keeps the forest (and its host view) alive

    def __len__(self):
        return self.array.shape[0]

    def _fields(self):
        a = self.array
        if a.dtype.names:
            return a["block"], a["x"], a["y"], a["z"], a["tag"], a["level"], a["info"]
        return tuple(a[:, j] for j in range(7))

    def findIndex(self, oc, use_nodes=False):
        """findIndex (TMR.pyx OctantArray, over TMROctantArray::contains,
        TMROctant.cpp:404-424): the index of the octant with oc's block,
        position and level (position alone with use_nodes), or None."""
        b, x, y, z, _tag, lev, _info = self._fields()
        m = (b == oc.block) & (x == oc.x) & (y == oc.y) & (z == oc.z)
        if not use_nodes:
            m &= lev == oc.level
        idx = np.flatnonzero(m)
        return int(idx[0]) if len(idx) else None

    def asArray7(self):
        """(n, 7) int32 copy {block, x, y, z, tag, level, info}."""
        if not self.array.dtype.names:
            return np.array(self.array, dtype=np.intc)
        return np.stack(self._fields(), axis=1).astype(np.intc)

    def __getitem__(self, k):
        n = len(self)
        if k < 0 or k >= n:
            raise IndexError("Octant array index %d out of range [0,%d)" % (k, n))
        r = self.array[k]
        return Octant(*(int(v) for v in (tuple(r) if self.array.dtype.names else r)))

    def __setitem__(self, k, oc):
        n = len(self)
        if k < 0 or k >= n:
            raise IndexError("Octant array index %d out of range [0,%d)" % (k, n))
        if not self.array.flags.writeable:
            raise ValueError("borrowed octant view is read-only")
        v = (oc.block, oc.x, oc.y, oc.z, oc.tag, oc.level, oc.info)
        self.array[k] = v if self.array.dtype.names else list(v)


class OctForest:
    """Forest of octrees on one GPU (TMROctForest, TMR.pyx:3393-3790)."""

    def __init__(self, comm=None, order=2, interp=GAUSS_LOBATTO_POINTS, stream=None,
                 _handle=None):
        self.comm = comm
        self._stream = stream
        if _handle is not None:
            self.ptr = _handle
        else:
            h = _vp()
            call("tmrg_forest_create", order, interp, _vp(self._stream_ptr()),
                 ctypes.byref(h))
            self.ptr = h

    def _stream_ptr(self):
        s = self._stream
        if s is None:
            return None
        return s.cuda_stream if hasattr(s, "cuda_stream") else int(s)

    def __del__(self):
        try:
            if getattr(self, "ptr", None):
                lib().tmrg_forest_destroy(self.ptr)
                self.ptr = None
        except Exception:
            pass

    # -- configuration -------------------------------------------------
    def setMeshOrder(self, order, interp=GAUSS_LOBATTO_POINTS):
        call("tmrg_forest_set_mesh_order", self.ptr, order, interp)

    def getMeshOrder(self):
        o = ctypes.c_int()
        call("tmrg_forest_get_mesh_order", self.ptr, ctypes.byref(o), None)
        return o.value

    def getInterpType(self):
        t = ctypes.c_int()
        call("tmrg_forest_get_mesh_order", self.ptr, None, ctypes.byref(t))
        return t.value

    def getInterpKnots(self):
        k = np.zeros(self.getMeshOrder(), np.float64)
        call("tmrg_forest_get_interp_knots", self.ptr, _ptr(k))
        return k

    def setConnectivity(self, conn):
        conn = np.ascontiguousarray(conn, dtype=np.intc)
        if conn.ndim != 2 or conn.shape[1] != 8:
            raise ValueError("Expected array of shape (n, 8)")
        num_nodes = int(conn.max()) + 1
        call("tmrg_forest_set_connectivity", self.ptr, num_nodes, _ptr(conn),
             conn.shape[0])

    def setFullConnectivity(self, conn, edge_conn, face_conn, num_nodes=None,
                            num_edges=None, num_faces=None):
        """TMROctForest::setFullConnectivity (TMROctForest.cpp:596-637):
        corner (n, 8), edge (n, 12) and face (n, 6) numbers of every block."""
        conn = np.ascontiguousarray(conn, dtype=np.intc)
        ec = np.ascontiguousarray(edge_conn, dtype=np.intc)
        fc = np.ascontiguousarray(face_conn, dtype=np.intc)
        nb = conn.shape[0]
        if conn.shape != (nb, 8) or ec.shape != (nb, 12) or fc.shape != (nb, 6):
            raise ValueError("Expected arrays of shape (n, 8), (n, 12), (n, 6)")
        nn = int(conn.max()) + 1 if num_nodes is None else num_nodes
        ne = int(ec.max()) + 1 if num_edges is None else num_edges
        nf = int(fc.max()) + 1 if num_faces is None else num_faces
        call("tmrg_forest_set_full_connectivity", self.ptr, nn, ne, nf, nb, _ptr(conn),
             _ptr(ec), _ptr(fc))

    def getConnectivity(self):
        """(block_conn (n,8), block_face_conn (n,6), block_edge_conn (n,12),
        block_face_ids (n,6), num_nodes, num_edges, num_faces) of the block
        connectivity (TMROctForest::getConnectivity); copies."""
        nb, nf, ne, nn = (ctypes.c_int() for _ in range(4))
        p = [_vp() for _ in range(4)]
        call("tmrg_forest_get_connectivity", self.ptr, ctypes.byref(nb), ctypes.byref(nf),
             ctypes.byref(ne), ctypes.byref(nn), *[ctypes.byref(q) for q in p])
        n = nb.value
        arr = [np.array(_host_view(q.value, n * w, np.intc)).reshape(n, w)
               for q, w in zip(p, (8, 6, 12, 6))]
        return (*arr, nn.value, ne.value, nf.value)

    def getInverseConnectivity(self):
        """{node,edge,face}_block (ptr, conn) CSR copies
        (TMROctForest::getInverseConnectivity)."""
        _, _, _, _, nn, ne, nf = self.getConnectivity()
        p = [_vp() for _ in range(6)]
        call("tmrg_forest_get_inverse_connectivity", self.ptr, *[ctypes.byref(q) for q in p])
        out = {}
        for (name, nitems), (pc, pp) in zip((("node", nn), ("edge", ne), ("face", nf)),
                                            ((p[0], p[1]), (p[2], p[3]), (p[4], p[5]))):
            ptr = np.array(_host_view(pp.value, nitems + 1, np.intc))
            out[name] = (ptr, np.array(_host_view(pc.value, int(ptr[-1]), np.intc)))
        return out

    def repartition(self, max_rank=-1):
        call("tmrg_forest_repartition", self.ptr, max_rank)

    # -- octants -------------------------------------------------------
    def createTrees(self, depth=0):
        call("tmrg_forest_create_trees", self.ptr, depth)

    def createRandomTrees(self, nrand=10, min_lev=0, max_lev=8, seed=0):
        """TMROctForest::createRandomTrees (TMROctForest.cpp:1838-1917) with a
        seeded generator in place of libc rand()."""
        call("tmrg_forest_create_random_trees", self.ptr, nrand, min_lev, max_lev, seed)

    def refine(self, refine=None, min_lev=0, max_lev=MAX_LEVEL):
        if refine is None:
            call("tmrg_forest_refine", self.ptr, None, 0, min_lev, max_lev)
        elif _is_torch(refine) and refine.is_cuda:
            import torch
            r = refine.to(torch.int32).contiguous()
            call("tmrg_forest_refine_device", self.ptr, _vp(r.data_ptr()), r.numel(),
                 min_lev, max_lev)
        else:
            r = np.ascontiguousarray(refine, dtype=np.intc)
            call("tmrg_forest_refine", self.ptr, _ptr(r), r.size, min_lev, max_lev)

    def duplicate(self):
        h = _vp()
        call("tmrg_forest_duplicate", self.ptr, ctypes.byref(h))
        return OctForest(self.comm, stream=self._stream, _handle=h)

    def coarsen(self):
        h = _vp()
        call("tmrg_forest_coarsen", self.ptr, ctypes.byref(h))
        return OctForest(self.comm, stream=self._stream, _handle=h)

    def balance(self, btype=0):
        call("tmrg_forest_balance", self.ptr, btype)

    def createNodes(self):
        call("tmrg_forest_create_nodes", self.ptr)

    def getNumOctants(self):
        n = ctypes.c_int64()
        call("tmrg_forest_num_octants", self.ptr, ctypes.byref(n))
        return n.value

    def getOctantsArray(self):
        """(n, 7) int32 array {block, x, y, z, tag, level, info}."""
        n = self.getNumOctants()
        out = np.zeros((n, 7), np.intc)
        if n:
            call("tmrg_forest_get_octants", self.ptr, _ptr(out), n)
        return out

    def getOctants(self):
        """Borrowed view of the octants in page-locked host memory
        (TMROctForest::getOctants, TMROctForest.cpp:1452), valid until the
        next call that changes this forest."""
        p = _vp()
        n = ctypes.c_int64()
        call("tmrg_forest_octants_host", self.ptr, ctypes.byref(p), ctypes.byref(n))
        return OctantArray(_host_view(p.value, n.value, OCTANT_DTYPE), owner=self)

    def getOctantsDevice(self):
        """Borrowed CUDA torch views of the octant arrays (block, x, y, z as
        int32; level, info as int16), valid until the next mutating call."""
        import torch
        n = self.getNumOctants()
        ptrs = [_vp() for _ in range(6)]
        call("tmrg_forest_octants_device", self.ptr, *[ctypes.byref(p) for p in ptrs])
        names = ("block", "x", "y", "z", "level", "info")
        types = ("<i4", "<i4", "<i4", "<i4", "<i2", "<i2")
        out = {}
        for name, p, t in zip(names, ptrs, types):
            out[name] = torch.as_tensor(_DeviceArray(p.value or 0, n, t), device="cuda")
        out["_owner"] = self
        return out

    # -- nodes ---------------------------------------------------------
    def _sizes(self):
        s = np.zeros(6, np.int64)
        call("tmrg_forest_node_sizes", self.ptr, _ptr(s))
        return s

    def getLocalNodeNumber(self, node):
        """TMROctForest::getLocalNodeNumber (TMROctForest.cpp:1486-1496)."""
        li = ctypes.c_int()
        call("tmrg_forest_get_local_node_number", self.ptr, int(node), ctypes.byref(li))
        return li.value

    def setBlockBoxes(self, boxes):
        """Axis-aligned box (origin xyz, extent xyz) of every block: the
        geometry getPoints maps node positions through; None removes it."""
        if boxes is None:
            call("tmrg_forest_set_block_boxes", self.ptr, None, 0)
            self._boxes = None
            return
        b = np.ascontiguousarray(boxes, dtype=np.float64)
        if b.ndim != 2 or b.shape[1] != 6:
            raise ValueError("Expected array of shape (n, 6)")
        call("tmrg_forest_set_block_boxes", self.ptr, _ptr(b), b.shape[0])
        self._boxes = b.copy()

    def getPoints(self):
        """Node locations (num_local_nodes, 3) (TMROctForest::getPoints):
        zeros without block boxes, as the reference without a topology."""
        n = int(self._sizes()[0])
        X = np.zeros((n, 3), np.float64)
        if n:
            call("tmrg_forest_get_points", self.ptr, _ptr(X), n)
        return X

    def evalInterp(self, pt, derivs=0):
        """TMROctForest::evalInterp (TMROctForest.cpp:1510-1631): N, or
        (N, N1, N2, N3) with derivs=1, or the ten arrays of the
        second-derivative form with derivs=2."""
        o = self.getMeshOrder()
        pt = np.ascontiguousarray(pt, dtype=np.float64)
        arrs = [np.zeros(o ** 3) for _ in range({0: 1, 1: 4, 2: 11}[derivs])]
        if derivs == 2:
            call("tmrg_forest_eval_interp2", self.ptr, _ptr(pt), *[_ptr(a) for a in arrs])
            return tuple(arrs)
        ptrs = [_ptr(a) for a in arrs] + [None] * (4 - len(arrs))
        call("tmrg_forest_eval_interp", self.ptr, _ptr(pt), *ptrs)
        return arrs[0] if derivs == 0 else tuple(arrs)

    def findEnclosing(self, order, knots, nodes):
        """TMROctForest::findEnclosing for nodes given as an OctantArray,
        an (n, 7) int array or a structured octant array; returns the index
        of the enclosing octant of this forest per node (-1: none)."""
        a = _octant_struct(nodes)
        k = np.ascontiguousarray(knots, dtype=np.float64)
        idx = np.zeros(len(a), np.int64)
        if len(a):
            call("tmrg_forest_find_enclosing", self.ptr, int(order), _ptr(k), _ptr(a), len(a),
                 _ptr(idx))
        return idx

    def transformNodes(self, nodes, edge_dir=-1):
        """TMROctForest::transformNode on every node (copy): returns the
        transformed structured octants, edge reversal flags and face ids."""
        a = _octant_struct(nodes).copy()
        rev = np.zeros(len(a), np.intc)
        fid = np.zeros(len(a), np.intc)
        if len(a):
            call("tmrg_forest_transform_nodes", self.ptr, _ptr(a), len(a), int(edge_dir),
                 _ptr(rev), _ptr(fid))
        return a, rev, fid

    def getNodeRange(self):
        return np.array([0, self._sizes()[1]], dtype=np.intc)

    def getExtPreOffset(self):
        return int(self._sizes()[3])

    def getMeshConn(self, copy=True):
        """(elements, order^3) global node numbers, dependent nodes -k-1.
        copy=False returns the borrowed read-only view of the forest's
        page-locked host connectivity (TMROctForest::getNodeConn,
        TMROctForest.cpp:5686), valid until the forest changes."""
        o = self.getMeshOrder()
        if not copy:
            p = _vp()
            ne = ctypes.c_int64()
            call("tmrg_forest_node_conn_host", self.ptr, ctypes.byref(p), ctypes.byref(ne))
            return _host_view(p.value, ne.value * o ** 3, np.intc).reshape(ne.value, o ** 3)
        s = self._sizes()
        n = int(s[4]) * o ** 3
        out = np.zeros(n, np.intc)
        if n:
            call("tmrg_forest_get_node_conn", self.ptr, _ptr(out), n)
        return out.reshape(int(s[4]), o ** 3)

    def getNodeNumbers(self):
        s = self._sizes()
        out = np.zeros(int(s[0]), np.intc)
        if out.size:
            call("tmrg_forest_get_node_numbers", self.ptr, _ptr(out), out.size)
        return out

    def getDepNodeConn(self, copy=True):
        """(ptr, conn, weights) of the dependent nodes; copy=False returns
        borrowed read-only views (TMROctForest::getDepNodeConn,
        TMROctForest.cpp:5717)."""
        if not copy:
            p, c, w = _vp(), _vp(), _vp()
            nd = ctypes.c_int64()
            call("tmrg_forest_dep_node_conn_host", self.ptr, ctypes.byref(p), ctypes.byref(c),
                 ctypes.byref(w), ctypes.byref(nd))
            ptr = _host_view(p.value, nd.value + 1, np.intc)
            nnz = int(ptr[-1]) if nd.value >= 0 else 0
            return ptr, _host_view(c.value, nnz, np.intc), _host_view(w.value, nnz, np.float64)
        s = self._sizes()
        ndep, nnz = int(s[2]), int(s[5])
        ptr = np.zeros(ndep + 1, np.intc)
        conn = np.zeros(max(nnz, 1), np.intc)
        w = np.zeros(max(nnz, 1), np.float64)
        call("tmrg_forest_get_dep_node_conn", self.ptr, _ptr(ptr), _ptr(conn), _ptr(w))
        return ptr, conn[:nnz], w[:nnz]

    def createInterpolation(self, forest, vec):
        if forest.ptr.value == self.ptr.value:
            raise ValueError("Cannot interpolate between the same object")
        vec._create(self, forest)

    def _block_node_points(self):
        """(block_conn, X): each block connectivity node at its owner
        block's corner (the lowest-numbered block touching it) mapped
        through that block's box, as the reference evaluates the owner's
        volume (node_block_owners, TMROctForest.cpp:1090-1143); None
        without block boxes."""
        boxes = getattr(self, "_boxes", None)
        if boxes is None:
            return None
        bc = self.getConnectivity()[0]
        nb = bc.shape[0]
        nn = int(bc.max()) + 1 if nb else 0
        owner = np.full(nn, nb, np.int64)
        np.minimum.at(owner, bc.ravel(), np.repeat(np.arange(nb), 8))
        X = np.zeros((nn, 3))
        for k in range(nn):
            b = owner[k]
            corner = next(c for c in range(8) if bc[b, c] == k)
            uvw = np.array([corner & 1, (corner >> 1) & 1, corner >> 2], np.float64)
            X[k] = boxes[b, :3] + boxes[b, 3:] * uvw
        return bc, X

    def writeToVTK(self, fname):
        """writeToVTK (TMROctForest.cpp:1149-1228): the block mesh as VTK
        hexahedra, each connectivity node at its owner block's corner
        through the block boxes (the topology's volumes in the reference),
        the block index as the cell scalar entity_index; nothing is written
        when no boxes are set (the reference needs a topology)."""
        bx = self._block_node_points()
        if bx is None:
            return
        bc, X = bx
        nb = bc.shape[0]
        with open(fname, "w") as fp:
            fp.write("# vtk DataFile Version 3.0\nvtk output\nASCII\n")
            fp.write("DATASET UNSTRUCTURED_GRID\nPOINTS %d float\n" % X.shape[0])
            for p in X:
                fp.write("%e %e %e\n" % (p[0], p[1], p[2]))
            fp.write("\nCELLS %d %d\n" % (nb, 9 * nb))
            for c in bc:
                fp.write("8 %d %d %d %d %d %d %d %d\n" % (c[0], c[1], c[3], c[2], c[4], c[5],
                                                          c[7], c[6]))
            fp.write("\nCELL_TYPES %d\n" % nb)
            fp.write("12\n" * nb)
            fp.write("CELL_DATA %d\nSCALARS entity_index float 1\nLOOKUP_TABLE default\n" % nb)
            for k in range(nb):
                fp.write("%e\n" % (1.0 * k))

    def writeToTecplot(self, fname):
        """writeToTecplot (TMROctForest.cpp:1233-1311): the block mesh as one
        Tecplot FEBRICK zone, each block connectivity node at its owner
        block's corner (the lowest-numbered block touching it) mapped
        through that block's volume, and the block index as a cell-centred
        variable.  The block boxes (setBlockBoxes) stand in for the
        topology's volumes; nothing is written when no boxes are set."""
        bx = self._block_node_points()
        if bx is None:
            return
        bc, X = bx
        nb, nn = bc.shape[0], X.shape[0]
        with open(fname, "w") as fp:
            fp.write("Variables = X,Y,Z,block\n")
            fp.write("Zone N = %d E = %d " % (nn, nb))
            fp.write("DATAPACKING=BLOCK, ZONETYPE=FEBRICK\n")
            fp.write("VARLOCATION = ([4]=CELLCENTERED)\n")
            for d in range(3):
                for k in range(nn):
                    fp.write("%e\n" % X[k, d])
            for k in range(nb):
                fp.write("%e\n" % (1.0 * k))
            for k in range(nb):
                c = bc[k] + 1
                fp.write("%d %d %d %d %d %d %d %d\n" % (c[0], c[1], c[3], c[2], c[4], c[5],
                                                         c[7], c[6]))

    def writeForestToVTK(self, fname):
        """writeForestToVTK (TMROctForest.cpp:1317-1384): every octant as a
        hexahedron with its own eight corner points (x fastest), mapped
        through the block's volume, and the block index as the cell scalar
        `entity_index`.  The block boxes (setBlockBoxes) stand in for the
        topology's volumes; like the reference without a topology, nothing
        is written when no boxes are set."""
        boxes = getattr(self, "_boxes", None)
        if boxes is None:
            return
        o = self.getOctantsArray()
        n = len(o)
        h = (1 << (30 - o[:, 5].astype(np.int64)))
        hmax = float(1 << 30)
        with open(fname, "w") as fp:
            fp.write("# vtk DataFile Version 3.0\nvtk output\nASCII\n")
            fp.write("DATASET UNSTRUCTURED_GRID\nPOINTS %d float\n" % (8 * n))
            for r, hh in zip(o, h):
                b = boxes[r[0]]
                for kk in range(2):
                    for jj in range(2):
                        for ii in range(2):
                            u = 1.0 * (r[1] + ii * hh) / hmax
                            v = 1.0 * (r[2] + jj * hh) / hmax
                            w = 1.0 * (r[3] + kk * hh) / hmax
                            fp.write("%e %e %e\n" % (b[0] + b[3] * u, b[1] + b[4] * v,
                                                     b[2] + b[5] * w))
            fp.write("\nCELLS %d %d\n" % (n, 9 * n))
            for k in range(n):
                c = 8 * k
                fp.write("8 %d %d %d %d %d %d %d %d\n" % (c, c + 1, c + 3, c + 2, c + 4, c + 5,
                                                          c + 7, c + 6))
            fp.write("\nCELL_TYPES %d\n" % n)
            fp.write("12\n" * n)
            fp.write("CELL_DATA %d\nSCALARS entity_index float 1\nLOOKUP_TABLE default\n" % n)
            for r in o:
                fp.write("%e\n" % (1.0 * r[0]))


class Quadrant:
    """TMRQuadrant value (TMRQuadrant.h:36-52)."""

    __slots__ = ("face", "x", "y", "tag", "level", "info")

    def __init__(self, face=0, x=0, y=0, tag=0, level=0, info=0):
        self.face, self.x, self.y = face, x, y
        self.tag, self.level, self.info = tag, level, info

    def __repr__(self):
        return "Quadrant(face=%d, x=%d, y=%d, tag=%d, level=%d, info=%d)" % (
            self.face, self.x, self.y, self.tag, self.level, self.info)


class QuadrantArray:
    """A forest's quadrants (TMR.pyx QuadrantArray) over an (n, 6) int32
    array {face, x, y, tag, level, info}."""

    def __init__(self, arr):
        self.array = arr

    def __len__(self):
        return self.array.shape[0]

    def __getitem__(self, k):
        n = len(self)
        if k < 0 or k >= n:
            raise IndexError("Quadrant array index %d out of range [0,%d)" % (k, n))
        return Quadrant(*(int(v) for v in self.array[k]))

    def findIndex(self, quad, use_nodes=False):
        """findIndex (TMR.pyx QuadrantArray, over TMRQuadrantArray::contains):
        the index of the quadrant with quad's face, position and level
        (position alone with use_nodes), or None."""
        a = self.array
        m = (a[:, 0] == quad.face) & (a[:, 1] == quad.x) & (a[:, 2] == quad.y)
        if not use_nodes:
            m &= a[:, 4] == quad.level
        idx = np.flatnonzero(m)
        return int(idx[0]) if len(idx) else None


class QuadForest:
    """Forest of quadtrees on one GPU (TMRQuadForest, TMR.pyx QuadForest):
    mesh orders 2 and 3, Gauss-Lobatto or uniform knots."""

    def __init__(self, comm=None, order=2, interp=GAUSS_LOBATTO_POINTS, stream=None,
                 _handle=None):
        self.comm = comm
        self._stream = stream
        if _handle is not None:
            self.ptr = _handle
        else:
            h = _vp()
            st = stream.cuda_stream if hasattr(stream, "cuda_stream") else stream
            call("tmrg_qforest_create", order, interp, _vp(st), ctypes.byref(h))
            self.ptr = h

    def __del__(self):
        try:
            if getattr(self, "ptr", None):
                lib().tmrg_qforest_destroy(self.ptr)
                self.ptr = None
        except Exception:
            pass

    def _child(self, name):
        h = _vp()
        call(name, self.ptr, ctypes.byref(h))
        return QuadForest(self.comm, stream=self._stream, _handle=h)

    def setMeshOrder(self, order, interp=GAUSS_LOBATTO_POINTS):
        call("tmrg_qforest_set_mesh_order", self.ptr, order, interp)

    def _order(self):
        o, t = ctypes.c_int(), ctypes.c_int()
        k = np.zeros(3)
        call("tmrg_qforest_get_mesh_order", self.ptr, ctypes.byref(o), ctypes.byref(t), _ptr(k))
        return o.value, t.value, k[: o.value]

    def getMeshOrder(self):
        return self._order()[0]

    def getInterpType(self):
        return self._order()[1]

    def getInterpKnots(self):
        return self._order()[2]

    def setConnectivity(self, conn):
        conn = np.ascontiguousarray(conn, dtype=np.intc)
        if conn.ndim != 2 or conn.shape[1] != 4:
            raise ValueError("Expected array of shape (n, 4)")
        call("tmrg_qforest_set_connectivity", self.ptr, int(conn.max()) + 1, _ptr(conn),
             conn.shape[0])

    def setFullConnectivity(self, conn, edge_conn, num_nodes=None, num_edges=None):
        conn = np.ascontiguousarray(conn, dtype=np.intc)
        ec = np.ascontiguousarray(edge_conn, dtype=np.intc)
        if conn.shape != ec.shape or conn.shape[1] != 4:
            raise ValueError("Expected arrays of shape (n, 4)")
        nn = int(conn.max()) + 1 if num_nodes is None else num_nodes
        ne = int(ec.max()) + 1 if num_edges is None else num_edges
        call("tmrg_qforest_set_full_connectivity", self.ptr, nn, ne, conn.shape[0], _ptr(conn),
             _ptr(ec))

    def getConnectivity(self):
        """(face_conn (n, 4), face_edge_conn (n, 4), num_nodes, num_edges)."""
        sz = np.zeros(3, np.intc)
        call("tmrg_qforest_get_connectivity", self.ptr, _ptr(sz), None, None)
        fc = np.zeros((sz[0], 4), np.intc)
        fe = np.zeros((sz[0], 4), np.intc)
        call("tmrg_qforest_get_connectivity", self.ptr, _ptr(sz), _ptr(fc), _ptr(fe))
        return fc, fe, int(sz[2]), int(sz[1])

    def createRandomTrees(self, nrand=10, min_lev=0, max_lev=8, seed=0):
        """TMRQuadForest::createRandomTrees (TMRQuadForest.cpp:1327-1407) with a
        seeded generator in place of libc rand()."""
        call("tmrg_qforest_create_random_trees", self.ptr, nrand, min_lev, max_lev, seed)

    def repartition(self):
        """TMRQuadForest::repartition: the forest lives on one GPU, nothing
        to redistribute."""
        return None

    def createTrees(self, depth=0):
        call("tmrg_qforest_create_trees", self.ptr, depth)

    def refine(self, refine=None, min_lev=0, max_lev=MAX_LEVEL):
        if refine is None:
            call("tmrg_qforest_refine", self.ptr, None, 0, min_lev, max_lev)
        elif _is_torch(refine) and refine.is_cuda:
            import torch
            r = refine.to(torch.int32).contiguous()
            call("tmrg_qforest_refine_device", self.ptr, _vp(r.data_ptr()), r.numel(),
                 min_lev, max_lev)
        else:
            r = np.ascontiguousarray(refine, dtype=np.intc)
            call("tmrg_qforest_refine", self.ptr, _ptr(r), r.size, min_lev, max_lev)

    def duplicate(self):
        return self._child("tmrg_qforest_duplicate")

    def coarsen(self):
        return self._child("tmrg_qforest_coarsen")

    def balance(self, btype=0):
        call("tmrg_qforest_balance", self.ptr, btype)

    def createNodes(self):
        call("tmrg_qforest_create_nodes", self.ptr)

    def getNumQuadrants(self):
        n = ctypes.c_int64(0)
        call("tmrg_qforest_num_quadrants", self.ptr, ctypes.byref(n))
        return n.value

    def getQuadrantsArray(self):
        """(n, 6) int32 {face, x, y, tag, level, info} in element order."""
        n = self.getNumQuadrants()
        out = np.zeros((n, 6), np.intc)
        if n:
            call("tmrg_qforest_get_quadrants", self.ptr, _ptr(out))
        return out

    def getQuadrants(self):
        return QuadrantArray(self.getQuadrantsArray())

    def _sizes(self):
        s = np.zeros(6, np.int64)
        call("tmrg_qforest_sizes", self.ptr, _ptr(s))
        return s

    def getNodeRange(self):
        return np.array([0, int(self._sizes()[1])], np.intc)

    def getExtPreOffset(self):
        return int(self._sizes()[3])

    def getMeshConn(self):
        s = self._sizes()
        o = self.getMeshOrder()
        out = np.zeros((int(s[4]), o * o), np.intc)
        call("tmrg_qforest_get_node_conn", self.ptr, _ptr(out))
        return out

    def getDepNodeConn(self):
        s = self._sizes()
        nd, nnz = int(s[2]), int(s[5])
        ptr = np.zeros(nd + 1, np.intc)
        conn = np.zeros(max(nnz, 1), np.intc)
        w = np.zeros(max(nnz, 1), np.float64)
        call("tmrg_qforest_get_dep_node_conn", self.ptr, _ptr(ptr), _ptr(conn), _ptr(w))
        return ptr, conn[:nnz], w[:nnz]

    def getNodeNumbers(self):
        """The local node numbers, sorted (dependent nodes negative)."""
        s = self._sizes()
        return np.arange(-int(s[2]), int(s[1]), dtype=np.intc)

    def getLocalNodeNumber(self, node):
        s = self._sizes()
        return int(node) + int(s[2]) if -int(s[2]) <= node < int(s[1]) else -1

    def createInterpolation(self, forest, vec):
        """P from `forest` (coarse) to this forest, into the VecInterp `vec`."""
        h = _vp()
        call("tmrg_qforest_create_interpolation", self.ptr, forest.ptr, ctypes.byref(h))
        vec.ptr = h
        return vec

    def setFaceBoxes(self, boxes):
        """A box (origin x, y, extent x, y) per face: the geometry getPoints
        maps nodes through; None removes it."""
        if boxes is None:
            call("tmrg_qforest_set_face_boxes", self.ptr, None, 0)
            return
        b = np.ascontiguousarray(boxes, dtype=np.float64)
        if b.ndim != 2 or b.shape[1] != 4:
            raise ValueError("Expected array of shape (n, 4)")
        call("tmrg_qforest_set_face_boxes", self.ptr, _ptr(b), b.shape[0])
        self._boxes = b.copy()

    def writeToVTK(self, fname):
        """writeToVTK (TMRQuadForest.cpp:651-720): the face mesh as VTK
        quadrilaterals, each connectivity node at its owner face's corner
        (the lowest-numbered face touching it) through the face boxes (the
        topology's surfaces in the reference), the face index as the cell
        scalar entity_index; nothing is written when no boxes are set."""
        boxes = getattr(self, "_boxes", None)
        if boxes is None:
            return
        fc = self.getConnectivity()[0]
        nf = fc.shape[0]
        nn = int(fc.max()) + 1 if nf else 0
        owner = np.full(nn, nf, np.int64)
        np.minimum.at(owner, fc.ravel(), np.repeat(np.arange(nf), 4))
        with open(fname, "w") as fp:
            fp.write("# vtk DataFile Version 3.0\nvtk output\nASCII\n")
            fp.write("DATASET UNSTRUCTURED_GRID\nPOINTS %d float\n" % nn)
            for k in range(nn):
                f = owner[k]
                corner = next(c for c in range(4) if fc[f, c] == k)
                p = boxes[f, :2] + boxes[f, 2:] * np.array([corner & 1, corner >> 1], np.float64)
                fp.write("%e %e %e\n" % (p[0], p[1], 0.0))
            fp.write("\nCELLS %d %d\n" % (nf, 5 * nf))
            for c in fc:
                fp.write("4 %d %d %d %d\n" % (c[0], c[1], c[3], c[2]))
            fp.write("\nCELL_TYPES %d\n" % nf)
            fp.write("9\n" * nf)
            fp.write("CELL_DATA %d\nSCALARS entity_index float 1\nLOOKUP_TABLE default\n" % nf)
            for k in range(nf):
                fp.write("%e\n" % (1.0 * k))

    def writeToTecplot(self, fname):
        """writeToTecplot (TMRQuadForest.cpp:729-804): the face mesh as one
        Tecplot FEQUADRILATERAL zone, nodes at their owner face's corner
        through the face boxes, the face index cell-centred; nothing is
        written when no boxes are set."""
        boxes = getattr(self, "_boxes", None)
        if boxes is None:
            return
        fc = self.getConnectivity()[0]
        nf = fc.shape[0]
        nn = int(fc.max()) + 1 if nf else 0
        owner = np.full(nn, nf, np.int64)
        np.minimum.at(owner, fc.ravel(), np.repeat(np.arange(nf), 4))
        X = np.zeros((nn, 3))
        for k in range(nn):
            f = owner[k]
            corner = next(c for c in range(4) if fc[f, c] == k)
            X[k, :2] = boxes[f, :2] + boxes[f, 2:] * np.array([corner & 1, corner >> 1],
                                                              np.float64)
        with open(fname, "w") as fp:
            fp.write("Variables = X,Y,Z,face\n")
            fp.write("Zone N = %d E = %d " % (nn, nf))
            fp.write("DATAPACKING=BLOCK, ZONETYPE=FEQUADRILATERAL\n")
            fp.write("VARLOCATION = ([4]=CELLCENTERED)\n")
            for d in range(3):
                for k in range(nn):
                    fp.write("%e\n" % X[k, d])
            for k in range(nf):
                fp.write("%e\n" % (1.0 * k))
            for c in fc:
                fp.write("%d %d %d %d\n" % (c[0] + 1, c[1] + 1, c[3] + 1, c[2] + 1))

    def writeForestToVTK(self, fname):
        """writeForestToVTK (TMRQuadForest.cpp:809-870): every quadrant as a
        quadrilateral with its own four corners (x fastest) through its
        face's box, the face index as the cell scalar entity_index; nothing
        is written when no boxes are set."""
        boxes = getattr(self, "_boxes", None)
        if boxes is None:
            return
        q = self.getQuadrantsArray()
        n = len(q)
        h = (1 << (30 - q[:, 4].astype(np.int64)))
        hmax = float(1 << 30)
        with open(fname, "w") as fp:
            fp.write("# vtk DataFile Version 3.0\nvtk output\nASCII\n")
            fp.write("DATASET UNSTRUCTURED_GRID\nPOINTS %d float\n" % (4 * n))
            for r, hh in zip(q, h):
                b = boxes[r[0]]
                for jj in range(2):
                    for ii in range(2):
                        u = 1.0 * (r[1] + ii * hh) / hmax
                        v = 1.0 * (r[2] + jj * hh) / hmax
                        fp.write("%e %e %e\n" % (b[0] + b[2] * u, b[1] + b[3] * v, 0.0))
            fp.write("\nCELLS %d %d\n" % (n, 5 * n))
            for k in range(n):
                c = 4 * k
                fp.write("4 %d %d %d %d\n" % (c, c + 1, c + 3, c + 2))
            fp.write("\nCELL_TYPES %d\n" % n)
            fp.write("9\n" * n)
            fp.write("CELL_DATA %d\nSCALARS entity_index float 1\nLOOKUP_TABLE default\n" % n)
            for r in q:
                fp.write("%e\n" % (1.0 * r[0]))

    def getPoints(self):
        s = self._sizes()
        X = np.zeros((int(s[0]), 3))
        call("tmrg_qforest_get_points", self.ptr, _ptr(X))
        return X

    def evalInterp(self, pt, derivs=0):
        """TMRQuadForest::evalInterp (:1069-1160) for the Lagrange knots:
        N (and the d/du, d/dv tables with derivs=1) at the parametric point
        pt in [-1, 1]^2, N[i + j order] = Nu[i] Nv[j]."""
        o = self.getMeshOrder()
        k = self.getInterpKnots()

        def lag(u):
            # lagrange_shape_func_derivative (TMRInterpolation.h), same
            # operation order
            N = [1.0] * o
            D = [0.0] * o
            for i in range(o):
                for j in range(o):
                    if i != j:
                        d = 1.0 / (k[i] - k[j])
                        N[i] *= (u - k[j]) * d
                        for m in range(o):
                            if m != i and m != j:
                                d *= (u - k[m]) / (k[i] - k[m])
                        D[i] += d
            return N, D
        k = [float(v) for v in k]
        Nu, Du = lag(float(pt[0]))
        Nv, Dv = lag(float(pt[1]))
        N = np.array([Nu[i] * Nv[j] for j in range(o) for i in range(o)])
        if not derivs:
            return N
        N1 = np.array([Du[i] * Nv[j] for j in range(o) for i in range(o)])
        N2 = np.array([Nu[i] * Dv[j] for j in range(o) for i in range(o)])
        return N, N1, N2


class VecInterp:
    """Prolongation operator P (fine rows x coarse columns); the TACS
    TACSBVecInterp role in TMR (createInterpolation target)."""

    def __init__(self):
        self.ptr = None

    def _create(self, fine, coarse):
        h = _vp()
        call("tmrg_interp_create", fine.ptr, coarse.ptr, ctypes.byref(h))
        self.ptr = h

    def __del__(self):
        try:
            if self.ptr:
                lib().tmrg_interp_destroy(self.ptr)
                self.ptr = None
        except Exception:
            pass

    def sizes(self):
        s = np.zeros(3, np.int64)
        call("tmrg_interp_sizes", self.ptr, _ptr(s))
        return int(s[0]), int(s[1]), int(s[2])

    def applyNnz(self):
        """Entries the applies use: P without its numerically-zero weights
        (|w| < 2^-49), which changes no product by more than 1e-13 of
        max |x|."""
        n = ctypes.c_int64(0)
        call("tmrg_interp_apply_nnz", self.ptr, ctypes.byref(n))
        return int(n.value)

    def getCSR(self):
        rows, cols, nnz = self.sizes()
        rp = np.zeros(rows + 1, np.intc)
        c = np.zeros(max(nnz, 1), np.intc)
        w = np.zeros(max(nnz, 1), np.float64)
        call("tmrg_interp_get_csr", self.ptr, _ptr(rp), _ptr(c), _ptr(w))
        return rp, c[:nnz], w[:nnz]

    def _apply(self, which, x, y):
        names = ("tmrg_interp_mult", "tmrg_interp_mult_transpose",
                 "tmrg_interp_mult_weight_transpose")
        rows, cols, _ = self.sizes()
        nin, nout = (cols, rows) if which == 0 else (rows, cols)
        nvec = _check_vectors(names[which], x, y, nin, nout, ("float64",))
        if _is_torch(x):
            call(names[which] + "_device", self.ptr, _vp(x.data_ptr()),
                 _vp(y.data_ptr()), nvec)
        else:
            x = np.ascontiguousarray(x, dtype=np.float64)
            direct = (isinstance(y, np.ndarray) and y.dtype == np.float64
                      and y.flags.c_contiguous)
            out = y if direct else np.zeros(y.shape, np.float64)
            call(names[which], self.ptr, _ptr(x), _ptr(out), nvec)
            if not direct:
                y[...] = out
        return y

    def mult(self, x, y):
        return self._apply(0, x, y)

    def multTranspose(self, x, y):
        return self._apply(1, x, y)

    def multWeightTranspose(self, x, y):
        return self._apply(2, x, y)


class MatrixFilter:
    """Matrix density filter (TMRMatrixFilter, TMR.pyx MatrixFilter).

    ``MatrixFilter(r, N, assemblers, filters)`` as in the reference; the
    assemblers are ignored (no TACS) and the filter is built on
    ``filters[0]`` (an OctForest whose blocks are cubes of side
    ``block_len``, or a QuadForest whose faces are squares of that side).  The
    remaining forests form the restriction hierarchy used by
    ``setDesignVars`` (TMRConformFilter.cpp:75-91).
    """

    def __init__(self, r, N, assemblers=None, filters=None, block_len=1.0, vpn=1):
        self.filters = list(filters)
        self.vpn = vpn
        h = _vp()
        name = ("tmrg_filter_create_quad" if isinstance(self.filters[0], QuadForest)
                else "tmrg_filter_create")
        call(name, self.filters[0].ptr, float(block_len), float(r), int(N), ctypes.byref(h))
        self.ptr = h
        self.interps = []
        for k in range(len(self.filters) - 1):
            I = VecInterp()
            self.filters[k].createInterpolation(self.filters[k + 1], I)
            self.interps.append(I)

    def __del__(self):
        try:
            if self.ptr:
                lib().tmrg_filter_destroy(self.ptr)
                self.ptr = None
        except Exception:
            pass

    def size(self):
        s = np.zeros(2, np.int64)
        call("tmrg_filter_sizes", self.ptr, _ptr(s))
        return int(s[0]), int(s[1])

    def getMatrix(self):
        n, nnz = self.size()
        rp = np.zeros(n + 1, np.intc)
        c = np.zeros(max(nnz, 1), np.intc)
        v = np.zeros(max(nnz, 1), np.float64)
        A = np.zeros(n, np.float64)
        B = np.zeros(n, np.float64)
        T = np.zeros(n, np.float64)
        call("tmrg_filter_get_matrix", self.ptr, _ptr(rp), _ptr(c), _ptr(v), _ptr(A),
             _ptr(B), _ptr(T))
        return rp, c[:nnz], v[:nnz], A, B, T

    def _apply(self, transpose, x, y, vpn=None):
        vpn = vpn or self.vpn
        n = self.size()[0]
        what = "MatrixFilter.applyTranspose" if transpose else "MatrixFilter.applyFilter"
        dts = ("float64", "float32") if _is_torch(x) else ("float64",)
        if _check_vectors(what, x, y, n, n, dts) != vpn:
            raise ValueError("%s: x holds %d values, expected %d nodes x vpn %d"
                             % (what, np.size(x) if not _is_torch(x) else x.numel(), n, vpn))
        if _is_torch(x):
            import torch
            if x.dtype == torch.float32:
                name = "tmrg_filter_apply_transpose_f32_device" if transpose else \
                    "tmrg_filter_apply_f32_device"
            else:
                name = "tmrg_filter_apply_transpose_device" if transpose else \
                    "tmrg_filter_apply_device"
            call(name, self.ptr, vpn, _vp(x.data_ptr()), _vp(y.data_ptr()))
        else:
            x = np.ascontiguousarray(x, dtype=np.float64)
            out = np.zeros(x.shape, np.float64)
            name = "tmrg_filter_apply_transpose" if transpose else "tmrg_filter_apply"
            call(name, self.ptr, vpn, _ptr(x), _ptr(out))
            y[...] = out
        return y

    def applyFilter(self, x, y, vpn=None):
        return self._apply(False, x, y, vpn)

    def applyTranspose(self, x, y, vpn=None):
        return self._apply(True, x, y, vpn)

    def setDesignVars(self, x):
        """Filter x on the finest filter level and restrict it down the
        hierarchy with the weight-normalised transpose
        (TMRMatrixFilter.cpp:272-320).  Returns the per-level vectors."""
        levels = [self._apply(False, x, _like(x))]
        for I in self.interps:
            rows, cols, _ = I.sizes()
            out = _zeros_like(x, cols * self.vpn)
            I.multWeightTranspose(levels[-1], out)
            levels.append(out)
        return levels

    def addValues(self, g):
        """Gradient with respect to the unfiltered design variables
        (TMRMatrixFilter.cpp:325-368)."""
        return self._apply(True, g, _like(g))


class ConformFilter:
    """TMRConformFilter (TMRConformFilter.cpp:33-168; TMR.pyx
    ConformFilter): the design variables live on the finest filter forest
    and are restricted level by level with the weight-normalised P^T
    (setDesignVars, :144-156).  ``assemblers`` are accepted and ignored
    (no TACS); ``filters`` is the list of forests, finest first, each
    balanced with nodes created.  applyFilter / applyTranspose are not
    implemented by the reference for this filter (TMRTopoFilter.h: message
    on stderr, no output), and likewise here."""

    _name = "TMRConformFilter"

    def __init__(self, assemblers=None, filters=None, vpn=1):
        if assemblers is not None and len(assemblers) != len(filters):
            raise ValueError("%s must have equal number of objects in lists" %
                             type(self).__name__)
        self.filters = list(filters)
        self.vpn = vpn
        self.interps = []
        for k in range(len(self.filters) - 1):
            I = VecInterp()
            self.filters[k].createInterpolation(self.filters[k + 1], I)
            self.interps.append(I)
        self.x = None

    def getFilter(self):
        return self.filters[0]

    def getNumLevels(self):
        return len(self.filters)

    def setDesignVars(self, x):
        """x on the finest level, then x[k+1] = P_k^T-weighted x[k]; returns
        the per-level vectors (the reference hands each to its level's
        assembler)."""
        levels = [x]
        for I in self.interps:
            rows, cols, _ = I.sizes()
            out = _zeros_like(x, cols * self.vpn)
            I.multWeightTranspose(levels[-1], out)
            levels.append(out)
        self.x = levels
        return levels

    def getDesignVars(self):
        return None if self.x is None else self.x[0]

    def addValues(self, g):
        """The gradient with respect to the finest-level variables: for this
        filter the reference only completes the vector's parallel
        assembly (addValues, :161-164), so it is returned unchanged."""
        return g

    def setValues(self, g):
        return g

    def writeSTLFile(self, k, cutoff, filename):
        """writeSTLFile (TMRConformFilter.h:58-61): the binary STL file of
        design component k of the finest-level design variables (set by
        setDesignVars) at level `cutoff`."""
        if self.x is not None:
            writeSTLToBin(filename, self.filters[0], self.x[0], index=k, cutoff=cutoff,
                          vpn=self.vpn)

    def applyFilter(self, x, y, vpn=None):
        import sys
        sys.stderr.write("TMR Filter Error: applyFilter() method is not implemented!\n")

    def applyTranspose(self, x, y, vpn=None):
        import sys
        sys.stderr.write("TMR Filter Error: applyTranspose() method is not implemented!\n")


class LagrangeFilter(ConformFilter):
    """TMRLagrangeFilter (TMRLagrangeFilter.cpp:31-150; TMR.pyx
    LagrangeFilter): the same level-by-level weight-normalised restriction
    of the design variables as ConformFilter (setDesignVars, :130-139)."""

    _name = "TMRLagrangeFilter"


class HelmholtzFilter(ConformFilter):
    """TMRHelmholtzFilter (TMRHelmholtzFilter.cpp:29-276; TMR.pyx
    HelmholtzFilter(radius, assemblers, filters)): the Helmholtz PDE filter
    psi = K^-1 M x on the finest filter forest, solved with conjugate
    gradients preconditioned by a multigrid V-cycle over the filter
    forests (OctForests, or QuadForests for the 2-D filter).
    ``assemblers`` are accepted and ignored (no TACS); every forest needs
    its nodes and block boxes (``setBlockBoxes`` / ``setFaceBoxes``): the
    boxes are the geometry the element integrals use."""

    _name = "TMRHelmholtzFilter"

    def __init__(self, r, assemblers=None, filters=None, vpn=1):
        ConformFilter.__init__(self, assemblers, filters, vpn)
        arr = (ctypes.c_void_p * len(self.filters))(*[f.ptr for f in self.filters])
        h = _vp()
        name = ("tmrg_helmholtz_create_quad" if isinstance(self.filters[0], QuadForest)
                else "tmrg_helmholtz_create")
        call(name, arr, len(self.filters), float(r), ctypes.byref(h))
        self.ptr = h
        self.r = r

    def __del__(self):
        try:
            if self.ptr:
                lib().tmrg_helmholtz_destroy(self.ptr)
                self.ptr = None
        except Exception:
            pass

    def sizes(self):
        """Per level (independent nodes, elements, dependent nodes,
        scatter-list entries)."""
        n = ctypes.c_int(0)
        out = np.zeros(4 * len(self.filters), np.int64)
        call("tmrg_helmholtz_sizes", self.ptr, ctypes.byref(n), _ptr(out))
        return out.reshape(-1, 4)[: n.value]

    def setTolerances(self, rtol=1e-12, atol=1e-30, max_iters=300):
        call("tmrg_helmholtz_set_tolerances", self.ptr, float(rtol), float(atol),
             int(max_iters))

    def setSmoother(self, degree_order2=5, degree_order3=6, lower_order2=0.05,
                    lower_order3=0.1, upper=1.1):
        """Chebyshev smoother of the multigrid preconditioner (degree and
        interval, as fractions of the largest eigenvalue estimate of
        D^-1 K, per level order); changes the iteration count only."""
        call("tmrg_helmholtz_set_smoother", self.ptr, int(degree_order2), int(degree_order3),
             float(lower_order2), float(lower_order3), float(upper))

    def lastSolve(self):
        """(iterations, residual norm per component) of the last solve."""
        it = ctypes.c_int(0)
        res = np.zeros(16)
        call("tmrg_helmholtz_last_solve", self.ptr, ctypes.byref(it), _ptr(res), 16)
        return it.value, res

    def _apply(self, transpose, x, y, vpn=None):
        vpn = vpn or self.vpn
        n = int(self.sizes()[0][0])
        what = "HelmholtzFilter.applyTranspose" if transpose else "HelmholtzFilter.applyFilter"
        if _check_vectors(what, x, y, n, n, ("float64",)) != vpn:
            raise ValueError("%s: vectors hold %d nodes x %d values, vpn is %d"
                             % (what, n, (x.numel() if _is_torch(x) else np.size(x)) // n, vpn))
        if _is_torch(x):
            name = ("tmrg_helmholtz_apply_transpose_device" if transpose
                    else "tmrg_helmholtz_apply_device")
            call(name, self.ptr, vpn, _vp(x.data_ptr()), _vp(y.data_ptr()))
        else:
            x = np.ascontiguousarray(x, dtype=np.float64)
            out = np.zeros(x.shape, np.float64)
            name = "tmrg_helmholtz_apply_transpose" if transpose else "tmrg_helmholtz_apply"
            call(name, self.ptr, vpn, _ptr(x), _ptr(out))
            y[...] = out
        return y

    def applyFilter(self, x, y, vpn=None):
        """applyFilter (:126-196): y = K^-1 M x per component."""
        return self._apply(False, x, y, vpn)

    def applyTranspose(self, x, y, vpn=None):
        """applyTranspose (:199-247): y = M K^-1 x per component."""
        return self._apply(True, x, y, vpn)

    def mult(self, level, which, x, y, nvec=1):
        """y = K x (which = 0) or M x (which = 1) on filter level `level`
        (torch CUDA tensors)."""
        sz = self.sizes()
        if not 0 <= level < len(sz):
            raise ValueError("HelmholtzFilter.mult: level %d of %d" % (level, len(sz)))
        n = int(sz[level][0])
        if not (_is_torch(x) and _is_torch(y)):
            raise ValueError("HelmholtzFilter.mult: x and y must be CUDA tensors")
        if _check_vectors("HelmholtzFilter.mult", x, y, n, n, ("float64",)) != nvec:
            raise ValueError("HelmholtzFilter.mult: vectors hold %d values, expected %d x %d"
                             % (x.numel(), n, nvec))
        call("tmrg_helmholtz_mult_device", self.ptr, int(level), int(which), int(nvec),
             _vp(x.data_ptr()), _vp(y.data_ptr()))
        return y

    def setDesignVars(self, x):
        """setDesignVars (:252-262): filter x, then restrict it level by
        level with the weight-normalised P^T; returns the per-level
        vectors."""
        return ConformFilter.setDesignVars(self, self._apply(False, x, _like(x)))

    def addValues(self, g):
        """addValues (:267-272): the gradient with respect to the unfiltered
        variables, applyTranspose of g."""
        return self._apply(True, g, _like(g))


def _stl_values(forest, x, vpn):
    n = forest.getNodeRange()[1]
    if vpn is None:
        vpn = max(1, len(x) // max(n, 1))
    if len(x) != n * vpn:
        raise ValueError("design vector length %d is not %d nodes x %d values" %
                         (len(x), n, vpn))
    return vpn


def getSTLTriangles(forest, x, offset=0, cutoff=0.5, root=0, vpn=None):
    """getSTLTriangles (TMR.pyx; TMR_GenerateSTLTriangles,
    TMR_STLTools.cpp:639-902): the points (3 ntris, 3) of the triangles of
    the level set x[offset] = cutoff, or np.array([[]]) when there are
    none.  x: numpy or torch CUDA array of vpn interleaved values per
    independent node of `forest`; `root` is accepted (one process)."""
    vpn = _stl_values(forest, x, vpn)
    n = ctypes.c_int64(0)
    if _is_torch(x):
        import torch
        fn, xp = "tmrg_stl_triangles_device", _vp(x.data_ptr())
        call(fn, forest.ptr, xp, vpn, int(offset), float(cutoff), ctypes.byref(n), None, 0)
        out = torch.empty(max(n.value, 1) * 9, dtype=torch.float64, device=x.device)
        call(fn, forest.ptr, xp, vpn, int(offset), float(cutoff), ctypes.byref(n),
             _vp(out.data_ptr()), n.value)
        pts = out[: 9 * n.value].reshape(-1, 3).cpu().numpy()
    else:
        xh = np.ascontiguousarray(x, dtype=np.float64)
        call("tmrg_stl_triangles", forest.ptr, _ptr(xh), vpn, int(offset), float(cutoff),
             ctypes.byref(n), None, 0)
        pts = np.zeros(max(n.value, 1) * 9)
        call("tmrg_stl_triangles", forest.ptr, _ptr(xh), vpn, int(offset), float(cutoff),
             ctypes.byref(n), _ptr(pts), n.value)
        pts = pts[: 9 * n.value].reshape(-1, 3)
    if n.value == 0:
        return np.array([[]])
    return pts


def writeSTLToBin(fname, forest, x, index=0, cutoff=0.5, vpn=None):
    """writeSTLToBin (TMR.pyx; TMR_GenerateBinFile): the triangles of the
    level set x[index] = cutoff to a binary file (int32 count, then 9
    doubles a triangle)."""
    xh = x.detach().cpu().numpy() if _is_torch(x) else x
    xh = np.ascontiguousarray(xh, dtype=np.float64)
    vpn = _stl_values(forest, xh, vpn)
    call("tmrg_generate_bin_file", str(fname).encode(), forest.ptr, _ptr(xh), vpn, int(index),
         float(cutoff))


def convertBinToSTL(binfile, stlfile):
    """TMR_ConvertBinToSTL (the reference's bstltostl converter): the ASCII
    STL file of a binary triangle file."""
    call("tmrg_convert_bin_to_stl", str(binfile).encode(), str(stlfile).encode())


def createTopoWeights(filter, forest):
    """Design -> analysis weights of TMROctTACSTopoCreator
    (TMR_TACSTopoCreator.cpp:55-183) as a VecInterp: rows = elements of
    `forest`, columns = owned nodes of `filter`; mult maps filter design
    values to element values."""
    I = VecInterp()
    h = _vp()
    call("tmrg_topo_weights_create", filter.ptr, forest.ptr, ctypes.byref(h))
    I.ptr = h
    return I


def interpolateDesignVec(orig_filter, orig_x, new_filter, new_x):
    """interpolateDesignVec (TopOptUtils.py:270-307): the design values on
    `orig_filter`'s nodes carried to `new_filter`'s nodes through
    new_filter.createInterpolation(orig_filter); vectors node-major with
    any number of values per node."""
    I = VecInterp()
    new_filter.createInterpolation(orig_filter, I)
    I.mult(orig_x, new_x)
    return new_x


def _like(x):
    if _is_torch(x):
        import torch
        return torch.empty_like(x)
    return np.zeros_like(x)


def _zeros_like(x, n):
    if _is_torch(x):
        import torch
        return torch.zeros(n, dtype=x.dtype, device=x.device)
    return np.zeros(n, dtype=np.float64)


def kernel_launch_count():
    return int(lib().tmrg_kernel_launch_count())


def host_sync_count():
    return int(lib().tmrg_host_sync_count())


def version():
    return lib().tmrg_version().decode()


def random_refinement(n, seed, stream, prob, device="cuda"):
    """Seeded 0/1 refinement indicator on the GPU (the synthetic
    workloads' U(seed, stream, i) < prob)."""
    import torch
    out = torch.empty(n, dtype=torch.int32, device=device)
    cs = torch.cuda.current_stream().cuda_stream
    call("tmrg_random_refinement_device", int(seed), int(stream), float(prob),
         _vp(out.data_ptr()), n, _vp(cs))
    return out


def bump_indicator(forest, centres, sigma, t_refine, t_coarsen, min_level, max_level):
    """Refine (+1) / coarsen (-1) / keep (0) flags of `forest`'s octants
    from a sum of Gaussian bumps at CUDA `centres` (K x 3, float64) with
    widths `sigma` (3), through the forest's block boxes.  Returns a CUDA
    int32 tensor; ordered on the forest's stream."""
    import torch
    n = forest.getNumOctants()
    out = torch.empty(max(n, 1), dtype=torch.int32, device="cuda")
    c = centres.contiguous()
    sg = np.ascontiguousarray(sigma, dtype=np.float64)
    call("tmrg_bump_indicator_device", forest.ptr, _vp(c.data_ptr()), int(c.shape[0]),
         _ptr(sg), float(t_refine), float(t_coarsen), int(min_level), int(max_level),
         _vp(out.data_ptr()))
    return out[:n]
