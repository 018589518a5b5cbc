"""CPU restatement of the iso-surface triangles of a design field
(TMR_GenerateSTLTriangles, TMR_STLTools.cpp:639-852) and of the reference's
binary and ASCII STL formats (TMR_GenerateBinFile :904-966,
TMR_ConvertBinToSTL :968-993, TriangleList::writeSTLFile :544-574).  Test
infrastructure only: tests, the smoke check and the benchmark's CPU
baseline use it; the product never imports it.

The element/cell traversal, corner values (dependent nodes through their
weights), boundary-face detection and the crossing-point formula
(vertex_interp, :339-356) follow the reference line by line.  The case
tables are rebuilt here from one rule (coded independently of the
library's C++ construction): on a face whose corners alternate
inside/outside (inside = value < cutoff) the inside corners are separated;
face segments run from the counter-clockwise boundary's exit crossing to
its entry crossing and chain into loops; each loop, from its lowest edge
number, and each boundary-face polygon (solid corners and crossings,
counter-clockwise from outside) is split into a fan.  Against the
reference's own tables (Bourke's, compiled in oracle/_ref) the crossing
points are bit-equal and the loops agree wherever the reference makes the
same face choice; tests compare per cell the vertex sets, triangle counts
and vector areas.
"""
import struct

import numpy as np

CORNER = [(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0), (0, 0, 1), (1, 0, 1), (1, 1, 1), (0, 1, 1)]
EDGE = [(0, 1), (1, 2), (2, 3), (3, 0), (4, 5), (5, 6), (6, 7), (7, 4), (0, 4), (1, 5), (2, 6),
        (3, 7)]
FACE = [(0, 4, 7, 3), (1, 2, 6, 5), (0, 1, 5, 4), (3, 7, 6, 2), (0, 3, 2, 1), (4, 5, 6, 7)]


def _edge_id(a, b):
    for e, (p, q) in enumerate(EDGE):
        if {p, q} == {a, b}:
            return e
    raise ValueError


def volume_table():
    """case -> list of (edge, edge, edge) triangles."""
    table = []
    for c in range(256):
        inside = [(c >> i) & 1 for i in range(8)]
        succ = {}
        for q in FACE:
            crossings = []  # (position on the face boundary, edge, kind)
            for k in range(4):
                a, b = q[k], q[(k + 1) % 4]
                if inside[a] != inside[b]:
                    crossings.append((k, _edge_id(a, b), "exit" if inside[a] else "entry"))
            for k_en, e_en, kind in crossings:
                if kind != "entry":
                    continue
                # the inside arc that starts here ends at the next exit
                exits = [(((k_ex - k_en) % 4), e_ex) for k_ex, e_ex, kd in crossings
                         if kd == "exit"]
                succ[min(exits)[1]] = e_en
        tris = []
        seen = set()
        for e0 in sorted(succ):
            if e0 in seen:
                continue
            loop = []
            e = e0
            while e not in seen:
                seen.add(e)
                loop.append(e)
                e = succ[e]
            tris += [(loop[0], loop[i], loop[i + 1]) for i in range(1, len(loop) - 1)]
        table.append(tris)
    return table


def face_table():
    """case (bit i: corner i of the face below the cutoff) -> triangles
    of vertex ids (0-3 corners, 4+i the crossing on face edge (i, i+1))."""
    table = []
    for c in range(16):
        poly = []
        for i in range(4):
            below_i, below_j = (c >> i) & 1, (c >> ((i + 1) % 4)) & 1
            if not below_i:
                poly.append(i)
            if below_i != below_j:
                poly.append(4 + i)
        table.append([(poly[0], poly[i], poly[i + 1]) for i in range(1, len(poly) - 1)])
    return table


def vertex_interp(iso, p1, p2, v1, v2):
    """vertex_interp (TMR_STLTools.cpp:339-356)."""
    if abs(iso - v1) <= 0.0:
        return p1
    if abs(iso - v2) <= 0.0:
        return p2
    if abs(v1 - v2) <= 0.0:
        return p1
    mu = (iso - v1) / (v2 - v1)
    return tuple(p1[a] + mu * (p2[a] - p1[a]) for a in range(3))


def boundary_faces(block_face, face_ptr):
    """6 flags per block: the block face is shared by one block."""
    bf = np.asarray(block_face).reshape(-1, 6)
    fp = np.asarray(face_ptr)
    return (fp[bf + 1] - fp[bf]) == 1


def triangles(octs, conn, dep, X, x, vpn, offset, cutoff, order, bface, cells=False):
    """The triangles (n, 3, 3) in the reference's order; with cells=True
    also the (element, cell) each triangle comes from."""
    vt, ft = volume_table(), face_table()
    dptr, dconn, dw = dep
    ndep = len(dptr) - 1
    o = order
    hmax = 1 << 30
    out, where = [], []
    x = np.asarray(x, np.float64)
    X = np.asarray(X, np.float64)
    for e in range(len(octs)):
        b, ox, oy, oz, _, lev, _ = (int(v) for v in octs[e])
        h = 1 << (30 - lev)
        fb = [bface[b, 0] and ox == 0, bface[b, 1] and ox + h == hmax,
              bface[b, 2] and oy == 0, bface[b, 3] and oy + h == hmax,
              bface[b, 4] and oz == 0, bface[b, 5] and oz + h == hmax]
        c = conn[e]
        lv, P = [], []
        for idx in range(o ** 3):
            g = int(c[idx])
            P.append(tuple(X[g + ndep]))
            if g >= 0:
                lv.append(x[g * vpn + offset])
            else:
                d = -g - 1
                s = 0.0
                for jp in range(dptr[d], dptr[d + 1]):
                    s += dw[jp] * x[dconn[jp] * vpn + offset]
                lv.append(s)
        cell_id = 0
        for iz in range(o - 1):
            for iy in range(o - 1):
                for ix in range(o - 1):
                    val, pts, onb = [0.0] * 8, [None] * 8, [False] * 8
                    for m, (ii, jj, kk) in enumerate(CORNER):
                        off = (ix + ii) + (iy + jj) * o + (iz + kk) * o * o
                        val[m] = lv[off]
                        pts[m] = P[off]
                        onb[m] = bool((fb[0] and ix == 0 and ii == 0) or
                                      (fb[1] and ix == o - 2 and ii == 1) or
                                      (fb[2] and iy == 0 and jj == 0) or
                                      (fb[3] and iy == o - 2 and jj == 1) or
                                      (fb[4] and iz == 0 and kk == 0) or
                                      (fb[5] and iz == o - 2 and kk == 1))
                    ci = sum(1 << m for m in range(8) if val[m] < cutoff)
                    for t in vt[ci]:
                        tri = [vertex_interp(cutoff, pts[EDGE[ed][0]], pts[EDGE[ed][1]],
                                             val[EDGE[ed][0]], val[EDGE[ed][1]]) for ed in t]
                        out.append(tri)
                        where.append((e, cell_id))
                    if any(onb):
                        for q in FACE:
                            if not all(onb[m] for m in q):
                                continue
                            fv = [val[m] for m in q]
                            fp = [pts[m] for m in q]
                            fi = sum(1 << i for i in range(4) if fv[i] < cutoff)
                            vert = fp + [vertex_interp(cutoff, fp[i], fp[(i + 1) % 4], fv[i],
                                                       fv[(i + 1) % 4]) for i in range(4)]
                            for t in ft[fi]:
                                out.append([vert[k] for k in t])
                                where.append((e, cell_id))
                    cell_id += 1
    tris = np.array(out, np.float64).reshape(-1, 3, 3)
    return (tris, np.array(where, np.int64).reshape(-1, 2)) if cells else tris


def write_bin(path, tris):
    """TMR_GenerateBinFile's layout: int32 count, then 9 doubles a triangle."""
    tris = np.ascontiguousarray(tris, np.float64).reshape(-1, 9)
    with open(path, "wb") as fp:
        fp.write(struct.pack("=i", len(tris)))
        fp.write(tris.tobytes())


def stl_ascii(tris):
    """TriangleList::writeSTLFile's text for the triangles."""
    lines = ["solid topology"]
    for t in np.asarray(tris, np.float64).reshape(-1, 3, 3):
        a = t[1] - t[0]
        b = t[2] - t[0]
        n = [a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]]
        norm = float(np.sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]))
        with np.errstate(invalid="ignore", divide="ignore"):
            n = [float(np.float64(v) / np.float64(norm)) for v in n]
        lines.append("facet normal %e %e %e" % tuple(n))
        lines.append("outer loop")
        for k in range(3):
            lines.append("vertex %e %e %e" % tuple(t[k]))
        lines.append("endloop")
        lines.append("endfacet")
    lines.append("endsolid topology")
    return "\n".join(lines) + "\n"
