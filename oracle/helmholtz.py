"""CPU restatement of the Helmholtz PDE density filter (test infrastructure
only: used by tests, the smoke check and the benchmark's CPU-baseline leg;
the product never imports it).

TMRHelmholtzFilter (TMRHelmholtzFilter.cpp:29-247) filters a design field
x on the finest filter forest by solving the Helmholtz problem

    K psi = M x,   K = int(r^2 grad N . grad N + N N),  M = int(N N)

with the element weak form of TMRHexaHelmholtzModel
(TMRHelmholtzModel.cpp:67-97: DUt = u, DUx = r^2 grad u) on the basis
TMROctTACSMatrixCreator gives each forest order (TMRMatrixCreator.h:76-92:
order 2 linear hexahedron, order 3 quadratic Bernstein hexahedron), and
condenses dependent (hanging) nodes onto the independent nodes they
interpolate, as TACS assembles through the forest's dependent weights.
applyFilter (:126-196) returns psi = K^-1 M x per design component;
applyTranspose (:199-247) returns M K^-1 x.

The element integrals restate the published TACS element loop
(TACSElement3D with a TACS hexahedral basis; TACS is a third-party library
that the reference builds against, unpinned, and that is absent from the
reference tree): Gauss quadrature with `order` points a direction, the
isoparametric map of the element's node coordinates, and the residual
weights wt * detJ.  The reference's own solve is GMRES(50) with a
geometric-multigrid preconditioner to a relative residual of 1e-12; this
restatement solves the assembled sparse system directly (scipy), which the
iterative answer matches to that tolerance.

Parity for this filter is unpinned against the reference itself (TACS is
not available to run); it is anchored on the restated integrals and on
exact properties: K 1 = M 1 (a constant field is unchanged), symmetry of K
and M, and the adjoint identity <y, F x> = <F^T y, x>.
"""
import numpy as np

_GAUSS = {
    2: (np.array([-1.0 / np.sqrt(3.0), 1.0 / np.sqrt(3.0)]), np.array([1.0, 1.0])),
    3: (np.array([-np.sqrt(0.6), 0.0, np.sqrt(0.6)]), np.array([5.0 / 9.0, 8.0 / 9.0, 5.0 / 9.0])),
}


def basis_1d(order, u):
    """Values and derivatives of the 1-D factors of the element basis at u:
    order 2 the linear Lagrange pair, order 3 the quadratic Bernstein
    polynomials on [-1, 1]."""
    if order == 2:
        return np.array([0.5 * (1.0 - u), 0.5 * (1.0 + u)]), np.array([-0.5, 0.5])
    if order == 3:
        N = np.array([0.25 * (1.0 - u) ** 2, 0.5 * (1.0 - u) * (1.0 + u), 0.25 * (1.0 + u) ** 2])
        D = np.array([-0.5 * (1.0 - u), -u, 0.5 * (1.0 + u)])
        return N, D
    raise ValueError("Helmholtz filter: forest order must be 2 or 3")


def element_points(oct_row, order, knots, boxes):
    """Node coordinates of one element (order^3 x 3), x fastest: the block
    box map of the octant's knot positions."""
    b, x, y, z, _, lev, _ = (int(v) for v in oct_row)
    s = 1.0 / (1 << 30)
    d = (1 << (30 - lev)) * s
    X = np.zeros((order ** 3, 3))
    for k in range(order):
        for j in range(order):
            for i in range(order):
                u = (x * s + 0.5 * d * (1.0 + knots[i]),
                     y * s + 0.5 * d * (1.0 + knots[j]),
                     z * s + 0.5 * d * (1.0 + knots[k]))
                for a in range(3):
                    X[i + order * j + order * order * k, a] = boxes[b, a] + boxes[b, 3 + a] * u[a]
    return X


def element_matrices(Xpts, order, r):
    """Element stiffness K_e and mass M_e by the TACS element loop: for each
    Gauss point, Xd = dX/dxi, J = Xd^-1, detJ, then
    K_e += wt detJ (r^2 (J^T dN)(J^T dN)^T + N N^T) and M_e += wt detJ N N^T."""
    pts, wts = _GAUSS[order]
    n = order ** 3
    Ke = np.zeros((n, n))
    Me = np.zeros((n, n))
    for kq in range(order):
        for jq in range(order):
            for iq in range(order):
                Nx, Dx = basis_1d(order, pts[iq])
                Ny, Dy = basis_1d(order, pts[jq])
                Nz, Dz = basis_1d(order, pts[kq])
                wt = wts[iq] * wts[jq] * wts[kq]
                N = np.einsum("k,j,i->kji", Nz, Ny, Nx).ravel()
                dN = np.stack([np.einsum("k,j,i->kji", Nz, Ny, Dx).ravel(),
                               np.einsum("k,j,i->kji", Nz, Dy, Nx).ravel(),
                               np.einsum("k,j,i->kji", Dz, Ny, Nx).ravel()], axis=1)
                Xd = Xpts.T @ dN  # Xd[a, c] = dX_a / dxi_c
                detJ = np.linalg.det(Xd)
                J = np.linalg.inv(Xd)
                G = dN @ J  # dN/dX
                h = wt * detJ
                Ke += h * (r * r * (G @ G.T) + np.outer(N, N))
                Me += h * np.outer(N, N)
    return Ke, Me


def slot_matrix(conn, dep_ptr, dep_conn, dep_w, num_nodes):
    """S (num_nodes x element slots): slot e*npe + a of an independent node g
    holds 1 in row g; a dependent slot holds its weights in the rows of the
    nodes it interpolates.  The global matrices are S blockdiag(A_e) S^T."""
    import scipy.sparse as sp
    conn = np.asarray(conn).ravel()
    dep_ptr = np.asarray(dep_ptr, np.int64)
    slots = np.arange(len(conn))
    ind = conn >= 0
    d = -conn[~ind] - 1
    cnt = dep_ptr[d + 1] - dep_ptr[d]
    first = np.repeat(dep_ptr[d], cnt)
    off = np.arange(cnt.sum()) - np.repeat(np.cumsum(cnt) - cnt, cnt)
    rows = np.concatenate([conn[ind], np.asarray(dep_conn)[first + off]])
    cols = np.concatenate([slots[ind], np.repeat(slots[~ind], cnt)])
    vals = np.concatenate([np.ones(ind.sum()), np.asarray(dep_w)[first + off]])
    return sp.csr_matrix((vals, (rows, cols)), shape=(num_nodes, len(conn)))


def assemble(octs, conn, dep_ptr, dep_conn, dep_w, num_nodes, order, knots, boxes, r):
    """Global K and M (scipy CSR, num_nodes square) with every dependent
    slot expanded through its weights."""
    import scipy.sparse as sp
    npe = order ** 3
    ne = len(octs)
    Ks = np.zeros((ne, npe, npe))
    Ms = np.zeros((ne, npe, npe))
    cache = {}  # the matrices depend only on the node offsets from node 0
    for e in range(ne):
        X = element_points(octs[e], order, knots, boxes)
        key = (X - X[0]).tobytes()
        if key not in cache:
            cache[key] = element_matrices(X, order, r)
        Ks[e], Ms[e] = cache[key]
    S = slot_matrix(conn, dep_ptr, dep_conn, dep_w, num_nodes)
    ip = np.arange(ne + 1)
    Kb = sp.bsr_matrix((Ks, np.arange(ne), ip), shape=(ne * npe, ne * npe))
    Mb = sp.bsr_matrix((Ms, np.arange(ne), ip), shape=(ne * npe, ne * npe))
    return (S @ Kb @ S.T).tocsr(), (S @ Mb @ S.T).tocsr()


def apply_filter(K, M, x, vpn=1):
    """applyFilter: psi = K^-1 M x for every interleaved component."""
    import scipy.sparse.linalg as sla
    x = np.asarray(x, np.float64).reshape(-1, vpn)
    lu = sla.splu(K.tocsc())
    return np.stack([lu.solve(M @ x[:, k]) for k in range(vpn)], axis=1).ravel()


def apply_transpose(K, M, x, vpn=1):
    """applyTranspose: M K^-1 x for every interleaved component."""
    import scipy.sparse.linalg as sla
    x = np.asarray(x, np.float64).reshape(-1, vpn)
    lu = sla.splu(K.tocsc())
    return np.stack([M @ lu.solve(x[:, k]) for k in range(vpn)], axis=1).ravel()


# ---------------------------------------------------------------------------
# The 2-D filter on quadtree forests (TMRQuadHelmholtzModel,
# TMRHelmholtzModel.cpp:23-59; TMRQuadTACSMatrixCreator's bilinear /
# quadratic Bernstein quadrilaterals).
def element_points2d(quad_row, order, knots, boxes):
    """Node coordinates of one quadrilateral (order^2 x 2), x fastest."""
    f, x, y = int(quad_row[0]), int(quad_row[1]), int(quad_row[2])
    lev = int(quad_row[4])
    s = 1.0 / (1 << 30)
    d = (1 << (30 - lev)) * s
    X = np.zeros((order ** 2, 2))
    for j in range(order):
        for i in range(order):
            u = (x * s + 0.5 * d * (1.0 + knots[i]), y * s + 0.5 * d * (1.0 + knots[j]))
            for a in range(2):
                X[i + order * j, a] = boxes[f, a] + boxes[f, 2 + a] * u[a]
    return X


def element_matrices2d(Xpts, order, r):
    pts, wts = _GAUSS[order]
    n = order ** 2
    Ke = np.zeros((n, n))
    Me = np.zeros((n, n))
    for jq in range(order):
        for iq in range(order):
            Nx, Dx = basis_1d(order, pts[iq])
            Ny, Dy = basis_1d(order, pts[jq])
            wt = wts[iq] * wts[jq]
            N = np.einsum("j,i->ji", Ny, Nx).ravel()
            dN = np.stack([np.einsum("j,i->ji", Ny, Dx).ravel(),
                           np.einsum("j,i->ji", Dy, Nx).ravel()], axis=1)
            Xd = Xpts.T @ dN
            detJ = np.linalg.det(Xd)
            G = dN @ np.linalg.inv(Xd)
            h = wt * detJ
            Ke += h * (r * r * (G @ G.T) + np.outer(N, N))
            Me += h * np.outer(N, N)
    return Ke, Me


def assemble2d(quads, conn, dep_ptr, dep_conn, dep_w, num_nodes, order, knots, boxes, r):
    """Global K and M of a quadtree forest (scipy CSR)."""
    import scipy.sparse as sp
    npe = order ** 2
    ne = len(quads)
    Ks = np.zeros((ne, npe, npe))
    Ms = np.zeros((ne, npe, npe))
    cache = {}
    for e in range(ne):
        X = element_points2d(quads[e], order, knots, boxes)
        key = (X - X[0]).tobytes()
        if key not in cache:
            cache[key] = element_matrices2d(X, order, r)
        Ks[e], Ms[e] = cache[key]
    S = slot_matrix(conn, dep_ptr, dep_conn, dep_w, num_nodes)
    ip = np.arange(ne + 1)
    Kb = sp.bsr_matrix((Ks, np.arange(ne), ip), shape=(ne * npe, ne * npe))
    Mb = sp.bsr_matrix((Ms, np.arange(ne), ip), shape=(ne * npe, ne * npe))
    return (S @ Kb @ S.T).tocsr(), (S @ Mb @ S.T).tocsr()
