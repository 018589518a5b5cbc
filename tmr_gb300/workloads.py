"""Seeded synthetic forests: the block connectivities and refinement
indicators of the benchmark configurations and the parity cases.

Every random draw is U(seed, stream, i) = splitmix64-based uniform on
[0, 1) (``uniform`` below, and the identical device generator behind
``TMR.random_refinement``), so a GPU run and a CPU run see the same input.
"""
import itertools

import numpy as np

HMAX = 1 << 30
_M64 = (1 << 64) - 1


def _splitmix64(x):
    x = (x + 0x9E3779B97F4A7C15) & _M64
    x = ((x ^ (x >> 30)) * 0xBF58476D1CE4E5B9) & _M64
    x = ((x ^ (x >> 27)) * 0x94D049BB133111EB) & _M64
    return x ^ (x >> 31)


def uniform(seed, stream, n):
    """U(seed, stream, i) for i < n, vectorised (uint64 arithmetic wraps)."""
    base = np.uint64(_splitmix64((seed * 0x100000001B3 + stream) & _M64))
    i = np.arange(n, dtype=np.uint64)
    with np.errstate(over="ignore"):
        x = base ^ (i * np.uint64(0xD6E8FEB86659FD93))
        x = x + np.uint64(0x9E3779B97F4A7C15)
        x = (x ^ (x >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        x = (x ^ (x >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        x = x ^ (x >> np.uint64(31))
    return (x >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def brick(nx, ny, nz):
    """Block connectivity of an nx x ny x nz brick of unit hexahedra; node
    (i, j, k) is numbered i + (nx+1)(j + (ny+1)k), block corners x fastest
    (the corner order of TMROctForest.cpp:29-37)."""
    def nid(i, j, k):
        return i + (nx + 1) * (j + (ny + 1) * k)
    conn = []
    for k in range(nz):
        for j in range(ny):
            for i in range(nx):
                conn.append([nid(i + (c & 1), j + ((c >> 1) & 1), k + (c >> 2))
                             for c in range(8)])
    return np.array(conn, dtype=np.intc)


def _rotations():
    R = []
    for perm in itertools.permutations(range(3)):
        for flips in range(8):
            M = np.zeros((3, 3), int)
            for a in range(3):
                M[a, perm[a]] = -1 if (flips >> a) & 1 else 1
            if round(np.linalg.det(M)) == 1:
                R.append(M)
    return R


def rotate_blocks(conn, seed):
    """Relabel each block's corners by a seeded cube rotation, so that
    neighbouring blocks meet with all face orientations and reversed
    edges."""
    R = _rotations()
    pick = (uniform(seed, 99, conn.shape[0]) * len(R)).astype(int)
    out = conn.copy()
    for b in range(conn.shape[0]):
        M = R[pick[b]]
        for c in range(8):
            v = np.array([c & 1, (c >> 1) & 1, c >> 2]) * 2 - 1
            w = M @ v
            src = (w[0] + 1) // 2 + 2 * ((w[1] + 1) // 2) + 4 * ((w[2] + 1) // 2)
            out[b, c] = conn[b, src]
    return out


def octant_centres(octs):
    """Block-local centres in [0, 1]^3 of an (n, 7) octant array."""
    h = (1 << (30 - octs[:, 5].astype(np.int64))).astype(np.float64)
    return (octs[:, 1:4].astype(np.float64) + 0.5 * h[:, None]) / float(HMAX)


def sphere_indicator(octs, centre=(0.5, 0.5, 0.5), radius=0.3):
    """1 where the octant centre lies within `radius` of `centre` (single
    unit-cube block, the configuration with ~300k octants)."""
    c = octant_centres(octs)
    return ((((c - np.asarray(centre)) ** 2).sum(1)) < radius * radius).astype(np.intc)


def point_indicator(octs, point):
    """1 where the octant contains the block-local point (in [0, 1)^3, on
    the 2^30 integer grid), in every block: one refinement path per block
    down to any depth."""
    p = np.floor(np.asarray(point, np.float64) * HMAX).astype(np.int64)
    h = (np.int64(1) << (30 - octs[:, 5].astype(np.int64)))
    xyz = octs[:, 1:4].astype(np.int64)
    inside = ((xyz <= p[None, :]) & (p[None, :] < xyz + h[:, None])).all(1)
    return inside.astype(np.intc)


def quad_point_indicator(quads, point):
    """The 2-D point_indicator over an (n, 6) {face, x, y, tag, level, info}
    quadrant array: 1 where the quadrant contains the face-local point."""
    p = np.floor(np.asarray(point, np.float64) * HMAX).astype(np.int64)
    h = (np.int64(1) << (30 - quads[:, 4].astype(np.int64)))
    xy = quads[:, 1:3].astype(np.int64)
    inside = ((xy <= p[None, :]) & (p[None, :] < xy + h[:, None])).all(1)
    return inside.astype(np.intc)


def random_indicator(n, seed, stream, prob):
    return (uniform(seed, stream, n) < prob).astype(np.intc)


def mixed_indicator(n, seed, stream, prob, coarsen_prob):
    """+1 (refine) where U < prob, -1 (coarsen) where U >= 1 - coarsen_prob,
    0 elsewhere."""
    u = uniform(seed, stream, n)
    out = np.zeros(n, np.intc)
    out[u < prob] = 1
    out[u >= 1.0 - coarsen_prob] = -1
    return out


# ---- the benchmark configurations ----------------------------------------
# C1: one tree, uniform level 4, 3 sphere passes to level 7, order 2.
C1 = dict(conn=lambda: brick(1, 1, 1), L0=4, passes=3, max_level=7, order=2,
          indicator="sphere", levels=2)
# C2: 8x4x4 brick, uniform level 2, 5 passes refining with p = 0.3 (seed 7)
# to level 9, order 3, 4-level hierarchy, P/P^T on 16 vectors.
C2 = dict(conn=lambda: brick(8, 4, 4), L0=2, passes=5, max_level=9, order=3,
          indicator="random", prob=0.3, seed=7, levels=4, nvec=16)


def brick2d(nx, ny):
    """Face connectivity of an nx x ny grid of unit squares: node (i, j) is
    numbered i + (nx+1) j, face corners x fastest (the corner order of
    TMRQuadForest.cpp:24-31)."""
    conn = []
    for j in range(ny):
        for i in range(nx):
            n0 = i + (nx + 1) * j
            conn.append([n0, n0 + 1, n0 + nx + 1, n0 + nx + 2])
    return np.array(conn, dtype=np.intc)


def rotate_faces(conn, seed):
    """Relabel each face's corners by a seeded symmetry of the square
    (rotations and reflections), so that neighbouring faces meet with
    reversed edges."""
    # corner (a, b) of the square -> index a + 2b; the 8 symmetries as maps
    # of (a, b)
    maps = [lambda a, b: (a, b), lambda a, b: (1 - b, a), lambda a, b: (1 - a, 1 - b),
            lambda a, b: (b, 1 - a), lambda a, b: (b, a), lambda a, b: (1 - a, b),
            lambda a, b: (a, 1 - b), lambda a, b: (1 - b, 1 - a)]
    rng = np.random.default_rng(seed)
    out = np.array(conn, dtype=np.intc).copy()
    for f in range(len(out)):
        m = maps[int(rng.integers(0, 8))]
        new = np.empty(4, np.intc)
        for c in range(4):
            a, b = c & 1, c >> 1
            na, nb = m(a, b)
            new[na + 2 * nb] = out[f, c]
        out[f] = new
    return out
