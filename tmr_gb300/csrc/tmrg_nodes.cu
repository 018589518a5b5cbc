// createNodes on the GPU (TMROctForest.cpp:3455-5519), hash-free:
//   1. hanging face/edge flags per octant by binary search in the sorted
//      octant keys (computeDepFacesAndEdges);
//   2. every element emits its corner (order 2) or 27 node objects in the
//      owner tree's frame (transformNode); one radix sort of the node keys
//      gives the node order of the reference (compareNode), and the unique
//      run index of each (element, object) entry is its local node;
//   3. dependent nodes are labelled, then one scan numbers independent
//      nodes 0.. and dependent nodes -1, -2, .. in node order;
//   4. the dependent-node CSR is sized by a scan; when several elements
//      write the same row the last one in element order wins, as in the
//      reference's sequential loop, resolved with a 64-bit atomicMax.
#include <vector>

#include "tmrg_tree.cuh"

namespace tmrg {

// Knots and the reciprocals 1/(k_i - k_j) (rounded once on the host, as
// the reference rounds them), so the device Lagrange basis needs no FP64
// division.
struct Knots {
  double k[TMRG_MAX_ORDER];
  double r[TMRG_MAX_ORDER][TMRG_MAX_ORDER];
  // Bernstein elements: bt[u + order - 1] are the coarse-edge weights of
  // refined control point u (bernstein_subdivision)
  int bern;
  double bt[2 * TMRG_MAX_ORDER - 1][TMRG_MAX_ORDER];
  // Lagrange elements: the 1-D weights of the dependent rows, by knot and
  // child side (lagrange_tables): le[k + order * side] for an edge node,
  // lf[k + order * side] for either direction of a face node
  double le[2 * TMRG_MAX_ORDER][TMRG_MAX_ORDER];
  double lf[2 * TMRG_MAX_ORDER][TMRG_MAX_ORDER];
};

// The Lagrange basis at u (TMRInterpolation.h:40-52): N_i the product over
// j != i, ascending, of (u - k_j) * (1 / (k_i - k_j)), in IEEE double
// without contraction, so the host values equal a device evaluation.
static void host_lagrange(int order, double u, const Knots &kn, double *N) {
  for (int i = 0; i < order; i++) {
    double v = 1.0;
    for (int j = 0; j < order; j++)
      if (i != j) v = v * ((u - kn.k[j]) * kn.r[i][j]);
    N[i] = v;
  }
}

// The 1-D weights of the dependent rows (createDependentConn,
// TMROctForest.cpp:5337-5519 with the knots of TMRInterpolation): an edge
// node at knot k of the half-edge on `side` (0 or 1) of its parent edge
// sits at u = (side - 1) + (1 + k_k) / 2 of the parent's [-1, 1]; a face
// node at u = (-1 + (1 + k_k) / 2) + side in each face direction.  The row
// kernel reads them instead of evaluating the basis per row.
static void lagrange_tables(int order, Knots &kn) {
  for (int side = 0; side < 2; side++)
    for (int k = 0; k < order; k++) {
      const double h = 0.5 * (1.0 + kn.k[k]);
      host_lagrange(order, (double)(side - 1) + h, kn, kn.le[k + order * side]);
      host_lagrange(order, (-1.0 + h) + (double)side, kn, kn.lf[k + order * side]);
    }
}

// Dependent-node weights of Bernstein elements (eval_bernstein_weights,
// TMRInterpolation.h:309-439, used by createDependentConn at
// TMROctForest.cpp:5364-5373 and 5453-5473): refined control point
// u in [-(order-1), order-1] of the two half-edges, by de Casteljau
// subdivision at t = 1/2.  Left half (u = r - (order-1)): C(r, i) / 2^r of
// coarse point i <= r; right half (u = r): C(order-1-r, i-r) / 2^(order-1-r)
// of coarse point i >= r.  Short dyadic fractions, exact in double, so they
// equal the reference's tabulated literals.  The reference tabulates orders
// 2-5; other orders are rejected before this is used.
static void bernstein_subdivision(int order, Knots &kn) {
  kn.bern = 1;
  const int p = order - 1;
  for (int u = -p; u <= p; u++) {
    double *N = kn.bt[u + p];
    for (int i = 0; i < TMRG_MAX_ORDER; i++) N[i] = 0.0;
    const int r = u <= 0 ? u + p : u, m = u <= 0 ? r : p - r, first = u <= 0 ? 0 : r;
    double c = 1.0;
    for (int i = 0; i <= m; i++) {
      N[first + i] = c / (double)(1 << m);
      c = c * (m - i) / (i + 1);
    }
  }
}

// Labels distinguish node objects at one position for order > 3
// (initLabel, TMROctForest.cpp:6798-6811).
struct Labels {
  int l[4];
  int bits;
};
static Labels make_labels(int order, int interp) {
  Labels L;
  if (order > 3 || (order >= 3 && interp == TMRG_BERNSTEIN_POINTS)) {
    for (int i = 0; i < 4; i++) L.l[i] = i;
    L.bits = 2;
  } else {
    for (int i = 0; i < 4; i++) L.l[i] = 0;
    L.bits = 0;
  }
  return L;
}

// ---------------------------------------------------------------------
// 1. Hanging flags.
template <typename Key>
__global__ void k_oct_keys(long long n, OctKeyT<Key> K, const int *__restrict__ blk,
                           const int *__restrict__ xs, const int *__restrict__ ys,
                           const int *__restrict__ zs,
                           const int16_t *__restrict__ lev, Key *keys) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) keys[i] = K.make(blk[i], xs[i], ys[i], zs[i], lev[i]);
}

template <typename Key>
__global__ void k_dep_info(long long n, ConnDev c, OctKeyT<Key> K,
                           const Key *__restrict__ keys,
                           const int *__restrict__ blk,
                           const int *__restrict__ xs, const int *__restrict__ ys,
                           const int *__restrict__ zs,
                           const int16_t *__restrict__ lev, int16_t *info) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  Oct o{blk[i], xs[i], ys[i], zs[i], lev[i]};
  if (o.level == 0) {
    info[i] = 0;
    return;
  }
  const int32_t hmax = TMRG_HMAX;
  auto exists = [&](const Oct &q) {
    return contains_key(keys, n, K.make(q.block, q.x, q.y, q.z, q.level));
  };
  int id = child_id(o);
  Oct p = parent_of(o);
  int bits = 0;
  for (int k = 0; k < 3; k++) {
    int fi = child_face(id, k);
    Oct nb = face_nbr(p, fi);
    bool hit = false;
    if (in_tree(nb)) {
      hit = exists(nb);
    } else {
      for_images(c, nb, side_of(nb.level), false, [&](const Oct &q) {
        if (!hit && exists(q)) hit = true;
      });
    }
    if (hit) bits |= 1 << k;
  }
  for (int k = 0; k < 3; k++) {
    int e = child_edge(id, k);
    Oct nb = edge_nbr(p, e);
    bool out = nb.x < 0 || nb.x >= hmax || nb.y < 0 || nb.y >= hmax ||
               nb.z < 0 || nb.z >= hmax;
    bool hit = false;
    if (!out) {
      hit = exists(nb);
    } else {
      for_images(c, nb, side_of(nb.level), false, [&](const Oct &q) {
        if (!hit && exists(q)) hit = true;
      });
    }
    if (hit) bits |= 1 << (k + 3);
  }
  info[i] = (int16_t)bits;
}

// decode_index_from_info (TMROctForest.cpp:250-276).
__device__ __forceinline__ void decode_info(int id, int info, int &fbits,
                                            int &ebits) {
  fbits = 0;
  ebits = 0;
  for (int k = 0; k < 3; k++) {
    if (info & (1 << k)) {
      fbits |= 1 << child_face(id, k);
      ebits |= 1 << child_face_edge(id, k, 0);
      ebits |= 1 << child_face_edge(id, k, 1);
    }
    if (info & (1 << (k + 3))) ebits |= 1 << child_edge(id, k);
  }
}

// ---------------------------------------------------------------------
// 2. Node objects.  Object j of an element: order 2 -> corner j
// (x fastest); order >= 3 -> (ii, jj, kk) = j % 3, j / 3 % 3, j / 9 on the
// half-size lattice.
struct NodeGen {
  int order, nobj;
  Labels lab;
  NodeKey NK;
};

__device__ __forceinline__ void object_of(const NodeGen &g, const Oct &e, int j,
                                          int32_t &x, int32_t &y, int32_t &z,
                                          int &label, int &mult, int &edge_dir) {
  edge_dir = -1;
  if (g.order == 2) {
    int32_t h = side_of(e.level);
    x = e.x + h * (j & 1);
    y = e.y + h * ((j >> 1) & 1);
    z = e.z + h * (j >> 2);
    label = g.lab.l[0];
    mult = 1;
    return;
  }
  int32_t h = (int32_t)1 << (TMRG_MAX_LEVEL - e.level - 1);
  int ii = j % 3, jj = (j / 3) % 3, kk = j / 9;
  x = e.x + h * ii;
  y = e.y + h * jj;
  z = e.z + h * kk;
  bool fx = ii != 1, fy = jj != 1, fz = kk != 1;
  int m = g.order - 2;
  if (fx && fy && fz) {
    label = g.lab.l[0];
    mult = 1;
  } else if ((fy && fz) || (fx && fz) || (fx && fy)) {
    label = g.lab.l[1];
    mult = m;
    edge_dir = !fx ? 0 : (!fy ? 1 : 2);
  } else if (fx || fy || fz) {
    label = g.lab.l[2];
    mult = m * m;
  } else {
    label = g.lab.l[3];
    mult = m * m * m;
  }
}

template <typename Key>
__global__ void k_node_keys(long long n, ConnDev c, NodeGen g,
                            const int *__restrict__ blk,
                            const int *__restrict__ xs, const int *__restrict__ ys,
                            const int *__restrict__ zs,
                            const int16_t *__restrict__ lev, Key *keys,
                            uint32_t *vals) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n * g.nobj) return;
  // t < 2^32 (it is stored as a 32-bit value): a 32-bit division
  const unsigned tu = (unsigned)t;
  long long e = tu / (unsigned)g.nobj;
  int j = (int)(tu - (unsigned)e * (unsigned)g.nobj);
  Oct o{blk[e], xs[e], ys[e], zs[e], lev[e]};
  int32_t b = o.block, x, y, z;
  int label, mult, ed;
  object_of(g, o, j, x, y, z, label, mult, ed);
  transform_node(c, b, x, y, z, -1, nullptr, nullptr);
  keys[t] = NodeKeyT<Key>{g.NK.Lg, g.NK.bb, g.NK.lb}.make(b, x, y, z, label);
  vals[t] = (uint32_t)t;
}

// Sorted node-object keys -> run index per (element, object) and the
// unique keys/multiplicities.
template <typename Key>
__global__ void k_node_unique(long long m, const Key *__restrict__ keys,
                              const uint32_t *__restrict__ vals,
                              const unsigned *__restrict__ pos, int lab_bits,
                              int order, Key *ukeys, unsigned *umult,
                              unsigned *obj_of) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) return;
  unsigned idx = pos[i + 1] - 1;  // inclusive count - 1
  obj_of[vals[i]] = idx;
  if (pos[i + 1] != pos[i]) {
    const Key k = keys[i];
    ukeys[idx] = k;
    int label = lab_bits ? (int)(klo64(k) & 3) : 0;
    int mm = order - 2;
    unsigned mult = (label == 0) ? 1u : (label == 1) ? mm : (label == 2) ? mm * mm : mm * mm * mm;
    umult[idx] = mult;
  }
}

// Flags for the unique pass (first entry of each run).
template <typename Key>
__global__ void k_first_of_run(long long m, const Key *__restrict__ keys, unsigned *flag) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < m) flag[i] = (i == 0 || keys[i] != keys[i - 1]) ? 1u : 0u;
}

// Element connectivity in local node numbers (createLocalConn,
// TMROctForest.cpp:4660-4867).
// Orders 2 and 3 (one node per object, objects in local-node order): conn
// entry i of the element-major array is the number of object i, one thread
// per entry so the object reads and conn writes are contiguous.
__global__ void k_local_conn_flat(long long m, const unsigned *__restrict__ obj_of,
                                  const unsigned *__restrict__ noff, int *lconn) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < m) lconn[i] = (int)noff[obj_of[i]];
}

// Order >= 4: one thread per element expands its edge/face/interior
// objects with the owner frame's edge reversal and face orientation.
__global__ void k_local_conn(long long n, ConnDev c, NodeGen g,
                             const int *__restrict__ blk,
                             const int *__restrict__ xs,
                             const int *__restrict__ ys,
                             const int *__restrict__ zs,
                             const int16_t *__restrict__ lev,
                             const unsigned *__restrict__ obj_of,
                             const unsigned *__restrict__ noff, int *lconn) {
  long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  const int o = g.order;
  const int npe = o * o * o;
  int *out = lconn + e * npe;
  const unsigned *ob = obj_of + e * g.nobj;
  Oct el{blk[e], xs[e], ys[e], zs[e], lev[e]};
  int rev[27], fid[27];
  for (int j = 0; j < 27; j++) {
    rev[j] = 0;
    fid[j] = 0;
    int32_t b = el.block, x, y, z;
    int label, mult, ed;
    object_of(g, el, j, x, y, z, label, mult, ed);
    int ii = j % 3, jj = (j / 3) % 3, kk = j / 9;
    int nmid = (ii == 1) + (jj == 1) + (kk == 1);
    if (nmid == 1)
      transform_node(c, b, x, y, z, ed, &rev[j], nullptr);
    else if (nmid == 2)
      transform_node(c, b, x, y, z, -1, nullptr, &fid[j]);
  }
  for (int kk = 0; kk < o; kk++)
    for (int jj = 0; jj < o; jj++)
      for (int ii = 0; ii < o; ii++) {
        int ci = (ii == 0) ? 0 : (ii == o - 1) ? 2 : 1;
        int cj = (jj == 0) ? 0 : (jj == o - 1) ? 2 : 1;
        int ck = (kk == 0) ? 0 : (kk == o - 1) ? 2 : 1;
        int j = ci + 3 * cj + 9 * ck;
        int base = (int)noff[ob[j]];
        int nmid = (ci == 1) + (cj == 1) + (ck == 1);
        int add = 0;
        if (nmid == 1) {
          int a = (ci == 1) ? ii : (cj == 1) ? jj : kk;
          add = rev[j] ? (o - 2 - a) : (a - 1);
        } else if (nmid == 2) {
          int a, b2;
          if (ci != 1) {
            a = jj;
            b2 = kk;
          } else if (cj != 1) {
            a = ii;
            b2 = kk;
          } else {
            a = ii;
            b2 = jj;
          }
          int32_t u, v;
          face_get(fid[j], o - 1, a, b2, u, v);
          add = (u - 1) + (v - 1) * (o - 2);
        } else if (nmid == 3) {
          add = (ii - 1) + (jj - 1) * (o - 2) + (kk - 1) * (o - 2) * (o - 2);
        }
        out[ii + jj * o + kk * o * o] = base + add;
      }
}

// ---------------------------------------------------------------------
// 3. Dependent labels (labelDependentNodes, TMROctForest.cpp:3711-3832).
__device__ __forceinline__ int edge_off(int o, int ei, int a) {
  if (ei < 4) return a + (o - 1) * (ei % 2) * o + (o - 1) * (ei / 2) * o * o;
  if (ei < 8) return (o - 1) * (ei % 2) + a * o + (o - 1) * ((ei - 4) / 2) * o * o;
  return (o - 1) * (ei % 2) + (o - 1) * ((ei - 8) / 2) * o + a * o * o;
}
__device__ __forceinline__ int face_off(int o, int fi, int a, int b) {
  if (fi < 2) return (o - 1) * (fi % 2) + a * o + b * o * o;
  if (fi < 4) return a + (o - 1) * (fi % 2) * o + b * o * o;
  return a + b * o + (o - 1) * (fi % 2) * o * o;
}

__global__ void k_label_dep(long long n, int order, int bern,
                            const int *__restrict__ xs,
                            const int *__restrict__ ys,
                            const int *__restrict__ zs,
                            const int16_t *__restrict__ lev,
                            const int16_t *__restrict__ info,
                            const int *__restrict__ lconn, unsigned *depflag) {
  long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  int inf = info[e];
  if (!inf) return;
  const int o = order;
  Oct el{0, xs[e], ys[e], zs[e], lev[e]};
  int id = child_id(el);
  int fb, eb;
  decode_info(id, inf, fb, eb);
  const int *c = lconn + e * (long long)(o * o * o);
  for (int fi = 0; fi < 6; fi++)
    if (fb & (1 << fi))
      for (int k = 0; k < 4; k++) eb |= 1 << face_edge(fi, k);
  bool m3 = (o == 3 && !bern);
  for (int ei = 0; ei < 12; ei++) {
    if (!(eb & (1 << ei))) continue;
    int sbit = (ei < 4) ? (id & 1) : (ei < 8) ? ((id >> 1) & 1) : (id >> 2);
    int st, en;
    if (sbit == 0) {
      st = 1;
      en = m3 ? o - 1 : o;
    } else {
      st = m3 ? 1 : 0;
      en = o - 1;
    }
    for (int a = st; a < en; a++) depflag[c[edge_off(o, ei, a)]] = 1u;
  }
  for (int fi = 0; fi < 6; fi++) {
    if (!(fb & (1 << fi))) continue;
    for (int b = 1; b < o - 1; b++)
      for (int a = 1; a < o - 1; a++) depflag[c[face_off(o, fi, a, b)]] = 1u;
  }
}

// ---------------------------------------------------------------------
// 4. Dependent CSR (createDependentConn, TMROctForest.cpp:5157-5519).
struct DepCtx {
  int order;
  Labels lab;
  NodeKey NK;  // the node key layout; 128-bit keys where wide
  ConnDev c;
  int wide;
  const uint64_t *ukeys;
  const U128 *ukeys_w;
  long long nobj;
  SampledKeys idx;
  SampledKeysT<U128> idx_w;
  const unsigned *noff;
  const unsigned *deprank;  // exclusive scan of dependent flags
  const unsigned *depflag;
  int *err;
};

__device__ __forceinline__ int dep_index(const DepCtx &d, int local) {
  return d.depflag[local] ? (int)d.deprank[local] : -1;
}

// Local node number of the object at (b, x, y, z) with `label`; also the
// owner-frame edge reversal / face orientation.
__device__ __forceinline__ int find_object(const DepCtx &d, int32_t b, int32_t x,
                                           int32_t y, int32_t z, int label,
                                           int edge_dir, int *rev, int *fid) {
  transform_node(d.c, b, x, y, z, edge_dir, rev, fid);
  long long i;
  bool found;
  if (d.wide) {
    const U128 k = NodeKeyT<U128>{d.NK.Lg, d.NK.bb, d.NK.lb}.make(b, x, y, z, label);
    i = d.idx_w.lower_bound(k);
    found = i < d.nobj && d.ukeys_w[i] == k;
  } else {
    const uint64_t k = d.NK.make(b, x, y, z, label);
    i = d.idx.lower_bound(k);
    found = i < d.nobj && d.ukeys[i] == k;
  }
  if (!found) {
    atomicExch(d.err, 1);
    return 0;
  }
  return (int)d.noff[i];
}

// getEdgeNodes (TMROctForest.cpp:4886-4963).
__device__ void parent_edge_nodes(const DepCtx &d, const Oct &p, int ei,
                                  int *out) {
  const int o = d.order;
  int32_t h = (int32_t)1 << (TMRG_MAX_LEVEL - p.level - 1);
  int32_t hp = side_of(p.level);
  int np = (o == 2) ? 2 : 3;
  int32_t step = (o == 2) ? hp : h;
  for (int ii = 0; ii < np; ii++) {
    int32_t x, y, z;
    if (ei < 4) {
      x = p.x + ii * step;
      y = p.y + hp * (ei % 2);
      z = p.z + hp * (ei / 2);
    } else if (ei < 8) {
      x = p.x + hp * (ei % 2);
      y = p.y + ii * step;
      z = p.z + hp * ((ei - 4) / 2);
    } else {
      x = p.x + hp * (ei % 2);
      y = p.y + hp * ((ei - 8) / 2);
      z = p.z + ii * step;
    }
    if (o == 2 || ii != 1) {
      int t = find_object(d, p.block, x, y, z, d.lab.l[0], -1, nullptr, nullptr);
      out[(o == 2) ? ii : (ii / 2) * (o - 1)] = t;
    } else {
      int rev = 0;
      int t = find_object(d, p.block, x, y, z, d.lab.l[1], ei / 4, &rev, nullptr);
      for (int k = 1; k < o - 1; k++) out[k] = t + (rev ? o - 2 - k : k - 1);
    }
  }
}

// getFaceNodes (TMROctForest.cpp:4984-5146).
__device__ void parent_face_nodes(const DepCtx &d, const Oct &p, int fi,
                                  int *out) {
  const int o = d.order;
  int32_t h = (int32_t)1 << (TMRG_MAX_LEVEL - p.level - 1);
  int np = (o == 2) ? 2 : 3;
  int32_t step = (o == 2) ? 2 * h : h;
  for (int jj = 0; jj < np; jj++)
    for (int ii = 0; ii < np; ii++) {
      int32_t x, y, z;
      if (fi < 2) {
        x = p.x + 2 * h * (fi % 2);
        y = p.y + ii * step;
        z = p.z + jj * step;
      } else if (fi < 4) {
        x = p.x + ii * step;
        y = p.y + 2 * h * (fi % 2);
        z = p.z + jj * step;
      } else {
        x = p.x + ii * step;
        y = p.y + jj * step;
        z = p.z + 2 * h * (fi % 2);
      }
      if (o == 2) {
        out[ii + 2 * jj] =
            find_object(d, p.block, x, y, z, d.lab.l[0], -1, nullptr, nullptr);
        continue;
      }
      bool ci = (ii != 1), cj = (jj != 1);
      if (ci && cj) {
        out[(ii / 2) * (o - 1) + (jj / 2) * (o - 1) * o] =
            find_object(d, p.block, x, y, z, d.lab.l[0], -1, nullptr, nullptr);
      } else if (ci || cj) {
        int e = (ii == 0) ? 0 : (ii == 2) ? 1 : (jj == 0) ? 2 : 3;
        int rev = 0;
        int t = find_object(d, p.block, x, y, z, d.lab.l[1],
                            face_edge(fi, e) / 4, &rev, nullptr);
        int incr = 1, start = (jj / 2) * (o - 1) * o;
        if (ii == 0 || ii == 2) {
          incr = o;
          start = (ii / 2) * (o - 1);
        }
        for (int k = 1; k < o - 1; k++)
          out[start + k * incr] = t + (rev ? o - 2 - k : k - 1);
      } else {
        int fid = 0;
        int t = find_object(d, p.block, x, y, z, d.lab.l[2], -1, nullptr, &fid);
        for (int k = 1; k < o - 1; k++)
          for (int j = 1; j < o - 1; j++) {
            int32_t u, v;
            face_get(fid, o - 1, j, k, u, v);
            out[j + k * o] = t + (u - 1) + (v - 1) * (o - 2);
          }
      }
    }
}

// Pass A: which dependent nodes sit on a hanging edge (row length order)
// or only on a hanging face (order^2).  Pass B: last writer per row, as
// (element+1) << 11 | (0..11 for an edge, 16..21 for a face) << 6 | position of
// the node on that edge/face; the maximum is the writer the reference's
// sequential loop (elements, then edges, then faces) leaves in place, and
// the position tells the row kernel which node of the edge/face it is.
template <int PASS>
__global__ void k_dep_rows(long long n, DepCtx d, const int *__restrict__ xs,
                           const int *__restrict__ ys,
                           const int *__restrict__ zs,
                           const int16_t *__restrict__ lev,
                           const int16_t *__restrict__ info,
                           const int *__restrict__ lconn, unsigned *has_edge,
                           unsigned *has_face, const int *__restrict__ dptr,
                           unsigned long long *writer) {
  long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  int inf = info[e];
  if (!inf) return;
  const int o = d.order;
  Oct el{0, xs[e], ys[e], zs[e], lev[e]};
  int id = child_id(el);
  int fb, eb;
  decode_info(id, inf, fb, eb);
  const int *c = lconn + e * (long long)(o * o * o);
  for (int ei = 0; ei < 12; ei++) {
    if (!(eb & (1 << ei))) continue;
    for (int k = 0; k < o; k++) {
      int di = dep_index(d, c[edge_off(o, ei, k)]);
      if (di < 0) continue;
      if (PASS == 0) {
        has_edge[di] = 1u;
      } else if (dptr[di + 1] - dptr[di] == o) {
        atomicMax(writer + di, ((unsigned long long)(e + 1) << 11) | ((unsigned)ei << 6) | (unsigned)k);
      }
    }
  }
  for (int fi = 0; fi < 6; fi++) {
    if (!(fb & (1 << fi))) continue;
    for (int b = 0; b < o; b++)
      for (int a = 0; a < o; a++) {
        int di = dep_index(d, c[face_off(o, fi, a, b)]);
        if (di < 0) continue;
        if (PASS == 0) {
          has_face[di] = 1u;
        } else if (dptr[di + 1] - dptr[di] == o * o) {
          atomicMax(writer + di, ((unsigned long long)(e + 1) << 11) |
                                     ((16u + (unsigned)fi) << 6) | (unsigned)(a + b * o));
        }
      }
  }
}

__global__ void k_dep_len(long long nd, int o, const unsigned *__restrict__ he,
                          const unsigned *__restrict__ hf, int *len) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < nd) len[i] = he[i] ? o : (hf[i] ? o * o : 0);
}

__global__ void __launch_bounds__(128, 12) k_dep_write(long long n, DepCtx d, Knots kn,
                            const int *__restrict__ blk,
                            const int *__restrict__ xs,
                            const int *__restrict__ ys,
                            const int *__restrict__ zs,
                            const int16_t *__restrict__ lev,
                            const int16_t *__restrict__ info,
                            const int *__restrict__ lconn,
                            const int *__restrict__ dptr,
                            const unsigned long long *__restrict__ writer,
                            const int *__restrict__ order, int *dconn, double *dw) {
  // One thread per dependent node: its winning writer (element, edge or
  // face, position) fixes the parent edge/face whose nodes form the row.
  // Threads take the nodes in `order` (edge rows first, then face rows),
  // so a warp runs one kind: an edge row takes `order` node lookups, a
  // face row order^2, and a warp of both kinds would run both paths.
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const long long di = order[t];
  const int o = d.order;
  unsigned long long w = writer[di];
  if (w == 0ULL) return;  // no writer: the row has length 0
  long long e = (long long)(w >> 11) - 1;
  int sub = (int)((w >> 6) & 31), pos = (int)(w & 63);
  Oct el{blk[e], xs[e], ys[e], zs[e], lev[e]};
  int id = child_id(el);
  int x = id % 2, y = (id % 4) / 2, z = id / 4;
  Oct p = parent_of(el);
  int ptr = dptr[di];
  if (dptr[di + 1] - ptr != (sub < 16 ? o : o * o)) return;
  if (sub < 16) {
    int ei = sub, k = pos;
    parent_edge_nodes(d, p, ei, dconn + ptr);
    int sb = (ei < 4) ? x : (ei < 8) ? y : z;
    const double *N = kn.bern ? kn.bt[(o - 1) * (sb - 1) + k + o - 1] : kn.le[k + o * sb];
    for (int j = 0; j < o; j++) dw[ptr + j] = N[j];
  } else {
    int fi = sub - 16, ii = pos % o, jj = pos / o;
    parent_face_nodes(d, p, fi, dconn + ptr);
    // the child offsets of the face's two directions; Bernstein: u =
    // -(order-1) + ii plus (order-1) times the offset, v likewise
    const int a = (fi < 2) ? y : x, b = (fi < 4) ? z : y;
    const double *Nu = kn.bern ? kn.bt[ii + (o - 1) * a] : kn.lf[ii + o * a];
    const double *Nv = kn.bern ? kn.bt[jj + (o - 1) * b] : kn.lf[jj + o * b];
    for (int j = 0; j < o * o; j++) dw[ptr + j] = __dmul_rn(Nu[j % o], Nv[j / o]);
  }
}

// Edge rows (writer on a parent edge) first, then the others, each in node
// order: flag, scan, then place.
__global__ void k_dep_edge_flag(long long n, const unsigned long long *__restrict__ writer,
                                unsigned *flag) {
  const long long di = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (di >= n) return;
  const unsigned long long w = writer[di];
  flag[di] = (w != 0ULL && ((w >> 6) & 31) < 16) ? 1u : 0u;
}
__global__ void k_dep_order(long long n, const unsigned long long *__restrict__ writer,
                            const unsigned *__restrict__ epos, int *order) {
  const long long di = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (di >= n) return;
  const unsigned long long w = writer[di];
  const bool edge = w != 0ULL && ((w >> 6) & 31) < 16;
  const long long k = edge ? (long long)epos[di] : (long long)epos[n] + (di - (long long)epos[di]);
  order[k] = (int)di;
}

// ---------------------------------------------------------------------
// Numbering and remap.
__global__ void k_number(long long nl, const unsigned *__restrict__ flag,
                         const unsigned *__restrict__ rank, int *num) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nl) return;
  num[i] = flag[i] ? -(int)rank[i] - 1 : (int)(i - (long long)rank[i]);
}
__global__ void k_remap(long long m, const int *__restrict__ num, int *a) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < m) a[i] = num[a[i]];
}

// ---------------------------------------------------------------------
// getPoints (TMROctForest.cpp:1476-1482, evaluateNodeLocations :5524-5680):
// each local node takes the position of its first (element, local index)
// in element order.  Without a geometry the reference leaves every point
// at 0; here a block may carry an axis-aligned box (origin, extent), the
// stand-in for TMRVolume::evalPoint on a box volume:
// X = origin + extent * (u + 0.5 d (1 + knot)), u = x / 2^30, d = h / 2^30.
__global__ void k_points_first_ref(long long n, int npe, long long num_dep,
                                   long long nlocal, const int *__restrict__ conn,
                                   unsigned long long *rep) {
  long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  const int *c = conn + e * npe;
  for (int l = 0; l < npe; l++) {
    long long li = (long long)__ldg(c + l) + num_dep;
    if (li >= 0 && li < nlocal)
      atomicMin(rep + li, ((unsigned long long)e << 8) | (unsigned)l);
  }
}
__global__ void k_points_eval(long long nlocal, int order, Knots kn,
                              const unsigned long long *__restrict__ rep,
                              const int *__restrict__ blk, const int *__restrict__ xs,
                              const int *__restrict__ ys, const int *__restrict__ zs,
                              const int16_t *__restrict__ lev,
                              const double *__restrict__ boxes, double *X) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nlocal) return;
  const unsigned long long r = rep[i];
  double p[3] = {0.0, 0.0, 0.0};
  if (r != ~0ULL && boxes) {
    const long long e = (long long)(r >> 8);
    const int l = (int)(r & 255u);
    const int ijk[3] = {l % order, (l / order) % order, l / (order * order)};
    const int32_t c[3] = {xs[e], ys[e], zs[e]};
    const double scale = 1.0 / (double)(1 << TMRG_MAX_LEVEL);
    const double d = (double)side_of(lev[e]) * scale;
    const double *bx = boxes + 6 * (long long)blk[e];
    for (int k = 0; k < 3; k++) {
      const double u = (double)c[k] * scale + 0.5 * d * (1.0 + kn.k[ijk[k]]);
      p[k] = bx[k] + bx[3 + k] * u;
    }
  }
  X[3 * i] = p[0];
  X[3 * i + 1] = p[1];
  X[3 * i + 2] = p[2];
}

void forest_get_points(Forest &f, const double *d_boxes, double *d_X) {
  if (!f.have_nodes) throw Error(TMRG_ERR_STATE, "getPoints: no nodes");
  cudaStream_t s = f.s;
  const int o = f.order, npe = o * o * o;
  const long long nlocal = f.num_local;
  DBuf<unsigned long long> rep(nlocal + 1, s);
  rep.fill_bytes(0xff);
  launch(k_points_first_ref, blocks_for(f.n, 256), 256, 0, s, f.n, npe, f.num_dep, nlocal,
         (const int *)f.econn.p, rep.p);
  Knots kn{};
  for (int i = 0; i < TMRG_MAX_ORDER; i++) kn.k[i] = i < o ? f.knots[i] : 0.0;
  launch(k_points_eval, blocks_for(nlocal, 256), 256, 0, s, nlocal, o, kn,
         (const unsigned long long *)rep.p, (const int *)f.block.p, (const int *)f.x.p,
         (const int *)f.y.p, (const int *)f.z.p, (const int16_t *)f.level.p, d_boxes, d_X);
  TMRG_CUDA(cudaStreamSynchronize(s));
}

// Hanging-face/edge flags of every octant (section 1 of createNodes).
template <typename Key>
static void hanging_flags(Forest &f, const OctKeyT<Key> &K) {
  cudaStream_t s = f.s;
  const long long n = f.n;
  DBuf<Key> okeys(n, s);
  launch(k_oct_keys<Key>, blocks_for(n, 256), 256, 0, s, n, K, (const int *)f.block.p,
         (const int *)f.x.p, (const int *)f.y.p, (const int *)f.z.p,
         (const int16_t *)f.level.p, okeys.p);
  launch(k_dep_info<Key>, blocks_for(n, 128), 128, 0, s, n, f.conn->dev, K,
         (const Key *)okeys.p, (const int *)f.block.p, (const int *)f.x.p,
         (const int *)f.y.p, (const int *)f.z.p, (const int16_t *)f.level.p, f.info.p);
}

// The distinct node objects (section 2): their sorted keys, multiplicities
// (in noff) and each (element, object)'s index.  Returns their number.
template <typename Key>
static long long node_objects(Forest &f, const NodeGen &g, long long m, DBuf<Key> &ukeys,
                              DBuf<unsigned> &noff, DBuf<unsigned> &obj_of) {
  cudaStream_t s = f.s;
  const long long n = f.n;
  DBuf<Key> keys(m, s);
  DBuf<uint32_t> vals(m, s);
  launch(k_node_keys<Key>, blocks_for(m, 256), 256, 0, s, n, f.conn->dev, g,
         (const int *)f.block.p, (const int *)f.x.p, (const int *)f.y.p,
         (const int *)f.z.p, (const int16_t *)f.level.p, keys.p, vals.p);
  sort_keys(keys, &vals, m, g.NK.total_bits(), s);
  DBuf<unsigned> pos(m + 1, s);
  launch(k_first_of_run<Key>, blocks_for(m, 256), 256, 0, s, m, (const Key *)keys.p, pos.p);
  exclusive_scan<unsigned>(pos.p, pos.p, m, s);
  const long long nobj = read_scalar(pos.p + m, s);
  ukeys.alloc(nobj, s);
  noff.alloc(nobj + 1, s);
  launch(k_node_unique<Key>, blocks_for(m, 256), 256, 0, s, m, (const Key *)keys.p,
         (const uint32_t *)vals.p, (const unsigned *)pos.p, g.lab.bits, g.order, ukeys.p,
         noff.p, obj_of.p);
  return nobj;
}

void forest_create_nodes(Forest &f) {
  Stage st("tmrg_create_nodes");
  if (!f.have_octs)
    throw Error(TMRG_ERR_STATE,
                "Cannot call createNodes(), no octants have been created");
  if (f.have_nodes) return;
  if (f.interp == TMRG_BERNSTEIN_POINTS && f.order > 5)
    throw Error(TMRG_ERR_UNSUPPORTED,
                "createNodes: Bernstein dependent weights exist for orders 2-5 "
                "(eval_bernstein_weights)");
  cudaStream_t s = f.s;
  const long long n = f.n;
  const int o = f.order, npe = o * o * o;
  ConnDev c = f.conn->dev;

  // 1. hanging flags
  const OctKey K = f.oct_key();
  if (K.total_bits() > 64)
    hanging_flags<U128>(f, OctKeyT<U128>{K.W, K.bb});
  else
    hanging_flags<uint64_t>(f, K);

  // 2. node objects
  NodeGen g;
  g.order = o;
  g.nobj = (o == 2) ? 8 : 27;
  g.lab = make_labels(o, f.interp);
  g.NK.Lg = f.maxlev + (o == 2 ? 0 : 1);
  g.NK.bb = f.conn->block_bits;
  g.NK.lb = g.lab.bits;
  if (g.NK.total_bits() > 128)
    throw Error(TMRG_ERR_KEY_RANGE, "node key needs " +
                                        std::to_string(g.NK.total_bits()) +
                                        " bits");
  if (o > 2 && f.maxlev >= TMRG_MAX_LEVEL)
    throw Error(TMRG_ERR_ARG, "createNodes: an order > 2 element at level " +
                                  std::to_string(TMRG_MAX_LEVEL) +
                                  " has no integer half-side for its nodes");
  const long long m = n * g.nobj;
  if (m >= (1LL << 32)) throw Error(TMRG_ERR_ARG, "createNodes: too many node objects");
  const bool wide = g.NK.total_bits() > 64;
  DBuf<uint64_t> ukeys;
  DBuf<U128> ukeys_w;
  DBuf<unsigned> noff;
  DBuf<unsigned> obj_of(m, s);
  long long nobj;
  if (wide)
    nobj = node_objects<U128>(f, g, m, ukeys_w, noff, obj_of);
  else
    nobj = node_objects<uint64_t>(f, g, m, ukeys, noff, obj_of);
  exclusive_scan<unsigned>(noff.p, noff.p, nobj, s);
  const long long nl = read_scalar(noff.p + nobj, s);
  f.num_local = nl;

  DBuf<int> lconn((size_t)n * npe, s);
  if (o == 2 || g.lab.bits == 0)  // g.nobj == npe
    launch(k_local_conn_flat, blocks_for(n * npe, 256), 256, 0, s, n * npe,
           (const unsigned *)obj_of.p, (const unsigned *)noff.p, lconn.p);
  else
    launch(k_local_conn, blocks_for(n, 128), 128, 0, s, n, c, g,
           (const int *)f.block.p, (const int *)f.x.p, (const int *)f.y.p,
           (const int *)f.z.p, (const int16_t *)f.level.p,
           (const unsigned *)obj_of.p, (const unsigned *)noff.p, lconn.p);
  obj_of.release();

  // 3. labels and numbering
  DBuf<unsigned> depflag(nl + 1, s);
  depflag.zero();
  launch(k_label_dep, blocks_for(n, 128), 128, 0, s, n, o,
         (int)(f.interp == TMRG_BERNSTEIN_POINTS), (const int *)f.x.p,
         (const int *)f.y.p, (const int *)f.z.p, (const int16_t *)f.level.p,
         (const int16_t *)f.info.p, (const int *)lconn.p, depflag.p);
  DBuf<unsigned> deprank(nl + 1, s);
  exclusive_scan<unsigned>(depflag.p, deprank.p, nl, s);
  const long long nd = read_scalar(deprank.p + nl, s);
  f.num_dep = nd;
  f.num_owned = nl - nd;
  f.ext_pre = nd;

  // 4. dependent CSR
  DBuf<int> err(1, s);
  err.zero();
  DepCtx d;
  d.order = o;
  d.lab = g.lab;
  d.NK = g.NK;
  d.c = c;
  d.wide = wide ? 1 : 0;
  d.ukeys = ukeys.p;
  d.ukeys_w = ukeys_w.p;
  d.nobj = nobj;
  const int S = 6;
  const long long ntop = (nobj + (1LL << S) - 1) >> S;
  DBuf<uint64_t> top;
  DBuf<U128> top_w;
  d.idx = SampledKeys{nullptr, 0, nullptr, 0, S};
  d.idx_w = SampledKeysT<U128>{nullptr, 0, nullptr, 0, S};
  if (wide) {
    top_w.alloc(ntop, s);
    launch(k_sample_keys<U128>, blocks_for(ntop, 256), 256, 0, s, ntop, S,
           (const U128 *)ukeys_w.p, top_w.p);
    d.idx_w = SampledKeysT<U128>{ukeys_w.p, nobj, top_w.p, ntop, S};
  } else {
    top.alloc(ntop, s);
    launch(k_sample_keys<uint64_t>, blocks_for(ntop, 256), 256, 0, s, ntop, S,
           (const uint64_t *)ukeys.p, top.p);
    d.idx = SampledKeys{ukeys.p, nobj, top.p, ntop, S};
  }
  d.noff = noff.p;
  d.deprank = deprank.p;
  d.depflag = depflag.p;
  d.err = err.p;
  DBuf<unsigned> he(nd + 1, s), hf(nd + 1, s);
  he.zero();
  hf.zero();
  f.dep_ptr.alloc(nd + 1, s);
  launch(k_dep_rows<0>, blocks_for(n, 128), 128, 0, s, n, d, (const int *)f.x.p,
         (const int *)f.y.p, (const int *)f.z.p, (const int16_t *)f.level.p,
         (const int16_t *)f.info.p, (const int *)lconn.p, he.p, hf.p,
         (const int *)nullptr, (unsigned long long *)nullptr);
  launch(k_dep_len, blocks_for(nd, 256), 256, 0, s, nd, o, (const unsigned *)he.p,
         (const unsigned *)hf.p, f.dep_ptr.p);
  exclusive_scan<int>(f.dep_ptr.p, f.dep_ptr.p, nd, s);
  const long long dnnz = read_scalar(f.dep_ptr.p + nd, s);
  f.dep_nnz = dnnz;
  DBuf<unsigned long long> writer(nd + 1, s);
  writer.zero();
  launch(k_dep_rows<1>, blocks_for(n, 128), 128, 0, s, n, d, (const int *)f.x.p,
         (const int *)f.y.p, (const int *)f.z.p, (const int16_t *)f.level.p,
         (const int16_t *)f.info.p, (const int *)lconn.p, he.p, hf.p,
         (const int *)f.dep_ptr.p, writer.p);
  f.dep_conn.alloc(dnnz + 1, s);
  f.dep_w.alloc(dnnz + 1, s);
  Knots kn{};
  for (int i = 0; i < TMRG_MAX_ORDER; i++) {
    kn.k[i] = f.knots[i];
    for (int j = 0; j < TMRG_MAX_ORDER; j++)
      kn.r[i][j] = (i != j && i < o && j < o) ? 1.0 / (f.knots[i] - f.knots[j]) : 0.0;
  }
  if (f.interp == TMRG_BERNSTEIN_POINTS)
    bernstein_subdivision(o, kn);
  else
    lagrange_tables(o, kn);
  DBuf<unsigned> epos(nd + 1, s);
  DBuf<int> order(nd + 1, s);
  launch(k_dep_edge_flag, blocks_for(nd, 256), 256, 0, s, nd,
         (const unsigned long long *)writer.p, epos.p);
  exclusive_scan<unsigned>(epos.p, epos.p, nd, s);
  launch(k_dep_order, blocks_for(nd, 256), 256, 0, s, nd, (const unsigned long long *)writer.p,
         (const unsigned *)epos.p, order.p);
  launch(k_dep_write, blocks_for(nd, 128), 128, 0, s, nd, d, kn,
         (const int *)f.block.p, (const int *)f.x.p, (const int *)f.y.p,
         (const int *)f.z.p, (const int16_t *)f.level.p,
         (const int16_t *)f.info.p, (const int *)lconn.p,
         (const int *)f.dep_ptr.p, (const unsigned long long *)writer.p,
         (const int *)order.p, f.dep_conn.p, f.dep_w.p);

  // 5. global numbers
  DBuf<int> num(nl + 1, s);
  launch(k_number, blocks_for(nl, 256), 256, 0, s, nl, (const unsigned *)depflag.p,
         (const unsigned *)deprank.p, num.p);
  launch(k_remap, blocks_for(n * npe, 256), 256, 0, s, n * npe,
         (const int *)num.p, lconn.p);
  launch(k_remap, blocks_for(dnnz, 256), 256, 0, s, dnnz, (const int *)num.p,
         f.dep_conn.p);
  if (read_scalar(err.p, s))
    throw Error(TMRG_ERR_INTERNAL, "createNodes: a parent node was not found");
  f.econn = std::move(lconn);
  f.have_nodes = true;
}

}  // namespace tmrg
