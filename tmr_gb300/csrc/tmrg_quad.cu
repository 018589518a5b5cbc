// Quadtree twin of the octree path (TMRQuadForest.cpp, TMRQuadrant.cpp) on
// the GPU: face connectivity, createTrees, refine, coarsen, duplicate, 2:1
// balance, createNodes with dependent (hanging-edge) weights and
// createInterpolation, for mesh orders 2 and 3 with Gauss-Lobatto or
// uniform knots.  Same design as the octree kernels, with 2-D keys:
// quadrants are a sorted structure of arrays keyed [face | morton(x, y) |
// level]; every set operation is a radix sort and a compaction; balance
// is the level-synchronous closure of child-0 families; node objects are
// sorted once and numbered by scans; P rows are built one fine node per
// thread.
#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "tmrg_quad.h"
#include "tmrg_tree.cuh"

namespace tmrg {

// Face edge -> its two corners (face_to_edge_nodes, TMRQuadForest.cpp:31).
__host__ __device__ __forceinline__ int q_edge_corner(int e, int k) {
  return (e < 2) ? (k == 0 ? e : e + 2) : (e == 2 ? k : 2 + k);
}

// ---------------------------------------------------------------------
// Keys.
HD uint64_t spread2(uint64_t v) {  // 31 bits -> every second bit
  v &= 0x7fffffffULL;
  v = (v | (v << 16)) & 0x0000ffff0000ffffULL;
  v = (v | (v << 8)) & 0x00ff00ff00ff00ffULL;
  v = (v | (v << 4)) & 0x0f0f0f0f0f0f0f0fULL;
  v = (v | (v << 2)) & 0x3333333333333333ULL;
  v = (v | (v << 1)) & 0x5555555555555555ULL;
  return v;
}
HD uint32_t compact2(uint64_t v) {
  v &= 0x5555555555555555ULL;
  v = (v | (v >> 1)) & 0x3333333333333333ULL;
  v = (v | (v >> 2)) & 0x0f0f0f0f0f0f0f0fULL;
  v = (v | (v >> 4)) & 0x00ff00ff00ff00ffULL;
  v = (v | (v >> 8)) & 0x0000ffff0000ffffULL;
  v = (v | (v >> 16)) & 0x00000000ffffffffULL;
  return (uint32_t)v;
}
// x-most-significant interleave: the order of TMRQuadrant::compare on
// positions (TMRQuadrant.cpp:108-140).
HD uint64_t morton2(uint32_t x, uint32_t y) { return (spread2(x) << 1) | spread2(y); }

struct Quad {
  int32_t block, x, y;
  int level;
};
HD Quad q_sibling(const Quad &o, int id) {
  int32_t h = side_of(o.level);
  Quad s = o;
  int32_t xr = (o.x & h) ? o.x - h : o.x, yr = (o.y & h) ? o.y - h : o.y;
  s.x = (id & 1) ? xr + h : xr;
  s.y = (id & 2) ? yr + h : yr;
  return s;
}
HD Quad q_parent(const Quad &o) {
  Quad p = o;
  if (o.level > 0) {
    int32_t h = side_of(o.level);
    p.level = o.level - 1;
    p.x = o.x & ~h;
    p.y = o.y & ~h;
  }
  return p;
}
HD Quad q_edge_nbr(const Quad &o, int e) {
  int32_t h = side_of(o.level);
  Quad n = o;
  n.x += (e == 0) ? -h : (e == 1) ? h : 0;
  n.y += (e == 2) ? -h : (e == 3) ? h : 0;
  return n;
}
HD Quad q_corner_nbr(const Quad &o, int c) {
  int32_t h = side_of(o.level);
  Quad n = o;
  n.x += (c & 1) ? h : -h;
  n.y += (c & 2) ? h : -h;
  return n;
}
HD bool q_in_tree(const Quad &q) {
  return q.x >= 0 && q.x < TMRG_HMAX && q.y >= 0 && q.y < TMRG_HMAX;
}
HD int cmp_position2(int32_t ab, int32_t ax, int32_t ay, int32_t bb, int32_t bx, int32_t by) {
  if (ab != bb) return ab < bb ? -1 : 1;
  uint32_t dx = (uint32_t)(ax ^ bx), dy = (uint32_t)(ay ^ by);
  uint32_t any = dx | dy;
  if (any == 0) return 0;
  int32_t d = (dx > (any ^ dx)) ? ax - bx : ay - by;
  return d > 0 ? 1 : (d < 0 ? -1 : 0);
}

// Keys are 64-bit where the face bits and levels fit and 128-bit (U128)
// otherwise; the Morton part (2 x 31 bits at most) always fits one word.
// [face | morton(2W) | level(5)]
template <typename Key>
struct QKeyT {
  int W, bb;
  HD int total_bits() const { return bb + 2 * W + 5; }
  HD Key make(int32_t b, int32_t x, int32_t y, int level) const {
    int s = TMRG_MAX_LEVEL - W;
    return (Key((uint64_t)(uint32_t)b) << (2 * W + 5)) |
           (Key(morton2((uint32_t)x >> s, (uint32_t)y >> s)) << 5) | Key((uint64_t)level);
  }
  HD Quad decode(Key k) const {
    int s = TMRG_MAX_LEVEL - W;
    Quad q;
    q.level = (int)(klo64(k) & 31);
    const uint64_t m = klo64((k >> 5) & kmask<Key>(2 * W));
    q.x = (int32_t)(compact2(m >> 1) << s);
    q.y = (int32_t)(compact2(m) << s);
    q.block = (int32_t)klo64(k >> (2 * W + 5));
    return q;
  }
};
// family position [face | morton(2W)]
template <typename Key>
struct QPos {
  int W, bb;
  HD Key make(int32_t b, int32_t x, int32_t y) const {
    int s = TMRG_MAX_LEVEL - W;
    return (Key((uint64_t)(uint32_t)b) << (2 * W)) |
           Key(morton2((uint32_t)x >> s, (uint32_t)y >> s));
  }
  HD Quad decode(Key k, int level) const {
    int s = TMRG_MAX_LEVEL - W;
    const uint64_t m = klo64(k & kmask<Key>(2 * W));
    Quad q;
    q.block = (int32_t)klo64(k >> (2 * W));
    q.x = (int32_t)(compact2(m >> 1) << s);
    q.y = (int32_t)(compact2(m) << s);
    q.level = level;
    return q;
  }
};
// node objects [face | morton(2(Lg+1))], coordinates on the node grid with
// hmax - 1 mapped to all ones (TMRQuadrant::compareNode order).
template <typename Key>
struct QNodeKeyT {
  int Lg, bb;
  HD uint32_t map(int32_t c) const {
    if (c == TMRG_HMAX - 1) return (1u << (Lg + 1)) - 1u;
    return ((uint32_t)c >> (TMRG_MAX_LEVEL - Lg)) << 1;
  }
  HD int total_bits() const { return bb + 2 * (Lg + 1); }
  HD Key make(int32_t b, int32_t x, int32_t y) const {
    return (Key((uint64_t)(uint32_t)b) << (2 * (Lg + 1))) | Key(morton2(map(x), map(y)));
  }
};
using QNodeKey = QNodeKeyT<uint64_t>;

QKey QForest::key() const {
  int W = std::max(maxlev, 1);
  QKey k{W, conn ? conn->block_bits : 1};
  if (k.total_bits() > 128)
    throw Error(TMRG_ERR_KEY_RANGE,
                "quadrant key needs " + std::to_string(k.total_bits()) + " bits");
  return k;
}
template <typename Key>
static QKeyT<Key> qkey_as(const QKey &k) {
  return QKeyT<Key>{k.W, k.bb};
}

// ---------------------------------------------------------------------
// Face connectivity (TMRQuadForest.cpp:318-650), host.
static void qconn_upload(QConn &c, cudaStream_t s) {
  std::vector<int> all;
  std::vector<size_t> off;
  for (auto *v : {&c.face_conn, &c.face_edge, &c.node_ptr, &c.node_ent, &c.edge_ptr,
                  &c.edge_ent}) {
    off.push_back(all.size());
    all.insert(all.end(), v->begin(), v->end());
  }
  c.d_all.alloc(std::max<size_t>(all.size(), 1), s);
  TMRG_CUDA(cudaMemcpyAsync(c.d_all.p, all.data(), all.size() * sizeof(int),
                            cudaMemcpyHostToDevice, s));
  int *d = c.d_all.p;
  c.dev.nf = c.nf;
  c.dev.face_conn = d + off[0];
  c.dev.face_edge = d + off[1];
  c.dev.node_ptr = d + off[2];
  c.dev.node_ent = d + off[3];
  c.dev.edge_ptr = d + off[4];
  c.dev.edge_ent = d + off[5];
  c.block_bits = bits_for(std::max(c.nf, 2));
  TMRG_CUDA(cudaStreamSynchronize(s));
}

std::shared_ptr<QConn> qconn_build(int num_nodes, const int *face_conn, int nf,
                                   const int *face_edge, int num_edges, cudaStream_t s) {
  if (nf <= 0 || num_nodes <= 0) throw Error(TMRG_ERR_ARG, "setConnectivity: empty mesh");
  auto c = std::make_shared<QConn>();
  c->nf = nf;
  c->num_nodes = num_nodes;
  c->face_conn.assign(face_conn, face_conn + 4 * (size_t)nf);
  for (int v : c->face_conn)
    if (v < 0 || v >= num_nodes) throw Error(TMRG_ERR_ARG, "setConnectivity: node out of range");
  // nodes -> faces (computeNodesToFaces :388-442)
  c->node_ptr.assign(num_nodes + 1, 0);
  for (int v : c->face_conn) c->node_ptr[v + 1]++;
  for (int i = 0; i < num_nodes; i++) c->node_ptr[i + 1] += c->node_ptr[i];
  c->node_ent.assign(c->node_ptr[num_nodes], 0);
  {
    std::vector<int> fill(c->node_ptr.begin(), c->node_ptr.end() - 1);
    for (int f = 0; f < nf; f++)
      for (int j = 0; j < 4; j++) {
        int node = c->face_conn[4 * f + j];
        int adj_index = 0;
        while (adj_index < 4 && c->face_conn[4 * f + adj_index] != node) adj_index++;
        c->node_ent[fill[node]++] = 4 * f + adj_index;
      }
  }
  auto en = [&](int f, int e, int k) { return c->face_conn[4 * f + q_edge_corner(e, k)]; };
  if (face_edge) {
    c->num_edges = num_edges;
    c->face_edge.assign(face_edge, face_edge + 4 * (size_t)nf);
    for (int v : c->face_edge)
      if (v < 0 || v >= num_edges)
        throw Error(TMRG_ERR_ARG, "setFullConnectivity: edge out of range");
  } else {
    // edges from nodes (computeEdgesFromNodes :533-608)
    c->face_edge.assign(4 * (size_t)nf, -1);
    int edge = 0;
    for (int i = 0; i < nf; i++)
      for (int j = 0; j < 4; j++) {
        if (c->face_edge[4 * i + j] >= 0) continue;
        int n1 = en(i, j, 0), n2 = en(i, j, 1);
        int idx[20], nidx = 1;
        idx[0] = 4 * i + j;
        int num = -1;
        for (int p = c->node_ptr[n1]; p < c->node_ptr[n1 + 1]; p++) {
          int ii = c->node_ent[p] / 4;
          for (int jj = 0; jj < 4; jj++) {
            int m1 = en(ii, jj, 0), m2 = en(ii, jj, 1);
            if ((n1 == m1 && n2 == m2) || (n1 == m2 && n2 == m1)) {
              if (c->face_edge[4 * ii + jj] >= 0)
                num = c->face_edge[4 * ii + jj];
              else if (nidx < 20)
                idx[nidx++] = 4 * ii + jj;
            }
          }
        }
        if (num < 0) num = edge++;
        for (int k = 0; k < nidx; k++) c->face_edge[idx[k]] = num;
      }
    c->num_edges = edge;
  }
  // edges -> faces (computeEdgesToFaces :444-531)
  const int ne = c->num_edges;
  c->edge_ptr.assign(ne + 1, 0);
  for (int v : c->face_edge) c->edge_ptr[v + 1]++;
  for (int i = 0; i < ne; i++) c->edge_ptr[i + 1] += c->edge_ptr[i];
  c->edge_ent.assign(c->edge_ptr[ne], 0);
  {
    std::vector<int> fill(c->edge_ptr.begin(), c->edge_ptr.end() - 1);
    for (int f = 0; f < nf; f++)
      for (int j = 0; j < 4; j++) c->edge_ent[fill[c->face_edge[4 * f + j]]++] = f;
  }
  for (int e = 0; e < ne; e++) {
    int owner = nf, oidx = 0;
    for (int p = c->edge_ptr[e]; p < c->edge_ptr[e + 1]; p++) {
      int f = c->edge_ent[p];
      if (f < owner) {
        owner = f;
        oidx = 0;
        while (oidx < 4 && c->face_edge[4 * f + oidx] != e) oidx++;
      }
    }
    int n1 = en(owner, oidx, 0), n2 = en(owner, oidx, 1);
    for (int p = c->edge_ptr[e]; p < c->edge_ptr[e + 1]; p++) {
      int f = c->edge_ent[p];
      for (int k = 0; k < 4; k++) {
        int m1 = en(f, k, 0), m2 = en(f, k, 1);
        if ((n1 == m1 && n2 == m2) || (n1 == m2 && n2 == m1)) {
          c->edge_ent[p] = 4 * f + k;
          break;
        }
      }
    }
  }
  qconn_upload(*c, s);
  return c;
}

// ---------------------------------------------------------------------
// Moves between trees.
// Box of side bs that crossed block edge ei of block b into the adjacent
// faces (addEdgeNeighbors :1994-2060, computeAdjacentDepEdges :2728-2790),
// or block corner ci (addCornerNeighbors :2080-2120).
template <typename F>
__device__ __forceinline__ void q_for_images(const QConnDev &c, const Quad &q, int32_t bs,
                                             bool allow_corner, F &&f) {
  const int32_t hmax = TMRG_HMAX;
  const int32_t ext = hmax - bs;
  const int b = q.block;
  const bool ex = (q.x < 0 || q.x >= hmax), ey = (q.y < 0 || q.y >= hmax);
  if (ex && ey) {
    if (!allow_corner) return;
    int ci = (q.x < 0 ? 0 : 1) + (q.y < 0 ? 0 : 2);
    int node = c.face_conn[4 * b + ci];
    for (int p = c.node_ptr[node]; p < c.node_ptr[node + 1]; p++) {
      int ab = c.node_ent[p] / 4, ac = c.node_ent[p] % 4;
      if (ab == b) continue;
      f(Quad{ab, ext * (ac % 2), ext * (ac / 2), q.level});
    }
    return;
  }
  const int ei = ex ? (q.x < 0 ? 0 : 1) : (q.y < 0 ? 2 : 3);
  const int edge = c.face_edge[4 * b + ei];
  const int32_t uc = (ei < 2) ? q.y : q.x;
  const int n1 = c.face_conn[4 * b + q_edge_corner(ei, 0)];
  const int n2 = c.face_conn[4 * b + q_edge_corner(ei, 1)];
  for (int p = c.edge_ptr[edge]; p < c.edge_ptr[edge + 1]; p++) {
    int ab = c.edge_ent[p] / 4, ae = c.edge_ent[p] % 4;
    if (ab == b) continue;
    int m1 = c.face_conn[4 * ab + q_edge_corner(ae, 0)];
    int m2 = c.face_conn[4 * ab + q_edge_corner(ae, 1)];
    int32_t u = (n1 == m2 && n2 == m1) ? ext - uc : uc;
    if (ae < 2)
      f(Quad{ab, ext * (ae % 2), u, q.level});
    else
      f(Quad{ab, u, ext * (ae % 2), q.level});
  }
}

// transformNode (TMRQuadForest.cpp:2874-2935): the owner face's frame of a
// node, hmax truncated to hmax - 1.
__device__ __forceinline__ void q_transform_node(const QConnDev &c, int32_t &b, int32_t &x,
                                                 int32_t &y) {
  const int32_t hmax = TMRG_HMAX;
  const bool fx0 = x == 0, fy0 = y == 0;
  const bool fx = fx0 || x == hmax, fy = fy0 || y == hmax;
  if (!(fx || fy)) return;
  if (fx && fy) {
    int node = c.face_conn[4 * b + (fx0 ? 0 : 1) + (fy0 ? 0 : 2)];
    int e = c.node_ent[c.node_ptr[node]];
    if (e / 4 != b) {
      int ac = e % 4;
      b = e / 4;
      x = hmax * (ac % 2);
      y = hmax * (ac / 2);
    }
  } else {
    int ei = fx ? (fx0 ? 0 : 1) : (fy0 ? 2 : 3);
    int edge = c.face_edge[4 * b + ei];
    int e = c.edge_ent[c.edge_ptr[edge]];
    if (e / 4 != b) {
      int ab = e / 4, ae = e % 4;
      int n1 = c.face_conn[4 * b + q_edge_corner(ei, 0)];
      int n2 = c.face_conn[4 * b + q_edge_corner(ei, 1)];
      int m1 = c.face_conn[4 * ab + q_edge_corner(ae, 0)];
      int m2 = c.face_conn[4 * ab + q_edge_corner(ae, 1)];
      int32_t u = (ei < 2) ? y : x;
      if (n1 == m2 && n2 == m1) u = hmax - u;
      b = ab;
      if (ae < 2) {
        x = hmax * (ae % 2);
        y = u;
      } else {
        x = u;
        y = hmax * (ae % 2);
      }
    }
  }
  if (x == hmax) x = hmax - 1;
  if (y == hmax) y = hmax - 1;
}

// ---------------------------------------------------------------------
static void q_alloc(QForest &f, long long n) {
  cudaStream_t s = f.s;
  f.block.alloc(std::max(1LL, n), s);
  f.x.alloc(std::max(1LL, n), s);
  f.y.alloc(std::max(1LL, n), s);
  f.level.alloc(std::max(1LL, n), s);
  f.info.alloc(std::max(1LL, n), s);
  f.n = n;
  f.have_quads = true;
}

void QForest::set_order(int o, int it) {
  if (o < 2 || o > 3) throw Error(TMRG_ERR_UNSUPPORTED, "QuadForest: mesh order must be 2 or 3");
  if (it != TMRG_GAUSS_LOBATTO_POINTS && it != TMRG_UNIFORM_POINTS)
    throw Error(TMRG_ERR_UNSUPPORTED,
                "QuadForest: Gauss-Lobatto or uniform interpolation points only");
  order = o;
  interp = it;
  // knots on [-1, 1] as setMeshOrder computes them (TMRQuadForest.cpp:948-990)
  for (int i = 0; i < 3; i++) knots[i] = 0.0;
  knots[0] = -1.0;
  knots[o - 1] = 1.0;
  for (int i = 1; i < o - 1; i++)
    knots[i] = (it == TMRG_GAUSS_LOBATTO_POINTS) ? -cos(M_PI * i / (o - 1))
                                                 : -1.0 + 2.0 * i / (o - 1);
  free_nodes();
}

__global__ void k_q_create_trees(long long n, int level, long long per, int *block, int *xs,
                                 int *ys, int16_t *lev, int16_t *info) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  long long b = t / per, m = t - b * per;
  int s = TMRG_MAX_LEVEL - level;
  block[t] = (int)b;
  xs[t] = (int32_t)(compact2((uint64_t)m >> 1) << s);
  ys[t] = (int32_t)(compact2((uint64_t)m) << s);
  lev[t] = (int16_t)level;
  info[t] = 0;
}
void qforest_create_trees(QForest &f, int level) {
  if (!f.conn) throw Error(TMRG_ERR_STATE, "createTrees: no connectivity");
  if (level < 0) level = 0;
  if (level >= TMRG_MAX_LEVEL) level = TMRG_MAX_LEVEL - 1;
  f.free_nodes();
  long long per = 1LL << (2 * level);
  long long n = per * f.conn->nf;
  q_alloc(f, n);
  f.maxlev = level;
  launch(k_q_create_trees, blocks_for(n, 256), 256, 0, f.s, n, level, per, f.block.p, f.x.p,
         f.y.p, f.level.p, f.info.p);
}

// refine (TMRQuadForest.cpp:1644-1800)
struct QRefineArgs {
  const int *ref;
  int min_level, max_level;
};
__device__ __forceinline__ int q_refine_target(const QRefineArgs &a, int r, int level,
                                               int &reps) {
  reps = 1;
  if (!a.ref) return (level < a.max_level) ? level + 1 : level;
  if (r == 0) return level;
  if (r < 0) {
    if (level > a.min_level) {
      int nl = level + r;
      return nl < a.min_level ? a.min_level : nl;
    }
    return level;
  }
  if (level < a.max_level) {
    int nl = level + r;
    if (nl > a.max_level) nl = a.max_level;
    int d = nl - level;
    reps = (d <= 0) ? 1 : (1 << (d - 1));
    return nl;
  }
  return level;
}
__global__ void k_q_refine_count(long long n, QRefineArgs a, const int16_t *__restrict__ lev,
                                 unsigned *cnt, int *maxlev) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  int ml = 0;
  if (i < n) {
    int reps;
    int nl = q_refine_target(a, a.ref ? a.ref[i] : 1, lev[i], reps);
    cnt[i] = (unsigned)(reps * reps);
    ml = nl;
  }
  for (int o = 16; o > 0; o >>= 1) ml = max(ml, __shfl_down_sync(0xffffffffu, ml, o));
  if ((threadIdx.x & 31) == 0 && ml > 0) atomicMax(maxlev, ml);
}
template <typename Key>
__global__ void k_q_refine_emit(long long n, QRefineArgs a, QKeyT<Key> K,
                                const int *__restrict__ blk, const int *__restrict__ xs,
                                const int *__restrict__ ys, const int16_t *__restrict__ lev,
                                const unsigned *__restrict__ offs, Key *keys, uint32_t *vals) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int level = lev[i];
  int reps;
  int nl = q_refine_target(a, a.ref ? a.ref[i] : 1, level, reps);
  unsigned o = offs[i];
  if (nl == level) {
    keys[o] = K.make(blk[i], xs[i], ys[i], level);
    vals[o] = (uint32_t)i | 0x80000000u;
    return;
  }
  int32_t h = side_of(nl);
  int32_t x0 = xs[i] - xs[i] % h, y0 = ys[i] - ys[i] % h;
  for (int ii = 0; ii < reps; ii++)
    for (int jj = 0; jj < reps; jj++) {
      keys[o] = K.make(blk[i], x0 + 2 * ii * h, y0 + 2 * jj * h, nl);
      vals[o] = (uint32_t)i;
      o++;
    }
}
// first of a run of equal keys, if that run is the finest at its position
template <typename Key>
__global__ void k_q_dedupe(long long n, const Key *__restrict__ keys, unsigned *flag) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const Key k = keys[i];
  unsigned keep = 0;
  if (i == 0 || keys[i - 1] != k) {
    long long e = i;
    while (e + 1 < n && keys[e + 1] == k) e++;
    keep = (e + 1 == n || (keys[e + 1] >> 5) != (k >> 5)) ? 1u : 0u;
  }
  flag[i] = keep;
}
template <typename Key>
__global__ void k_q_compact(long long n, QKeyT<Key> K, const Key *__restrict__ keys,
                            const uint32_t *__restrict__ vals, const unsigned *__restrict__ pos,
                            const int16_t *__restrict__ old_info, int *blk, int *xs, int *ys,
                            int16_t *lev, int16_t *info) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || pos[i + 1] == pos[i]) return;
  unsigned o = pos[i];
  Quad q = K.decode(keys[i]);
  blk[o] = q.block;
  xs[o] = q.x;
  ys[o] = q.y;
  lev[o] = (int16_t)q.level;
  uint32_t v = vals ? vals[i] : 0u;
  info[o] = (vals && old_info && (v & 0x80000000u)) ? old_info[v & 0x7fffffffu] : (int16_t)0;
}

template <typename Key>
static void q_refine_sort_compact(QForest &f, const QRefineArgs &a, const QKeyT<Key> &K,
                                  const DBuf<unsigned> &cnt, unsigned total) {
  cudaStream_t s = f.s;
  const long long n = f.n;
  DBuf<Key> keys(total, s);
  DBuf<uint32_t> vals(total, s);
  launch(k_q_refine_emit<Key>, blocks_for(n, 256), 256, 0, s, n, a, K, (const int *)f.block.p,
         (const int *)f.x.p, (const int *)f.y.p, (const int16_t *)f.level.p,
         (const unsigned *)cnt.p, keys.p, vals.p);
  sort_keys(keys, &vals, total, K.total_bits(), s);
  DBuf<unsigned> pos(total + 1, s);
  launch(k_q_dedupe<Key>, blocks_for(total, 256), 256, 0, s, (long long)total,
         (const Key *)keys.p, pos.p);
  exclusive_scan<unsigned>(pos.p, pos.p, total, s);
  const unsigned m = read_scalar(pos.p + total, s);
  DBuf<int16_t> old_info = std::move(f.info);
  q_alloc(f, m);
  launch(k_q_compact<Key>, blocks_for(total, 256), 256, 0, s, (long long)total, K,
         (const Key *)keys.p, (const uint32_t *)vals.p, (const unsigned *)pos.p,
         (const int16_t *)old_info.p, f.block.p, f.x.p, f.y.p, f.level.p, f.info.p);
}

void qforest_refine(QForest &f, const int *d_ref, long long nref, int min_level,
                    int max_level) {
  Stage st("tmrg_quad_refine");
  if (!f.have_quads) throw Error(TMRG_ERR_STATE, "refine: no quadrants");
  if (d_ref && nref != f.n)
    throw Error(TMRG_ERR_ARG, "refine: refinement array length " + std::to_string(nref) +
                                  " != quadrants " + std::to_string(f.n));
  f.free_nodes();
  if (min_level < 0) min_level = 0;
  if (max_level > TMRG_MAX_LEVEL) max_level = TMRG_MAX_LEVEL;
  if (min_level > max_level) min_level = max_level;
  const long long n = f.n;
  if (n == 0) return;
  cudaStream_t s = f.s;
  QRefineArgs a{d_ref, min_level, max_level};
  DBuf<unsigned> cnt(n + 1, s);
  DBuf<int> ml(1, s);
  ml.zero();
  launch(k_q_refine_count, blocks_for(n, 256), 256, 0, s, n, a, (const int16_t *)f.level.p,
         cnt.p, ml.p);
  exclusive_scan<unsigned>(cnt.p, cnt.p, n, s);
  const unsigned total = read_scalar(cnt.p + n, s);
  f.maxlev = std::max(f.maxlev, std::max(read_scalar(ml.p, s), 0));
  const QKey K = f.key();
  if (K.total_bits() > 64)
    q_refine_sort_compact<U128>(f, a, qkey_as<U128>(K), cnt, total);
  else
    q_refine_sort_compact<uint64_t>(f, a, K, cnt, total);
}

// createRandomTrees (TMRQuadForest.cpp:1327-1407): nrand quadrants per face
// at a random level in [min_level, max_level] and a random anchor of that
// level, sorted, and made unique on position keeping the finest (the
// reference's TMRQuadrantArray::sort).  The reference draws from libc
// rand(); here quadrant i of face f draws U(seed, f, 3i + k), k = 0..2.
template <typename Key>
__global__ void k_q_random_quads(long long total, int nrand, int min_level, int max_level,
                                 uint64_t seed, QKeyT<Key> K, Key *keys) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= total) return;
  const unsigned tu = (unsigned)t;  // total < 2^32
  const int b = (int)(tu / (unsigned)nrand), i = (int)(tu - (unsigned)b * (unsigned)nrand);
  const uint64_t base = 3ULL * (uint64_t)i;
  int level = min_level + (int)(seeded_uniform(seed, b, base) * (max_level - min_level + 1));
  if (level > max_level) level = max_level;
  const int32_t h = side_of(level);
  const double cells = (double)(1 << level);
  int32_t c[2];
  for (int k = 0; k < 2; k++) {
    int32_t q = (int32_t)(seeded_uniform(seed, b, base + 1 + k) * cells);
    if (q >= (1 << level)) q = (1 << level) - 1;
    c[k] = h * q;
  }
  keys[t] = K.make(b, c[0], c[1], level);
}
template <typename Key>
static void q_random_sort_compact(QForest &f, long long total, int nrand, int min_level,
                                  int max_level, uint64_t seed, const QKeyT<Key> &K) {
  cudaStream_t s = f.s;
  DBuf<Key> keys(std::max(1LL, total), s);
  launch(k_q_random_quads<Key>, blocks_for(total, 256), 256, 0, s, total, nrand, min_level,
         max_level, seed, K, keys.p);
  sort_keys(keys, nullptr, total, K.total_bits(), s);
  DBuf<unsigned> pos(total + 1, s);
  launch(k_q_dedupe<Key>, blocks_for(total, 256), 256, 0, s, total, (const Key *)keys.p, pos.p);
  exclusive_scan<unsigned>(pos.p, pos.p, total, s);
  const unsigned m = total ? read_scalar(pos.p + total, s) : 0u;
  q_alloc(f, m);
  launch(k_q_compact<Key>, blocks_for(total, 256), 256, 0, s, total, K, (const Key *)keys.p,
         (const uint32_t *)nullptr, (const unsigned *)pos.p, (const int16_t *)nullptr, f.block.p,
         f.x.p, f.y.p, f.level.p, f.info.p);
}
void qforest_create_random_trees(QForest &f, int nrand, int min_level, int max_level,
                                 uint64_t seed) {
  Stage st("tmrg_quad_create_random_trees");
  if (!f.conn) throw Error(TMRG_ERR_STATE, "createRandomTrees: no connectivity");
  if (nrand < 0) throw Error(TMRG_ERR_ARG, "createRandomTrees: nrand < 0");
  if (min_level < 0) min_level = 0;
  if (max_level >= TMRG_MAX_LEVEL) max_level = TMRG_MAX_LEVEL - 1;
  if (min_level > max_level) min_level = max_level;
  f.free_nodes();
  const long long total = (long long)f.conn->nf * nrand;
  if (total >= (1LL << 32)) throw Error(TMRG_ERR_ARG, "createRandomTrees: too many quadrants");
  f.maxlev = max_level;
  const QKey K = f.key();
  if (K.total_bits() > 64)
    q_random_sort_compact<U128>(f, total, nrand, min_level, max_level, seed, qkey_as<U128>(K));
  else
    q_random_sort_compact<uint64_t>(f, total, nrand, min_level, max_level, seed, K);
  TMRG_CUDA(cudaStreamSynchronize(f.s));
}

// coarsen (TMRQuadForest.cpp:1594-1640)
__global__ void k_q_coarsen_flags(long long n, const int *__restrict__ xs,
                                  const int *__restrict__ ys, const int16_t *__restrict__ lev,
                                  unsigned *flag) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int l = lev[i];
  unsigned keep = 1;
  if (l > 0) {
    int32_t h = side_of(l);
    keep = ((xs[i] & h) | (ys[i] & h)) ? 0u : 1u;
  }
  flag[i] = keep;
}
__global__ void k_q_coarsen_emit(long long n, const unsigned *__restrict__ pos,
                                 const int *__restrict__ blk, const int *__restrict__ xs,
                                 const int *__restrict__ ys, const int16_t *__restrict__ lev,
                                 const int16_t *__restrict__ info, int *ob, int *ox, int *oy,
                                 int16_t *ol, int16_t *oi) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || pos[i + 1] == pos[i]) return;
  unsigned o = pos[i];
  int l = lev[i];
  ob[o] = blk[i];
  if (l > 0) {
    int32_t h = side_of(l);
    ox[o] = xs[i] & ~h;
    oy[o] = ys[i] & ~h;
    ol[o] = (int16_t)(l - 1);
    oi[o] = 0;
  } else {
    ox[o] = xs[i];
    oy[o] = ys[i];
    ol[o] = (int16_t)l;
    oi[o] = info[i];
  }
}
void qforest_coarsen(QForest &f, QForest &out) {
  if (!f.have_quads) throw Error(TMRG_ERR_STATE, "coarsen: no quadrants");
  out.conn = f.conn;
  out.set_order(f.order, f.interp);
  cudaStream_t s = out.s;
  TMRG_CUDA(cudaStreamSynchronize(f.s));
  const long long n = f.n;
  DBuf<unsigned> pos(n + 1, s);
  launch(k_q_coarsen_flags, blocks_for(n, 256), 256, 0, s, n, (const int *)f.x.p,
         (const int *)f.y.p, (const int16_t *)f.level.p, pos.p);
  exclusive_scan<unsigned>(pos.p, pos.p, n, s);
  const unsigned m = n ? read_scalar(pos.p + n, s) : 0;
  q_alloc(out, m);
  launch(k_q_coarsen_emit, blocks_for(n, 256), 256, 0, s, n, (const unsigned *)pos.p,
         (const int *)f.block.p, (const int *)f.x.p, (const int *)f.y.p,
         (const int16_t *)f.level.p, (const int16_t *)f.info.p, out.block.p, out.x.p,
         out.y.p, out.level.p, out.info.p);
  out.maxlev = std::max(f.maxlev - 1, 0);
}
void qforest_duplicate(QForest &f, QForest &out) {
  out.conn = f.conn;
  out.set_order(f.order, f.interp);
  if (!f.have_quads) return;
  TMRG_CUDA(cudaStreamSynchronize(f.s));
  q_alloc(out, f.n);
  cudaStream_t s = out.s;
  size_t n = (size_t)f.n;
  TMRG_CUDA(cudaMemcpyAsync(out.block.p, f.block.p, n * 4, cudaMemcpyDeviceToDevice, s));
  TMRG_CUDA(cudaMemcpyAsync(out.x.p, f.x.p, n * 4, cudaMemcpyDeviceToDevice, s));
  TMRG_CUDA(cudaMemcpyAsync(out.y.p, f.y.p, n * 4, cudaMemcpyDeviceToDevice, s));
  TMRG_CUDA(cudaMemcpyAsync(out.level.p, f.level.p, n * 2, cudaMemcpyDeviceToDevice, s));
  TMRG_CUDA(cudaMemcpyAsync(out.info.p, f.info.p, n * 2, cudaMemcpyDeviceToDevice, s));
  out.maxlev = f.maxlev;
}

// ---------------------------------------------------------------------
// 2:1 balance (TMRQuadForest.cpp:2137-2410): the child-0 families closed
// level by level from the finest down, S_L = seeds_L U gen(S_{L+1}), then
// the siblings of every family that are not themselves refined.
template <typename Key>
__global__ void k_q_seed_keys(long long n, QPos<Key> P, const int *__restrict__ blk,
                              const int *__restrict__ xs, const int *__restrict__ ys,
                              const int16_t *__restrict__ lev, Key *keys) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  Quad o{blk[i], xs[i], ys[i], lev[i]};
  Quad q = q_sibling(o, 0);
  keys[i] = (Key((uint64_t)o.level) << (P.bb + 2 * P.W)) | P.make(q.block, q.x, q.y);
}
template <typename Key>
__global__ void k_q_unique_flags(long long n, const Key *__restrict__ keys, unsigned *flag) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) flag[i] = (i == 0 || keys[i - 1] != keys[i]) ? 1u : 0u;
}
template <typename Key>
__global__ void k_q_unique_emit(long long n, const Key *__restrict__ keys,
                                const unsigned *__restrict__ pos, Key mask, Key *out) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || pos[i + 1] == pos[i]) return;
  out[pos[i]] = keys[i] & mask;
}
template <typename Key>
__global__ void k_q_mask_copy(long long n, const Key *__restrict__ in, Key mask, Key *out) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = in[i] & mask;
}
template <typename Key>
__global__ void k_q_level_starts(long long n, const Key *__restrict__ keys, int shift,
                                 long long *starts) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int l = (int)klo64(keys[i] >> shift);
  if (i == 0 || (int)klo64(keys[i - 1] >> shift) != l) starts[l] = i;
}
// children-0 of the parent's edge (and corner) neighbours of family q
template <bool WRITE, typename Key>
__device__ __forceinline__ unsigned q_gen_family(const QConnDev &c, QPos<Key> P, const Quad &q,
                                                 int corner, Key *out) {
  unsigned cnt = 0;
  Quad p = q_parent(q);
  const int32_t bs = 2 * side_of(p.level);
  auto emit = [&](const Quad &r) {
    if (WRITE) out[cnt] = P.make(r.block, r.x, r.y);
    cnt++;
  };
  for (int e = 0; e < 4; e++) {
    Quad r = q_sibling(q_edge_nbr(p, e), 0);
    if (q_in_tree(r))
      emit(r);
    else
      q_for_images(c, r, bs, false, emit);
  }
  if (corner)
    for (int k = 0; k < 4; k++) {
      Quad r = q_sibling(q_corner_nbr(p, k), 0);
      if (q_in_tree(r))
        emit(r);
      else
        q_for_images(c, r, bs, true, emit);
    }
  return cnt;
}
// n bounds the families; *m (device) is their number (entries past it
// count 0), so it need not be read back before the count.
template <typename Key>
__global__ void k_q_gen_count(long long n, const unsigned *__restrict__ m, QConnDev c,
                              QPos<Key> P, int level, int corner, const Key *__restrict__ cur,
                              unsigned *cnt) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (i >= (long long)*m) {
    cnt[i] = 0;
    return;
  }
  cnt[i] = q_gen_family<false, Key>(c, P, P.decode(cur[i], level), corner, nullptr);
}
template <typename Key>
__global__ void k_q_gen_write(long long n, const unsigned *__restrict__ m, QConnDev c,
                              QPos<Key> P, int level, int corner, const Key *__restrict__ cur,
                              const unsigned *__restrict__ offs, Key *out) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || i >= (long long)*m) return;
  q_gen_family<true, Key>(c, P, P.decode(cur[i], level), corner, out + offs[i]);
}
template <typename Key>
__global__ void k_q_leaves(long long n, QPos<Key> P, QKeyT<Key> K, int level,
                           const Key *__restrict__ cur, const Key *__restrict__ finer,
                           long long nfiner, Key *out, unsigned long long *counter) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  Key mine[4];
  int m = 0;
  if (i < n) {
    Quad q = P.decode(cur[i], level);
    int ns = (level == 0) ? 1 : 4;
    for (int j = 0; j < ns; j++) {
      Quad sb = (level == 0) ? q : q_sibling(q, j);
      if (!contains_key(finer, nfiner, P.make(sb.block, sb.x, sb.y)))
        mine[m++] = K.make(sb.block, sb.x, sb.y, level);
    }
  }
  int lane = threadIdx.x & 31;
  int incl = m;
  for (int o = 1; o < 32; o <<= 1) {
    int y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += y;
  }
  int tot = __shfl_sync(0xffffffffu, incl, 31);
  unsigned long long base = 0;
  if (lane == 31 && tot > 0) base = atomicAdd(counter, (unsigned long long)tot);
  base = __shfl_sync(0xffffffffu, base, 31);
  unsigned long long o = base + (incl - m);
  for (int j = 0; j < m; j++) out[o + j] = mine[j];
}
template <typename Key>
__global__ void k_q_decode(long long n, QKeyT<Key> K, const Key *__restrict__ keys, int *blk,
                           int *xs, int *ys, int16_t *lev, int16_t *info) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  Quad q = K.decode(keys[i]);
  blk[i] = q.block;
  xs[i] = q.x;
  ys[i] = q.y;
  lev[i] = (int16_t)q.level;
  info[i] = 0;
}
template <typename Key>
static long long q_sort_unique(DBuf<Key> &keys, long long n, int nbits, Key mask,
                               DBuf<Key> &out, cudaStream_t s) {
  if (n == 0) {
    out.release();
    return 0;
  }
  sort_keys(keys, nullptr, n, nbits, s);
  DBuf<unsigned> pos(n + 1, s);
  launch(k_q_unique_flags<Key>, blocks_for(n, 256), 256, 0, s, n, (const Key *)keys.p, pos.p);
  exclusive_scan<unsigned>(pos.p, pos.p, n, s);
  long long m = read_scalar(pos.p + n, s);
  out.alloc(std::max(1LL, m), s);
  launch(k_q_unique_emit<Key>, blocks_for(n, 256), 256, 0, s, n, (const Key *)keys.p,
         (const unsigned *)pos.p, mask, out.p);
  return m;
}

template <typename Key>
static void q_balance_impl(QForest &f, int corner, const QKeyT<Key> K) {
  const long long n = f.n;
  cudaStream_t s = f.s;
  QPos<Key> P{K.W, K.bb};
  const int pbits = K.bb + 2 * K.W;
  const Key pmask = kmask<Key>(pbits);
  const Key all = kmask<Key>(8 * (int)sizeof(Key));
  QConnDev c = f.conn->dev;
  DBuf<Key> sk(n, s);
  launch(k_q_seed_keys<Key>, blocks_for(n, 256), 256, 0, s, n, P, (const int *)f.block.p,
         (const int *)f.x.p, (const int *)f.y.p, (const int16_t *)f.level.p, sk.p);
  DBuf<Key> seeds;
  const long long ns = q_sort_unique<Key>(sk, n, pbits + 5, all, seeds, s);
  sk.release();
  DBuf<long long> starts(TMRG_MAX_LEVEL + 2, s);
  starts.fill_bytes(0xff);
  launch(k_q_level_starts<Key>, blocks_for(ns, 256), 256, 0, s, ns, (const Key *)seeds.p, pbits,
         starts.p);
  std::vector<long long> st(TMRG_MAX_LEVEL + 2);
  TMRG_CUDA(cudaMemcpyAsync(st.data(), starts.p, st.size() * sizeof(long long),
                            cudaMemcpyDeviceToHost, s));
  TMRG_CUDA(cudaStreamSynchronize(s));
  const int L = f.maxlev;
  std::vector<long long> lo(L + 2, 0), hi(L + 2, 0);
  {
    long long next = ns;
    for (int l = TMRG_MAX_LEVEL + 1; l >= 0; l--) {
      if (st[l] >= 0) {
        if (l <= L + 1) {
          lo[l] = st[l];
          hi[l] = next;
        }
        next = st[l];
      }
    }
  }
  std::vector<DBuf<Key>> S(L + 2);
  std::vector<long long> Sn(L + 2, 0);
  DBuf<Key> gen;
  long long ngen = 0;
  // one wait per level, as in the octree balance
  for (int l = L; l >= 0; l--) {
    const long long nseed = hi[l] - lo[l];
    const long long tot = nseed + ngen;
    DBuf<unsigned> upos;  // unique positions; upos[tot] = Sn[l]
    if (tot > 0) {
      DBuf<Key> cat(tot, s);
      if (nseed)
        launch(k_q_mask_copy<Key>, blocks_for(nseed, 256), 256, 0, s, nseed,
               (const Key *)(seeds.p + lo[l]), pmask, cat.p);
      if (ngen)
        TMRG_CUDA(cudaMemcpyAsync(cat.p + nseed, gen.p, ngen * sizeof(Key),
                                  cudaMemcpyDeviceToDevice, s));
      sort_keys(cat, nullptr, tot, pbits, s);
      upos.alloc(tot + 1, s);
      launch(k_q_unique_flags<Key>, blocks_for(tot, 256), 256, 0, s, tot, (const Key *)cat.p,
             upos.p);
      exclusive_scan<unsigned>(upos.p, upos.p, tot, s);
      S[l].alloc(tot, s);
      launch(k_q_unique_emit<Key>, blocks_for(tot, 256), 256, 0, s, tot, (const Key *)cat.p,
             (const unsigned *)upos.p, all, S[l].p);
    }
    gen.release();
    ngen = 0;
    Sn[l] = 0;
    if (tot == 0) continue;
    if (l >= 2) {
      DBuf<unsigned> cnt(tot + 1, s);
      launch(k_q_gen_count<Key>, blocks_for(tot, 128), 128, 0, s, tot,
             (const unsigned *)upos.p + tot, c, P, l, corner, (const Key *)S[l].p, cnt.p);
      exclusive_scan<unsigned>(cnt.p, cnt.p, tot, s);
      const unsigned *dv[2] = {upos.p + tot, cnt.p + tot};
      unsigned hv[2];
      read_scalars(dv, hv, s);
      Sn[l] = hv[0];
      ngen = hv[1];
      gen.alloc(std::max(1LL, ngen), s);
      launch(k_q_gen_write<Key>, blocks_for(tot, 128), 128, 0, s, tot,
             (const unsigned *)upos.p + tot, c, P, l, corner, (const Key *)S[l].p,
             (const unsigned *)cnt.p, gen.p);
    } else {
      Sn[l] = read_scalar(upos.p + tot, s);
    }
  }
  seeds.release();
  long long cap = 0;
  for (int l = 0; l <= L; l++) cap += (l == 0 ? 1 : 4) * Sn[l];
  DBuf<Key> leaves(std::max(1LL, cap), s);
  DBuf<unsigned long long> counter(1, s);
  counter.zero();
  for (int l = 0; l <= L; l++) {
    if (!Sn[l]) continue;
    launch(k_q_leaves<Key>, blocks_for(Sn[l], 256), 256, 0, s, Sn[l], P, K, l,
           (const Key *)S[l].p, (const Key *)S[l + 1].p, Sn[l + 1], leaves.p, counter.p);
  }
  const long long m = (long long)read_scalar(counter.p, s);
  S.clear();
  sort_keys(leaves, nullptr, m, K.total_bits(), s);
  q_alloc(f, m);
  launch(k_q_decode<Key>, blocks_for(m, 256), 256, 0, s, m, K, (const Key *)leaves.p, f.block.p,
         f.x.p, f.y.p, f.level.p, f.info.p);
}

void qforest_balance(QForest &f, int corner) {
  Stage stage("tmrg_quad_balance");
  if (!f.have_quads)
    throw Error(TMRG_ERR_STATE, "Cannot call balance(), no quadrants have been created");
  f.free_nodes();
  if (f.n == 0) return;
  const QKey K = f.key();
  if (K.total_bits() > 64)
    q_balance_impl<U128>(f, corner, qkey_as<U128>(K));
  else
    q_balance_impl<uint64_t>(f, corner, K);
}


// ---------------------------------------------------------------------
// createNodes (TMRQuadForest.cpp:2996-3860).
// 1. hanging edges: bit e of info when the quadrant's edge e lies on its
//    parent's edge e and the parent's neighbour across it is a leaf
//    (computeDepEdges :2658-2726, seen from the finer side).
template <typename Key>
__global__ void k_q_keys(long long n, QKeyT<Key> K, const int *__restrict__ blk,
                         const int *__restrict__ xs, const int *__restrict__ ys,
                         const int16_t *__restrict__ lev, Key *keys) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) keys[i] = K.make(blk[i], xs[i], ys[i], lev[i]);
}
template <typename Key>
__global__ void k_q_dep_info(long long n, QConnDev c, QKeyT<Key> K, const Key *__restrict__ keys,
                             const int *__restrict__ blk, const int *__restrict__ xs,
                             const int *__restrict__ ys, const int16_t *__restrict__ lev,
                             int16_t *info) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  Quad o{blk[i], xs[i], ys[i], lev[i]};
  if (o.level == 0) {
    info[i] = 0;
    return;
  }
  auto exists = [&](const Quad &q) {
    return contains_key(keys, n, K.make(q.block, q.x, q.y, q.level));
  };
  const int32_t h = side_of(o.level);
  const int id = ((o.x & h) ? 1 : 0) | ((o.y & h) ? 2 : 0);
  Quad p = q_parent(o);
  int bits = 0;
  const int edges[2] = {(id & 1) ? 1 : 0, (id & 2) ? 3 : 2};
  for (int k = 0; k < 2; k++) {
    const int e = edges[k];
    Quad nb = q_edge_nbr(p, e);
    bool hit = false;
    if (q_in_tree(nb)) {
      hit = exists(nb);
    } else {
      q_for_images(c, nb, side_of(nb.level), false, [&](const Quad &q) {
        if (!hit && exists(q)) hit = true;
      });
    }
    if (hit) bits |= 1 << e;
  }
  info[i] = (int16_t)bits;
}

// 2. node objects: order 2 the 4 corners, order 3 the 3 x 3 lattice of
//    half-size steps (createLocalNodes :3218-3480), in the owner's frame.
__device__ __forceinline__ void q_object(int order, const Quad &e, int j, int32_t &x,
                                         int32_t &y) {
  if (order == 2) {
    int32_t h = side_of(e.level);
    x = e.x + h * (j & 1);
    y = e.y + h * (j >> 1);
  } else {
    int32_t h = (int32_t)1 << (TMRG_MAX_LEVEL - e.level - 1);
    x = e.x + h * (j % 3);
    y = e.y + h * (j / 3);
  }
}
template <typename Key>
__global__ void k_q_node_keys(long long n, QConnDev c, QNodeKeyT<Key> NK, int order,
                              const int *__restrict__ blk, const int *__restrict__ xs,
                              const int *__restrict__ ys, const int16_t *__restrict__ lev,
                              Key *keys, uint32_t *vals) {
  const int npe = order * order;
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n * npe) return;
  const unsigned tu = (unsigned)t;
  const long long e = tu / (unsigned)npe;
  const int j = (int)(tu - (unsigned)e * (unsigned)npe);
  Quad o{blk[e], xs[e], ys[e], lev[e]};
  int32_t b = o.block, x, y;
  q_object(order, o, j, x, y);
  q_transform_node(c, b, x, y);
  keys[t] = NK.make(b, x, y);
  vals[t] = (uint32_t)t;
}
// sorted object keys -> run index of every (element, local node) entry
template <typename Key>
__global__ void k_q_node_runs(long long m, const Key *__restrict__ keys,
                              const uint32_t *__restrict__ vals, const unsigned *__restrict__ pos,
                              Key *ukeys, int *lconn) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) return;
  unsigned idx = pos[i + 1] - 1;
  lconn[vals[i]] = (int)idx;
  if (pos[i + 1] != pos[i]) ukeys[idx] = keys[i];
}

// 3. dependent labels (labelDependentNodes :2806-2866)
__device__ __forceinline__ int q_edge_offset(int o, int e, int k) {
  return (e < 2) ? (e % 2) * (o - 1) + k * o : k + (e % 2) * (o - 1) * o;
}
__global__ void k_q_label_dep(long long n, int order, const int *__restrict__ lconn,
                              const int *__restrict__ xs, const int *__restrict__ ys,
                              const int16_t *__restrict__ lev, const int16_t *__restrict__ info,
                              unsigned *dep) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || !info[i]) return;
  const int o = order;
  const int32_t h = side_of(lev[i]);
  const int id = ((xs[i] & h) ? 1 : 0) | ((ys[i] & h) ? 2 : 0);
  for (int e = 0; e < 4; e++) {
    if (!(info[i] & (1 << e))) continue;
    int start, end;
    if ((e < 2 && id / 2 == 0) || (e >= 2 && id % 2 == 0)) {
      start = 1;
      end = (o == 3) ? o - 1 : o;
    } else {
      start = (o == 3) ? 1 : 0;
      end = o - 1;
    }
    for (int k = start; k < end; k++) dep[lconn[i * o * o + q_edge_offset(o, e, k)]] = 1;
  }
}
__global__ void k_q_widen(long long n, const unsigned *__restrict__ a, long long *b) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) b[i] = a[i];
}
// independent nodes 0, 1, ..; dependent nodes -1, -2, .. in node order
__global__ void k_q_number(long long nl, const unsigned *__restrict__ dep,
                           const long long *__restrict__ dscan, int *num) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nl) return;
  long long d = dscan[i];
  num[i] = dep[i] ? (int)(-(d + 1)) : (int)(i - d);
}
__global__ void k_q_remap(long long m, const int *__restrict__ num, const int *__restrict__ in,
                          int *out) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < m) out[i] = num[in[i]];
}

// 4. dependent rows (createDependentConn :3673-3860): every row holds the
//    `order` nodes of the parent edge with the Lagrange weights of the
//    dependent node's position on it.
struct QKnots {
  double k[3];
  double r[3][3];
};
template <typename Key>
__device__ __forceinline__ long long q_find_node(const Key *ukeys, long long nl, Key key) {
  long long i = lower_bound_key(ukeys, nl, key);
  return (i < nl && ukeys[i] == key) ? i : -1;
}
template <typename Key>
__global__ void k_q_dep_rows(long long n, QConnDev c, QNodeKeyT<Key> NK, int order, QKnots kn,
                             const int *__restrict__ blk, const int *__restrict__ xs,
                             const int *__restrict__ ys, const int16_t *__restrict__ lev,
                             const int16_t *__restrict__ info, const int *__restrict__ lconn,
                             const int *__restrict__ num, const Key *__restrict__ ukeys,
                             long long nl, int *dconn, double *dw, int *err) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || !info[i]) return;
  const int o = order;
  Quad q{blk[i], xs[i], ys[i], lev[i]};
  const int32_t h = side_of(q.level);
  const int id = ((q.x & h) ? 1 : 0) | ((q.y & h) ? 2 : 0);
  Quad p = q_parent(q);
  for (int e = 0; e < 4; e++) {
    if (!(info[i] & (1 << e))) continue;
    int en[3];
    for (int ii = 0; ii < o; ii++) {
      // parent edge nodes at 2h (order 2) or h (order 3) steps
      int32_t step = (o == 2) ? 2 * h : h;
      int32_t x, y, b = p.block;
      if (e < 2) {
        x = p.x + 2 * h * (e % 2);
        y = p.y + step * ii;
      } else {
        x = p.x + step * ii;
        y = p.y + 2 * h * (e % 2);
      }
      q_transform_node(c, b, x, y);
      long long t = q_find_node<Key>(ukeys, nl, NK.make(b, x, y));
      if (t < 0) {
        atomicExch(err, 1);
        return;
      }
      en[ii] = num[t];
    }
    for (int k = 0; k < o; k++) {
      int local = lconn[i * o * o + q_edge_offset(o, e, k)];
      int nk = num[local];
      if (nk >= 0) continue;
      long long row = -nk - 1;
      double u = __dadd_rn(1.0 * (double)(-1 + ((e < 2) ? id / 2 : id % 2)),
                           __dmul_rn(0.5, __dadd_rn(1.0, kn.k[k])));
      for (int a = 0; a < o; a++) {
        double v = 1.0;
        for (int b2 = 0; b2 < o; b2++)
          if (a != b2) v = __dmul_rn(v, __dmul_rn(__dsub_rn(u, kn.k[b2]), kn.r[a][b2]));
        dconn[row * o + a] = en[a];
        dw[row * o + a] = v;
      }
    }
  }
}

// Hanging-edge flags (section 1 of createNodes).
template <typename Key>
static void q_hanging(QForest &f, const QKeyT<Key> &K) {
  cudaStream_t s = f.s;
  const long long n = f.n;
  DBuf<Key> qk(std::max(1LL, n), s);
  launch(k_q_keys<Key>, blocks_for(n, 256), 256, 0, s, n, K, (const int *)f.block.p,
         (const int *)f.x.p, (const int *)f.y.p, (const int16_t *)f.level.p, qk.p);
  launch(k_q_dep_info<Key>, blocks_for(n, 128), 128, 0, s, n, f.conn->dev, K,
         (const Key *)qk.p, (const int *)f.block.p, (const int *)f.x.p, (const int *)f.y.p,
         (const int16_t *)f.level.p, f.info.p);
}

// Node objects, numbering and the dependent rows (the node keys are 64- or
// 128-bit).
template <typename Key>
static void q_nodes(QForest &f, const QNodeKeyT<Key> &NK) {
  cudaStream_t s = f.s;
  const long long n = f.n;
  const int o = f.order;
  QConnDev c = f.conn->dev;
  const long long m = n * o * o;
  DBuf<Key> keys(std::max(1LL, m), s);
  DBuf<uint32_t> vals(std::max(1LL, m), s);
  launch(k_q_node_keys<Key>, blocks_for(m, 256), 256, 0, s, n, c, NK, o,
         (const int *)f.block.p, (const int *)f.x.p, (const int *)f.y.p,
         (const int16_t *)f.level.p, keys.p, vals.p);
  sort_keys(keys, &vals, m, NK.total_bits(), s);
  DBuf<unsigned> pos(m + 1, s);
  launch(k_q_unique_flags<Key>, blocks_for(m, 256), 256, 0, s, m, (const Key *)keys.p, pos.p);
  // pos[i + 1] - 1 is then the run (node) index of entry i
  exclusive_scan<unsigned>(pos.p, pos.p, m, s);
  const long long nl = read_scalar(pos.p + m, s);
  DBuf<Key> ukeys(std::max(1LL, nl), s);
  DBuf<int> lconn(std::max(1LL, m), s);
  launch(k_q_node_runs<Key>, blocks_for(m, 256), 256, 0, s, m, (const Key *)keys.p,
         (const uint32_t *)vals.p, (const unsigned *)pos.p, ukeys.p, lconn.p);
  keys.release();
  vals.release();
  pos.release();
  DBuf<unsigned> dep(std::max(1LL, nl), s);
  dep.zero();
  launch(k_q_label_dep, blocks_for(n, 256), 256, 0, s, n, o, (const int *)lconn.p,
         (const int *)f.x.p, (const int *)f.y.p, (const int16_t *)f.level.p,
         (const int16_t *)f.info.p, dep.p);
  DBuf<long long> dscan(nl + 1, s);
  launch(k_q_widen, blocks_for(nl, 256), 256, 0, s, nl, (const unsigned *)dep.p, dscan.p);
  exclusive_scan<long long>(dscan.p, dscan.p, nl, s);
  const long long ndep = read_scalar(dscan.p + nl, s);
  DBuf<int> num(std::max(1LL, nl), s);
  launch(k_q_number, blocks_for(nl, 256), 256, 0, s, nl, (const unsigned *)dep.p,
         (const long long *)dscan.p, num.p);
  f.num_local = nl;
  f.num_dep = ndep;
  f.num_owned = nl - ndep;
  f.dep_nnz = ndep * o;
  f.econn.alloc(std::max(1LL, m), s);
  launch(k_q_remap, blocks_for(m, 256), 256, 0, s, m, (const int *)num.p, (const int *)lconn.p,
         f.econn.p);
  f.dep_ptr.alloc(ndep + 1, s);
  {
    std::vector<int> hp(ndep + 1);
    for (long long k = 0; k <= ndep; k++) hp[k] = (int)(k * o);
    TMRG_CUDA(cudaMemcpyAsync(f.dep_ptr.p, hp.data(), sizeof(int) * (ndep + 1),
                              cudaMemcpyHostToDevice, s));
    TMRG_CUDA(cudaStreamSynchronize(s));
  }
  f.dep_conn.alloc(std::max(1LL, f.dep_nnz), s);
  f.dep_w.alloc(std::max(1LL, f.dep_nnz), s);
  QKnots kn{};
  for (int a = 0; a < o; a++) {
    kn.k[a] = f.knots[a];
    for (int b = 0; b < o; b++) kn.r[a][b] = (a != b) ? 1.0 / (f.knots[a] - f.knots[b]) : 0.0;
  }
  DBuf<int> err(1, s);
  err.zero();
  if (ndep)
    launch(k_q_dep_rows<Key>, blocks_for(n, 128), 128, 0, s, n, c, NK, o, kn,
           (const int *)f.block.p, (const int *)f.x.p, (const int *)f.y.p,
           (const int16_t *)f.level.p, (const int16_t *)f.info.p, (const int *)lconn.p,
           (const int *)num.p, (const Key *)ukeys.p, nl, f.dep_conn.p, f.dep_w.p, err.p);
  if (read_scalar(err.p, s))
    throw Error(TMRG_ERR_INTERNAL, "createNodes: a parent edge node is missing");
  f.node_num = std::move(num);
  f.have_nodes = true;
  TMRG_CUDA(cudaStreamSynchronize(s));
}

void qforest_create_nodes(QForest &f) {
  Stage st("tmrg_quad_create_nodes");
  if (!f.have_quads)
    throw Error(TMRG_ERR_STATE, "Cannot call createNodes(), no quadrants have been created");
  if (f.have_nodes) return;
  const long long n = f.n;
  const int o = f.order;
  const QKey K = f.key();
  if (K.total_bits() > 64)
    q_hanging<U128>(f, qkey_as<U128>(K));
  else
    q_hanging<uint64_t>(f, K);
  if (n * o * o >= (1LL << 32))
    throw Error(TMRG_ERR_ARG, "createNodes: too many element nodes");
  if (o == 3 && f.maxlev >= TMRG_MAX_LEVEL)
    throw Error(TMRG_ERR_ARG, "createNodes: an order-3 element at level " +
                                  std::to_string(TMRG_MAX_LEVEL) +
                                  " has no integer half-side for its nodes");
  const QNodeKey NK{f.maxlev + (o == 3 ? 1 : 0), f.conn->block_bits};
  if (NK.total_bits() > 128) throw Error(TMRG_ERR_KEY_RANGE, "createNodes: node key range");
  if (NK.total_bits() > 64)
    q_nodes<U128>(f, QNodeKeyT<U128>{NK.Lg, NK.bb});
  else
    q_nodes<uint64_t>(f, NK);
}

// ---------------------------------------------------------------------
// createInterpolation (TMRQuadForest.cpp:4338-4845): one fine node per
// thread, from the first (element, local node) that uses it.
__global__ void k_q_first_ref(long long n, int npe, long long rows, const int *__restrict__ econn,
                              unsigned long long *rep) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n * npe) return;
  long long e = t / npe;
  int j = (int)(t - e * npe);
  int g = econn[t];
  if (g >= 0 && g < rows) atomicMin(rep + g, ((unsigned long long)e << 8) | (unsigned)j);
}
struct QInterpCtx {
  int fo, co;
  double fk1[3], ck[3], crk[3][3];
  const int *fb, *fx, *fy;
  const int16_t *fl;
  long long cn;
  const int4 *c4;  // coarse (face | level << 26, x, y, 0)
  const int *cconn, *cdptr, *cdconn;
  const double *cdw;
  const unsigned long long *rep;
  int *err;
};
__global__ void k_q_pack(long long n, const int *__restrict__ b, const int *__restrict__ x,
                         const int *__restrict__ y, const int16_t *__restrict__ l, int4 *out) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = make_int4(b[i] | ((int)l[i] << 26), x[i], y[i], 0);
}
// 2^e as a double from its exponent (exact; e >= -1022).
__device__ __forceinline__ double q_pow2(int e) { return __hiloint2double((1023 + e) << 20, 0); }
// A non-negative int32 as a double assembled from its bits with integer
// operations (exactly (double)v): GB300 issues int-to-double conversions on
// its FP64 pipe.
__device__ __forceinline__ double q_exact(int32_t v) {
  if (v <= 0) return 0.0;
  const int e = 31 - __clz(v);
  const unsigned long long m =
      ((unsigned long long)(uint32_t)v << (52 - e)) & ((1ULL << 52) - 1ULL);
  return __longlong_as_double((long long)(((unsigned long long)(1023 + e) << 52) | m));
}
// findEnclosing (:4338-4440)
__device__ long long q_find_enclosing(const QInterpCtx &I, const Quad &node, int info) {
  const int order = I.fo;
  const int32_t h = side_of(node.level);
  const int ii = info % order, jj = info / order;
  int32_t xi = -1, yi = -1;
  if (ii == 0 || ii == order - 1)
    xi = node.x + (ii / (order - 1)) * h;
  else if (order % 2 == 1 && ii == order / 2)
    xi = node.x + h / 2;
  if (jj == 0 || jj == order - 1)
    yi = node.y + (jj / (order - 1)) * h;
  else if (order % 2 == 1 && jj == order / 2)
    yi = node.y + h / 2;
  int32_t xl = xi, xh = xi, yl = yi, yh = yi;
  if (xi < 0) {
    double xd = __dadd_rn(q_exact(node.x), __dmul_rn(q_pow2(TMRG_MAX_LEVEL - 1 - node.level), I.fk1[ii]));
    xl = (int32_t)floor(xd);
    xh = (int32_t)ceil(xd);
  }
  if (yi < 0) {
    double yd = __dadd_rn(q_exact(node.y), __dmul_rn(q_pow2(TMRG_MAX_LEVEL - 1 - node.level), I.fk1[jj]));
    yl = (int32_t)floor(yd);
    yh = (int32_t)ceil(yd);
  }
  long long low = 0, high = I.cn - 1, mid = low + (high - low) / 2;
  while (mid != low) {
    int4 q = I.c4[mid];
    int32_t hm = side_of(q.x >> 26);
    int32_t ab = q.x & 0x3ffffff;
    if (node.block == ab && node.x >= q.y && node.x < q.y + hm && node.y >= q.z &&
        node.y < q.z + hm)
      break;
    int st = cmp_position2(ab, q.y, q.z, node.block, node.x, node.y);
    if (st == 0) break;
    if (st < 0)
      low = mid + 1;
    else
      high = mid - 1;
    mid = low + (high - low) / 2;
  }
  const int32_t bx = node.x + h, by = node.y + h;
  while (mid < I.cn) {
    int4 q = I.c4[mid];
    int32_t ab = q.x & 0x3ffffff;
    if (cmp_position2(ab, q.y, q.z, node.block, bx, by) > 0) break;
    if (ab == node.block) {
      int32_t hm = side_of(q.x >> 26);
      if (q.y <= xl && xh <= q.y + hm && q.z <= yl && yh <= q.z + hm) return mid;
    }
    mid++;
  }
  return -1;
}
// the coarse index range [s, e) of one direction (an exact hit of the
// element's side keeps one index)
__device__ __forceinline__ void q_range(const QInterpCtx &I, int i, int32_t nx, int nlev,
                                        int32_t ox, int clev, int &s, int &e) {
  const int mo = I.fo, co = I.co;
  const int32_t h = side_of(nlev), hc = side_of(clev);
  if ((i == 0 && ox == nx) || (i == mo - 1 && ox == nx + h)) {
    s = 0;
    e = 1;
  } else if ((i == 0 && ox + hc == nx) || (i == mo - 1 && ox + hc == nx + h)) {
    s = co - 1;
    e = co;
  } else {
    s = 0;
    e = co;
  }
}
// one direction of computeElemInterp (:4486-4640, Lagrange branch)
__device__ __forceinline__ void q_dir(const QInterpCtx &I, int i, int32_t nx, int nlev,
                                      int32_t ox, int clev, int &s, int &e, double *N) {
  const int32_t h = side_of(nlev), hc = side_of(clev);
  const int mo = I.fo, co = I.co;
  if ((i == 0 && ox == nx) || (i == mo - 1 && ox == nx + h)) {
    s = 0;
    e = 1;
    N[0] = 1.0;
  } else if ((i == 0 && ox + hc == nx) || (i == mo - 1 && ox + hc == nx + h)) {
    s = co - 1;
    e = co;
    N[co - 1] = 1.0;
  } else {
    s = 0;
    e = co;
    // u = -1 + 2 (x + 0.5 h (1 + k_i) - ox) / hc: the scalings by 0.5 h and
    // 2 / hc are powers of two, so the products round as the reference's
    // expression does
    double t = __dadd_rn(q_exact(nx), __dmul_rn(q_pow2(TMRG_MAX_LEVEL - 1 - nlev), I.fk1[i]));
    double u = __dadd_rn(-1.0, __dmul_rn(__dsub_rn(t, q_exact(ox)), q_pow2(clev - TMRG_MAX_LEVEL + 1)));
    for (int a = 0; a < co; a++) {
      double v = 1.0;
      for (int b = 0; b < co; b++)
        if (a != b) v = __dmul_rn(v, __dmul_rn(__dsub_rn(u, I.ck[b]), I.crk[a][b]));
      N[a] = v;
    }
  }
}
// the row's entries (uniqueSort: stable by column, duplicates summed in
// order); returns the count, and with WEIGHTS writes the columns and
// weights (the count pass needs only the columns).  The enclosing coarse
// element is searched when *tp < 0 and returned in *tp.
template <bool WEIGHTS>
__device__ int q_row(const QInterpCtx &I, long long row, int *tp, int *cols, double *w) {
  unsigned long long rr = I.rep[row];
  long long e = (long long)(rr >> 8);
  int info = (int)(rr & 255u);
  Quad node{I.fb[e], I.fx[e], I.fy[e], I.fl[e]};
  long long t = *tp;
  if (t < 0) {
    t = q_find_enclosing(I, node, info);
    if (t < 0) {
      atomicExch(I.err, 1);
      return 0;
    }
    *tp = (int)t;
  }
  int4 cq = I.c4[t];
  const int mo = I.fo, co = I.co;
  double Nu[3], Nv[3];
  int is, ie, js, je;
  if (WEIGHTS) {
    q_dir(I, info % mo, node.x, node.level, cq.y, cq.x >> 26, is, ie, Nu);
    q_dir(I, info / mo, node.y, node.level, cq.z, cq.x >> 26, js, je, Nv);
  } else {
    q_range(I, info % mo, node.x, node.level, cq.y, cq.x >> 26, is, ie);
    q_range(I, info / mo, node.y, node.level, cq.z, cq.x >> 26, js, je);
  }
  int ic[27];
  double iw[WEIGHTS ? 27 : 1];
  int m = 0;
  const int *c = I.cconn + t * co * co;
  for (int jj = js; jj < je; jj++)
    for (int ii = is; ii < ie; ii++) {
      double wt = WEIGHTS ? __dmul_rn(Nu[ii], Nv[jj]) : 0.0;
      int g = c[ii + jj * co];
      if (g >= 0) {
        ic[m] = g;
        if (WEIGHTS) iw[m] = wt;
        m++;
      } else {
        int d = -g - 1;
        for (int p = I.cdptr[d]; p < I.cdptr[d + 1] && m < 27; p++) {
          ic[m] = I.cdconn[p];
          if (WEIGHTS) iw[m] = __dmul_rn(wt, I.cdw[p]);
          m++;
        }
      }
    }
  // stable insertion sort by column
  for (int a = 1; a < m; a++) {
    int kc = ic[a];
    double kw = WEIGHTS ? iw[a] : 0.0;
    int b = a - 1;
    while (b >= 0 && ic[b] > kc) {
      ic[b + 1] = ic[b];
      if (WEIGHTS) iw[b + 1] = iw[b];
      b--;
    }
    ic[b + 1] = kc;
    if (WEIGHTS) iw[b + 1] = kw;
  }
  int k = 0;
  for (int a = 0; a < m; a++) {
    double sum = WEIGHTS ? iw[a] : 0.0;
    while (a + 1 < m && ic[a + 1] == ic[a]) {
      ++a;
      if (WEIGHTS) sum = __dadd_rn(sum, iw[a]);
    }
    if (WEIGHTS) {
      cols[k] = ic[a];
      w[k] = sum;
    }
    k++;
  }
  return k;
}
__global__ void k_q_row_count(long long rows, QInterpCtx I, int *cnt, int *encl) {
  long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= rows) return;
  int t = -1;
  cnt[r] = q_row<false>(I, r, &t, nullptr, nullptr);
  encl[r] = t;
}
__global__ void k_q_row_fill(long long rows, QInterpCtx I, const int *__restrict__ rp,
                             const int *__restrict__ encl, int *cols, double *w,
                             unsigned long long *nonzero) {
  long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  unsigned nz = 0;
  if (r < rows) {
    int t = encl[r];
    int k = q_row<true>(I, r, &t, cols + rp[r], w + rp[r]);
    for (int a = 0; a < k; a++) nz += apply_keeps(w[rp[r] + a]);
  }
  // one atomic per warp
  for (int o = 16; o; o >>= 1) nz += __shfl_xor_sync(0xffffffffu, nz, o);
  if ((threadIdx.x & 31) == 0 && nz) atomicAdd(nonzero, (unsigned long long)nz);
}

void qinterp_create(QForest &fine, QForest &coarse, Interp &I) {
  Stage st("tmrg_quad_create_interpolation");
  if (&fine == &coarse) throw Error(TMRG_ERR_ARG, "Cannot interpolate between the same object");
  if (fine.interp != coarse.interp)
    throw Error(TMRG_ERR_ARG, "Interpolation types between meshes are not identical");
  qforest_create_nodes(fine);
  qforest_create_nodes(coarse);
  TMRG_CUDA(cudaStreamSynchronize(coarse.s));
  cudaStream_t s = fine.s;
  I.s = s;
  I.have_colsum = false;
  I.colsum.release();
  const long long rows = fine.num_owned;
  I.rows = rows;
  I.cols = coarse.num_owned;
  const int fnpe = fine.order * fine.order;
  DBuf<unsigned long long> rep(rows + 1, s);
  rep.fill_bytes(0xff);
  launch(k_q_first_ref, blocks_for(fine.n * fnpe, 256), 256, 0, s, fine.n, fnpe, rows,
         (const int *)fine.econn.p, rep.p);
  if (coarse.conn->nf >= (1 << 26))
    throw Error(TMRG_ERR_KEY_RANGE, "createInterpolation: more than 2^26 faces");
  DBuf<int4> c4(std::max(1LL, coarse.n), s);
  launch(k_q_pack, blocks_for(coarse.n, 256), 256, 0, s, coarse.n, (const int *)coarse.block.p,
         (const int *)coarse.x.p, (const int *)coarse.y.p, (const int16_t *)coarse.level.p, c4.p);
  DBuf<int> err(1, s);
  err.zero();
  QInterpCtx c{};
  c.fo = fine.order;
  c.co = coarse.order;
  for (int a = 0; a < 3; a++) {
    c.fk1[a] = 1.0 + fine.knots[a];
    c.ck[a] = coarse.knots[a];
    for (int b = 0; b < 3; b++)
      c.crk[a][b] = (a != b && a < coarse.order && b < coarse.order)
                        ? 1.0 / (coarse.knots[a] - coarse.knots[b])
                        : 0.0;
  }
  c.fb = fine.block.p;
  c.fx = fine.x.p;
  c.fy = fine.y.p;
  c.fl = fine.level.p;
  c.cn = coarse.n;
  c.c4 = c4.p;
  c.cconn = coarse.econn.p;
  c.cdptr = coarse.dep_ptr.p;
  c.cdconn = coarse.dep_conn.p;
  c.cdw = coarse.dep_w.p;
  c.rep = rep.p;
  c.err = err.p;
  DBuf<int> cnt(rows + 1, s);
  // compulsory per row: its reference entry, the fine element fields, the
  // coarse element it lands in (packed quad and connectivity) and the row
  // count (the fill pass adds 12 bytes per entry written)
  const long long row_bytes = rows * (8LL + 14 + 16 + 4LL * coarse.order * coarse.order + 8);
  prof_bytes(row_bytes);
  DBuf<int> encl(std::max(1LL, rows), s);
  launch(k_q_row_count, blocks_for(rows, 128), 128, 0, s, rows, c, cnt.p, encl.p);
  exclusive_scan<int>(cnt.p, cnt.p, rows, s);
  const long long nnz = read_scalar(cnt.p + rows, s);
  if (read_scalar(err.p, s))
    throw Error(TMRG_ERR_INTERNAL, "createInterpolation: no enclosing coarse quadrant");
  I.nnz = nnz;
  I.rowptr = std::move(cnt);
  I.colidx.alloc(std::max(1LL, nnz), s);
  I.vals.alloc(std::max(1LL, nnz), s);
  DBuf<unsigned long long> nzc(1, s);
  nzc.zero();
  prof_bytes(row_bytes + 12 * nnz);
  launch(k_q_row_fill, blocks_for(rows, 128), 128, 0, s, rows, c, (const int *)I.rowptr.p,
         (const int *)encl.p, I.colidx.p, I.vals.p, nzc.p);
  const long long nonzeros = (long long)read_scalar(nzc.p, s);
  interp_finish(I, nonzeros, s);
  TMRG_CUDA(cudaStreamSynchronize(s));
}

// ---------------------------------------------------------------------
// getPoints with a box per face (origin x, y, extent x, y): the first
// (element, local node) using each node places it; z = 0.
__global__ void k_q_points_first(long long n, int npe, long long num_dep, long long nl,
                                 const int *__restrict__ econn, unsigned long long *rep) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n * npe) return;
  long long e = t / npe;
  int j = (int)(t - e * npe);
  long long li = econn[t] + num_dep;
  if (li >= 0 && li < nl) atomicMin(rep + li, ((unsigned long long)e << 8) | (unsigned)j);
}
__global__ void k_q_points(long long nl, int o, QKnots kn, const unsigned long long *__restrict__ rep,
                           const int *__restrict__ blk, const int *__restrict__ xs,
                           const int *__restrict__ ys, const int16_t *__restrict__ lev,
                           const double *__restrict__ boxes, double *X) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nl) return;
  unsigned long long r = rep[i];
  if (r == ~0ULL) {
    X[3 * i] = X[3 * i + 1] = X[3 * i + 2] = 0.0;
    return;
  }
  long long e = (long long)(r >> 8);
  int j = (int)(r & 255u);
  const double sc = 1.0 / 1073741824.0;
  double d = (double)side_of(lev[e]) * sc;
  const double *bx = boxes + 4LL * blk[e];
  double u = (double)xs[e] * sc + 0.5 * d * (1.0 + kn.k[j % o]);
  double v = (double)ys[e] * sc + 0.5 * d * (1.0 + kn.k[j / o]);
  X[3 * i] = bx[0] + bx[2] * u;
  X[3 * i + 1] = bx[1] + bx[3] * v;
  X[3 * i + 2] = 0.0;
}
void qforest_get_points(QForest &f, double *d_X) {
  if (!f.have_nodes) throw Error(TMRG_ERR_STATE, "getPoints: no nodes");
  cudaStream_t s = f.s;
  const long long nl = f.num_local;
  if (f.conn->boxes.empty()) {
    TMRG_CUDA(cudaMemsetAsync(d_X, 0, sizeof(double) * 3 * nl, s));
    TMRG_CUDA(cudaStreamSynchronize(s));
    return;
  }
  const int o = f.order, npe = o * o;
  DBuf<unsigned long long> rep(nl + 1, s);
  rep.fill_bytes(0xff);
  launch(k_q_points_first, blocks_for(f.n * npe, 256), 256, 0, s, f.n, npe, f.num_dep, nl,
         (const int *)f.econn.p, rep.p);
  QKnots kn{};
  for (int a = 0; a < o; a++) kn.k[a] = f.knots[a];
  launch(k_q_points, blocks_for(nl, 256), 256, 0, s, nl, o, kn,
         (const unsigned long long *)rep.p, (const int *)f.block.p, (const int *)f.x.p,
         (const int *)f.y.p, (const int16_t *)f.level.p, (const double *)f.conn->d_boxes.p, d_X);
  TMRG_CUDA(cudaStreamSynchronize(s));
}

}  // namespace tmrg
