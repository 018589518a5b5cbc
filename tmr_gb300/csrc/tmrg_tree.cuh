// Device-side moves between trees: mapping an octant box or a node across
// a block face, edge or corner with the connectivity tables.
#pragma once

#include "tmrg_internal.h"

namespace tmrg {

// Box of side `bs` whose anchor lies across block face fi of block b,
// placed in adjacent block ab whose matching face is af
// (addFaceNeighbors TMROctForest.cpp:2525-2584, checkAdjacentFaces
// :3464-3513).  (u, v) are the box coordinates on the owner's face.
__device__ __forceinline__ Oct box_on_face(const ConnDev &c, int ab, int af,
                                           int32_t ext, int32_t u, int32_t v,
                                           int level) {
  int aid = c.face_ids[6 * ab + af];
  Oct n;
  n.block = ab;
  n.level = level;
  if (af < 2) {
    n.x = ext * (af % 2);
    face_set(aid, ext, u, v, n.y, n.z);
  } else if (af < 4) {
    n.y = ext * (af % 2);
    face_set(aid, ext, u, v, n.x, n.z);
  } else {
    n.z = ext * (af % 2);
    face_set(aid, ext, u, v, n.x, n.y);
  }
  return n;
}
__device__ __forceinline__ void face_uv(const ConnDev &c, int b, int fi,
                                        int32_t ext, const Oct &q, int32_t &u,
                                        int32_t &v) {
  int id = c.face_ids[6 * b + fi];
  if (fi < 2)
    face_get(id, ext, q.y, q.z, u, v);
  else if (fi < 4)
    face_get(id, ext, q.x, q.z, u, v);
  else
    face_get(id, ext, q.x, q.y, u, v);
}
// Box along block edge ae of block ab (addEdgeNeighbors
// TMROctForest.cpp:2601-2671).
__device__ __forceinline__ Oct box_on_edge(const ConnDev &c, int b, int ei,
                                           int ab, int ae, int32_t ext,
                                           int32_t uc, int level) {
  int a1, a2, c1, c2;
  edge_corners(ei, a1, a2);
  edge_corners(ae, c1, c2);
  int n1 = c.block_conn[8 * b + a1], n2 = c.block_conn[8 * b + a2];
  int m1 = c.block_conn[8 * ab + c1], m2 = c.block_conn[8 * ab + c2];
  int32_t u = (n1 == m2 && n2 == m1) ? ext - uc : uc;
  Oct n;
  n.block = ab;
  n.level = level;
  if (ae < 4) {
    n.x = u;
    n.y = ext * (ae % 2);
    n.z = ext * (ae / 2);
  } else if (ae < 8) {
    n.x = ext * (ae % 2);
    n.y = u;
    n.z = ext * ((ae - 4) / 2);
  } else {
    n.x = ext * (ae % 2);
    n.y = ext * ((ae - 8) / 2);
    n.z = u;
  }
  return n;
}

// Visit every image of the box `q` (side bs = ext_sub, i.e. ext = hmax -
// bs) in the trees across the block boundary it crossed.  `f` is called
// with each image.  allow_corner selects corner crossings
// (balanceOctant TMROctForest.cpp:2763-2895 and computeDepFacesAndEdges
// :3619-3702 use the same classification).
template <typename F>
__device__ __forceinline__ void for_images(const ConnDev &c, const Oct &q,
                                           int32_t bs, bool allow_corner,
                                           F &&f) {
  const int32_t hmax = TMRG_HMAX;
  int32_t ext = hmax - bs;
  int b = q.block;
  bool ex = (q.x < 0 || q.x >= hmax), ey = (q.y < 0 || q.y >= hmax),
       ez = (q.z < 0 || q.z >= hmax);
  if (allow_corner && ex && ey && ez) {
    int ci = (q.x < 0 ? 0 : 1) + (q.y < 0 ? 0 : 2) + (q.z < 0 ? 0 : 4);
    int node = c.block_conn[8 * b + ci];
    for (int p = c.node_ptr[node]; p < c.node_ptr[node + 1]; p++) {
      int ab = c.node_ent[p] / 8, ac = c.node_ent[p] % 8;
      if (ab == b) continue;
      Oct n;
      n.block = ab;
      n.level = q.level;
      n.x = ext * (ac % 2);
      n.y = ext * ((ac % 4) / 2);
      n.z = ext * (ac / 4);
      f(n);
    }
  } else if ((ex && ey) || (ex && ez) || (ey && ez)) {
    int ei;
    if (ey && ez)
      ei = (q.y < 0 ? 0 : 1) + (q.z < 0 ? 0 : 2);
    else if (ex && ez)
      ei = (q.x < 0 ? 4 : 5) + (q.z < 0 ? 0 : 2);
    else
      ei = (q.x < 0 ? 8 : 9) + (q.y < 0 ? 0 : 2);
    int edge = c.block_edge[12 * b + ei];
    int32_t uc = (ei < 4) ? q.x : (ei < 8) ? q.y : q.z;
    for (int p = c.edge_ptr[edge]; p < c.edge_ptr[edge + 1]; p++) {
      int ab = c.edge_ent[p] / 12, ae = c.edge_ent[p] % 12;
      if (ab == b) continue;
      f(box_on_edge(c, b, ei, ab, ae, ext, uc, q.level));
    }
  } else {
    int fi;
    if (ex)
      fi = q.x < 0 ? 0 : 1;
    else if (ey)
      fi = q.y < 0 ? 2 : 3;
    else
      fi = q.z < 0 ? 4 : 5;
    int face = c.block_face[6 * b + fi];
    int32_t u, v;
    face_uv(c, b, fi, ext, q, u, v);
    for (int p = c.face_ptr[face]; p < c.face_ptr[face + 1]; p++) {
      int ab = c.face_ent[p] / 6, af = c.face_ent[p] % 6;
      if (ab == b) continue;
      f(box_on_face(c, ab, af, ext, u, v, q.level));
    }
  }
}

// Canonical frame of a node: the lowest-numbered block sharing the face,
// edge or corner it lies on, with the hmax -> hmax-1 truncation
// (transformNode, TMROctForest.cpp:3847-4039).  Optionally reports
// whether an edge runs reversed in the owner frame (edge_dir = 0,1,2 for
// the edge direction) and the face orientation id.
__device__ __forceinline__ void transform_node(const ConnDev &c, int32_t &block,
                                               int32_t &x, int32_t &y,
                                               int32_t &z, int edge_dir,
                                               int *edge_rev, int *face_id) {
  const int32_t hmax = TMRG_HMAX;
  bool fx0 = x == 0, fy0 = y == 0, fz0 = z == 0;
  bool fx = fx0 || x == hmax, fy = fy0 || y == hmax, fz = fz0 || z == hmax;
  if (edge_rev) *edge_rev = 0;
  if (face_id) *face_id = 0;
  if (!(fx || fy || fz)) return;
  int b = block;
  if (fx && fy && fz) {
    int corner = (fx0 ? 0 : 1) + (fy0 ? 0 : 2) + (fz0 ? 0 : 4);
    int node = c.block_conn[8 * b + corner];
    int e = c.node_ent[c.node_ptr[node]];
    if (e / 8 != b) {
      int ac = e % 8;
      block = e / 8;
      x = hmax * (ac % 2);
      y = hmax * ((ac % 4) / 2);
      z = hmax * (ac / 4);
    }
  } else if ((fy && fz) || (fx && fz) || (fx && fy)) {
    int ei;
    int32_t u;
    if (fy && fz) {
      ei = (fy0 ? 0 : 1) + (fz0 ? 0 : 2);
      u = x;
    } else if (fx && fz) {
      ei = (fx0 ? 4 : 5) + (fz0 ? 0 : 2);
      u = y;
    } else {
      ei = (fx0 ? 8 : 9) + (fy0 ? 0 : 2);
      u = z;
    }
    int edge = c.block_edge[12 * b + ei];
    int e = c.edge_ent[c.edge_ptr[edge]];
    if (e / 12 != b) {
      int ab = e / 12, ae = e % 12;
      int a1, a2, c1, c2;
      edge_corners(ei, a1, a2);
      edge_corners(ae, c1, c2);
      int n1 = c.block_conn[8 * b + a1], n2 = c.block_conn[8 * b + a2];
      int m1 = c.block_conn[8 * ab + c1], m2 = c.block_conn[8 * ab + c2];
      int rev = (n1 == m2 && n2 == m1);
      if (edge_rev) *edge_rev = rev;
      int32_t uo = rev ? hmax - u : u;
      block = ab;
      if (ae < 4) {
        x = uo;
        y = hmax * (ae % 2);
        z = hmax * (ae / 2);
      } else if (ae < 8) {
        x = hmax * (ae % 2);
        y = uo;
        z = hmax * ((ae - 4) / 2);
      } else {
        x = hmax * (ae % 2);
        y = hmax * ((ae - 8) / 2);
        z = uo;
      }
    }
  } else {
    int fi = fx ? (fx0 ? 0 : 1) : fy ? (fy0 ? 2 : 3) : (fz0 ? 4 : 5);
    int face = c.block_face[6 * b + fi];
    int e = c.face_ent[c.face_ptr[face]];
    if (e / 6 != b) {
      int id = c.face_ids[6 * b + fi];
      if (face_id) *face_id = id;
      int32_t u, v;
      if (fi < 2)
        face_get(id, hmax, y, z, u, v);
      else if (fi < 4)
        face_get(id, hmax, x, z, u, v);
      else
        face_get(id, hmax, x, y, u, v);
      if (edge_rev) {
        int32_t ux = 0, uy = 0, uz = 0;
        if (edge_dir == 0)
          ux = 1;
        else if (edge_dir == 1)
          uy = 1;
        else if (edge_dir == 2)
          uz = 1;
        if (fi < 2)
          face_get(id, 0, uy, uz, uy, uz);
        else if (fi < 4)
          face_get(id, 0, ux, uz, ux, uz);
        else
          face_get(id, 0, ux, uy, ux, uy);
        *edge_rev = (ux < 0 || uy < 0 || uz < 0);
      }
      int ab = e / 6, af = e % 6;
      block = ab;
      if (af < 2) {
        x = hmax * (af % 2);
        y = u;
        z = v;
      } else if (af < 4) {
        x = u;
        y = hmax * (af % 2);
        z = v;
      } else {
        x = u;
        y = v;
        z = hmax * (af % 2);
      }
    }
  }
  if (x == hmax) x = hmax - 1;
  if (y == hmax) y = hmax - 1;
  if (z == hmax) z = hmax - 1;
}

// lower_bound over a sorted key array (uint64_t or U128).
template <typename K>
__device__ __forceinline__ long long lower_bound_key(const K *a, long long n, K v) {
  long long lo = 0, hi = n;
  while (lo < hi) {
    long long mid = (lo + hi) >> 1;
    if (a[mid] < v)
      lo = mid + 1;
    else
      hi = mid;
  }
  return lo;
}
template <typename K>
__device__ __forceinline__ bool contains_key(const K *a, long long n, K v) {
  long long i = lower_bound_key(a, n, v);
  return i < n && a[i] == v;
}
__device__ __forceinline__ long long lower_bound_u64(const uint64_t *a, long long n,
                                                     uint64_t v) {
  return lower_bound_key(a, n, v);
}
__device__ __forceinline__ bool contains_u64(const uint64_t *a, long long n, uint64_t v) {
  return contains_key(a, n, v);
}

// Two-level search over a large sorted array: `top` samples every
// 2^S-th key (small enough to stay in L2), so a lookup touches the big
// array only inside one 2^S-key segment.
template <typename K>
struct SampledKeysT {
  const K *keys;
  long long n;
  const K *top;
  long long ntop;
  int S;
  __device__ __forceinline__ long long lower_bound(K v) const {
    // last sample <= v
    long long lo = 0, hi = ntop;
    while (lo < hi) {
      long long mid = (lo + hi) >> 1;
      if (kldg(top + mid) <= v)
        lo = mid + 1;
      else
        hi = mid;
    }
    long long seg = lo - 1;
    if (seg < 0) return 0;
    long long a = seg << S, b = min(n, (seg + 1) << S);
    while (a < b) {
      long long mid = (a + b) >> 1;
      if (kldg(keys + mid) < v)
        a = mid + 1;
      else
        b = mid;
    }
    return a;
  }
};
using SampledKeys = SampledKeysT<uint64_t>;

template <typename K>
__global__ void k_sample_keys(long long ntop, int S, const K *__restrict__ keys, K *top) {
  long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (j < ntop) top[j] = keys[j << S];
}

}  // namespace tmrg
