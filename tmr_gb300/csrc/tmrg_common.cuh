// Shared definitions for the GB300 octree-forest library: octant algebra,
// block geometry, Morton keys and the error type.  Everything here is
// host+device inline so that kernels and host setup agree bit for bit.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <stdexcept>
#include <string>

#include "../../include/tmrg.h"

#define TMRG_MAX_LEVEL 30
#define TMRG_HMAX (1 << TMRG_MAX_LEVEL)
#define TMRG_MAX_ORDER 6

#define HD __host__ __device__ __forceinline__

namespace tmrg {

// Error carried from internal code to the C ABI, which turns it into a
// status code.  Nothing in the library aborts the process.
struct Error : public std::runtime_error {
  int status;
  Error(int s, const std::string &m) : std::runtime_error(m), status(s) {}
};

#define TMRG_CUDA(call)                                                    \
  do {                                                                     \
    cudaError_t _e = (call);                                               \
    if (_e != cudaSuccess)                                                 \
      throw ::tmrg::Error(TMRG_ERR_CUDA, std::string(#call) + ": " +       \
                                             cudaGetErrorString(_e));      \
  } while (0)
#define TMRG_CHECK_LAUNCH() TMRG_CUDA(cudaGetLastError())

HD int32_t side_of(int level) { return (int32_t)1 << (TMRG_MAX_LEVEL - level); }

// Corner nodes of block edge e: edges 0-3 run along x, 4-7 along y,
// 8-11 along z (TMROctForest.cpp:29-31).
HD void edge_corners(int e, int &n1, int &n2) {
  if (e < 4) {
    n1 = 2 * (e & 1) + 4 * (e >> 1);
    n2 = n1 + 1;
  } else if (e < 8) {
    n1 = (e & 1) + 4 * ((e - 4) >> 1);
    n2 = n1 + 2;
  } else {
    n1 = e - 8;
    n2 = n1 + 4;
  }
}
// Corner k of face f, first free coordinate fastest (TMROctForest.cpp:37).
HD int face_corner(int f, int k) {
  int d = f >> 1, s = f & 1, a = k & 1, b = k >> 1;
  if (d == 0) return s + 2 * a + 4 * b;
  if (d == 1) return a + 2 * s + 4 * b;
  return a + 2 * b + 4 * s;
}
// Parent face / edge touched by child `id` in direction k
// (child_id_to_face_index / child_id_to_edge_index).
HD int child_face(int id, int k) { return 2 * k + ((id >> k) & 1); }
HD int child_edge(int id, int k) {
  int x = id & 1, y = (id >> 1) & 1, z = id >> 2;
  if (k == 0) return y + 2 * z;
  if (k == 1) return 4 + x + 2 * z;
  return 8 + x + 2 * y;
}
HD int child_face_edge(int id, int k, int j) {
  int d0 = (k == 2) ? 1 : 2;  // directions other than k, descending
  int d1 = (k == 0) ? 1 : 0;
  return child_edge(id, j == 0 ? d0 : d1);
}
// Edge e (0..3) of face f (face_to_edge_index): entries 0,1 run along the
// face's second free coordinate, 2,3 along the first.
HD int face_edge(int f, int e) {
  int d = f >> 1, s = f & 1, side = e & 1, dir, a, b;
  if (d == 0)
    dir = (e < 2) ? 2 : 1;
  else if (d == 1)
    dir = (e < 2) ? 2 : 0;
  else
    dir = (e < 2) ? 1 : 0;
  if (dir == 0) {
    a = (d == 1) ? s : side;
    b = (d == 2) ? s : side;
  } else if (dir == 1) {
    a = (d == 0) ? s : side;
    b = (d == 2) ? s : side;
  } else {
    a = (d == 0) ? s : side;
    b = (d == 1) ? s : side;
  }
  return 4 * dir + a + 2 * b;
}

// The 8 face transforms between matched block faces
// (TMROctForest.cpp:78-198).  `ext` is hmax - h for an octant of side h,
// hmax for a node.
HD void face_get(int id, int32_t ext, int32_t x, int32_t y, int32_t &u,
                 int32_t &v) {
  switch (id) {
    case 0: u = x; v = y; break;
    case 1: u = ext - y; v = x; break;
    case 2: u = ext - x; v = ext - y; break;
    case 3: u = y; v = ext - x; break;
    case 4: u = y; v = x; break;
    case 5: u = x; v = ext - y; break;
    case 6: u = ext - y; v = ext - x; break;
    default: u = ext - x; v = y; break;
  }
}
HD void face_set(int id, int32_t ext, int32_t u, int32_t v, int32_t &x,
                 int32_t &y) {
  switch (id) {
    case 0: x = u; y = v; break;
    case 1: x = v; y = ext - u; break;
    case 2: x = ext - u; y = ext - v; break;
    case 3: x = ext - v; y = u; break;
    case 4: x = v; y = u; break;
    case 5: x = u; y = ext - v; break;
    case 6: x = ext - v; y = ext - u; break;
    default: x = ext - u; y = v; break;
  }
}

// Lightweight octant value (the SoA arrays hold the same fields).
struct Oct {
  int32_t block, x, y, z;
  int level;
};

HD int child_id(const Oct &o) {
  int32_t h = side_of(o.level);
  return ((o.x & h) ? 1 : 0) | ((o.y & h) ? 2 : 0) | ((o.z & h) ? 4 : 0);
}
HD Oct sibling(const Oct &o, int id) {
  int32_t h = side_of(o.level);
  Oct s = o;
  int32_t xr = (o.x & h) ? o.x - h : o.x, yr = (o.y & h) ? o.y - h : o.y,
          zr = (o.z & h) ? o.z - h : o.z;
  s.x = (id & 1) ? xr + h : xr;
  s.y = (id & 2) ? yr + h : yr;
  s.z = (id & 4) ? zr + h : zr;
  return s;
}
HD Oct parent_of(const Oct &o) {
  Oct p = o;
  if (o.level > 0) {
    int32_t h = side_of(o.level);
    p.level = o.level - 1;
    p.x = o.x & ~h;
    p.y = o.y & ~h;
    p.z = o.z & ~h;
  }
  return p;
}
HD Oct face_nbr(const Oct &o, int f) {
  int32_t h = side_of(o.level);
  Oct n = o;
  n.x += (f == 0) ? -h : (f == 1) ? h : 0;
  n.y += (f == 2) ? -h : (f == 3) ? h : 0;
  n.z += (f == 4) ? -h : (f == 5) ? h : 0;
  return n;
}
HD Oct edge_nbr(const Oct &o, int e) {
  int32_t h = side_of(o.level);
  Oct n = o;
  int32_t a = (e & 1) ? h : -h, b = (e & 2) ? h : -h;
  if (e < 4) {
    n.y += a;
    n.z += b;
  } else if (e < 8) {
    n.x += a;
    n.z += b;
  } else {
    n.x += a;
    n.y += b;
  }
  return n;
}
HD Oct corner_nbr(const Oct &o, int c) {
  int32_t h = side_of(o.level);
  Oct n = o;
  n.x += (c & 1) ? h : -h;
  n.y += (c & 2) ? h : -h;
  n.z += (c & 4) ? h : -h;
  return n;
}
HD bool in_tree(const Oct &q) {
  return q.x >= 0 && q.x < TMRG_HMAX && q.y >= 0 && q.y < TMRG_HMAX &&
         q.z >= 0 && q.z < TMRG_HMAX;
}
// Morton position order with x-priority ties (TMROctant.cpp:171-204).
HD int cmp_position(int32_t ab, int32_t ax, int32_t ay, int32_t az, int32_t bb,
                    int32_t bx, int32_t by, int32_t bz) {
  if (ab != bb) return ab < bb ? -1 : 1;
  uint32_t dx = (uint32_t)(ax ^ bx), dy = (uint32_t)(ay ^ by),
           dz = (uint32_t)(az ^ bz);
  uint32_t any = dx | dy | dz;
  if (any == 0) return 0;
  int32_t d;
  if (dx > (any ^ dx))
    d = ax - bx;
  else if (dy > (any ^ dy))
    d = ay - by;
  else
    d = az - bz;
  return d > 0 ? 1 : (d < 0 ? -1 : 0);
}

// ---------------------------------------------------------------------
// 64-bit Morton keys.  Coordinates are interleaved x-most-significant in
// each bit triple, which reproduces TMROctant::compare on positions.
HD uint64_t spread3(uint64_t v) {  // 21 bits -> every third bit
  v &= 0x1fffffULL;
  v = (v | (v << 32)) & 0x1f00000000ffffULL;
  v = (v | (v << 16)) & 0x1f0000ff0000ffULL;
  v = (v | (v << 8)) & 0x100f00f00f00f00fULL;
  v = (v | (v << 4)) & 0x10c30c30c30c30c3ULL;
  v = (v | (v << 2)) & 0x1249249249249249ULL;
  return v;
}
HD uint32_t compact3(uint64_t v) {
  v &= 0x1249249249249249ULL;
  v = (v ^ (v >> 2)) & 0x10c30c30c30c30c3ULL;
  v = (v ^ (v >> 4)) & 0x100f00f00f00f00fULL;
  v = (v ^ (v >> 8)) & 0x1f0000ff0000ffULL;
  v = (v ^ (v >> 16)) & 0x1f00000000ffffULL;
  v = (v ^ (v >> 32)) & 0x1fffffULL;
  return (uint32_t)v;
}
HD uint64_t morton3(uint32_t x, uint32_t y, uint32_t z) {
  return (spread3(x) << 2) | (spread3(y) << 1) | spread3(z);
}

// 128-bit keys for forests whose octant or node keys outgrow 64 bits
// (deep levels times many blocks).  Only the operations the key kernels
// use: shifts, or, and, compare, and the low words.
struct alignas(16) U128 {
  uint64_t lo, hi;
  HD U128() : lo(0), hi(0) {}
  HD U128(uint64_t v) : lo(v), hi(0) {}
  HD U128(uint64_t h, uint64_t l) : lo(l), hi(h) {}
};
HD U128 operator|(U128 a, U128 b) { return U128(a.hi | b.hi, a.lo | b.lo); }
HD U128 operator&(U128 a, U128 b) { return U128(a.hi & b.hi, a.lo & b.lo); }
HD bool operator==(U128 a, U128 b) { return a.lo == b.lo && a.hi == b.hi; }
HD bool operator!=(U128 a, U128 b) { return !(a == b); }
HD bool operator<(U128 a, U128 b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }
HD bool operator<=(U128 a, U128 b) { return !(b < a); }
HD U128 operator<<(U128 a, int s) {
  if (s <= 0) return a;
  if (s >= 128) return U128();
  if (s >= 64) return U128(a.lo << (s - 64), 0);
  return U128((a.hi << s) | (a.lo >> (64 - s)), a.lo << s);
}
HD U128 operator>>(U128 a, int s) {
  if (s <= 0) return a;
  if (s >= 128) return U128();
  if (s >= 64) return U128(0, a.hi >> (s - 64));
  return U128(a.hi >> s, (a.lo >> s) | (a.hi << (64 - s)));
}
HD uint64_t klo64(uint64_t k) { return k; }
HD uint64_t klo64(U128 k) { return k.lo; }
// all ones in the low `bits` bits
template <typename K>
HD K kmask(int bits);
template <>
HD uint64_t kmask<uint64_t>(int bits) {
  return bits >= 64 ? ~0ULL : ((1ULL << bits) - 1ULL);
}
template <>
HD U128 kmask<U128>(int bits) {
  if (bits >= 128) return U128(~0ULL, ~0ULL);
  if (bits >= 64) return U128(kmask<uint64_t>(bits - 64), ~0ULL);
  return U128(0, kmask<uint64_t>(bits));
}
// Morton code of coordinates of up to 21 (uint64_t) or 30 (U128) bits.
template <typename K>
HD K kmorton3(uint32_t x, uint32_t y, uint32_t z);
template <>
HD uint64_t kmorton3<uint64_t>(uint32_t x, uint32_t y, uint32_t z) {
  return morton3(x, y, z);
}
template <>
HD U128 kmorton3<U128>(uint32_t x, uint32_t y, uint32_t z) {
  const uint32_t m21 = 0x1fffffu;
  return U128(morton3(x & m21, y & m21, z & m21)) |
         (U128(morton3(x >> 21, y >> 21, z >> 21)) << 63);
}
// Every third bit of v (from bit 0), compacted.
HD uint32_t kcompact3(uint64_t v) { return compact3(v); }
HD uint32_t kcompact3(U128 v) {
  return compact3(v.lo & 0x7fffffffffffffffULL) | (compact3((v >> 63).lo) << 21);
}
// 16-byte aligned read-only load
__device__ __forceinline__ uint64_t kldg(const uint64_t *p) { return __ldg(p); }
__device__ __forceinline__ U128 kldg(const U128 *p) {
  const ulonglong2 v = __ldg(reinterpret_cast<const ulonglong2 *>(p));
  return U128(v.y, v.x);
}

// Key layout for octants: [block | morton(3W) | level(5)], W = bits per
// coordinate (the finest level present).  Element order = key order.
// K = uint64_t where bb + 3W + 5 <= 64, else U128.
template <typename K>
struct OctKeyT {
  int W;  // coordinate bits
  int bb; // block bits
  HD int total_bits() const { return bb + 3 * W + 5; }
  HD K make(int32_t block, int32_t x, int32_t y, int32_t z, int level) const {
    int s = TMRG_MAX_LEVEL - W;
    K m = kmorton3<K>((uint32_t)x >> s, (uint32_t)y >> s, (uint32_t)z >> s);
    return (K((uint64_t)(uint32_t)block) << (3 * W + 5)) | (m << 5) | K((uint64_t)level);
  }
  HD K pos(K key) const { return key >> 5; }
  HD Oct decode(K key) const {
    Oct o;
    int s = TMRG_MAX_LEVEL - W;
    o.level = (int)(klo64(key) & 31);
    K m = (key >> 5) & kmask<K>(3 * W);
    o.x = (int32_t)(kcompact3(m >> 2) << s);
    o.y = (int32_t)(kcompact3(m >> 1) << s);
    o.z = (int32_t)(kcompact3(m) << s);
    o.block = (int32_t)klo64(key >> (3 * W + 5));
    return o;
  }
};
using OctKey = OctKeyT<uint64_t>;

// Key layout for node objects: [block | morton(3Wn) | label(lb)].  Node
// coordinates are multiples of 2^(30-Lg) or the truncated boundary value
// hmax-1; they map to 2c/s and to all-ones, which keeps the order of the
// truncated 30-bit coordinates (TMROctForest.cpp:4029-4037).
template <typename K>
struct NodeKeyT {
  int Lg;  // node grid level
  int bb;  // block bits
  int lb;  // label bits (0 or 2)
  HD int W() const { return Lg + 1; }
  HD int total_bits() const { return bb + 3 * (Lg + 1) + lb; }
  HD uint32_t map(int32_t c) const {
    if (c == TMRG_HMAX - 1) return (1u << (Lg + 1)) - 1u;
    return ((uint32_t)c >> (TMRG_MAX_LEVEL - Lg)) << 1;
  }
  HD K make(int32_t block, int32_t x, int32_t y, int32_t z, int label) const {
    K m = kmorton3<K>(map(x), map(y), map(z));
    return (K((uint64_t)(uint32_t)block) << (3 * (Lg + 1) + lb)) | (m << lb) |
           K((uint64_t)label);
  }
};
using NodeKey = NodeKeyT<uint64_t>;

// Seeded uniform U(seed, stream, i) in [0, 1): splitmix64 of the seed and
// stream, mixed with the index (same function as oo_uniform and
// workloads.uniform).
__device__ __forceinline__ double seeded_uniform(uint64_t seed, uint64_t stream, uint64_t i) {
  auto sm = [](uint64_t x) {
    x += 0x9E3779B97F4A7C15ULL;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ULL;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBULL;
    return x ^ (x >> 31);
  };
  uint64_t r = sm(sm(seed * 0x100000001B3ULL + stream) ^ (i * 0xD6E8FEB86659FD93ULL));
  return (double)(r >> 11) * (1.0 / 9007199254740992.0);
}

HD int bits_for(long long n) {  // bits to hold values 0..n-1 (>= 1)
  int b = 1;
  while ((1LL << b) < n) b++;
  return b;
}

}  // namespace tmrg
