// Forest construction and adaptation on the GPU: createTrees, refine,
// coarsen, duplicate and 2:1 balance.  Octants are kept as a sorted
// structure of arrays; every set operation is a 64-bit Morton-key radix
// sort followed by a compaction.
#include <algorithm>
#include <vector>

#include "tmrg_tree.cuh"

namespace tmrg {

std::atomic<long long> g_kernel_launches{0};
std::atomic<long long> g_host_syncs{0};
std::atomic<long long> g_device_allocs{0};
std::atomic<bool> g_profile_on{false};
thread_local long long g_prof_bytes = 0;
thread_local long long g_prof_flops = 0;

void Forest::set_order(int o, int it) {
  free_nodes();
  if (o < 2) o = 2;
  if (o > TMRG_MAX_ORDER) o = TMRG_MAX_ORDER;
  order = o;
  interp = it;
  // Knots on [-1, 1] (TMROctForest.cpp:1409-1426); computed with the
  // host's cos so both sides of a comparison share them.
  for (int i = 0; i < TMRG_MAX_ORDER; i++) knots[i] = 0.0;
  knots[0] = -1.0;
  knots[o - 1] = 1.0;
  for (int i = 1; i < o - 1; i++) {
    if (it == TMRG_GAUSS_LOBATTO_POINTS || it == TMRG_BERNSTEIN_POINTS)
      knots[i] = -cos(M_PI * i / (o - 1));
    else
      knots[i] = -1.0 + 2.0 * i / (o - 1);
  }
}

// The octant key layout; the kernels take 64-bit keys where it fits and
// 128-bit keys (U128) otherwise.
OctKey Forest::oct_key() const {
  OctKey k;
  k.W = std::max(maxlev, 1);
  k.bb = conn->block_bits;
  if (k.total_bits() > 128)
    throw Error(TMRG_ERR_KEY_RANGE,
                "octant key needs " + std::to_string(k.total_bits()) + " bits");
  return k;
}
template <typename Key>
static OctKeyT<Key> key_as(const OctKey &k) {
  return OctKeyT<Key>{k.W, k.bb};
}

static void alloc_octs(Forest &f, long long n) {
  f.block.alloc(n, f.s);
  f.x.alloc(n, f.s);
  f.y.alloc(n, f.s);
  f.z.alloc(n, f.s);
  f.level.alloc(n, f.s);
  f.info.alloc(n, f.s);
  f.n = n;
}

// ---------------------------------------------------------------------
// createTrees: every block refined uniformly to `level`, generated
// directly in Morton order (TMROctForest.cpp:1744-1833).
__global__ void k_create_trees(long long n, int level, int *block, int *x,
                               int *y, int *z, int16_t *lev, int16_t *info) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  long long b = i >> (3 * level);  // 8^level octants per block
  uint64_t m = (uint64_t)(i - (b << (3 * level)));
  int s = TMRG_MAX_LEVEL - level;
  block[i] = (int)b;
  x[i] = (int)(compact3(m >> 2) << s);
  y[i] = (int)(compact3(m >> 1) << s);
  z[i] = (int)(compact3(m) << s);
  lev[i] = (int16_t)level;
  info[i] = 0;
}

void forest_create_trees(Forest &f, int level) {
  if (!f.conn) throw Error(TMRG_ERR_STATE, "createTrees: no connectivity");
  if (level < 0) level = 0;
  if (level >= TMRG_MAX_LEVEL) level = TMRG_MAX_LEVEL - 1;
  if (level > 20) throw Error(TMRG_ERR_ARG, "createTrees: level too large");
  f.free_nodes();
  long long n = (long long)f.conn->nb << (3 * level);
  alloc_octs(f, n);
  launch(k_create_trees, blocks_for(n, 256), 256, 0, f.s, n, level, f.block.p,
         f.x.p, f.y.p, f.z.p, f.level.p, f.info.p);
  f.maxlev = level;
  f.have_octs = true;
}

// ---------------------------------------------------------------------
// refine(refinement[], min, max) (TMROctForest.cpp:2169-2329).  Each
// octant emits itself, its coarsened ancestor or the child-0 seeds of its
// refinement; the set is made unique on (position, level) keeping the
// first emitted, then on position keeping the finest.
struct RefineArgs {
  const int *ref;  // nullptr: refine every octant by one level
  int min_level, max_level;
};

__device__ __forceinline__ int refine_target(const RefineArgs &a, int r,
                                             int level, int &reps) {
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

__global__ void k_refine_count(long long n, RefineArgs a,
                               const int16_t *__restrict__ lev,
                               unsigned *__restrict__ cnt, int *maxlev) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  int ml = 0;
  if (i < n) {
    int reps;
    int nl = refine_target(a, a.ref ? a.ref[i] : 1, lev[i], reps);
    cnt[i] = (unsigned)(reps * reps * reps);
    ml = nl;
  }
  for (int o = 16; o > 0; o >>= 1) ml = max(ml, __shfl_down_sync(0xffffffffu, ml, o));
  if ((threadIdx.x & 31) == 0 && ml > 0) atomicMax(maxlev, ml);
}

// Payload: source index; bit 31 set when the octant keeps its info.
template <typename Key>
__global__ void k_refine_emit(long long n, RefineArgs a, OctKeyT<Key> K,
                              const int *__restrict__ blk,
                              const int *__restrict__ xs,
                              const int *__restrict__ ys,
                              const int *__restrict__ zs,
                              const int16_t *__restrict__ lev,
                              const unsigned *__restrict__ offs, Key *keys,
                              uint32_t *vals) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int level = lev[i];
  int r = a.ref ? a.ref[i] : 1;
  int reps;
  int nl = refine_target(a, r, level, reps);
  unsigned o = offs[i];
  int32_t x = xs[i], y = ys[i], z = zs[i];
  if (nl == level) {
    keys[o] = K.make(blk[i], x, y, z, level);
    vals[o] = (uint32_t)i | 0x80000000u;
    return;
  }
  int32_t h = side_of(nl);
  int32_t x0 = x - x % h, y0 = y - y % h, z0 = z - z % h;
  for (int ii = 0; ii < reps; ii++)
    for (int jj = 0; jj < reps; jj++)
      for (int kk = 0; kk < reps; kk++) {
        keys[o] = K.make(blk[i], x0 + 2 * ii * h, y0 + 2 * jj * h,
                         z0 + 2 * kk * h, nl);
        vals[o] = (uint32_t)i;
        o++;
      }
}

// Keep entry i of the sorted keys if it opens its run of equal keys and
// that run is the last (finest) one at its position.
template <typename Key>
__global__ void k_dedupe_flags(long long n, const Key *__restrict__ keys,
                               unsigned *__restrict__ flag) {
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
__global__ void k_compact_octs(long long n, OctKeyT<Key> K,
                               const Key *__restrict__ keys,
                               const uint32_t *__restrict__ vals,
                               const unsigned *__restrict__ pos,
                               const int16_t *__restrict__ old_info, int *blk,
                               int *xs, int *ys, int *zs, int16_t *lev,
                               int16_t *info) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (pos[i + 1] == pos[i]) return;
  unsigned o = pos[i];
  Oct q = K.decode(keys[i]);
  blk[o] = q.block;
  xs[o] = q.x;
  ys[o] = q.y;
  zs[o] = q.z;
  lev[o] = (int16_t)q.level;
  uint32_t v = vals ? vals[i] : 0u;
  info[o] = (vals && old_info && (v & 0x80000000u)) ? old_info[v & 0x7fffffffu]
                                                   : (int16_t)0;
}

template <typename Key>
static void refine_sort_compact(Forest &f, const RefineArgs &a, const OctKeyT<Key> &K,
                                const DBuf<unsigned> &cnt, unsigned total) {
  cudaStream_t s = f.s;
  const long long n = f.n;
  DBuf<Key> keys(total, s);
  DBuf<uint32_t> vals(total, s);
  launch(k_refine_emit<Key>, blocks_for(n, 256), 256, 0, s, n, a, K,
         (const int *)f.block.p, (const int *)f.x.p, (const int *)f.y.p,
         (const int *)f.z.p, (const int16_t *)f.level.p, (const unsigned *)cnt.p,
         keys.p, vals.p);
  sort_keys(keys, &vals, total, K.total_bits(), s);
  DBuf<unsigned> pos(total + 1, s);
  launch(k_dedupe_flags<Key>, blocks_for(total, 256), 256, 0, s, (long long)total,
         (const Key *)keys.p, pos.p);
  exclusive_scan<unsigned>(pos.p, pos.p, total, s);
  unsigned m = read_scalar(pos.p + total, s);
  DBuf<int16_t> old_info = std::move(f.info);
  alloc_octs(f, m);
  launch(k_compact_octs<Key>, blocks_for(total, 256), 256, 0, s, (long long)total, K,
         (const Key *)keys.p, (const uint32_t *)vals.p,
         (const unsigned *)pos.p, (const int16_t *)old_info.p, f.block.p, f.x.p,
         f.y.p, f.z.p, f.level.p, f.info.p);
}

void forest_refine(Forest &f, const int *d_ref, long long nref, int min_level,
                   int max_level) {
  Stage st("tmrg_refine");
  if (!f.have_octs) throw Error(TMRG_ERR_STATE, "refine: no octants");
  if (d_ref && nref != f.n)
    throw Error(TMRG_ERR_ARG, "refine: refinement array length " +
                                  std::to_string(nref) + " != octants " +
                                  std::to_string(f.n));
  f.free_nodes();
  if (min_level < 0) min_level = 0;
  if (max_level > TMRG_MAX_LEVEL) max_level = TMRG_MAX_LEVEL;
  if (min_level > max_level) min_level = max_level;
  long long n = f.n;
  if (n == 0) return;
  cudaStream_t s = f.s;
  RefineArgs a{d_ref, min_level, max_level};
  DBuf<unsigned> cnt(n + 1, s);
  DBuf<int> ml(1, s);
  ml.zero();
  launch(k_refine_count, blocks_for(n, 256), 256, 0, s, n, a,
         (const int16_t *)f.level.p, cnt.p, ml.p);
  exclusive_scan<unsigned>(cnt.p, cnt.p, n, s);
  unsigned total = read_scalar(cnt.p + n, s);
  int newmax = read_scalar(ml.p, s);
  f.maxlev = std::max(newmax, 0);
  const OctKey K = f.oct_key();
  if (K.total_bits() > 64)
    refine_sort_compact<U128>(f, a, key_as<U128>(K), cnt, total);
  else
    refine_sort_compact<uint64_t>(f, a, K, cnt, total);
}

// ---------------------------------------------------------------------
// coarsen (TMROctForest.cpp:2119-2164): the parent of every child-0,
// level-0 octants unchanged, in array order.
__global__ void k_coarsen_flags(long long n, const int *__restrict__ xs,
                                const int *__restrict__ ys,
                                const int *__restrict__ zs,
                                const int16_t *__restrict__ lev,
                                unsigned *flag) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int l = lev[i];
  unsigned keep = 1;
  if (l > 0) {
    int32_t h = side_of(l);
    keep = ((xs[i] & h) | (ys[i] & h) | (zs[i] & h)) ? 0u : 1u;
  }
  flag[i] = keep;
}
__global__ void k_coarsen_emit(long long n, const unsigned *__restrict__ pos,
                               const int *__restrict__ blk,
                               const int *__restrict__ xs,
                               const int *__restrict__ ys,
                               const int *__restrict__ zs,
                               const int16_t *__restrict__ lev,
                               const int16_t *__restrict__ info, int *ob,
                               int *ox, int *oy, int *oz, int16_t *ol,
                               int16_t *oi) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || pos[i + 1] == pos[i]) return;
  unsigned o = pos[i];
  int l = lev[i];
  ob[o] = blk[i];
  if (l > 0) {
    int32_t h = side_of(l);
    ox[o] = xs[i] & ~h;
    oy[o] = ys[i] & ~h;
    oz[o] = zs[i] & ~h;
    ol[o] = (int16_t)(l - 1);
    oi[o] = 0;
  } else {
    ox[o] = xs[i];
    oy[o] = ys[i];
    oz[o] = zs[i];
    ol[o] = (int16_t)l;
    oi[o] = info[i];
  }
}

void forest_coarsen(Forest &f, Forest &out) {
  if (!f.have_octs) throw Error(TMRG_ERR_STATE, "coarsen: no octants");
  out.conn = f.conn;
  out.set_order(f.order, f.interp);
  cudaStream_t s = out.s;
  TMRG_CUDA(cudaStreamSynchronize(f.s));
  long long n = f.n;
  DBuf<unsigned> pos(n + 1, s);
  launch(k_coarsen_flags, blocks_for(n, 256), 256, 0, s, n, (const int *)f.x.p,
         (const int *)f.y.p, (const int *)f.z.p, (const int16_t *)f.level.p,
         pos.p);
  exclusive_scan<unsigned>(pos.p, pos.p, n, s);
  unsigned m = n ? read_scalar(pos.p + n, s) : 0;
  alloc_octs(out, m);
  launch(k_coarsen_emit, blocks_for(n, 256), 256, 0, s, n,
         (const unsigned *)pos.p, (const int *)f.block.p, (const int *)f.x.p,
         (const int *)f.y.p, (const int *)f.z.p, (const int16_t *)f.level.p,
         (const int16_t *)f.info.p, out.block.p, out.x.p, out.y.p, out.z.p,
         out.level.p, out.info.p);
  out.maxlev = std::max(f.maxlev - 1, 0);
  out.have_octs = true;
}

void forest_duplicate(Forest &f, Forest &out) {
  out.conn = f.conn;
  out.set_order(f.order, f.interp);
  if (!f.have_octs) return;
  TMRG_CUDA(cudaStreamSynchronize(f.s));
  alloc_octs(out, f.n);
  cudaStream_t s = out.s;
  size_t n = (size_t)f.n;
  TMRG_CUDA(cudaMemcpyAsync(out.block.p, f.block.p, n * 4, cudaMemcpyDeviceToDevice, s));
  TMRG_CUDA(cudaMemcpyAsync(out.x.p, f.x.p, n * 4, cudaMemcpyDeviceToDevice, s));
  TMRG_CUDA(cudaMemcpyAsync(out.y.p, f.y.p, n * 4, cudaMemcpyDeviceToDevice, s));
  TMRG_CUDA(cudaMemcpyAsync(out.z.p, f.z.p, n * 4, cudaMemcpyDeviceToDevice, s));
  TMRG_CUDA(cudaMemcpyAsync(out.level.p, f.level.p, n * 2, cudaMemcpyDeviceToDevice, s));
  TMRG_CUDA(cudaMemcpyAsync(out.info.p, f.info.p, n * 2, cudaMemcpyDeviceToDevice, s));
  out.maxlev = f.maxlev;
  out.have_octs = true;
}

// ---------------------------------------------------------------------
// 2:1 balance (TMROctForest.cpp:2525-3089).
//
// The reference grows a hash of child-0 octants to a fixed point: every
// child-0 q at level L > 1 adds the child-0 of each face/edge(/corner)
// neighbour of its parent, across tree boundaries through the block
// tables.  That rule only maps level L to level L-1, so the fixed point is
// reached level by level from the finest down: S_L = seeds_L U gen(S_{L+1}),
// each level one generate + sort + unique.  The balanced forest is then
// the set of siblings of all S_L members that are not themselves refined
// (a sibling s at level L is refined iff S_{L+1} holds a child-0 at s's
// anchor), which is exactly what the reference's sibling expansion and
// finest-per-position sort leave.

// Position key of a family: [block | morton(3W)].
template <typename Key>
struct PosKey {
  int W, bb;
  __device__ __forceinline__ Key make(int32_t b, int32_t x, int32_t y, int32_t z) const {
    int s = TMRG_MAX_LEVEL - W;
    return (Key((uint64_t)(uint32_t)b) << (3 * W)) |
           kmorton3<Key>((uint32_t)x >> s, (uint32_t)y >> s, (uint32_t)z >> s);
  }
  __device__ __forceinline__ Oct decode(Key k, int level) const {
    int s = TMRG_MAX_LEVEL - W;
    Key m = k & kmask<Key>(3 * W);
    Oct o;
    o.block = (int32_t)klo64(k >> (3 * W));
    o.x = (int32_t)(kcompact3(m >> 2) << s);
    o.y = (int32_t)(kcompact3(m >> 1) << s);
    o.z = (int32_t)(kcompact3(m) << s);
    o.level = level;
    return o;
  }
};

// Seeds: the child-0 of every octant, keyed level-major.
template <typename Key>
__global__ void k_seed_keys(long long n, PosKey<Key> P, const int *__restrict__ blk,
                            const int *__restrict__ xs,
                            const int *__restrict__ ys,
                            const int *__restrict__ zs,
                            const int16_t *__restrict__ lev, Key *keys) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  Oct o{blk[i], xs[i], ys[i], zs[i], lev[i]};
  Oct q = sibling(o, 0);
  keys[i] = (Key((uint64_t)o.level) << (P.bb + 3 * P.W)) | P.make(q.block, q.x, q.y, q.z);
}

// Unique flags over sorted keys (first of each run).
template <typename Key>
__global__ void k_unique_flags(long long n, const Key *__restrict__ keys, unsigned *flag) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  flag[i] = (i == 0 || keys[i - 1] != keys[i]) ? 1u : 0u;
}
template <typename Key>
__global__ void k_unique_emit(long long n, const Key *__restrict__ keys,
                              const unsigned *__restrict__ pos, Key mask, Key *out) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || pos[i + 1] == pos[i]) return;
  out[pos[i]] = keys[i] & mask;
}
template <typename Key>
__global__ void k_mask_copy(long long n, const Key *__restrict__ in, Key mask, Key *out) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = in[i] & mask;
}
template <typename Key>
__global__ void k_level_starts(long long n, const Key *__restrict__ keys, int shift,
                               long long *starts) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int l = (int)klo64(keys[i] >> shift);
  if (i == 0 || (int)klo64(keys[i - 1] >> shift) != l) starts[l] = i;
}

// Children-0 of the parent's neighbours of family q (level L >= 2).
template <bool WRITE, typename Key>
__device__ __forceinline__ unsigned gen_family(const ConnDev &c, PosKey<Key> P,
                                               const Oct &q, int corner, Key *out) {
  unsigned cnt = 0;
  Oct p = parent_of(q);
  int32_t bs = 2 * side_of(p.level);  // side of the generated family's box
  auto emit = [&](const Oct &r) {
    if (WRITE) out[cnt] = P.make(r.block, r.x, r.y, r.z);
    cnt++;
  };
  for (int f = 0; f < 6; f++) {
    Oct r = sibling(face_nbr(p, f), 0);
    if (in_tree(r))
      emit(r);
    else
      for_images(c, r, bs, false, emit);
  }
  for (int e = 0; e < 12; e++) {
    Oct r = sibling(edge_nbr(p, e), 0);
    if (in_tree(r))
      emit(r);
    else
      for_images(c, r, bs, false, emit);
  }
  if (corner) {
    for (int k = 0; k < 8; k++) {
      Oct r = sibling(corner_nbr(p, k), 0);
      if (in_tree(r))
        emit(r);
      else
        for_images(c, r, bs, true, emit);
    }
  }
  return cnt;
}

// n bounds the families; *m (device) is their number, so the count of the
// families need not be read back first (entries past it count 0).
template <typename Key>
__global__ void k_gen_count(long long n, const unsigned *__restrict__ m, ConnDev c,
                            PosKey<Key> P, int level, int corner, const Key *__restrict__ cur,
                            unsigned *cnt) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (i >= (long long)*m) {
    cnt[i] = 0;
    return;
  }
  Oct q = P.decode(cur[i], level);
  cnt[i] = gen_family<false, Key>(c, P, q, corner, nullptr);
}
template <typename Key>
__global__ void k_gen_write(long long n, const unsigned *__restrict__ m, ConnDev c,
                            PosKey<Key> P, int level, int corner, const Key *__restrict__ cur,
                            const unsigned *__restrict__ offs, Key *out) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || i >= (long long)*m) return;
  Oct q = P.decode(cur[i], level);
  gen_family<true, Key>(c, P, q, corner, out + offs[i]);
}

// Leaves of level L: siblings of each family in S_L whose anchor does not
// hold a finer family (or the root itself at level 0).
template <typename Key>
__global__ void k_leaves(long long n, PosKey<Key> P, OctKeyT<Key> K, int level,
                         const Key *__restrict__ cur, const Key *__restrict__ finer,
                         long long nfiner, Key *out, unsigned long long *counter) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  Key mine[8];
  int m = 0;
  if (i < n) {
    Oct q = P.decode(cur[i], level);
    int ns = (level == 0) ? 1 : 8;
    for (int j = 0; j < ns; j++) {
      Oct sb = (level == 0) ? q : sibling(q, j);
      const Key pk = P.make(sb.block, sb.x, sb.y, sb.z);
      if (!contains_key(finer, nfiner, pk))
        mine[m++] = K.make(sb.block, sb.x, sb.y, sb.z, level);
    }
  }
  // warp-aggregated append
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
__global__ void k_decode_octs(long long n, OctKeyT<Key> K, const Key *__restrict__ keys,
                              int *blk,
                              int *xs, int *ys, int *zs, int16_t *lev,
                              int16_t *info) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  Oct q = K.decode(keys[i]);
  blk[i] = q.block;
  xs[i] = q.x;
  ys[i] = q.y;
  zs[i] = q.z;
  lev[i] = (int16_t)q.level;
  info[i] = 0;
}

// Sort `keys` (n entries, nbits) and keep one of each value (masked).
template <typename Key>
static long long sort_unique(DBuf<Key> &keys, long long n, int nbits, Key mask, DBuf<Key> &out,
                             cudaStream_t s) {
  if (n == 0) {
    out.release();
    return 0;
  }
  sort_keys(keys, nullptr, n, nbits, s);
  DBuf<unsigned> pos(n + 1, s);
  launch(k_unique_flags<Key>, blocks_for(n, 256), 256, 0, s, n, (const Key *)keys.p, pos.p);
  exclusive_scan<unsigned>(pos.p, pos.p, n, s);
  long long m = read_scalar(pos.p + n, s);
  out.alloc(m, s);
  launch(k_unique_emit<Key>, blocks_for(n, 256), 256, 0, s, n, (const Key *)keys.p,
         (const unsigned *)pos.p, mask, out.p);
  return m;
}

template <typename Key>
static void balance_impl(Forest &f, int corner, const OctKeyT<Key> K) {
  const long long n = f.n;
  cudaStream_t s = f.s;
  PosKey<Key> P{K.W, K.bb};
  const int pbits = K.bb + 3 * K.W;
  const Key pmask = kmask<Key>(pbits);
  const Key all = kmask<Key>(8 * (int)sizeof(Key));
  ConnDev c = f.conn->dev;

  // Seeds, unique, grouped by level.
  DBuf<Key> sk(n, s);
  launch(k_seed_keys<Key>, blocks_for(n, 256), 256, 0, s, n, P, (const int *)f.block.p,
         (const int *)f.x.p, (const int *)f.y.p, (const int *)f.z.p,
         (const int16_t *)f.level.p, sk.p);
  DBuf<Key> seeds;
  long long ns = sort_unique<Key>(sk, n, pbits + 5, all, seeds, s);
  sk.release();
  DBuf<long long> starts(TMRG_MAX_LEVEL + 2, s);
  starts.fill_bytes(0xff);
  launch(k_level_starts<Key>, blocks_for(ns, 256), 256, 0, s, ns, (const Key *)seeds.p, pbits,
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

  // Fixed point, finest level first.
  std::vector<DBuf<Key>> S(L + 2);
  std::vector<long long> Sn(L + 2, 0);
  DBuf<Key> gen;
  long long ngen = 0;
  // One wait per level: the level's distinct families stay counted on the
  // device (S[l] sized by the level's input), the next level's generated
  // families are counted over that bound, and both counts come back
  // together.
  for (int l = L; l >= 0; l--) {
    long long nseed = hi[l] - lo[l];
    long long tot = nseed + ngen;
    DBuf<unsigned> upos;  // unique positions; upos[tot] = Sn[l]
    if (tot > 0) {
      DBuf<Key> cat(tot, s);
      if (nseed)
        launch(k_mask_copy<Key>, blocks_for(nseed, 256), 256, 0, s, nseed,
               (const Key *)(seeds.p + lo[l]), pmask, cat.p);
      if (ngen)
        TMRG_CUDA(cudaMemcpyAsync(cat.p + nseed, gen.p, ngen * sizeof(Key),
                                  cudaMemcpyDeviceToDevice, s));
      sort_keys(cat, nullptr, tot, pbits, s);
      upos.alloc(tot + 1, s);
      launch(k_unique_flags<Key>, blocks_for(tot, 256), 256, 0, s, tot, (const Key *)cat.p,
             upos.p);
      exclusive_scan<unsigned>(upos.p, upos.p, tot, s);
      S[l].alloc(tot, s);
      launch(k_unique_emit<Key>, blocks_for(tot, 256), 256, 0, s, tot, (const Key *)cat.p,
             (const unsigned *)upos.p, all, S[l].p);
    }
    gen.release();
    ngen = 0;
    Sn[l] = 0;
    if (tot == 0) continue;
    if (l >= 2) {
      DBuf<unsigned> cnt(tot + 1, s);
      launch(k_gen_count<Key>, blocks_for(tot, 128), 128, 0, s, tot,
             (const unsigned *)upos.p + tot, c, P, l, corner, (const Key *)S[l].p, cnt.p);
      exclusive_scan<unsigned>(cnt.p, cnt.p, tot, s);
      const unsigned *dv[2] = {upos.p + tot, cnt.p + tot};
      unsigned hv[2];
      read_scalars(dv, hv, s);
      Sn[l] = hv[0];
      ngen = hv[1];
      gen.alloc(ngen, s);
      launch(k_gen_write<Key>, blocks_for(tot, 128), 128, 0, s, tot,
             (const unsigned *)upos.p + tot, c, P, l, corner, (const Key *)S[l].p,
             (const unsigned *)cnt.p, gen.p);
    } else {
      Sn[l] = read_scalar(upos.p + tot, s);
    }
  }
  seeds.release();

  // Leaves of every level, then one sort into element order.
  long long cap = 0;
  for (int l = 0; l <= L; l++) cap += (l == 0 ? 1 : 8) * Sn[l];
  DBuf<Key> leaves(cap, s);
  DBuf<unsigned long long> counter(1, s);
  counter.zero();
  for (int l = 0; l <= L; l++) {
    if (!Sn[l]) continue;
    launch(k_leaves<Key>, blocks_for(Sn[l], 256), 256, 0, s, Sn[l], P, K, l,
           (const Key *)S[l].p, (const Key *)S[l + 1].p, Sn[l + 1], leaves.p, counter.p);
  }
  long long m = (long long)read_scalar(counter.p, s);
  S.clear();
  sort_keys(leaves, nullptr, m, K.total_bits(), s);
  alloc_octs(f, m);
  launch(k_decode_octs<Key>, blocks_for(m, 256), 256, 0, s, m, K, (const Key *)leaves.p,
         f.block.p, f.x.p, f.y.p, f.z.p, f.level.p, f.info.p);
}

void forest_balance(Forest &f, int corner) {
  Stage stage("tmrg_balance");
  if (!f.have_octs)
    throw Error(TMRG_ERR_STATE,
                "Cannot call balance(), no octants have been created");
  f.free_nodes();
  if (f.n == 0) return;
  const OctKey K = f.oct_key();
  if (K.total_bits() > 64)
    balance_impl<U128>(f, corner, key_as<U128>(K));
  else
    balance_impl<uint64_t>(f, corner, K);
}

// ---------------------------------------------------------------------
__global__ void k_random_refinement(uint64_t seed, uint64_t stream, double prob,
                                    int *out, long long n) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  out[i] = (seeded_uniform(seed, stream, (uint64_t)i) < prob) ? 1 : 0;
}

// ---------------------------------------------------------------------
// createRandomTrees (TMROctForest.cpp:1838-1917): nrand octants per block
// at a random level in [min_level, max_level] and a random anchor of that
// level, sorted, and made unique on position keeping the finest (the
// reference's TMROctantArray::sort).  The reference draws from libc rand();
// here octant i of block b draws U(seed, b, 4i + k), k = 0..3.
template <typename Key>
__global__ void k_random_octs(long long total, int nrand, int min_level, int max_level,
                              uint64_t seed, OctKeyT<Key> K, Key *keys) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= total) return;
  const unsigned tu = (unsigned)t;  // total < 2^32
  const int b = (int)(tu / (unsigned)nrand), i = (int)(tu - (unsigned)b * (unsigned)nrand);
  const uint64_t base = 4ULL * (uint64_t)i;
  int level = min_level + (int)(seeded_uniform(seed, b, base) * (max_level - min_level + 1));
  if (level > max_level) level = max_level;
  const int32_t h = side_of(level);
  const double cells = (double)(1 << level);
  int32_t c[3];
  for (int k = 0; k < 3; k++) {
    int32_t q = (int32_t)(seeded_uniform(seed, b, base + 1 + k) * cells);
    if (q >= (1 << level)) q = (1 << level) - 1;
    c[k] = h * q;
  }
  keys[t] = K.make(b, c[0], c[1], c[2], level);
}

template <typename Key>
static void random_sort_compact(Forest &f, long long total, int nrand, int min_level,
                                int max_level, uint64_t seed, const OctKeyT<Key> &K) {
  cudaStream_t s = f.s;
  DBuf<Key> keys(total, s);
  launch(k_random_octs<Key>, blocks_for(total, 256), 256, 0, s, total, nrand, min_level,
         max_level, seed, K, keys.p);
  sort_keys(keys, nullptr, total, K.total_bits(), s);
  DBuf<unsigned> pos(total + 1, s);
  launch(k_dedupe_flags<Key>, blocks_for(total, 256), 256, 0, s, total, (const Key *)keys.p,
         pos.p);
  exclusive_scan<unsigned>(pos.p, pos.p, total, s);
  const unsigned m = total ? read_scalar(pos.p + total, s) : 0u;
  alloc_octs(f, m);
  launch(k_compact_octs<Key>, blocks_for(total, 256), 256, 0, s, total, K, (const Key *)keys.p,
         (const uint32_t *)nullptr, (const unsigned *)pos.p, (const int16_t *)nullptr,
         f.block.p, f.x.p, f.y.p, f.z.p, f.level.p, f.info.p);
}

void forest_create_random_trees(Forest &f, int nrand, int min_level, int max_level,
                                uint64_t seed) {
  Stage st("tmrg_create_random_trees");
  if (!f.conn) throw Error(TMRG_ERR_STATE, "createRandomTrees: no connectivity");
  if (nrand < 0) throw Error(TMRG_ERR_ARG, "createRandomTrees: nrand < 0");
  if (min_level < 0) min_level = 0;
  if (max_level >= TMRG_MAX_LEVEL) max_level = TMRG_MAX_LEVEL - 1;
  if (min_level > max_level) min_level = max_level;
  f.free_nodes();
  cudaStream_t s = f.s;
  const long long total = (long long)f.conn->nb * nrand;
  if (total >= (1LL << 32)) throw Error(TMRG_ERR_ARG, "createRandomTrees: too many octants");
  f.maxlev = max_level;
  const OctKey K = f.oct_key();
  if (K.total_bits() > 64)
    random_sort_compact<U128>(f, total, nrand, min_level, max_level, seed, key_as<U128>(K));
  else
    random_sort_compact<uint64_t>(f, total, nrand, min_level, max_level, seed, K);
  f.have_octs = true;
  TMRG_CUDA(cudaStreamSynchronize(s));
}

// ---------------------------------------------------------------------
// transformNode (TMROctForest.cpp:3847-4039) on a batch of nodes in place:
// block, x, y, z of each node become those of its owner frame; edge_dir
// as in the reference; optional per-node edge reversal and face id.
__global__ void k_transform_nodes(long long n, ConnDev c, tmrg_octant *o, int edge_dir,
                                  int *rev, int *fid) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  tmrg_octant q = o[i];
  int32_t b = q.block, x = q.x, y = q.y, z = q.z;
  int r = 0, id = 0;
  transform_node(c, b, x, y, z, edge_dir, rev ? &r : nullptr, fid ? &id : nullptr);
  q.block = b;
  q.x = x;
  q.y = y;
  q.z = z;
  o[i] = q;
  if (rev) rev[i] = r;
  if (fid) fid[i] = id;
}

void forest_transform_nodes(Forest &f, tmrg_octant *d_octs, long long n, int edge_dir,
                            int *d_rev, int *d_fid) {
  if (!f.conn) throw Error(TMRG_ERR_STATE, "transformNode: no connectivity");
  launch(k_transform_nodes, blocks_for(n, 256), 256, 0, f.s, n, f.conn->dev, d_octs,
         edge_dir, d_rev, d_fid);
}

// Refinement indicator of the large adaptive workload: the sum of K
// Gaussian bumps at the octant centre (physical position through the
// per-block boxes) gives +1 above t_refine (below max_level), -1 below
// t_coarsen (above min_level), 0 otherwise.
__global__ void k_bump_indicator(long long n, const int *__restrict__ blk,
                                 const int *__restrict__ xs, const int *__restrict__ ys,
                                 const int *__restrict__ zs, const int16_t *__restrict__ lev,
                                 const double *__restrict__ boxes,
                                 const double *__restrict__ centres, int K, double sx,
                                 double sy, double sz, double t_refine, double t_coarsen,
                                 int min_level, int max_level, int *out) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double *bx = boxes + 6 * (long long)blk[i];
  const int l = lev[i];
  const double half = 0.5 * (double)side_of(l);
  const double sc = 1.0 / (double)(1 << TMRG_MAX_LEVEL);
  const double px = bx[0] + bx[3] * (((double)xs[i] + half) * sc);
  const double py = bx[1] + bx[4] * (((double)ys[i] + half) * sc);
  const double pz = bx[2] + bx[5] * (((double)zs[i] + half) * sc);
  double v = 0.0;
  for (int k = 0; k < K; k++) {
    const double dx = (px - centres[3 * k]) / sx, dy = (py - centres[3 * k + 1]) / sy,
                 dz = (pz - centres[3 * k + 2]) / sz;
    v += exp(-0.5 * (dx * dx + dy * dy + dz * dz));
  }
  out[i] = (v > t_refine && l < max_level) ? 1 : ((v < t_coarsen && l > min_level) ? -1 : 0);
}

void bump_indicator(Forest &f, const double *d_centres, int K, const double sigma[3],
                    double t_refine, double t_coarsen, int min_level, int max_level,
                    int *d_out) {
  if (!f.have_octs) throw Error(TMRG_ERR_STATE, "bump indicator: no octants");
  if (f.conn->boxes.empty()) throw Error(TMRG_ERR_STATE, "bump indicator: no block boxes");
  launch(k_bump_indicator, blocks_for(f.n, 256), 256, 0, f.s, f.n, (const int *)f.block.p,
         (const int *)f.x.p, (const int *)f.y.p, (const int *)f.z.p,
         (const int16_t *)f.level.p, (const double *)f.conn->d_boxes.p, d_centres, K,
         sigma[0], sigma[1], sigma[2], t_refine, t_coarsen, min_level, max_level, d_out);
}

// Batched forests (several independent forests as one forest over the
// disjoint union of their blocks): the first octant of each forest, and a
// per-forest seeded refinement array in which octant j of forest k draws
// U(seed, k * 1024 + pass, j) < prob[k] (zero for inactive forests), the
// same draws the forest alone gets from random_refinement.
__global__ void k_forest_starts(int nforests, const int *__restrict__ first_block,
                                long long n, const int *__restrict__ blk,
                                long long *start) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k > nforests) return;
  const int b = first_block[k];
  long long lo = 0, hi = n;
  while (lo < hi) {
    long long mid = (lo + hi) >> 1;
    if (blk[mid] < b)
      lo = mid + 1;
    else
      hi = mid;
  }
  start[k] = lo;
}
__global__ void k_batch_refinement(long long n, const int *__restrict__ blk,
                                   const int *__restrict__ block_forest,
                                   const long long *__restrict__ start,
                                   const double *__restrict__ prob,
                                   const int *__restrict__ active, uint64_t seed,
                                   uint64_t pass, int *out) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int k = block_forest[blk[i]];
  const uint64_t j = (uint64_t)(i - start[k]);
  out[i] = (active[k] && seeded_uniform(seed, (uint64_t)k * 1024 + pass, j) < prob[k]) ? 1 : 0;
}

void batch_refinement(Forest &f, int nforests, const int *d_first_block,
                      const int *d_block_forest, const double *d_prob, const int *d_active,
                      uint64_t seed, uint64_t pass, long long *d_start, int *d_out) {
  if (!f.have_octs) throw Error(TMRG_ERR_STATE, "batch refinement: no octants");
  launch(k_forest_starts, blocks_for(nforests + 1, 128), 128, 0, f.s, nforests, d_first_block,
         f.n, (const int *)f.block.p, d_start);
  launch(k_batch_refinement, blocks_for(f.n, 256), 256, 0, f.s, f.n, (const int *)f.block.p,
         d_block_forest, (const long long *)d_start, d_prob, d_active, seed, pass, d_out);
}

void random_refinement(uint64_t seed, uint64_t stream, double prob, int *out,
                       long long n, cudaStream_t s) {
  launch(k_random_refinement, blocks_for(n, 256), 256, 0, s, seed, stream, prob,
         out, n);
}

}  // namespace tmrg
