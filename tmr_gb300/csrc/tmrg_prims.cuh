// Device memory, launch accounting and the data-parallel primitives the
// octree kernels are built from: exclusive scan and a stable LSD radix
// sort of 64-bit keys with 32-bit payloads.  Header-only templates.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <nvtx3/nvToolsExt.h>

#include <algorithm>
#include <atomic>
#include <functional>
#include <utility>

#include "tmrg_common.cuh"

namespace tmrg {

// NVTX range for a pipeline stage (visible to ncu --nvtx and profilers;
// a no-op when no tool is attached).
struct Stage {
  explicit Stage(const char *name) { nvtxRangePushA(name); }
  ~Stage() { nvtxRangePop(); }
};

extern std::atomic<long long> g_kernel_launches;
// device-to-host reads that wait for the stream (read_scalar)
extern std::atomic<long long> g_host_syncs;
// Device allocations made through DBuf (the library's only device allocator).
extern std::atomic<long long> g_device_allocs;

// Optional per-kernel timing (tmrg_profile_begin/end): CUDA events recorded
// on the launching stream around each launch, with the launch's
// algorithmic byte count when the launch site states one.
extern std::atomic<bool> g_profile_on;
extern thread_local long long g_prof_bytes;
extern thread_local long long g_prof_flops;
cudaEvent_t prof_event();
void prof_push(const char *name, cudaEvent_t a, cudaEvent_t b, long long bytes,
               long long flops);
inline void prof_bytes(long long b) { g_prof_bytes = b; }
inline void prof_flops(long long f) { g_prof_flops = f; }

// Launch a kernel on `s`, count it and check the launch.  Use through the
// `launch(kernel, grid, block, smem, stream, args...)` macro.
template <typename... KArgs, typename... Args>
inline void launch_impl(const char *name, void (*k)(KArgs...), dim3 grid,
                        dim3 block, size_t smem, cudaStream_t s,
                        Args &&...args) {
  long long bytes = g_prof_bytes, flops = g_prof_flops;
  g_prof_bytes = 0;
  g_prof_flops = 0;
  if (grid.x == 0 || grid.y == 0 || grid.z == 0) return;
  const bool prof = g_profile_on.load(std::memory_order_relaxed);
  cudaEvent_t a = nullptr;
  if (prof) {
    a = prof_event();
    TMRG_CUDA(cudaEventRecord(a, s));
  }
  k<<<grid, block, smem, s>>>(std::forward<Args>(args)...);
  g_kernel_launches.fetch_add(1, std::memory_order_relaxed);
  TMRG_CHECK_LAUNCH();
  if (prof) {
    cudaEvent_t b = prof_event();
    TMRG_CUDA(cudaEventRecord(b, s));
    prof_push(name, a, b, bytes, flops);
  }
}
#define launch(k, ...) ::tmrg::launch_impl(#k, k, __VA_ARGS__)

inline unsigned blocks_for(long long n, int per_block) {
  long long b = (n + per_block - 1) / per_block;
  return (unsigned)(b > 0 ? b : 0);
}

// Stream-ordered device buffer (cudaMallocAsync / cudaFreeAsync).
template <typename T>
struct DBuf {
  T *p = nullptr;
  size_t n = 0;
  cudaStream_t s = 0;
  DBuf() {}
  DBuf(size_t count, cudaStream_t st) { alloc(count, st); }
  DBuf(const DBuf &) = delete;
  DBuf &operator=(const DBuf &) = delete;
  DBuf(DBuf &&o) noexcept : p(o.p), n(o.n), s(o.s) {
    o.p = nullptr;
    o.n = 0;
  }
  DBuf &operator=(DBuf &&o) noexcept {
    if (this != &o) {
      release();
      p = o.p;
      n = o.n;
      s = o.s;
      o.p = nullptr;
      o.n = 0;
    }
    return *this;
  }
  ~DBuf() { release(); }
  void alloc(size_t count, cudaStream_t st) {
    release();
    s = st;
    n = count;
    if (count) {
      g_device_allocs.fetch_add(1, std::memory_order_relaxed);
      cudaError_t e = cudaMallocAsync((void **)&p, count * sizeof(T), s);
      if (e != cudaSuccess) {
        p = nullptr;
        n = 0;
        cudaGetLastError();
        throw Error(TMRG_ERR_NOMEM, std::string("device allocation of ") +
                                        std::to_string(count * sizeof(T)) +
                                        " bytes failed");
      }
    }
  }
  void release() {
    if (p) cudaFreeAsync(p, s);
    p = nullptr;
    n = 0;
  }
  void zero() {
    if (n) TMRG_CUDA(cudaMemsetAsync(p, 0, n * sizeof(T), s));
  }
  void fill_bytes(int v) {
    if (n) TMRG_CUDA(cudaMemsetAsync(p, v, n * sizeof(T), s));
  }
  T *get() const { return p; }
  void swap(DBuf &o) {
    std::swap(p, o.p);
    std::swap(n, o.n);
    std::swap(s, o.s);
  }
};

// Several device scalars after one wait for the stream.
template <typename T, int K>
inline void read_scalars(const T *const (&d)[K], T (&h)[K], cudaStream_t s) {
  g_host_syncs.fetch_add(1, std::memory_order_relaxed);
  for (int k = 0; k < K; k++)
    TMRG_CUDA(cudaMemcpyAsync(&h[k], d[k], sizeof(T), cudaMemcpyDeviceToHost, s));
  TMRG_CUDA(cudaStreamSynchronize(s));
}

template <typename T>
inline T read_scalar(const T *d, cudaStream_t s) {
  T v;
  g_host_syncs.fetch_add(1, std::memory_order_relaxed);
  TMRG_CUDA(cudaMemcpyAsync(&v, d, sizeof(T), cudaMemcpyDeviceToHost, s));
  TMRG_CUDA(cudaStreamSynchronize(s));
  return v;
}

// ---------------------------------------------------------------------
// Exclusive scan: out[i] = sum(in[0..i-1]) for i <= n (out has n+1
// entries; out[n] is the total).  Tiles of 2048 items, reduce-then-scan.
constexpr int SCAN_THREADS = 256;
constexpr int SCAN_ITEMS = 8;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;

template <typename T>
__device__ __forceinline__ T block_exclusive_scan(T v, T *warp_tot, T &total) {
  int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  T x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    T y = __shfl_up_sync(0xffffffff, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_tot[warp] = x;
  __syncthreads();
  if (warp == 0) {
    T w = (lane < SCAN_THREADS / 32) ? warp_tot[lane] : T(0);
    T ws = w;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      T y = __shfl_up_sync(0xffffffff, ws, o);
      if (lane >= o) ws += y;
    }
    if (lane < SCAN_THREADS / 32) warp_tot[lane] = ws - w;
    if (lane == SCAN_THREADS / 32 - 1) warp_tot[SCAN_THREADS / 32] = ws;
  }
  __syncthreads();
  T r = x - v + warp_tot[warp];
  total = warp_tot[SCAN_THREADS / 32];
  __syncthreads();
  return r;
}

template <typename T>
__global__ void __launch_bounds__(SCAN_THREADS)
    k_scan_reduce(const T *__restrict__ in, long long n, T *__restrict__ sums) {
  __shared__ T red[SCAN_THREADS / 32];
  long long base = (long long)blockIdx.x * SCAN_TILE;
  T s = 0;
  for (int i = threadIdx.x; i < SCAN_TILE; i += SCAN_THREADS) {
    long long idx = base + i;
    if (idx < n) s += in[idx];
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffff, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    T t = 0;
    for (int w = 0; w < SCAN_THREADS / 32; w++) t += red[w];
    sums[blockIdx.x] = t;
  }
}

template <typename T>
__global__ void __launch_bounds__(SCAN_THREADS)
    k_scan_down(const T *in, T *out, long long n, const T *__restrict__ offs) {
  __shared__ T tile[SCAN_TILE];
  __shared__ T warp_tot[SCAN_THREADS / 32 + 1];
  long long base = (long long)blockIdx.x * SCAN_TILE;
  for (int i = threadIdx.x; i < SCAN_TILE; i += SCAN_THREADS) {
    long long idx = base + i;
    tile[i] = (idx < n) ? in[idx] : T(0);
  }
  __syncthreads();
  T loc[SCAN_ITEMS];
  T ts = 0;
#pragma unroll
  for (int j = 0; j < SCAN_ITEMS; j++) {
    loc[j] = tile[threadIdx.x * SCAN_ITEMS + j];
    ts += loc[j];
  }
  T total;
  T pre = block_exclusive_scan<T>(ts, warp_tot, total);
  T off = offs ? offs[blockIdx.x] : T(0);
  pre += off;
#pragma unroll
  for (int j = 0; j < SCAN_ITEMS; j++) {
    tile[threadIdx.x * SCAN_ITEMS + j] = pre;
    pre += loc[j];
  }
  __syncthreads();
  for (int i = threadIdx.x; i < SCAN_TILE; i += SCAN_THREADS) {
    long long idx = base + i;
    if (idx < n) out[idx] = tile[i];
  }
  if (threadIdx.x == 0 && base + SCAN_TILE >= n) out[n] = off + total;
}

// out must hold n+1 elements; `in` may alias `out`.
template <typename T>
void exclusive_scan(const T *in, T *out, long long n, cudaStream_t s) {
  if (n <= 0) {
    TMRG_CUDA(cudaMemsetAsync(out, 0, sizeof(T), s));
    return;
  }
  unsigned nb = blocks_for(n, SCAN_TILE);
  if (nb == 1) {
    launch(k_scan_down<T>, 1, SCAN_THREADS, 0, s, in, out, n, (const T *)nullptr);
    return;
  }
  DBuf<T> sums(nb + 1, s);
  launch(k_scan_reduce<T>, nb, SCAN_THREADS, 0, s, in, n, sums.p);
  exclusive_scan<T>(sums.p, sums.p, (long long)nb, s);
  launch(k_scan_down<T>, nb, SCAN_THREADS, 0, s, in, out, n,
         (const T *)sums.p);
}

// ---------------------------------------------------------------------
// Stable LSD radix sort, 8-bit digits.  Tiles of 4096 keys: 8 warps, each
// owning a contiguous run of 512 keys read lane-striped.  Ranks inside a
// warp come from __match_any_sync peer groups in key order, across warps
// from a per-digit prefix in shared memory, across tiles from a
// digit-major scan of the tile histograms.
constexpr int RS_THREADS = 512;
constexpr int RS_WARPS = RS_THREADS / 32;
constexpr int RS_ITEMS = 8;
constexpr int RS_TILE = RS_THREADS * RS_ITEMS;

template <typename K>
__global__ void __launch_bounds__(RS_THREADS)
    k_radix_hist(const K *__restrict__ kin, long long n, int shift,
                 uint32_t *__restrict__ hist, unsigned nblocks) {
  __shared__ uint32_t wh[RS_WARPS][256];
  for (int i = threadIdx.x; i < RS_WARPS * 256; i += RS_THREADS) (&wh[0][0])[i] = 0;
  __syncthreads();
  int warp = threadIdx.x >> 5;
  long long base = (long long)blockIdx.x * RS_TILE;
  for (int i = threadIdx.x; i < RS_TILE; i += RS_THREADS) {
    long long idx = base + i;
    if (idx < n) atomicAdd(&wh[warp][(uint32_t)(kin[idx] >> shift) & 0xFFu], 1u);
  }
  __syncthreads();
  for (int d = threadIdx.x; d < 256; d += RS_THREADS) {
    uint32_t t = 0;
    for (int w = 0; w < RS_WARPS; w++) t += wh[w][d];
    hist[(size_t)d * nblocks + blockIdx.x] = t;
  }
}

// Per digit (one block each): the exclusive scan of its row of tile counts
// in place (the tile's offset inside the digit's run) and the digit's
// total.  One launch per pass instead of a multi-level scan of the whole
// digit-major table.
constexpr int RS_SCAN_THREADS = 1024;
static __global__ void __launch_bounds__(RS_SCAN_THREADS)
    k_radix_scan_digits(uint32_t *__restrict__ hist, unsigned nblocks,
                        uint32_t *__restrict__ dtot) {
  __shared__ uint32_t wsum[RS_SCAN_THREADS / 32];
  uint32_t *row = hist + (size_t)blockIdx.x * nblocks;
  const unsigned per = (nblocks + RS_SCAN_THREADS - 1) / RS_SCAN_THREADS;
  const unsigned a = threadIdx.x * per, b = min(nblocks, a + per);
  uint32_t sum = 0;
  for (unsigned i = a; i < b; i++) sum += row[i];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t incl = sum;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += y;
  }
  if (lane == 31) wsum[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    uint32_t w = wsum[lane];
    uint32_t wi = w;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, wi, o);
      if (lane >= o) wi += y;
    }
    wsum[lane] = wi - w;
    if (lane == 31) dtot[blockIdx.x] = wi;
  }
  __syncthreads();
  uint32_t run = wsum[warp] + incl - sum;
  for (unsigned i = a; i < b; i++) {
    const uint32_t c = row[i];
    row[i] = run;
    run += c;
  }
}

// One tile of RS_TILE keys per block of THREADS threads, RS_TILE / THREADS
// keys per lane, at least MINB blocks per SM (the launch shapes the
// autotuner picks from: 512 x 8 keys at 2 or 3 blocks, 1024 x 4 keys at 2).
// Ranks inside the tile come from __match_any_sync per warp-row and
// per-warp digit counters; keys (and values) are staged in tile order of
// their digit and written out as one contiguous run per digit.  K: 64-bit
// keys, or 32-bit keys where the sorted bits fit (half the key traffic of
// every pass).
template <typename K, bool VALS, int THREADS, int MINB>
__global__ void __launch_bounds__(THREADS, MINB)
    k_radix_scatter(const K *__restrict__ kin,
                    const uint32_t *__restrict__ vin, K *__restrict__ kout,
                    uint32_t *__restrict__ vout, long long n, int shift,
                    const uint32_t *__restrict__ offs, const uint32_t *__restrict__ dtot,
                    unsigned nblocks) {
  constexpr int NW = THREADS / 32, ITEMS = RS_TILE / THREADS;
  static_assert(THREADS >= 256 && RS_TILE % THREADS == 0, "scatter shape");
  __shared__ uint16_t wcnt[NW][256];
  __shared__ uint32_t tile_off[256];
  __shared__ uint32_t gbase[256];
  __shared__ uint32_t wsum[8];
  __shared__ uint32_t dsum[8];
  __shared__ K stage[RS_TILE];
  __shared__ uint8_t stage_d[RS_TILE];
  for (int i = threadIdx.x; i < NW * 256; i += THREADS) (&wcnt[0][0])[i] = 0;
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const unsigned lt = (1u << lane) - 1u;
  const long long base = (long long)blockIdx.x * RS_TILE + (long long)warp * 32 * ITEMS;
  K k[ITEMS];
  uint32_t v[ITEMS];
  uint32_t rank[ITEMS];
#pragma unroll
  for (int j = 0; j < ITEMS; j++) {
    long long idx = base + j * 32 + lane;
    k[j] = (idx < n) ? kin[idx] : K(0);
    if (VALS) v[j] = (idx < n) ? vin[idx] : 0u;
  }
#pragma unroll
  for (int j = 0; j < ITEMS; j++) {
    long long idx = base + j * 32 + lane;
    bool ok = idx < n;
    uint32_t d = ok ? ((uint32_t)(k[j] >> shift) & 0xFFu) : (256u + lane);
    unsigned peers = __match_any_sync(0xffffffffu, d);
    int leader = __ffs(peers) - 1;
    uint32_t b = 0;
    if (ok && lane == leader) {
      b = wcnt[warp][d];
      wcnt[warp][d] = (uint16_t)(b + __popc(peers));
    }
    b = __shfl_sync(0xffffffffu, b, leader);
    rank[j] = b + __popc(peers & lt);
    __syncwarp();
  }
  __syncthreads();
  // Per digit (threads 0..255): prefix over warps, then the tile's digit
  // offsets (exclusive scan over digits) and the digit's global base.
  // The digit's global base: the exclusive prefix of the digit totals.
  uint32_t run = 0, incl = 0, dt = 0, dincl = 0;
  if (threadIdx.x < 256) {
    const int d = threadIdx.x;
    for (int w = 0; w < NW; w++) {
      uint32_t c = wcnt[w][d];
      wcnt[w][d] = (uint16_t)run;
      run += c;
    }
    incl = run;
    dt = dtot[d];
    dincl = dt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
      uint32_t z = __shfl_up_sync(0xffffffffu, dincl, o);
      if (lane >= o) incl += y, dincl += z;
    }
    if (lane == 31) wsum[warp] = incl, dsum[warp] = dincl;
  }
  __syncthreads();
  if (threadIdx.x < 256) {
    uint32_t pre = 0, dpre = 0;
    for (int w = 0; w < warp; w++) pre += wsum[w], dpre += dsum[w];
    tile_off[threadIdx.x] = pre + incl - run;
    gbase[threadIdx.x] = dpre + dincl - dt + offs[(size_t)threadIdx.x * nblocks + blockIdx.x];
  }
  __syncthreads();
  const long long tile_base = (long long)blockIdx.x * RS_TILE;
  const int cnt = (int)min((long long)RS_TILE, n - tile_base);
#pragma unroll
  for (int j = 0; j < ITEMS; j++) {
    long long idx = base + j * 32 + lane;
    if (idx < n) {
      uint32_t d = (uint32_t)(k[j] >> shift) & 0xFFu;
      uint32_t tp = tile_off[d] + wcnt[warp][d] + rank[j];
      rank[j] = tp;
      stage[tp] = k[j];
      stage_d[tp] = (uint8_t)d;
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < cnt; i += THREADS) {
    uint32_t d = stage_d[i];
    kout[gbase[d] + (i - tile_off[d])] = stage[i];
  }
  if (VALS) {
    __syncthreads();
    uint32_t *vstage = reinterpret_cast<uint32_t *>(stage);
#pragma unroll
    for (int j = 0; j < ITEMS; j++) {
      long long idx = base + j * 32 + lane;
      if (idx < n) vstage[rank[j]] = v[j];
    }
    __syncthreads();
    for (int i = threadIdx.x; i < cnt; i += THREADS) {
      uint32_t d = stage_d[i];
      vout[gbase[d] + (i - tile_off[d])] = vstage[i];
    }
  }
}

// Autotuner (tmrg_tune.cu): a size class of an operation with `ncand`
// candidate shapes.  tune_run runs the operation with the class's chosen
// candidate, timing all of them the first time the class is seen on the
// device; tune_lookup returns the cached choice (or the fallback).
struct TuneKey {
  int kind, a, b, c, d;
  int fallback;
};
enum TuneKind {
  TUNE_P = 1,
  TUNE_PT = 2,
  TUNE_FILTER3_F32 = 3,
  TUNE_FILTER3_F64 = 4,
  TUNE_RADIX = 5
};
int tune_run(const TuneKey &k, int ncand, const std::function<void(int)> &run,
             cudaStream_t s);
int tune_lookup(const TuneKey &k);

template <typename K, bool VALS>
inline void radix_scatter_shape(int shape, unsigned nb, cudaStream_t s, const K *kin,
                                const uint32_t *vin, K *kout, uint32_t *vout, long long n,
                                int shift, const uint32_t *offs, const uint32_t *dtot) {
  switch (shape) {
    case 1:
      launch((k_radix_scatter<K, VALS, 512, 3>), nb, 512, 0, s, kin, vin, kout, vout, n, shift,
             offs, dtot, nb);
      break;
    case 2:
      launch((k_radix_scatter<K, VALS, 1024, 2>), nb, 1024, 0, s, kin, vin, kout, vout, n, shift,
             offs, dtot, nb);
      break;
    default:
      launch((k_radix_scatter<K, VALS, 512, 2>), nb, 512, 0, s, kin, vin, kout, vout, n, shift,
             offs, dtot, nb);
  }
}

// Sorts keys[0..n) (and vals alongside, if given) by bits [0, nbits).
// Buffers are swapped with internal scratch, so the sorted data ends in
// `keys`/`vals`.  n < 2^32.
template <typename K>
inline void radix_sort(DBuf<K> &keys, DBuf<uint32_t> *vals, long long n, int nbits,
                       cudaStream_t s) {
  static_assert(sizeof(K) == 4 || sizeof(K) == 8, "radix sort keys are 32 or 64 bits");
  if (n <= 1 || nbits <= 0) return;
  if (n >= (1LL << 32)) throw Error(TMRG_ERR_ARG, "radix sort size >= 2^32");
  if (nbits > 8 * (int)sizeof(K)) throw Error(TMRG_ERR_ARG, "radix sort: bits beyond the key");
  unsigned nb = blocks_for(n, RS_TILE);
  DBuf<K> k2(n, s);
  DBuf<uint32_t> v2;
  if (vals) v2.alloc(n, s);
  DBuf<uint32_t> hist((size_t)256 * nb + 256, s);
  uint32_t *dtot = hist.p + (size_t)256 * nb;
  constexpr long long KB = sizeof(K);
  for (int shift = 0; shift < nbits; shift += 8) {
    prof_bytes(KB * n);
    launch(k_radix_hist<K>, nb, RS_THREADS, 0, s, (const K *)keys.p, n, shift, hist.p, nb);
    prof_bytes(8LL * 256 * nb);
    launch(k_radix_scan_digits, 256, RS_SCAN_THREADS, 0, s, hist.p, nb, dtot);
    // the scatter is out of place and every shape writes the same result,
    // so the first pass of a size class times the shapes on its own data
    const TuneKey tk{TUNE_RADIX, (int)KB, vals ? 1 : 0, bits_for(n), 0, 0};
    tune_run(tk, 3, [&](int shape) {
      prof_bytes((vals ? 2 * KB + 8 : 2 * KB) * n);
      if (vals)
        radix_scatter_shape<K, true>(shape, nb, s, (const K *)keys.p, (const uint32_t *)vals->p,
                                     k2.p, v2.p, n, shift, (const uint32_t *)hist.p,
                                     (const uint32_t *)dtot);
      else
        radix_scatter_shape<K, false>(shape, nb, s, (const K *)keys.p, nullptr, k2.p, nullptr,
                                      n, shift, (const uint32_t *)hist.p,
                                      (const uint32_t *)dtot);
    }, s);
    keys.swap(k2);
    if (vals) vals->swap(v2);
  }
}

// Key sort over the two key widths: 64-bit keys go straight to the radix
// sort; 128-bit keys are sorted as two stable LSD stages (the low word,
// then the high word's remaining bits) that carry a permutation, which then
// gathers the keys and values.
inline void sort_keys(DBuf<uint64_t> &keys, DBuf<uint32_t> *vals, long long n, int nbits,
                      cudaStream_t s) {
  radix_sort(keys, vals, n, nbits, s);
}
static __global__ void k_split128(long long n, const U128 *__restrict__ k, uint64_t *lo,
                                  uint64_t *hi, uint32_t *perm) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const U128 v = k[i];
  lo[i] = v.lo;
  hi[i] = v.hi;
  perm[i] = (uint32_t)i;
}
template <typename T>
__global__ void k_gather_perm(long long n, const uint32_t *__restrict__ perm,
                              const T *__restrict__ in, T *out) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = in[perm[i]];
}
inline void sort_keys(DBuf<U128> &keys, DBuf<uint32_t> *vals, long long n, int nbits,
                      cudaStream_t s) {
  if (n <= 1 || nbits <= 0) return;
  if (n >= (1LL << 32)) throw Error(TMRG_ERR_ARG, "radix sort size >= 2^32");
  DBuf<uint64_t> lo(n, s), hi(n, s);
  DBuf<uint32_t> perm(n, s);
  launch(k_split128, blocks_for(n, 256), 256, 0, s, n, (const U128 *)keys.p, lo.p, hi.p,
         perm.p);
  radix_sort(lo, &perm, n, std::min(nbits, 64), s);
  if (nbits > 64) {
    launch(k_gather_perm<uint64_t>, blocks_for(n, 256), 256, 0, s, n,
           (const uint32_t *)perm.p, (const uint64_t *)hi.p, lo.p);
    radix_sort(lo, &perm, n, nbits - 64, s);
  }
  lo.release();
  hi.release();
  DBuf<U128> k2(n, s);
  launch(k_gather_perm<U128>, blocks_for(n, 256), 256, 0, s, n, (const uint32_t *)perm.p,
         (const U128 *)keys.p, k2.p);
  keys.swap(k2);
  if (vals) {
    DBuf<uint32_t> v2(n, s);
    launch(k_gather_perm<uint32_t>, blocks_for(n, 256), 256, 0, s, n, (const uint32_t *)perm.p,
           (const uint32_t *)vals->p, v2.p);
    vals->swap(v2);
  }
}

}  // namespace tmrg
