// Matrix density filter (TMRMatrixFilter.cpp:30-235) on the GPU.
//
// Setup: the consistent mass matrix M of the trilinear (octree) or
// bilinear (quadtree) elements of an order-2 forest, with dependent nodes
// condensed onto the independent nodes they interpolate.  Each element
// first merges its 8x8 (4x4) element
// matrix, expanded through the dependent-node weights, into a dense
// block over its distinct independent nodes; the blocks of all elements
// are then sorted by (row, column) and summed in element order.  Then
// D = M 1, Ainv = 1/(1 + r^2/D^(2/3)), B = Ainv r^2/(D^(2/3) D) (in 2-D
// Ainv = 1/(1 + r^2/D), B = Ainv r^2/(D D)) and Tinv = 1/(F~ 1).
//
// Apply: Horner's recurrence out = B.(M out) + t1 (forward) or
// out = M(B.out) + t1 (transpose), one fused CSR kernel per term over all
// `vpn` interleaved design components, so M is read once per term.
#include <mutex>
#include <string>

#include "tmrg_quad.h"
#include "tmrg_tree.cuh"

namespace tmrg {

constexpr int FMAXK = 27;  // distinct independent nodes one element touches

struct FilterCtx {
  const int *conn;
  const int *dptr, *dconn;
  const double *dw;
  double block_len;
  const int16_t *lev;
  int *err;
  int npe, dim;  // 8 and 3 (octree) or 4 and 2 (quadtree)
};

// Merged element block: distinct nodes U[0..K) in first-appearance order
// and L[u][v] summed over (a, b, p, q) in loop order.
__device__ int element_block(const FilterCtx &c, long long e, int *U,
                             double (*L)[FMAXK]) {
  const int npe = c.npe;
  const int *ec = c.conn + e * npe;
  int ni[8][4];
  double nw[8][4];
  int nc[8];
  int K = 0;
  for (int a = 0; a < npe; a++) {
    int g = ec[a];
    if (g >= 0) {
      nc[a] = 1;
      ni[a][0] = g;
      nw[a][0] = 1.0;
    } else {
      int d = -g - 1;
      int p0 = c.dptr[d], p1 = c.dptr[d + 1];
      nc[a] = p1 - p0;
      if (nc[a] > 4) {
        atomicExch(c.err, 1);
        nc[a] = 4;
      }
      for (int p = 0; p < nc[a]; p++) {
        ni[a][p] = c.dconn[p0 + p];
        nw[a][p] = c.dw[p0 + p];
      }
    }
    for (int p = 0; p < nc[a]; p++) {
      int u = 0;
      while (u < K && U[u] != ni[a][p]) u++;
      if (u == K) {
        if (K == FMAXK) {
          atomicExch(c.err, 1);
          return K;
        }
        U[K++] = ni[a][p];
      }
    }
  }
  if (!L) return K;
  for (int u = 0; u < K; u++)
    for (int v = 0; v < K; v++) L[u][v] = 0.0;
  double side = c.block_len / (double)(1 << c.lev[e]);
  double s3 = __dmul_rn(__dmul_rn(side, side), side);
  const double s2 = __dmul_rn(side, side);
  // exact mass of the linear element (corner a = i + 2j + 4k): the 1-D
  // entries s/3 and s/6 multiplied over the directions, nd of which differ
  for (int a = 0; a < npe; a++)
    for (int b = 0; b < npe; b++) {
      int nd = ((a ^ b) & 1) + (((a ^ b) >> 1) & 1) + ((a ^ b) >> 2);
      double mab = c.dim == 3 ? __ddiv_rn(s3, 27.0 * (double)(1 << nd))
                              : __ddiv_rn(s2, 9.0 * (double)(1 << nd));
      for (int p = 0; p < nc[a]; p++) {
        int u = 0;
        while (U[u] != ni[a][p]) u++;
        double t = __dmul_rn(mab, nw[a][p]);
        for (int q = 0; q < nc[b]; q++) {
          int v = 0;
          while (U[v] != ni[b][q]) v++;
          L[u][v] = __dadd_rn(L[u][v], __dmul_rn(t, nw[b][q]));
        }
      }
    }
  return K;
}

__global__ void k_fe_count(long long n, FilterCtx c, unsigned *cnt) {
  long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  int U[FMAXK];
  int K = element_block(c, e, U, nullptr);
  cnt[e] = (unsigned)(K * K);
}
__global__ void __launch_bounds__(64)
    k_fe_write(long long n, FilterCtx c, int cb, const unsigned *__restrict__ offs,
               uint64_t *keys, uint32_t *perm, double *vals) {
  long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  int U[FMAXK];
  double L[FMAXK][FMAXK];
  int K = element_block(c, e, U, L);
  unsigned o = offs[e];
  for (int u = 0; u < K; u++)
    for (int v = 0; v < K; v++) {
      keys[o] = ((uint64_t)(uint32_t)U[u] << cb) | (uint64_t)(uint32_t)U[v];
      perm[o] = o;
      vals[o] = L[u][v];
      o++;
    }
}
// Sum each run of equal (row, col) keys in element order.
__global__ void k_fe_reduce(long long E, const uint64_t *__restrict__ keys,
                            const uint32_t *__restrict__ perm,
                            const double *__restrict__ v,
                            const unsigned *__restrict__ pos, int cb,
                            int *cols, double *out, int *rowcnt) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= E || pos[i + 1] == pos[i]) return;
  uint64_t k = keys[i];
  double s = v[perm[i]];
  for (long long j = i + 1; j < E && keys[j] == k; j++) s = __dadd_rn(s, v[perm[j]]);
  unsigned o = pos[i];
  cols[o] = (int)(k & ((1ULL << cb) - 1));
  out[o] = s;
  atomicAdd(rowcnt + (k >> cb), 1);
}
__global__ void k_fe_first(long long E, const uint64_t *__restrict__ keys,
                           unsigned *flag) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < E) flag[i] = (i == 0 || keys[i] != keys[i - 1]) ? 1u : 0u;
}

// ---------------------------------------------------------------------
// Orders 3 and 4 (the quadratic and cubic Bernstein hexahedra the
// reference's matrix creator picks, TMRMatrixCreator.h:80-85): one warp per
// element.  The element's expansion list (each node, dependent nodes
// through their CSR rows) is staged in shared memory; its distinct
// independent nodes U are numbered in first-appearance order; then
//   T[a][v] = sum over entries (b, w) with node U[v] of M_e[a][b] w
// (entries in list order) and the merged block row u is
//   L[u][v] = sum over entries (a, w) with node U[u] of w T[a][v]
// (entries in list order), written as K x K (row, column, value) triplets
// that the common sort-and-sum pass adds up in element order.  M_e[a][b] =
// ((s^3 m[ia][ib]) m[ja][jb]) m[ka][kb] with m the 1-D Bernstein mass on
// [0, 1] (exact on axis-aligned cubes).  The sums run in a different
// order than the per-pair loop of the order-2 kernel; the results agree to
// rounding.
struct FGen {
  int o, npe;
  int cap;    // staged entries per warp
  int kcap;   // distinct nodes per element
  int tcols;  // columns of T in shared memory (0 in the count pass)
  double m1[4][4];
};
constexpr int FG_WARPS = 2;

// Shared-memory layout of one warp (bytes, 8-aligned).
struct FGLayout {
  size_t node, w, a, u, ord, U, ust, T, total;
};
__host__ __device__ inline FGLayout fg_layout(const FGen &g) {
  FGLayout L;
  size_t o = 0;
  auto take = [&](size_t bytes) {
    size_t r = o;
    o += (bytes + 7) & ~(size_t)7;
    return r;
  };
  L.w = take(sizeof(double) * g.cap);
  L.T = take(sizeof(double) * (size_t)g.npe * g.tcols);
  L.node = take(sizeof(int) * g.cap);
  L.U = take(sizeof(int) * g.kcap);
  L.u = take(sizeof(uint16_t) * g.cap);
  L.ord = take(sizeof(uint16_t) * g.cap);
  L.ust = take(sizeof(uint16_t) * (g.kcap + 1));
  L.a = take(g.cap);
  L.total = o;
  return L;
}

// Expansion list and distinct nodes of element e; returns K (0 with the
// error flag set when the element outgrows the stage).
__device__ int fg_stage(const FilterCtx &c, const FGen &g, long long e, unsigned char *sm,
                        const FGLayout &L) {
  const int lane = threadIdx.x & 31;
  int *s_node = (int *)(sm + L.node);
  double *s_w = (double *)(sm + L.w);
  uint8_t *s_a = (uint8_t *)(sm + L.a);
  uint16_t *s_u = (uint16_t *)(sm + L.u), *s_first = (uint16_t *)(sm + L.ord);
  int *s_U = (int *)(sm + L.U);
  const int *ec = c.conn + e * g.npe;
  int total = 0;
  for (int a0 = 0; a0 < g.npe; a0 += 32) {
    const int a = a0 + lane;
    int gv = 0, len = 0, d0 = 0;
    if (a < g.npe) {
      gv = __ldg(ec + a);
      if (gv >= 0) {
        len = 1;
      } else {
        d0 = __ldg(c.dptr - gv - 1);
        len = __ldg(c.dptr - gv) - d0;
      }
    }
    int incl = len;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += y;
    }
    const int off = total + incl - len;
    if (off + len <= g.cap) {
      for (int p = 0; p < len; p++) {
        s_node[off + p] = gv >= 0 ? gv : __ldg(c.dconn + d0 + p);
        s_w[off + p] = gv >= 0 ? 1.0 : __ldg(c.dw + d0 + p);
        s_a[off + p] = (uint8_t)a;
      }
    }
    total += __shfl_sync(0xffffffffu, incl, 31);
  }
  if (total > g.cap) {
    if (lane == 0) atomicExch(c.err, 1);
    return 0;
  }
  __syncwarp();
  // first occurrence of each entry's node
  for (int i = lane; i < total; i += 32) {
    const int nd = s_node[i];
    int j = 0;
    while (s_node[j] != nd) j++;
    s_first[i] = (uint16_t)j;
  }
  __syncwarp();
  int K = 0;
  for (int i0 = 0; i0 < total; i0 += 32) {
    const int i = i0 + lane;
    const bool first = i < total && s_first[i] == i;
    const unsigned m = __ballot_sync(0xffffffffu, first);
    if (first) {
      const int k = K + __popc(m & ((1u << lane) - 1u));
      if (k < g.kcap) s_U[k] = s_node[i];
      s_u[i] = (uint16_t)k;
    }
    K += __popc(m);
  }
  if (K > g.kcap) {
    if (lane == 0) atomicExch(c.err, 1);
    return 0;
  }
  __syncwarp();
  for (int i = lane; i < total; i += 32)
    if (s_first[i] != i) s_u[i] = s_u[s_first[i]];
  __syncwarp();
  return K | (total << 16);
}

// Largest expansion list of an element (sizes the stage).
__global__ void k_fe_gen_emax(long long ne, FilterCtx c, int npe, int *emax) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ne) return;
  const int *ec = c.conn + e * npe;
  int t = 0;
  for (int a = 0; a < npe; a++) {
    const int gv = __ldg(ec + a);
    t += gv >= 0 ? 1 : __ldg(c.dptr - gv) - __ldg(c.dptr - gv - 1);
  }
  atomicMax(emax, t);
}
// Pass 0: K^2 triplets per element (and the largest K).
__global__ void __launch_bounds__(FG_WARPS * 32)
    k_fe_gen_count(long long ne, FilterCtx c, FGen g, long long *cnt, int *kmax) {
  extern __shared__ __align__(16) unsigned char fg_smem[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const long long e = (long long)blockIdx.x * FG_WARPS + warp;
  if (e >= ne) return;
  const FGLayout L = fg_layout(g);
  const int r = fg_stage(c, g, e, fg_smem + warp * L.total, L);
  const int K = r & 0xffff;
  if (lane == 0) {
    cnt[e] = (long long)K * K;
    atomicMax(kmax, K);
  }
}
// Pass 1: the triplets at offs[e].
__global__ void __launch_bounds__(FG_WARPS * 32)
    k_fe_gen_write(long long ne, FilterCtx c, FGen g, int cb, const long long *__restrict__ offs,
                   uint64_t *keys, uint32_t *perm, double *vals) {
  extern __shared__ __align__(16) unsigned char fg_smem[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const long long e = (long long)blockIdx.x * FG_WARPS + warp;
  if (e >= ne) return;
  const FGLayout L = fg_layout(g);
  unsigned char *sm = fg_smem + warp * L.total;
  const int r = fg_stage(c, g, e, sm, L);
  const int K = r & 0xffff, total = r >> 16;
  if (K == 0) return;
  const double *s_w = (const double *)(sm + L.w);
  const uint8_t *s_a = (const uint8_t *)(sm + L.a);
  const uint16_t *s_u = (const uint16_t *)(sm + L.u);
  uint16_t *s_ord = (uint16_t *)(sm + L.ord), *s_ust = (uint16_t *)(sm + L.ust);
  const int *s_U = (const int *)(sm + L.U);
  double *T = (double *)(sm + L.T);
  const int o = g.o, npe = g.npe;
  const double side = c.block_len / (double)(1 << c.lev[e]);
  const double s3 = __dmul_rn(__dmul_rn(side, side), side);
  // T = M_e W over the K distinct nodes; lanes own rows a
  for (int a = lane; a < npe; a += 32)
    for (int v = 0; v < K; v++) T[a * K + v] = 0.0;
  for (int i = 0; i < total; i++) {
    const int b = s_a[i], v = s_u[i];
    const double wb = s_w[i];
    const int ib = b % o, jb = (b / o) % o, kb = b / (o * o);
    for (int a = lane; a < npe; a += 32) {
      const int ia = a % o, ja = (a / o) % o, ka = a / (o * o);
      const double mab =
          __dmul_rn(__dmul_rn(__dmul_rn(s3, g.m1[ia][ib]), g.m1[ja][jb]), g.m1[ka][kb]);
      T[a * K + v] = __fma_rn(mab, wb, T[a * K + v]);
    }
  }
  // entries ordered by distinct node (stable), and each node's first slot
  for (int i = lane; i < total; i += 32) {
    const int ui = s_u[i];
    int pos = 0;
    for (int j = 0; j < total; j++) {
      const int uj = s_u[j];
      pos += (uj < ui) || (uj == ui && j < i);
    }
    s_ord[pos] = (uint16_t)i;
  }
  __syncwarp();
  for (int p = lane; p < total; p += 32) {
    const int up = s_u[s_ord[p]];
    if (p == 0 || s_u[s_ord[p - 1]] != up) s_ust[up] = (uint16_t)p;
  }
  if (lane == 0) s_ust[K] = (uint16_t)total;
  __syncwarp();
  // row u of the merged block: lanes own columns v
  const long long base = offs[e];
  for (int u = 0; u < K; u++) {
    const int p0 = s_ust[u], p1 = s_ust[u + 1];
    const uint64_t rk = (uint64_t)(uint32_t)s_U[u] << cb;
    for (int v = lane; v < K; v += 32) {
      double acc = 0.0;
      for (int p = p0; p < p1; p++) {
        const int i = s_ord[p];
        acc = __fma_rn(s_w[i], T[s_a[i] * K + v], acc);
      }
      const long long q = base + (long long)u * K + v;
      keys[q] = rk | (uint64_t)(uint32_t)s_U[v];
      perm[q] = (uint32_t)q;
      vals[q] = acc;
    }
  }
}

// D, Ainv, B (TMRMatrixFilter.cpp:121-147).
__global__ void k_fe_scalings(long long n, int dim, const int *__restrict__ rp,
                              const double *__restrict__ vals, double r,
                              double *Ainv, double *B) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double D = 0.0;
  for (int p = rp[i]; p < rp[i + 1]; p++) D = __dadd_rn(D, vals[p]);
  if (D == 0.0) {
    Ainv[i] = 1.0;
    B[i] = 0.0;
  } else if (dim == 2) {
    double rr = __dmul_rn(r, r);
    double a = __ddiv_rn(1.0, __dadd_rn(1.0, __ddiv_rn(rr, D)));
    Ainv[i] = a;
    B[i] = __ddiv_rn(__dmul_rn(__dmul_rn(a, r), r), __dmul_rn(D, D));
  } else {
    double t = pow(D, 2.0 / 3.0);
    double rr = __dmul_rn(r, r);
    double a = __ddiv_rn(1.0, __dadd_rn(1.0, __ddiv_rn(rr, t)));
    Ainv[i] = a;
    B[i] = __ddiv_rn(__dmul_rn(__dmul_rn(a, r), r), __dmul_rn(t, D));
  }
}
__global__ void k_fe_tinv(long long n, const double *__restrict__ y, double *T) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) T[i] = (y[i] != 0.0) ? __ddiv_rn(1.0, y[i]) : 0.0;
}
template <typename T>
__global__ void k_to_f32(long long n, const double *__restrict__ a, T *b) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) b[i] = (T)a[i];
}

// ---------------------------------------------------------------------
__device__ __forceinline__ double fmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double fadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
// The Horner terms accumulate M x with fused multiply-adds: half the FP64
// instructions (a scarce pipe on GB300) and one rounding per term.
__device__ __forceinline__ double ffma(double a, double b, double c) { return __fma_rn(a, b, c); }
__device__ __forceinline__ float ffma(float a, float b, float c) { return __fmaf_rn(a, b, c); }

// t1 = s . in ; returns t1 (the first Horner iterate).
template <typename T>
__global__ void k_fe_scale(long long n, int vpn, const T *__restrict__ s,
                           const T *__restrict__ in, T *out) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n * vpn) return;
  out[i] = fmul(s[i / vpn], in[i]);
}

// One Horner term over all components:
//   forward:   y = B.(M x) + t1
//   transpose: y = M(B.x) + t1
// then y *= post (the final Tinv or Ainv) when post != nullptr.
// ---------------------------------------------------------------------
// Sliced-ELL copy of M (see Filter): per slice the longest row length,
// then per position its row's entries at soff[slice] + 32 k + lane (CSR
// order; the tail of a shorter row holds column = row, value 0, never
// read).
__global__ void k_sell_len(long long npos, long long n, const int *__restrict__ perm,
                           const int *__restrict__ rp, int *srl, long long *ssz) {
  const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= npos) return;
  int len = 0;
  if (p < n) {
    const int row = perm[p];
    len = rp[row + 1] - rp[row];
  }
  srl[p] = len;
  // slice length: the longest row of the 32 positions (one warp)
  int m = len;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((p & 31) == 0) ssz[p >> 5] = 32LL * m;
}
template <typename T>
__global__ void k_sell_fill(long long npos, long long n, const int *__restrict__ perm,
                            const int *__restrict__ rp, const int *__restrict__ cols,
                            const T *__restrict__ vals, const long long *__restrict__ soff,
                            int *scol, T *sval) {
  const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= npos) return;
  const long long sl = p >> 5;
  const int L = (int)((soff[sl + 1] - soff[sl]) >> 5);
  const long long base = soff[sl] + (p & 31);
  const int row = p < n ? perm[p] : 0;
  const int p0 = p < n ? rp[row] : 0, len = p < n ? rp[row + 1] - p0 : 0;
  for (int k = 0; k < L; k++) {
    scol[base + 32LL * k] = k < len ? cols[p0 + k] : row;
    sval[base + 32LL * k] = k < len ? vals[p0 + k] : T(0);
  }
}

// One Horner term on the sliced copy: thread p <-> row sperm[p], its
// entries in CSR order (the same FMA sequence as k_fe_step).
template <typename T, int VPN, bool TR>
__global__ void __launch_bounds__(256)
    k_fe_sell(long long n, int vpn_rt, const int *__restrict__ perm, const int *__restrict__ srl,
              const long long *__restrict__ soff, const int *__restrict__ scol,
              const T *__restrict__ sval, const T *__restrict__ B, const T *__restrict__ t1,
              const T *__restrict__ x, T *__restrict__ y, const T *__restrict__ post) {
  const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  const long long i = perm[p];
  const int len = srl[p];
  const long long base = soff[p >> 5] + (p & 31);
  const int vpn = VPN > 0 ? VPN : vpn_rt;
  T acc[VPN > 0 ? VPN : 4];
  for (int c0 = 0; c0 < vpn; c0 += (VPN > 0 ? VPN : 4)) {
    const int nc = (VPN > 0) ? VPN : min(4, vpn - c0);
#pragma unroll
    for (int v = 0; v < (VPN > 0 ? VPN : 4); v++) acc[v] = T(0);
#pragma unroll 4
    for (int k = 0; k < len; k++) {
      const int j = __ldg(scol + base + 32LL * k);
      const T m = __ldg(sval + base + 32LL * k);
      const T bj = TR ? __ldg(B + j) : T(1);
#pragma unroll
      for (int v = 0; v < (VPN > 0 ? VPN : 4); v++) {
        if (v < nc) {
          T xv = __ldg(x + (long long)j * vpn + c0 + v);
          if (TR) xv = fmul(bj, xv);
          acc[v] = ffma(m, xv, acc[v]);
        }
      }
    }
    const T bi = TR ? T(1) : B[i];
    const T pi = post ? post[i] : T(1);
#pragma unroll
    for (int v = 0; v < (VPN > 0 ? VPN : 4); v++) {
      if (v < nc) {
        const long long o = i * vpn + c0 + v;
        T r = TR ? fadd(acc[v], t1[o]) : fadd(fmul(bi, acc[v]), t1[o]);
        if (post) r = fmul(r, pi);
        y[o] = r;
      }
    }
  }
}

// Three components per node (the design fields of the C3 workload) are
// carried through the Horner terms padded to four: a node's values are one
// 16-byte (FP32) or two 16-byte (FP64) loads per gathered neighbour instead
// of three scalar loads.  Only the first scaling reads and only the last
// term writes the caller's 3-component layout.  Same operation sequence per
// component as k_fe_sell, so the results are the same bits.
template <typename T>
__device__ __forceinline__ void load4(const T *p, T (&v)[4]);
template <>
__device__ __forceinline__ void load4<float>(const float *p, float (&v)[4]) {
  const float4 q = __ldg((const float4 *)p);
  v[0] = q.x, v[1] = q.y, v[2] = q.z, v[3] = q.w;
}
template <>
__device__ __forceinline__ void load4<double>(const double *p, double (&v)[4]) {
  const double2 a = __ldg((const double2 *)p), b = __ldg((const double2 *)p + 1);
  v[0] = a.x, v[1] = a.y, v[2] = b.x, v[3] = b.y;
}
template <typename T>
__device__ __forceinline__ void store4(T *p, T a, T b, T c);
template <>
__device__ __forceinline__ void store4<float>(float *p, float a, float b, float c) {
  *(float4 *)p = make_float4(a, b, c, 0.0f);
}
template <>
__device__ __forceinline__ void store4<double>(double *p, double a, double b, double c) {
  ((double2 *)p)[0] = make_double2(a, b);
  ((double2 *)p)[1] = make_double2(c, 0.0);
}
// t1 (padded) = s . in (3 components)
template <typename T>
__global__ void k_fe_scale3p(long long n, const T *__restrict__ s, const T *__restrict__ in,
                             T *out) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const T si = s[i];
  store4<T>(out + 4 * i, fmul(si, in[3 * i]), fmul(si, in[3 * i + 1]),
            fmul(si, in[3 * i + 2]));
}
// One Horner term, padded input; output padded (ypad) or in the caller's
// 3-component layout (the last term).
template <typename T, bool TR>
__global__ void __launch_bounds__(256)
    k_fe_sell3p(long long n, const int *__restrict__ perm, const int *__restrict__ srl,
                const long long *__restrict__ soff, const int *__restrict__ scol,
                const T *__restrict__ sval, const T *__restrict__ B, const T *__restrict__ t1,
                const T *__restrict__ x, T *__restrict__ y, bool ypad,
                const T *__restrict__ post) {
  const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  const long long i = perm[p];
  const int len = srl[p];
  const long long base = soff[p >> 5] + (p & 31);
  T a0 = T(0), a1 = T(0), a2 = T(0);
#pragma unroll 4
  for (int k = 0; k < len; k++) {
    const int j = __ldg(scol + base + 32LL * k);
    const T m = __ldg(sval + base + 32LL * k);
    T xv[4];
    load4<T>(x + 4LL * j, xv);
    if (TR) {
      const T bj = __ldg(B + j);
      xv[0] = fmul(bj, xv[0]), xv[1] = fmul(bj, xv[1]), xv[2] = fmul(bj, xv[2]);
    }
    a0 = ffma(m, xv[0], a0);
    a1 = ffma(m, xv[1], a1);
    a2 = ffma(m, xv[2], a2);
  }
  T tv[4];
  load4<T>(t1 + 4 * i, tv);
  T r0, r1, r2;
  if (TR) {
    r0 = fadd(a0, tv[0]), r1 = fadd(a1, tv[1]), r2 = fadd(a2, tv[2]);
  } else {
    const T bi = B[i];
    r0 = fadd(fmul(bi, a0), tv[0]), r1 = fadd(fmul(bi, a1), tv[1]), r2 = fadd(fmul(bi, a2), tv[2]);
  }
  if (post) {
    const T pi = post[i];
    r0 = fmul(r0, pi), r1 = fmul(r1, pi), r2 = fmul(r2, pi);
  }
  if (ypad) {
    store4<T>(y + 4 * i, r0, r1, r2);
  } else {
    y[3 * i] = r0, y[3 * i + 1] = r1, y[3 * i + 2] = r2;
  }
}

template <typename T>
static const T *sell_vals(const Filter &F);
template <>
const double *sell_vals<double>(const Filter &F) {
  return F.sval.p;
}
template <>
const float *sell_vals<float>(const Filter &F) {
  return F.sval32.p;
}

// One Horner term (all vpn components) on the sliced copy of M.
template <typename T, bool TR>
static void launch_sell(const Filter &F, int vpn, const T *B, const T *t1, const T *x, T *y,
                        const T *post, cudaStream_t s) {
  const long long n = F.n;
  const unsigned g = blocks_for(n, 256);
  // compulsory traffic of one term: M (value + column), B, t1, one read of
  // x and one write of y (all vpn components)
  prof_bytes((long long)(sizeof(T) + 4) * F.nnz + 4 * (n + 1) + (long long)sizeof(T) * n +
             3LL * sizeof(T) * n * vpn + (post ? (long long)sizeof(T) * n : 0));
  prof_flops(2LL * vpn * F.nnz);
  const T *sv = sell_vals<T>(F);
#define TMRG_SELL(V)                                                                         \
  launch((k_fe_sell<T, V, TR>), g, 256, 0, s, n, vpn, (const int *)F.sperm.p,               \
         (const int *)F.srl.p, (const long long *)F.soff.p, (const int *)F.scol.p, sv, B, t1, \
         x, y, post)
  switch (vpn) {
    case 1: TMRG_SELL(1); break;
    case 2: TMRG_SELL(2); break;
    case 3: TMRG_SELL(3); break;
    case 4: TMRG_SELL(4); break;
    default: TMRG_SELL(0);
  }
#undef TMRG_SELL
}

// applyFilter / applyTranspose for three components per node, padded
// (k_fe_sell3p); F.N >= 1.
template <typename T>
static void horner3p(Filter &F, bool tr, const T *in, T *out, const T *Ainv, const T *B,
                     const T *Tinv) {
  cudaStream_t s = F.s;
  const long long n = F.n;
  DBuf<T> t1(4 * n, s), ta(4 * n, s), tb(4 * n, s);
  const T *pre = tr ? Tinv : Ainv;
  const T *post = tr ? Ainv : Tinv;
  prof_bytes((long long)sizeof(T) * (3 * n + 4 * n + n));
  launch(k_fe_scale3p<T>, blocks_for(n, 256), 256, 0, s, n, pre, in, t1.p);
  const T *sv = sell_vals<T>(F);
  const T *x = t1.p;
  for (int k = 0; k < F.N; k++) {
    const bool last = (k == F.N - 1);
    T *y = last ? out : ((k % 2 == 0) ? ta.p : tb.p);
    // compulsory traffic of one term: M (value + column), B, t1 and one read
    // of x (padded), one write of y (padded, or 3 components)
    prof_bytes((long long)(sizeof(T) + 4) * F.nnz + 4 * (n + 1) + (long long)sizeof(T) * n +
               (long long)sizeof(T) * n * (4 + 4 + (last ? 3 : 4)) +
               (last ? (long long)sizeof(T) * n : 0));
    prof_flops(6LL * F.nnz);
    if (tr)
      launch((k_fe_sell3p<T, true>), blocks_for(n, 256), 256, 0, s, n, (const int *)F.sperm.p,
             (const int *)F.srl.p, (const long long *)F.soff.p, (const int *)F.scol.p, sv, B,
             (const T *)t1.p, x, y, !last, last ? post : (const T *)nullptr);
    else
      launch((k_fe_sell3p<T, false>), blocks_for(n, 256), 256, 0, s, n, (const int *)F.sperm.p,
             (const int *)F.srl.p, (const long long *)F.soff.p, (const int *)F.scol.p, sv, B,
             (const T *)t1.p, x, y, !last, last ? post : (const T *)nullptr);
    x = y;
  }
}

template <typename T>
static void horner_generic(Filter &F, bool tr, int vpn, const T *in, T *out, const T *Ainv,
                           const T *B, const T *Tinv);

// applyFilter / applyTranspose (TMRMatrixFilter.cpp:191-235).
template <typename T>
static void horner(Filter &F, bool tr, int vpn, const T *in, T *out, const T *Ainv,
                   const T *B, const T *Tinv) {
  cudaStream_t s = F.s;
  const long long n = F.n;
  if (n == 0) return;
  if (vpn == 3 && F.N > 0) {
    // three components: padded (candidate 0) or sliced-ELL with three
    // scalar loads per neighbour (candidate 1), chosen by the autotuner per
    // precision and size (both give the same bits)
    int lr = 0;
    while ((1LL << (lr + 1)) <= n) lr++;
    const TuneKey key{sizeof(T) == 4 ? TUNE_FILTER3_F32 : TUNE_FILTER3_F64, lr, (int)tr, 0, 0, 0};
    auto run = [&](int c) {
      if (c == 0)
        horner3p<T>(F, tr, in, out, Ainv, B, Tinv);
      else
        horner_generic<T>(F, tr, vpn, in, out, Ainv, B, Tinv);
    };
    // tuning runs the apply several times: not on an in-place call
    if ((const void *)in == (const void *)out)
      run(tune_lookup(key));
    else
      tune_run(key, 2, run, s);
    return;
  }
  horner_generic<T>(F, tr, vpn, in, out, Ainv, B, Tinv);
}

template <typename T>
static void horner_generic(Filter &F, bool tr, int vpn, const T *in, T *out, const T *Ainv,
                           const T *B, const T *Tinv) {
  cudaStream_t s = F.s;
  long long n = F.n, len = n * vpn;
  DBuf<T> t1(len, s), tmp(len, s);
  const T *pre = tr ? Tinv : Ainv;
  const T *post = tr ? Ainv : Tinv;
  prof_bytes(2LL * sizeof(T) * len + (long long)sizeof(T) * n);
  launch(k_fe_scale<T>, blocks_for(len, 256), 256, 0, s, n, vpn, pre, in, t1.p);
  if (F.N == 0) {
    prof_bytes(2LL * sizeof(T) * len + (long long)sizeof(T) * n);
    launch(k_fe_scale<T>, blocks_for(len, 256), 256, 0, s, n, vpn, post,
           (const T *)t1.p, out);
    return;
  }
  // ping-pong so that the last term lands in `out`
  const T *x = t1.p;
  for (int k = 0; k < F.N; k++) {
    bool last = (k == F.N - 1);
    T *y = ((F.N - 1 - k) % 2 == 0) ? out : tmp.p;
    if (tr)
      launch_sell<T, true>(F, vpn, B, t1.p, x, y, last ? post : nullptr, s);
    else
      launch_sell<T, false>(F, vpn, B, t1.p, x, y, last ? post : nullptr, s);
    x = y;
  }
}

void filter_apply(Filter &F, bool tr, int vpn, const double *in, double *out) {
  Stage st(tr ? "tmrg_filter_apply_transpose" : "tmrg_filter_apply");
  horner<double>(F, tr, vpn, in, out, F.Ainv.p, F.B.p, F.Tinv.p);
}
void filter_apply_f32(Filter &F, bool tr, int vpn, const float *in, float *out) {
  horner<float>(F, tr, vpn, in, out, F.Ainv32.p, F.B32.p, F.Tinv32.p);
}

// ---------------------------------------------------------------------
// Allocation-free apply.  Some callers cannot allocate device memory at
// the point where they filter: a framework whose caching allocator owns
// the GPU's memory, or a section that must not call cudaMalloc/cudaFree
// because those can synchronise the device.  This variant takes its two
// Horner work vectors (t1 and the ping-pong term) from a static device
// array instead of the stream-ordered pool.
//
// The array holds 2 x FILTER_STATIC_MAX doubles (16 MiB) and stays
// resident on every GPU that loads the library until the process exits.
// Every call shares it and it keeps the last call's contents; nothing in
// it has to start at zero (each call writes t1 and every Horner term in
// full before reading them).  Calls that overlap on the GPU (different
// streams, or different filters sharing a device) race on the array.
constexpr long long FILTER_STATIC_MAX = 1LL << 20;
static __device__ __align__(256) double g_filter_static[2 * FILTER_STATIC_MAX];

// Device address of the array on the current device, looked up once per
// device: in host code `g_filter_static` names a host-side stand-in, not
// device memory.  The first call on a device performs the lookup, so it
// should come before any stream capture.
static double *filter_static_scratch() {
  static std::mutex mu;
  static double *addr[256] = {nullptr};
  int dev = 0;
  TMRG_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 256) throw Error(TMRG_ERR_ARG, "device ordinal out of range");
  std::lock_guard<std::mutex> lk(mu);
  if (!addr[dev]) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_filter_static);
    if (e != cudaSuccess)
      throw Error(TMRG_ERR_CUDA, std::string("cudaGetSymbolAddress(filter scratch): ") +
                                     cudaGetErrorString(e));
    addr[dev] = (double *)p;
  }
  return addr[dev];
}

void filter_apply_static(Filter &F, bool tr, int vpn, const double *in, double *out) {
  const long long n = F.n, len = n * vpn;
  if (len > FILTER_STATIC_MAX)
    throw Error(TMRG_ERR_ARG,
                "allocation-free filter apply: " + std::to_string(len) +
                    " values (nodes x vpn) exceed the static scratch limit of " +
                    std::to_string(FILTER_STATIC_MAX));
  Stage st(tr ? "tmrg_filter_apply_static_transpose" : "tmrg_filter_apply_static");
  double *t1 = filter_static_scratch();
  double *tmp = t1 + FILTER_STATIC_MAX;
  if (n == 0) return;
  cudaStream_t s = F.s;
  const double *pre = tr ? F.Tinv.p : F.Ainv.p;
  const double *post = tr ? F.Ainv.p : F.Tinv.p;
  prof_bytes(2LL * sizeof(double) * len + (long long)sizeof(double) * n);
  launch(k_fe_scale<double>, blocks_for(len, 256), 256, 0, s, n, vpn, pre, in, t1);
  if (F.N == 0) {
    prof_bytes(2LL * sizeof(double) * len + (long long)sizeof(double) * n);
    launch(k_fe_scale<double>, blocks_for(len, 256), 256, 0, s, n, vpn, post,
           (const double *)t1, out);
    return;
  }
  const double *x = t1;
  for (int k = 0; k < F.N; k++) {
    bool last = (k == F.N - 1);
    double *y = ((F.N - 1 - k) % 2 == 0) ? out : tmp;
    if (tr)
      launch_sell<double, true>(F, vpn, F.B.p, t1, x, y, last ? post : nullptr, s);
    else
      launch_sell<double, false>(F, vpn, F.B.p, t1, x, y, last ? post : nullptr, s);
    x = y;
  }
}

// What the filter needs from an octree or quadtree forest (nodes created).
struct FSource {
  cudaStream_t s;
  int order, npe, dim;
  long long ne, nn;
  const int *econn, *dptr, *dconn;
  const double *dw;
  const int16_t *level;
};
static void filter_build(const FSource &f, double len, double r, int N, Filter &F);

// 1-D Bernstein mass of degree p on [0, 1]:
// C(p, i) C(p, j) / ((2p + 1) C(2p, i + j)), one division.
static double bernstein_mass_1d(int p, int i, int j) {
  double ci = 1.0, cj = 1.0, c2 = 1.0;
  for (int k = 1; k <= i; k++) ci = ci * (p - k + 1) / k;
  for (int k = 1; k <= j; k++) cj = cj * (p - k + 1) / k;
  for (int k = 1; k <= i + j; k++) c2 = c2 * (2 * p - k + 1) / k;
  return (ci * cj) / ((2 * p + 1) * c2);
}

void filter_create(Forest &f, double len, double r, int N, Filter &F) {
  Stage st("tmrg_filter_create");
  if (f.order < 2 || f.order > 4)
    throw Error(TMRG_ERR_UNSUPPORTED,
                "matrix filter: forests of order 2-4 (the element bases the reference's "
                "matrix creator provides)");
  forest_create_nodes(f);
  filter_build(FSource{f.s, f.order, f.order * f.order * f.order, 3, f.n, f.num_owned,
                       f.econn.p, f.dep_ptr.p, f.dep_conn.p, f.dep_w.p, f.level.p},
               len, r, N, F);
}
void filter_create_quad(QForest &f, double len, double r, int N, Filter &F) {
  Stage st("tmrg_filter_create");
  if (f.order != 2)
    throw Error(TMRG_ERR_UNSUPPORTED, "matrix filter: order-2 forests only");
  qforest_create_nodes(f);
  filter_build(FSource{f.s, 2, 4, 2, f.n, f.num_owned, f.econn.p, f.dep_ptr.p, f.dep_conn.p,
                       f.dep_w.p, f.level.p},
               len, r, N, F);
}

static void filter_build(const FSource &f, double len, double r, int N, Filter &F) {
  cudaStream_t s = f.s;
  F.s = s;
  F.N = N;
  F.r = r;
  const long long n = f.nn, ne = f.ne;
  F.n = n;
  DBuf<int> err(1, s);
  err.zero();
  FilterCtx c{f.econn, f.dptr, f.dconn, f.dw, len, f.level, err.p, f.npe, f.dim};
  const int cb = bits_for(n + 1);
  if (2 * cb > 64) throw Error(TMRG_ERR_KEY_RANGE, "filter key range");
  long long E = 0;
  DBuf<uint64_t> keys;
  DBuf<uint32_t> perm;
  DBuf<double> ev;
  if (f.order == 2) {
    DBuf<unsigned> cnt(ne + 1, s);
    launch(k_fe_count, blocks_for(ne, 128), 128, 0, s, ne, c, cnt.p);
    exclusive_scan<unsigned>(cnt.p, cnt.p, ne, s);
    E = read_scalar(cnt.p + ne, s);
    keys.alloc(E, s);
    perm.alloc(E, s);
    ev.alloc(E, s);
    launch(k_fe_write, blocks_for(ne, 64), 64, 0, s, ne, c, cb,
           (const unsigned *)cnt.p, keys.p, perm.p, ev.p);
  } else {
    FGen g{};
    g.o = f.order;
    g.npe = f.npe;
    for (int i = 0; i < g.o; i++)
      for (int j = 0; j < g.o; j++) g.m1[i][j] = bernstein_mass_1d(g.o - 1, i, j);
    DBuf<int> mx(2, s);
    mx.zero();
    launch(k_fe_gen_emax, blocks_for(ne, 256), 256, 0, s, ne, c, g.npe, mx.p);
    const int emax = read_scalar(mx.p, s);
    // count pass: the list and its distinct nodes (at most the list length)
    g.cap = std::max(32, emax);
    g.kcap = g.cap;
    g.tcols = 0;
    const size_t sm_c = fg_layout(g).total * FG_WARPS;
    if (g.cap > 65535 || sm_c > 200 * 1024)
      throw Error(TMRG_ERR_UNSUPPORTED, "matrix filter: an element expands to " +
                                            std::to_string(emax) + " entries");
    DBuf<long long> cnt(ne + 1, s);
    TMRG_CUDA(cudaFuncSetAttribute(k_fe_gen_count, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)sm_c));
    launch(k_fe_gen_count, blocks_for(ne, FG_WARPS), FG_WARPS * 32, sm_c, s, ne, c, g, cnt.p,
           mx.p + 1);
    const int kmax = read_scalar(mx.p + 1, s);
    if (read_scalar(err.p, s))
      throw Error(TMRG_ERR_UNSUPPORTED, "matrix filter: an element touches too many nodes");
    exclusive_scan<long long>(cnt.p, cnt.p, ne, s);
    E = read_scalar(cnt.p + ne, s);
    if (E >= (1LL << 32))
      throw Error(TMRG_ERR_ARG, "matrix filter: more than 2^32 element-matrix entries");
    // write pass: T over the largest number of distinct nodes
    g.kcap = std::max(1, kmax);
    g.tcols = g.kcap;
    const size_t smem = fg_layout(g).total * FG_WARPS;
    if (smem > 227 * 1024)
      throw Error(TMRG_ERR_UNSUPPORTED, "matrix filter: an element touches " +
                                            std::to_string(kmax) + " independent nodes");
    keys.alloc(E, s);
    perm.alloc(E, s);
    ev.alloc(E, s);
    TMRG_CUDA(cudaFuncSetAttribute(k_fe_gen_write, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)smem));
    launch(k_fe_gen_write, blocks_for(ne, FG_WARPS), FG_WARPS * 32, smem, s, ne, c, g, cb,
           (const long long *)cnt.p, keys.p, perm.p, ev.p);
  }
  radix_sort(keys, &perm, E, 2 * cb, s);
  DBuf<unsigned> pos(E + 1, s);
  launch(k_fe_first, blocks_for(E, 256), 256, 0, s, E, (const uint64_t *)keys.p,
         pos.p);
  exclusive_scan<unsigned>(pos.p, pos.p, E, s);
  const long long nnz = read_scalar(pos.p + E, s);
  F.nnz = nnz;
  F.colidx.alloc(nnz + 1, s);
  F.vals.alloc(nnz + 1, s);
  F.rowptr.alloc(n + 1, s);
  F.rowptr.zero();
  launch(k_fe_reduce, blocks_for(E, 256), 256, 0, s, E, (const uint64_t *)keys.p,
         (const uint32_t *)perm.p, (const double *)ev.p, (const unsigned *)pos.p,
         cb, F.colidx.p, F.vals.p, F.rowptr.p);
  keys.release();
  perm.release();
  ev.release();
  pos.release();
  exclusive_scan<int>(F.rowptr.p, F.rowptr.p, n, s);
  if (read_scalar(err.p, s))
    throw Error(TMRG_ERR_INTERNAL, "matrix filter: element touches too many nodes");
  F.Ainv.alloc(n, s);
  F.B.alloc(n, s);
  F.Tinv.alloc(n, s);
  launch(k_fe_scalings, blocks_for(n, 256), 256, 0, s, n, f.dim, (const int *)F.rowptr.p,
         (const double *)F.vals.p, r, F.Ainv.p, F.B.p);
  // the sliced-ELL copy the Horner steps read
  {
    const long long nsl = (n + 31) / 32;
    F.npos = nsl * 32;
    F.sperm.alloc(std::max(1LL, n), s);
    F.srl.alloc(std::max(1LL, F.npos), s);
    F.soff.alloc(nsl + 1, s);
    if (n) len_order(n, (const int *)F.rowptr.p, F.sperm.p, s);
    launch(k_sell_len, blocks_for(F.npos, 256), 256, 0, s, F.npos, n, (const int *)F.sperm.p,
           (const int *)F.rowptr.p, F.srl.p, F.soff.p);
    exclusive_scan<long long>(F.soff.p, F.soff.p, nsl, s);
    F.nsell = read_scalar(F.soff.p + nsl, s);
    F.scol.alloc(std::max(1LL, F.nsell), s);
    F.sval.alloc(std::max(1LL, F.nsell), s);
    launch((k_sell_fill<double>), blocks_for(F.npos, 256), 256, 0, s, F.npos, n,
           (const int *)F.sperm.p, (const int *)F.rowptr.p, (const int *)F.colidx.p,
           (const double *)F.vals.p, (const long long *)F.soff.p, F.scol.p, F.sval.p);
  }
  // Tinv = 1 / (F~ 1) with Tinv = 1 during the evaluation.
  {
    DBuf<double> ones(n, s), y(n, s);
    std::vector<double> h1(n, 1.0);
    TMRG_CUDA(cudaMemcpyAsync(ones.p, h1.data(), n * sizeof(double),
                              cudaMemcpyHostToDevice, s));
    TMRG_CUDA(cudaMemcpyAsync(F.Tinv.p, h1.data(), n * sizeof(double),
                              cudaMemcpyHostToDevice, s));
    filter_apply(F, false, 1, ones.p, y.p);
    launch(k_fe_tinv, blocks_for(n, 256), 256, 0, s, n, (const double *)y.p,
           F.Tinv.p);
    TMRG_CUDA(cudaStreamSynchronize(s));
  }
  F.sval32.alloc(std::max(1LL, F.nsell), s);
  launch(k_to_f32<float>, blocks_for(F.nsell, 256), 256, 0, s, F.nsell,
         (const double *)F.sval.p, F.sval32.p);
  F.Ainv32.alloc(n, s);
  F.B32.alloc(n, s);
  F.Tinv32.alloc(n, s);
  launch(k_to_f32<float>, blocks_for(n, 256), 256, 0, s, n,
         (const double *)F.Ainv.p, F.Ainv32.p);
  launch(k_to_f32<float>, blocks_for(n, 256), 256, 0, s, n,
         (const double *)F.B.p, F.B32.p);
  launch(k_to_f32<float>, blocks_for(n, 256), 256, 0, s, n,
         (const double *)F.Tinv.p, F.Tinv32.p);
  TMRG_CUDA(cudaStreamSynchronize(s));
}

}  // namespace tmrg
