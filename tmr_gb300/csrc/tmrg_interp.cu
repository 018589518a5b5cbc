// createInterpolation and the P / P^T applies on the GPU.
//
// P (coarse -> fine) has one row per owned fine node.  A node is handled
// through the first (element, local node) that references it in element
// order (TMROctForest.cpp:6654-6688): the reference's findEnclosing search
// over the sorted coarse octants, computeElemInterp's tensor-product
// Lagrange weights with the coarse dependent-node expansion, and a sort and
// merge of the entries by column (TMRIndexWeight::uniqueSort).
//
// The sort is done once per coarse element instead of once per row.  The
// entries of a row are, in computeElemInterp's order (kk, jj, ii, then the
// dependent entries in CSR order), the in-box subsequence of its element's
// full expansion sequence.  A stable sort by column commutes with taking a
// subsequence, so each coarse element's expansion is stably sorted by
// column once, and a row is the in-box filter of that list with adjacent
// equal columns summed in order.  Rows are written in two passes (exact
// count, then write at the scanned offsets).  P^T is the apply copy
// re-sorted by (column, row), so transpose applies gather without atomics
// and sum in a fixed order.
#include <cuda.h>  // CUtensorMap (the encoder is fetched from the driver at run time)

#include <algorithm>

#include "tmrg_tree.cuh"

namespace tmrg {

constexpr int IMAX_CO = 3;   // coarse orders built for createInterpolation
constexpr int IMAX_E = 256;  // entries of one coarse element's expansion
constexpr uint8_t KEY_INDEP = 0x80;  // list entry is an independent node

struct InterpCtx {
  int fo, co;  // fine / coarse order
  double fk1[TMRG_MAX_ORDER], ck[TMRG_MAX_ORDER];  // 1 + fine knot, coarse knot
  double crk[TMRG_MAX_ORDER][TMRG_MAX_ORDER];     // 1/(ck_i - ck_j)
  int fk1i[TMRG_MAX_ORDER];  // 1 + fine knot rounded to 0, 1 or 2 (orders 2, 3)
  int fodd;                  // bit i: 1 + fine knot i is not that integer
  // fine octants
  const int *fb, *fx, *fy, *fz;
  const int16_t *fl;
  // coarse octants {block | level << 26, x, y, z}
  long long cn;
  const int4 *c4;
  // per coarse element: offsets of its sorted expansion list, the list
  // (column, dependent weight, local node | KEY_INDEP) and its kind
  // (0: co^3 independent distinct nodes, 1: dependent entries, 2: a
  // column repeats)
  const long long *eoff;
  const int *lcol;
  const double *ldw;
  const uint8_t *lkey;
  const uint8_t *ekind;
  const unsigned long long *rep;  // fine node -> element*npe + local index
  int *err;
  // weight products by direction states (k_uvw_table), or null
  const double *uvw;
  int *wide;  // set when a fine element lies two or more levels below its coarse element
};

__global__ void k_pack_octs(long long n, const int *__restrict__ b,
                            const int *__restrict__ x, const int *__restrict__ y,
                            const int *__restrict__ z,
                            const int16_t *__restrict__ l, int4 *out) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = make_int4(b[i] | ((int)l[i] << 26), x[i], y[i], z[i]);
}

// First reference of every owned fine node in (element, local index)
// order, packed element << 8 | local (npe <= 216): decoding takes shifts,
// not a 64-bit division (which GB300 runs on its scarce FP64 pipe).
__global__ void k_first_ref(long long n, int npe, long long nowned,
                            const int *__restrict__ conn,
                            unsigned long long *rep) {
  long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  const int *c = conn + e * npe;
  for (int l = 0; l < npe; l++) {
    int v = __ldg(c + l);
    if (v >= 0 && v < nowned) atomicMin(rep + v, ((unsigned long long)e << 8) | (unsigned)l);
  }
}

// ---------------------------------------------------------------------
// Coarse element expansion lists.
__global__ void k_elist_count(long long n, int cnpe, const int *__restrict__ conn,
                              const int *__restrict__ dptr, long long *cnt) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const int *c = conn + t * cnpe;
  long long e = 0;
  for (int l = 0; l < cnpe; l++) {
    int cv = __ldg(c + l);
    e += (cv >= 0) ? 1 : (__ldg(dptr - cv) - __ldg(dptr - cv - 1));
  }
  cnt[t] = e;
}

// One warp per coarse element: lane l expands local node l (l = ii + jj*co
// + kk*co^2, so lanes run in computeElemInterp's loop order) into shared
// memory, then a stable rank sort by column writes the list.
constexpr int EL_WARPS = 4;
__global__ void __launch_bounds__(EL_WARPS * 32, 16)
    k_elist_fill(long long n, int cnpe, const int *__restrict__ conn,
                 const int *__restrict__ dptr, const int *__restrict__ dconn,
                 const double *__restrict__ dw, const long long *__restrict__ eoff,
                 int *lcol, double *ldw, uint8_t *lkey, uint8_t *ekind, int *err) {
  __shared__ int s_col[EL_WARPS][IMAX_E];
  __shared__ double s_dw[EL_WARPS][IMAX_E];
  __shared__ uint8_t s_key[EL_WARPS][IMAX_E];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const long long t = (long long)blockIdx.x * EL_WARPS + warp;
  if (t >= n) return;
  const long long eo = eoff[t];
  const int E = (int)(eoff[t + 1] - eo);
  if (E > IMAX_E) {
    if (lane == 0) atomicExch(err, 2);
    return;
  }
  int cv = 0, myn = 0, d0 = 0;
  if (lane < cnpe) {
    cv = __ldg(conn + t * cnpe + lane);
    if (cv >= 0) {
      myn = 1;
    } else {
      d0 = __ldg(dptr - cv - 1);
      myn = __ldg(dptr - cv) - d0;
    }
  }
  int incl = myn;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += y;
  }
  const int off = incl - myn;
  if (lane < cnpe) {
    if (cv >= 0) {
      s_col[warp][off] = cv;
      s_dw[warp][off] = 1.0;
      s_key[warp][off] = (uint8_t)(lane | KEY_INDEP);
    } else {
      for (int p = 0; p < myn; p++) {
        s_col[warp][off + p] = __ldg(dconn + d0 + p);
        s_dw[warp][off + p] = __ldg(dw + d0 + p);
        s_key[warp][off + p] = (uint8_t)lane;
      }
    }
  }
  const bool anydep = __any_sync(0xffffffffu, lane < cnpe && cv < 0);
  __syncwarp();
  bool dup = false;
  for (int a = lane; a < E; a += 32) {
    const int col = s_col[warp][a];
    int rk = 0;
    for (int b = 0; b < E; b++) {
      const int cb = s_col[warp][b];
      rk += (cb < col) || (cb == col && b < a);
      dup |= (cb == col && b != a);
    }
    lcol[eo + rk] = col;
    ldw[eo + rk] = s_dw[warp][a];
    lkey[eo + rk] = s_key[warp][a];
  }
  const bool anydup = __any_sync(0xffffffffu, dup);
  if (lane == 0) ekind[t] = anydup ? 2 : (anydep ? 1 : 0);
}

// ---------------------------------------------------------------------
// 1-D Lagrange basis (TMRInterpolation.h:40-52) for two or three knots:
// N_i = prod_{j != i, ascending} (u - k_j) * rk[i][j], where rk[i][j] holds
// 1/(k_i - k_j), rounded once on the host exactly as the reference rounds
// it.  The product starts from its first factor (1.0 * f == f exactly), so
// an order-3 basis takes 12 FP64 operations (FP64 is a scarce pipe on
// GB300).
__device__ __forceinline__ void lagrange3(int order, double u, const double *kn,
                                          const double (*rk)[TMRG_MAX_ORDER],
                                          double &n0, double &n1, double &n2) {
  const double d0 = __dsub_rn(u, kn[0]), d1 = __dsub_rn(u, kn[1]);
  if (order == 2) {
    n0 = __dmul_rn(d1, rk[0][1]);
    n1 = __dmul_rn(d0, rk[1][0]);
    n2 = 1.0;
    return;
  }
  const double d2 = __dsub_rn(u, kn[2]);
  n0 = __dmul_rn(__dmul_rn(d1, rk[0][1]), __dmul_rn(d2, rk[0][2]));
  n1 = __dmul_rn(__dmul_rn(d0, rk[1][0]), __dmul_rn(d2, rk[1][2]));
  n2 = __dmul_rn(__dmul_rn(d0, rk[2][0]), __dmul_rn(d1, rk[2][1]));
}
// 2^e as a double from its exponent (exact; e >= -1022).
__device__ __forceinline__ double pow2(int e) { return __hiloint2double((1023 + e) << 20, 0); }
// A non-negative int32 as a double, assembled from its bits with integer
// operations (exactly (double)v): GB300 issues int-to-double conversions on
// its FP64 pipe.
__device__ __forceinline__ double exact_double(int32_t v) {
  if (v <= 0) return 0.0;
  const int e = 31 - __clz(v);  // leading bit
  const unsigned long long m = ((unsigned long long)(uint32_t)v << (52 - e)) &
                               ((1ULL << 52) - 1ULL);
  return __longlong_as_double((long long)(((unsigned long long)(1023 + e) << 52) | m));
}

// Integer bounds [lo, hi] of a node coordinate at a knot that is not an
// octant-grid point (orders >= 4): x + (0.5 h)(1 + k) in double as the
// reference rounds it, with 0.5 h = 2^(29 - level) exact.  An integer a
// satisfies a <= xd iff a <= floor(xd), and xd <= b iff ceil(xd) <= b, so
// the containment tests below stay in integers.  Kept out of line: GB300
// runs integer-to-double conversions on its FP64 pipe, and the exact
// (grid-point) case must not pay for them.
__device__ __noinline__ void knot_bounds(int32_t x, int level, double fk1, int32_t &lo,
                                         int32_t &hi) {
  const double xd = __dadd_rn((double)x, __dmul_rn(pow2(TMRG_MAX_LEVEL - 1 - level), fk1));
  lo = (int32_t)floor(xd);
  hi = (int32_t)ceil(xd);
}

// findEnclosing (TMROctForest.cpp:6228-6377): binary search for the node's
// element octant, then a forward scan up to the bounding position.
__device__ long long find_enclosing(const InterpCtx &I, const Oct &node, int info) {
  const int order = I.fo;
  int32_t h = side_of(node.level);
  int ii = info % order, jj = (info % (order * order)) / order,
      kk = info / (order * order);
  int32_t xi = -1, yi = -1, zi = -1;
  if (ii == 0 || ii == order - 1)
    xi = node.x + (ii / (order - 1)) * h;
  else if (order % 2 == 1 && ii == order / 2)
    xi = node.x + h / 2;
  if (jj == 0 || jj == order - 1)
    yi = node.y + (jj / (order - 1)) * h;
  else if (order % 2 == 1 && jj == order / 2)
    yi = node.y + h / 2;
  if (kk == 0 || kk == order - 1)
    zi = node.z + (kk / (order - 1)) * h;
  else if (order % 2 == 1 && kk == order / 2)
    zi = node.z + h / 2;
  int32_t xl = xi, xh = xi, yl = yi, yh = yi, zl = zi, zh = zi;
  if (xi < 0) knot_bounds(node.x, node.level, I.fk1[ii], xl, xh);
  if (yi < 0) knot_bounds(node.y, node.level, I.fk1[jj], yl, yh);
  if (zi < 0) knot_bounds(node.z, node.level, I.fk1[kk], zl, zh);
  long long low = 0, high = I.cn - 1, mid = low + (high - low) / 2;
  while (mid != low) {
    int4 q = __ldg(I.c4 + mid);
    int32_t hm = side_of(q.x >> 26);
    int32_t ab = q.x & 0x3ffffff, ax = q.y, ay = q.z, az = q.w;
    if (node.block == ab && node.x >= ax && node.x < ax + hm && node.y >= ay &&
        node.y < ay + hm && node.z >= az && node.z < az + hm)
      break;
    int st = cmp_position(ab, ax, ay, az, node.block, node.x, node.y, node.z);
    if (st == 0) break;
    if (st < 0)
      low = mid + 1;
    else
      high = mid - 1;
    mid = low + (high - low) / 2;
  }
  int32_t bx = node.x + h, by = node.y + h, bz = node.z + h;
  while (mid < I.cn) {
    int4 q = __ldg(I.c4 + mid);
    int32_t ab = q.x & 0x3ffffff;
    if (cmp_position(ab, q.y, q.z, q.w, node.block, bx, by, bz) > 0) break;
    if (ab == node.block) {
      int32_t hm = side_of(q.x >> 26);
      int32_t ax = q.y, ay = q.z, az = q.w;
      const bool xin = ax <= xl && xh <= ax + hm;
      const bool yin = ay <= yl && yh <= ay + hm;
      const bool zin = az <= zl && zh <= az + hm;
      if (xin && yin && zin) return mid;
    }
    mid++;
  }
  return -1;
}

// The index range [s, e) of one coordinate direction of computeElemInterp
// (TMROctForest.cpp:6497-6548, Lagrange branch) as s | e << 2: an exact
// face hit keeps one coarse index.
__device__ __forceinline__ int dir_range(int i, int mo, int co, int32_t nx, int32_t h,
                                         int32_t ox, int32_t hc) {
  if ((i == 0 && ox == nx) || (i == mo - 1 && ox == nx + h)) return 0 | (1 << 2);
  if ((i == 0 && ox + hc == nx) || (i == mo - 1 && ox + hc == nx + h))
    return (co - 1) | (co << 2);
  return 0 | (co << 2);
}
// The weights of that direction (1.0 at a face hit).
// u = -1 + 2 (x + 0.5 h (1 + k_i) - ox) / hc as the reference rounds it:
// 0.5 h and 2 / hc are powers of two, so those scalings are exact.
__device__ __forceinline__ void dir_weights(const InterpCtx &I, int i, int range,
                                            int32_t nx, double half, int32_t ox,
                                            double two_ihc, double &n0, double &n1,
                                            double &n2) {
  if (((range >> 2) - (range & 3)) == 1) {
    n0 = n1 = n2 = 1.0;
    return;
  }
  double t = __dadd_rn(exact_double(nx), __dmul_rn(half, I.fk1[i]));
  double u = __dadd_rn(-1.0, __dmul_rn(__dsub_rn(t, exact_double(ox)), two_ihc));
  lagrange3(I.co, u, I.ck, I.crk, n0, n1, n2);
}

// Direction states.  Fine orders 2 and 3 have 1 + k_i equal to 0, 1 or 2,
// or (the middle Gauss-Lobatto knot -cos(pi/2)) 1 - 2^-53.  Where the fine
// level lf is at most one below the coarse level lc and not above it when
// a knot is of the second kind, the u that dir_weights computes is one of:
//   s = 0..4: u = -1 + s/2 exactly.  With t = nx + 0.5 h (1 + k_i) exact
//     (integers; for the inexact knot and nx >= h the 2^-53 term is below
//     half an ulp of nx + h/2), num = 2 (nx - ox) + h (1 + k_i) - hc is a
//     multiple of 2^(30 - max(lf, lc)) and u = num / hc.
//   s = 6: the inexact knot at nx = ox = 0, lf = lc: u = -1 + (1 - 2^-53),
//     which is -2^-53 whatever the level.  (At lf = lc + 1 the sum
//     -1 + (1/2 - 2^-54) is a tie that rounds to -1/2, s = 1; the host
//     checks it.)
//   s = 5: an exact face hit (weights 1).
// A row's three states index k_uvw_table's products, which repeat the
// double sequence of dir_weights and the Nu Nv then Nw products on the same
// u, so they are the same bits.
__device__ __forceinline__ int dir_state(const InterpCtx &I, int i, int range, int32_t nx,
                                         int32_t h, int lf, int32_t ox, int32_t hc, int lc) {
  if (((range >> 2) - (range & 3)) == 1) return 5;
  if (((I.fodd >> i) & 1) && nx == 0 && lf == lc) return 6;
  const long long num = 2LL * (nx - ox) + (long long)h * I.fk1i[i] - hc;
  const int lm = max(lf, lc);
  const int m = (int)(num >> (TMRG_MAX_LEVEL - lm));
  return m * (1 << (1 - (lm - lc))) + 2;
}
constexpr int UVW_DIR = 7, UVW_STATES = UVW_DIR * UVW_DIR * UVW_DIR;
// tab[(su*49 + sv*7 + sw) * co^3 + ii + co*jj + co^2*kk] = (Nu[ii] Nv[jj]) Nw[kk];
// fk1odd is 1 + the inexact fine knot (state 6).
__global__ void k_uvw_table(InterpCtx I, double fk1odd, double *tab) {
  const int co = I.co, cn3 = co * co * co;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= UVW_STATES * cn3) return;
  const int st = t / cn3, li = t - st * cn3;
  const int ss[3] = {st / (UVW_DIR * UVW_DIR), (st / UVW_DIR) % UVW_DIR, st % UVW_DIR};
  const int ix[3] = {li % co, (li / co) % co, li / (co * co)};
  double w[3];
  for (int d = 0; d < 3; d++) {
    double n[3] = {1.0, 1.0, 1.0};
    if (ss[d] < 5) {
      lagrange3(co, -1.0 + 0.5 * ss[d], I.ck, I.crk, n[0], n[1], n[2]);
    } else if (ss[d] == 6) {
      // dir_weights' sequence at nx = ox = 0, lf = lc = 10
      const double tt = __dadd_rn(0.0, __dmul_rn(pow2(TMRG_MAX_LEVEL - 11), fk1odd));
      const double u = __dadd_rn(-1.0, __dmul_rn(__dsub_rn(tt, 0.0), pow2(11 - TMRG_MAX_LEVEL)));
      lagrange3(co, u, I.ck, I.crk, n[0], n[1], n[2]);
    }
    w[d] = n[ix[d]];
  }
  tab[t] = __dmul_rn(__dmul_rn(w[0], w[1]), w[2]);
}
// Bit l of the mask is set when local coarse node l = ii + jj*co + kk*co^2
// lies in the row's box.
__device__ __forceinline__ unsigned box_mask(int co, int rx, int ry, int rz) {
  unsigned mu = ((1u << (rx >> 2)) - 1u) & ~((1u << (rx & 3)) - 1u);
  unsigned m = 0;
  for (int kk = rz & 3; kk < (rz >> 2); kk++)
    for (int jj = ry & 3; jj < (ry >> 2); jj++) m |= mu << (jj * co + kk * co * co);
  return m;
}

// The row's element and box.  Returns the element (or -1 with the error
// flag set) and the box mask in `bm`.
__device__ __forceinline__ long long row_box(const InterpCtx &I, long long row,
                                             Oct &node, int &info, int4 &cq,
                                             int r[3], unsigned &bm) {
  const int mo = I.fo, co = I.co;
  unsigned long long rr = I.rep[row];
  long long e = (long long)(rr >> 8);
  info = (int)(rr & 255u);
  node = Oct{I.fb[e], I.fx[e], I.fy[e], I.fz[e], I.fl[e]};
  long long t = find_enclosing(I, node, info);
  bm = 0;
  if (t < 0) {
    atomicExch(I.err, 1);
    return -1;
  }
  cq = __ldg(I.c4 + t);
  int32_t h = side_of(node.level), hc = side_of(cq.x >> 26);
  int i = info % mo, j = (info % (mo * mo)) / mo, k = info / (mo * mo);
  r[0] = dir_range(i, mo, co, node.x, h, cq.y, hc);
  r[1] = dir_range(j, mo, co, node.y, h, cq.z, hc);
  r[2] = dir_range(k, mo, co, node.z, h, cq.w, hc);
  bm = box_mask(co, r[0], r[1], r[2]);
  return t;
}

// Pass 1, one lane per row: findEnclosing, kept in `trow`, and the exact
// number of merged entries of the row in `cnt`.
__global__ void k_interp_count(long long rows, InterpCtx I, int *trow, long long *cnt) {
  long long row = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (row >= rows) return;
  Oct node;
  int info, r[3];
  int4 cq;
  unsigned bm;
  long long t = row_box(I, row, node, info, cq, r, bm);
  trow[row] = (int)t;
  long long ne = 0;
  if (t >= 0) {
    const int kind = I.ekind[t];
    if (kind == 0) {
      ne = __popc(bm);
    } else {
      const long long eo = I.eoff[t], e1 = I.eoff[t + 1];
      int prev = -1;
      for (long long j = eo; j < e1; j++) {
        int key = I.lkey[j];
        if ((bm >> (key & 31)) & 1u) {
          if (kind == 1) {
            ne++;
          } else {
            int col = I.lcol[j];
            ne += (col != prev);
            prev = col;
          }
        }
      }
    }
  }
  cnt[row] = ne;
}


// Pass 2, 32 consecutive rows per warp; their entries form one contiguous
// segment of the CSR.  Phase A, one lane per row: the element, its list
// range, the box mask and the direction weights, with the products
// Nu[ii]*Nv[jj] formed once per row (computeElemInterp multiplies Nu*Nv
// first).  Phase B walks the 32 rows' element lists as one concatenated
// sequence, 64 entries per step with all loads independent, and stages the
// in-box entries in order (ballot + popc) in shared memory.  A flush forms
// the staged weights on full warps (a masked FP64 warp instruction costs
// the GB300 FP64 pipe as much as a full one), sums each run of equal
// (row, column) in order and writes the run heads in order; the last run
// of a non-final flush stays staged because it may continue.  *nzcount
// gets the number of nonzero values written.
//
// This is the general kernel (any level gap, any knots of orders 2-3);
// k_interp_elem covers the multigrid case with less work.
constexpr int IW_WARPS = 4;
constexpr int IW_CAP = 256;  // staged entries per warp
__global__ void __launch_bounds__(IW_WARPS * 32)
    k_interp_rows(long long rows, InterpCtx I, const int *__restrict__ trow,
                  const long long *__restrict__ roff, int *cols, double *vals,
                  unsigned long long *nzcount) {
  __shared__ double s_uv[IW_WARPS][32][IMAX_CO * IMAX_CO];
  __shared__ double s_nw[IW_WARPS][32][IMAX_CO];
  __shared__ long long s_eo[IW_WARPS][32];
  __shared__ int s_vs[IW_WARPS][33];  // start of each row's list in the sequence
  __shared__ unsigned s_bm[IW_WARPS][32];
  __shared__ int s_c[IW_WARPS][IW_CAP];
  __shared__ double s_v[IW_WARPS][IW_CAP];
  __shared__ uint16_t s_k[IW_WARPS][IW_CAP];  // row slot << 8 | kk << 4 | ii + co*jj
  __shared__ uint16_t s_rs[IW_WARPS][IW_CAP / 2];  // start and length of each
  __shared__ uint8_t s_rl[IW_WARPS][IW_CAP / 2];   // run to sum
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const unsigned lt = (1u << lane) - 1u;
  const long long base = ((long long)blockIdx.x * IW_WARPS + warp) * 32;
  if (base >= rows) return;
  const int mo = I.fo, co = I.co, co2 = co * co;
  // phase A
  {
    long long row = base + lane;
    int E = 0;
    long long eo = 0;
    unsigned bm = 0;
    if (row < rows) {
      const int t = trow[row];
      if (t >= 0) {
        eo = I.eoff[t];
        E = (int)(I.eoff[t + 1] - eo);
        unsigned long long rr = I.rep[row];
        long long e = (long long)(rr >> 8);
        int info = (int)(rr & 255u);
        Oct node{I.fb[e], I.fx[e], I.fy[e], I.fz[e], I.fl[e]};
        int4 cq = __ldg(I.c4 + t);
        int cl = cq.x >> 26;
        int32_t h = side_of(node.level), hc = side_of(cl);
        int i = info % mo, j = (info % (mo * mo)) / mo, k = info / (mo * mo);
        int rx = dir_range(i, mo, co, node.x, h, cq.y, hc);
        int ry = dir_range(j, mo, co, node.y, h, cq.z, hc);
        int rz = dir_range(k, mo, co, node.z, h, cq.w, hc);
        bm = box_mask(co, rx, ry, rz);
        const double half = pow2(TMRG_MAX_LEVEL - 1 - node.level);
        const double two_ihc = pow2(cl + 1 - TMRG_MAX_LEVEL);
        double u0, u1, u2, v0, v1, v2, w0, w1, w2;
        dir_weights(I, i, rx, node.x, half, cq.y, two_ihc, u0, u1, u2);
        dir_weights(I, j, ry, node.y, half, cq.z, two_ihc, v0, v1, v2);
        dir_weights(I, k, rz, node.z, half, cq.w, two_ihc, w0, w1, w2);
        const double nu[3] = {u0, u1, u2}, nv[3] = {v0, v1, v2};
#pragma unroll
        for (int b = 0; b < IMAX_CO; b++)
#pragma unroll
          for (int a = 0; a < IMAX_CO; a++)
            if (a < co && b < co) s_uv[warp][lane][a + co * b] = __dmul_rn(nu[a], nv[b]);
        s_nw[warp][lane][0] = w0;
        s_nw[warp][lane][1] = w1;
        s_nw[warp][lane][2] = w2;
      }
    }
    int incl = E;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int y = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += y;
    }
    s_vs[warp][lane] = incl - E;
    if (lane == 31) s_vs[warp][32] = incl;
    s_eo[warp][lane] = eo;
    s_bm[warp][lane] = bm;
  }
  __syncwarp();
  const int vtot = s_vs[warp][32];
  // phase B
  const long long lim = roff[min(base + 32, rows)];  // end of the warp's segment
  long long out = roff[base];
  int nbuf = 0, nzc = 0;
  auto flush = [&](bool final) {
    __syncwarp();
    int end = nbuf;
    if (!final && nbuf > 0) {
      // keep the last run (at most co^3 entries: one per local node)
      const int c1 = s_c[warp][nbuf - 1], q1 = s_k[warp][nbuf - 1] >> 8;
      while (end > 1 && s_c[warp][end - 2] == c1 && (s_k[warp][end - 2] >> 8) == q1) end--;
      end--;
    }
    for (int k = lane; k < end; k += 32) {
      const int sk = s_k[warp][k];
      const int q = sk >> 8;
      s_v[warp][k] = __dmul_rn(__dmul_rn(s_uv[warp][q][sk & 15], s_nw[warp][q][(sk >> 4) & 15]),
                               s_v[warp][k]);
    }
    __syncwarp();
    // runs of equal (row, column) longer than one entry, listed densely so
    // that their in-order sums run on as many lanes as there are runs
    int nruns = 0;
    for (int c0 = 0; c0 < end; c0 += 32) {
      const int k = c0 + lane;
      int len = 0;
      if (k < end) {
        const int col = s_c[warp][k], q = s_k[warp][k] >> 8;
        if ((k == 0) || (s_c[warp][k - 1] != col) || ((s_k[warp][k - 1] >> 8) != q)) {
          len = 1;
          while (k + len < end && s_c[warp][k + len] == col && (s_k[warp][k + len] >> 8) == q)
            len++;
        }
      }
      const unsigned m = __ballot_sync(0xffffffffu, len > 1);
      if (len > 1) {
        const int r = nruns + __popc(m & lt);
        s_rs[warp][r] = (uint16_t)k;
        s_rl[warp][r] = (uint8_t)len;
      }
      nruns += __popc(m);
    }
    __syncwarp();
    for (int r = lane; r < nruns; r += 32) {
      const int st = s_rs[warp][r], len = s_rl[warp][r];
      double acc = s_v[warp][st];
      for (int i = 1; i < len; i++) acc = __dadd_rn(acc, s_v[warp][st + i]);
      s_v[warp][st] = acc;
    }
    __syncwarp();
    for (int c0 = 0; c0 < end; c0 += 32) {
      const int k = c0 + lane;
      bool head = false;
      int col = 0;
      if (k < end) {
        col = s_c[warp][k];
        const int q = s_k[warp][k] >> 8;
        head = (k == 0) || (s_c[warp][k - 1] != col) || ((s_k[warp][k - 1] >> 8) != q);
      }
      const unsigned m = __ballot_sync(0xffffffffu, head);
      if (head) {
        const double acc = s_v[warp][k];
        const long long o = out + __popc(m & lt);
        if (o < lim) {
          cols[o] = col;
          vals[o] = acc;
          nzc += apply_keeps(acc);
        } else {
          atomicExch(I.err, 3);
        }
      }
      out += __popc(m);
    }
    // move the kept run (shorter than the flushed part) to the front
    int keep = nbuf - end;
    if (keep > 32) {  // a run has at most one entry per local node
      atomicExch(I.err, 3);
      keep = 0;
    }
    int kc = 0, kk = 0;
    double kv = 0.0;
    if (lane < keep) {
      kc = s_c[warp][end + lane];
      kk = s_k[warp][end + lane];
      kv = s_v[warp][end + lane];
    }
    __syncwarp();
    if (lane < keep) {
      s_c[warp][lane] = kc;
      s_k[warp][lane] = (uint16_t)kk;
      s_v[warp][lane] = kv;
    }
    __syncwarp();
    nbuf = keep;
  };
  // the row slot of sequence position v: the last q with s_vs[q] <= v
  auto slot = [&](int v) {
    int q = 0;
#pragma unroll
    for (int step = 16; step > 0; step >>= 1)
      if (q + step < 32 && s_vs[warp][q + step] <= v) q += step;
    return q;
  };
  for (int v0 = 0; v0 < vtot; v0 += 64) {
    int key[2] = {0, 0}, col[2] = {0, 0}, qs[2] = {0, 0};
    double dw[2] = {0.0, 0.0};
#pragma unroll
    for (int u = 0; u < 2; u++) {
      const int v = v0 + 32 * u + lane;
      if (v < vtot) {
        const int q = slot(v);
        const long long a = s_eo[warp][q] + (v - s_vs[warp][q]);
        qs[u] = q;
        key[u] = I.lkey[a];
        col[u] = I.lcol[a];
        dw[u] = I.ldw[a];
      }
    }
#pragma unroll
    for (int u = 0; u < 2; u++) {
      const int v = v0 + 32 * u + lane;
      const bool in = v < vtot && ((s_bm[warp][qs[u]] >> (key[u] & 31)) & 1u);
      const unsigned m = __ballot_sync(0xffffffffu, in);
      if (in) {
        const int li = key[u] & 31;
        const int kk = li >= 2 * co2 ? 2 : (li >= co2 ? 1 : 0);
        const int o = nbuf + __popc(m & lt);
        s_c[warp][o] = col[u];
        // (Nu Nv Nw) * 1.0 is the independent node's weight exactly
        s_v[warp][o] = (key[u] & KEY_INDEP) ? 1.0 : dw[u];
        s_k[warp][o] = (uint16_t)((qs[u] << 8) | (kk << 4) | (li - kk * co2));
      }
      nbuf += __popc(m);
    }
    if (nbuf > IW_CAP - 64) flush(false);
  }
  flush(true);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) nzc += __shfl_xor_sync(0xffffffffu, nzc, o);
  if (lane == 0 && nzc) atomicAdd(nzcount, (unsigned long long)nzc);
}

// ---------------------------------------------------------------------
// P rows grouped by coarse element (the direction-state case: every fine
// element at most one level below its coarse element).  All rows whose
// node lies in one coarse element filter the same sorted expansion list,
// so one warp per coarse element loads the list into shared memory once
// and handles its rows one after the other: a ballot compaction of the
// in-box entries (list order kept), their weights (table product times the
// dependent weight, as in k_interp_rows), and the in-order sums of equal
// columns.  Same entries, same arithmetic, same bits as k_interp_rows.

// Pass 1: each row's element (findEnclosing), the rows per element, and
// the row's box mask and direction states packed as bm | state << 32
// (state = su*49 + sv*7 + sw, or 0xffff where the states do not cover the
// row: its element is too coarse, and the host takes the per-row kernel).
__global__ void k_interp_find(long long rows, InterpCtx I, int *trow, unsigned *ecnt,
                              unsigned long long *rinfo) {
  long long row = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (row >= rows) return;
  const unsigned long long rr = I.rep[row];
  const long long e = (long long)(rr >> 8);
  const int info = (int)(rr & 255u);
  const Oct node{I.fb[e], I.fx[e], I.fy[e], I.fz[e], I.fl[e]};
  const long long t = find_enclosing(I, node, info);
  trow[row] = (int)t;
  if (t < 0) {
    atomicExch(I.err, 1);
    return;
  }
  atomicAdd(ecnt + t, 1u);
  const int4 cq = __ldg(I.c4 + t);
  const int cl = cq.x >> 26;
  const int gap = node.level - cl;
  const bool wide = gap > 1 || (gap < 0 && I.fodd);
  if (wide && *(volatile int *)I.wide == 0) atomicOr(I.wide, 1);
  const int mo = I.fo, co = I.co;
  const int32_t h = side_of(node.level), hc = side_of(cl);
  const int i = info % mo, j = (info % (mo * mo)) / mo, k = info / (mo * mo);
  const int rx = dir_range(i, mo, co, node.x, h, cq.y, hc);
  const int ry = dir_range(j, mo, co, node.y, h, cq.z, hc);
  const int rz = dir_range(k, mo, co, node.z, h, cq.w, hc);
  unsigned sidx = 0xffffu;
  if (!wide) {
    const int su = dir_state(I, i, rx, node.x, h, node.level, cq.y, hc, cl);
    const int sv = dir_state(I, j, ry, node.y, h, node.level, cq.z, hc, cl);
    const int sw = dir_state(I, k, rz, node.z, h, node.level, cq.w, hc, cl);
    if ((unsigned)su < UVW_DIR && (unsigned)sv < UVW_DIR && (unsigned)sw < UVW_DIR)
      sidx = (unsigned)((su * UVW_DIR + sv) * UVW_DIR + sw);
  }
  rinfo[row] = (unsigned long long)box_mask(co, rx, ry, rz) |
               ((unsigned long long)sidx << 32);
}
// Rows by element: erows[estart[t] ..] lists the rows of element t (in no
// particular order: each row's output place is fixed by its offset), with
// their packed box mask and states beside them in einfo.
__global__ void k_group_rows(long long rows, const int *__restrict__ trow,
                             const unsigned long long *__restrict__ rinfo,
                             const unsigned *__restrict__ estart, unsigned *ecur, int *erows,
                             unsigned long long *einfo) {
  long long row = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (row >= rows) return;
  const int t = trow[row];
  if (t < 0) return;
  const unsigned pos = estart[t] + atomicAdd(ecur + t, 1u);
  erows[pos] = (int)row;
  einfo[pos] = rinfo[row];
}
// Passes 2 (FILL = false: each row's merged length in cnt) and 3 (FILL:
// the rows at roff, each row's apply_keeps entries counted in cnt).  One warp per
// coarse element, its rows 32 at a time, lane r <-> row r for the set-up
// (box mask, direction states, CSR offsets).
// An element of kind 0 (co^3 distinct independent nodes: each entry's
// weight is the table value itself) emits its rows one after another, lane
// j <-> list entry j: the in-box lanes write consecutive CSR slots, so a
// row is one contiguous store, with no FP64 instruction.
// Other elements walk the sorted list in step (broadcast shared-memory
// reads), lane r <-> row r:
//   stage: the in-box (row, entry) pairs of list entries k0.. in list
//     order, with each entry's rows mask and first pair;
//   weights: the pairs' products on full warps (table value times the
//     dependent weight, as in k_interp_rows; a masked FP64 warp
//     instruction costs the GB300 FP64 pipe as much as a full one);
//   merge: lane r takes its pairs in list order and sums equal columns in
//     that order; an add is issued only at list entries that repeat the
//     previous entry's column (the list is sorted, so no other entry can
//     continue a run).
constexpr int EW_WARPS = 4;
constexpr int EW_CAP = 256;  // staged pairs per warp
template <bool FILL>
__global__ void __launch_bounds__(EW_WARPS * 32)
    k_interp_elem(long long n, InterpCtx I, const unsigned *__restrict__ estart,
                  const int *__restrict__ erows, const unsigned long long *__restrict__ einfo,
                  long long *cnt, const long long *__restrict__ roff, int *cols,
                  double *vals) {
  constexpr int FW = FILL ? EW_WARPS : 1;
  __shared__ int s_col[EW_WARPS][IMAX_E];
  __shared__ uint8_t s_key[EW_WARPS][IMAX_E];
  __shared__ unsigned s_mk[FW][IMAX_E];   // rows (lanes) taking entry k
  __shared__ uint16_t s_bk[FW][IMAX_E];   // staged position of its first pair
  __shared__ uint8_t s_pr[FW][EW_CAP];    // staged pair: row lane
  __shared__ uint8_t s_pk[FW][EW_CAP];    // staged pair: list entry
  __shared__ double s_pv[FW][EW_CAP];     // staged pair: weight
  __shared__ int s_st[FW][32];            // row state * co^3
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const unsigned lt = (1u << lane) - 1u;
  const long long t = (long long)blockIdx.x * EW_WARPS + warp;
  if (t >= n) return;
  const unsigned r0 = estart[t], r1 = estart[t + 1];
  if (r0 == r1) return;
  const long long eo = I.eoff[t];
  const int E = (int)(I.eoff[t + 1] - eo);
  if (E > IMAX_E) return;  // k_elist_fill flagged it; the host throws
  const int kind = I.ekind[t];
  for (int k = lane; k < E; k += 32) {
    s_col[warp][k] = I.lcol[eo + k];
    s_key[warp][k] = I.lkey[eo + k];
  }
  const double *ldw = I.ldw + eo;  // the element's dependent weights (L1)
  const int fw = FILL ? warp : 0;
  const int co = I.co, cn3 = co * co * co;
  for (unsigned b0 = r0; b0 < r1; b0 += 32) {
    const int nb = (int)min(32u, r1 - b0);
    const bool mine = lane < nb;
    int nzc = 0;  // this lane's row: entries the applies keep
    unsigned bm = 0;
    int row = 0;
    long long out = 0, lim = 0;
    __syncwarp();
    if (mine) {
      row = erows[b0 + lane];
      const unsigned long long inf = einfo[b0 + lane];
      bm = (unsigned)inf;
      if (FILL) {
        unsigned sidx = (unsigned)(inf >> 32);
        if (sidx >= (unsigned)UVW_STATES) {
          atomicExch(I.err, 4);  // outside the table: reported, never read
          sidx = 0;
        }
        s_st[fw][lane] = (int)sidx * cn3;
        out = roff[row];
        lim = roff[row + 1];
      }
    }
    __syncwarp();
    if constexpr (!FILL) {
      long long ne = 0;
      if (kind == 0) {
        ne = __popc(bm);
      } else {
        int pcol = -1;
        for (int k = 0; k < E; k++) {
          const int col = s_col[warp][k];
          if ((bm >> (s_key[warp][k] & 31)) & 1u) {
            ne += (kind == 1 || col != pcol);
            pcol = col;
          }
        }
      }
      if (mine) cnt[row] = ne;
    } else if (kind == 0) {
      // E == co^3 <= 27: one list entry per lane
      const int ekey = lane < E ? (s_key[warp][lane] & 31) : 0;
      const int ecol = lane < E ? s_col[warp][lane] : 0;
      for (int r = 0; r < nb; r++) {
        const unsigned rbm = __shfl_sync(0xffffffffu, bm, r);
        const int rs = s_st[fw][r];
        const long long o = __shfl_sync(0xffffffffu, out, r);
        const long long rlim = __shfl_sync(0xffffffffu, lim, r);
        const bool in = lane < E && ((rbm >> ekey) & 1u);
        const unsigned m = __ballot_sync(0xffffffffu, in);
        double v = 0.0;
        if (in) {
          v = __ldg(I.uvw + rs + ekey);
          const long long p = o + __popc(m & lt);
          if (p < rlim) {
            cols[p] = ecol;
            vals[p] = v;
          } else {
            atomicExch(I.err, 3);
          }
        }
        const int kept = __popc(__ballot_sync(0xffffffffu, in && apply_keeps(v)));
        if (lane == r) {
          if (o + __popc(m) != rlim) atomicExch(I.err, 3);
          cnt[row] = kept;
        }
      }
    } else {
      int pcol = -1;
      double acc = 0.0;
      for (int k0 = 0; k0 < E;) {
        // stage entries k0..k1-1 (at most EW_CAP pairs)
        int k1 = k0, nst = 0;
        __syncwarp();
        while (k1 < E && nst + 32 <= EW_CAP) {
          const bool in = (bm >> (s_key[warp][k1] & 31)) & 1u;
          const unsigned m = __ballot_sync(0xffffffffu, in);
          if (in) {
            const int p = nst + __popc(m & lt);
            s_pr[fw][p] = (uint8_t)lane;
            s_pk[fw][p] = (uint8_t)k1;
          }
          if (lane == 0) {
            s_mk[fw][k1] = m;
            s_bk[fw][k1] = (uint16_t)nst;
          }
          nst += __popc(m);
          k1++;
        }
        __syncwarp();
        for (int p = lane; p < nst; p += 32) {
          const int k = s_pk[fw][p];
          const double w = __ldg(I.uvw + s_st[fw][s_pr[fw][p]] + (s_key[warp][k] & 31));
          s_pv[fw][p] = kind == 0 ? w : __dmul_rn(w, __ldg(ldw + k));
        }
        __syncwarp();
        for (int k = k0; k < k1; k++) {
          const unsigned m = s_mk[fw][k];
          const int col = s_col[warp][k];
          const bool in = (m >> lane) & 1u;
          const bool cont = kind == 2 && k > 0 && s_col[warp][k - 1] == col;  // uniform
          if (in) {
            const double v = s_pv[fw][s_bk[fw][k] + __popc(m & lt)];
            if (cont && col == pcol) {
              acc = __dadd_rn(acc, v);
            } else {
              if (pcol >= 0) {
                if (out < lim) {
                  cols[out] = pcol;
                  vals[out] = acc;
                  nzc += apply_keeps(acc);
                } else {
                  atomicExch(I.err, 3);
                }
                out++;
              }
              pcol = col;
              acc = v;
            }
          }
        }
        k0 = k1;
      }
      if (pcol >= 0) {
        if (out < lim) {
          cols[out] = pcol;
          vals[out] = acc;
          nzc += apply_keeps(acc);
        } else {
          atomicExch(I.err, 3);
        }
        out++;
      }
      if (mine && out != lim) atomicExch(I.err, 3);
      if (mine) cnt[row] = nzc;
    }
  }
}

// Entries the applies keep, per row (8 lanes per row).
__global__ void k_nz_count(long long rows, const int *__restrict__ rp,
                           const double *__restrict__ v, long long *cnt) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long r = t >> 3;
  const int g8 = threadIdx.x & 7;
  int c = 0;
  if (r < rows)
    for (int p = __ldg(rp + r) + g8; p < __ldg(rp + r + 1); p += 8) c += apply_keeps(__ldg(v + p));
  c += __shfl_xor_sync(0xffffffffu, c, 1);
  c += __shfl_xor_sync(0xffffffffu, c, 2);
  c += __shfl_xor_sync(0xffffffffu, c, 4);
  if (r < rows && g8 == 0) cnt[r] = c;
}

__global__ void k_ptr32(long long n, const long long *__restrict__ in, int *out) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i <= n) out[i] = (int)in[i];
}

// ---------------------------------------------------------------------
// Double-float arithmetic for the applies.  A value v is carried as two
// floats, hi = v rounded to 24 bits and lo = v - hi rounded to 24 bits
// (|v - hi - lo| <= 2^-48 |v|), and a CSR product sum as a pair (sh, sl)
// updated with an exact product (TwoProduct by FMA) and an exact sum
// (TwoSum), renormalised every four terms.  Measured against exact sums
// on order-3 Gauss-Lobatto prolongations (rows up to 27 entries, transpose
// rows up to 616) the error stays below 3e-14 of max(1, |y|), inside the
// 1e-13 bar, for about 13 FP32 operations per entry and vector instead of
// one FP64 FMA: GB300 issues FP64 at 1/64 of its FP32 rate, which bounds
// an FP64 apply at 2 FMAs per 12 bytes of matrix far below its HBM rate.
//
// The split takes the exponent and mantissa bits apart with integer
// operations (no FP64 instruction).  Values are represented when their
// biased exponent lies in [emin, emin + erange) or they are zero; the
// windows below keep every partial product and sum a normal float.
constexpr unsigned DF_X_EMIN = 1023 - 40, DF_X_ERANGE = 100;  // 2^-40 <= |x| < 2^60
constexpr unsigned DF_W_EMIN = 1023 - 49, DF_W_ERANGE = 66;   // 2^-49 <= |w| < 2^17
__device__ __forceinline__ bool df_split(double v, unsigned emin, unsigned erange, float &hi,
                                         float &lo) {
  const unsigned h = (unsigned)__double2hiint(v), l = (unsigned)__double2loint(v);
  const unsigned E = (h >> 20) & 0x7ffu, sgn = h & 0x80000000u;
  const bool zero = ((h & 0x7fffffffu) | l) == 0u;
  const bool in = (E - emin) < erange;
  // top 24 bits rounded (a carry into the exponent is the correct rounding)
  const unsigned rb = (l >> 28) & 1u;
  const unsigned hb = (sgn | ((((h & 0x7fffffffu) - (896u << 20)) << 3) | (l >> 29))) + rb;
  // the remainder v - hi: the low 29 mantissa bits, less 2^29 when rounded
  // up, in units of 2^(E - 1075)
  const int m = (int)(l & 0x1fffffffu) - (int)(rb << 29);
  const float sc = __uint_as_float(sgn | ((E - 948u) << 23));
  hi = in ? __uint_as_float(hb) : 0.0f;
  lo = in ? __fmul_rn(__int2float_rn(m), sc) : 0.0f;
  return in || zero;
}
// A weight of the apply copy: weights below the window (< 2^-49, the
// apply_keeps residue kept when P has few of them) become 0, which changes
// a row by at most 2^-49 |x| per such entry; weights above it (or Inf/NaN)
// set the flag that sends the applies to FP64.
__device__ __forceinline__ float2 df_weight(double w, int *flag) {
  float hi, lo;
  if (!df_split(w, DF_W_EMIN, DF_W_ERANGE, hi, lo) &&
      ((unsigned)(__double2hiint(w) >> 20) & 0x7ffu) >= DF_W_EMIN + DF_W_ERANGE)
    atomicOr(flag, 1);
  return make_float2(hi, lo);
}
// (sh, sl) += (wh + wl)(xh + xl), the wl xl term (below 2^-48 |w x|) left out.
__device__ __forceinline__ void df_fma(float wh, float wl, float xh, float xl, float &sh,
                                       float &sl) {
  const float p = __fmul_rn(wh, xh);
  const float e = __fmaf_rn(wh, xh, -p);
  const float c = __fmaf_rn(wh, xl, __fmaf_rn(wl, xh, e));
  const float t = __fadd_rn(sh, p);
  const float bp = __fsub_rn(t, sh);
  const float err = __fadd_rn(__fsub_rn(sh, __fsub_rn(t, bp)), __fsub_rn(p, bp));
  sl = __fadd_rn(sl, __fadd_rn(err, c));
  sh = t;
}
__device__ __forceinline__ void df_renorm(float &sh, float &sl) {
  const float t = __fadd_rn(sh, sl);
  sl = __fsub_rn(sl, __fsub_rn(t, sh));
  sh = t;
}
// (sh, sl) += (oh, ol)
__device__ __forceinline__ void df_add(float &sh, float &sl, float oh, float ol) {
  const float t = __fadd_rn(sh, oh);
  const float bp = __fsub_rn(t, sh);
  const float err = __fadd_rn(__fsub_rn(sh, __fsub_rn(t, bp)), __fsub_rn(oh, bp));
  sl = __fadd_rn(sl, __fadd_rn(err, ol));
  sh = t;
  df_renorm(sh, sl);
}
// sh + sl as a double, from the bits with integer operations (the FP64 pipe
// carries no work of the applies but rare special cases).  (sh, sl) is
// normalised, |sl| <= ulp(sh) / 2, so sl lies 24 or more binades below sh:
// the double of sh plus sl in units of the double ulp at sh's exponent
// (exact up to a gap of 29 binades, rounded half away from zero beyond;
// when sh is a power of two and sl has the other sign the result falls
// into the binade below, whose ulp is half as large).
__device__ __forceinline__ double df_value(float sh, float sl) {
  const unsigned bh = __float_as_uint(sh), bl = __float_as_uint(sl);
  const int eh = (int)((bh >> 23) & 0xffu), el = (int)((bl >> 23) & 0xffu);
  if (eh == 0 || eh == 255 || (el == 0 && (bl & 0x7fffffffu) != 0u) || el == 255)
    return __dadd_rn((double)sh, (double)sl);  // zeros/subnormal sh, Inf, NaN
  const unsigned long long hd = ((unsigned long long)(bh & 0x80000000u) << 32) |
                                ((unsigned long long)(eh + 896) << 52) |
                                ((unsigned long long)(bh & 0x7fffffu) << 29);
  if (el == 0) return __longlong_as_double((long long)hd);  // sl = +-0
  const int g = eh - el;
  const bool neg = ((bh ^ bl) >> 31) != 0u;
  const bool pow2 = (bh & 0x7fffffu) == 0u;
  const int sft = (neg && pow2 ? 30 : 29) - g;
  const unsigned long long ml = (unsigned long long)((bl & 0x7fffffu) | 0x800000u);
  unsigned long long d;
  if (sft >= 0)
    d = ml << sft;
  else if (sft > -26)
    d = (ml + (1ULL << (-sft - 1))) >> (-sft);
  else
    d = 0;
  return __longlong_as_double((long long)(neg ? hd - d : hd + d));
}

// The apply copy's weights when it shares P's structure (nnz_nz == nnz).
__global__ void k_df_weights(long long n, const double *__restrict__ v, float2 *w, int *flag) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) w[i] = df_weight(__ldg(v + i), flag);
}
// An apply's input vector as (hi, lo) pairs; flag set when a value lies
// outside the window (that apply then runs in FP64).
__global__ void k_df_split_x(long long n, const double *__restrict__ x, float2 *xs, int *flag) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float hi, lo;
  if (!df_split(__ldg(x + i), DF_X_EMIN, DF_X_ERANGE, hi, lo)) atomicOr(flag, 1);
  xs[i] = make_float2(hi, lo);
}

// The apply copy of P: 8 lanes per row keep the apply_keeps entries in order.
// Each kept entry also gets its transpose sort record: key = column,
// value = its position in the copy, erow = its row (k_t_keys' output).
__global__ void k_nz_fill(long long rows, const int *__restrict__ rp,
                          const int *__restrict__ ci, const double *__restrict__ v,
                          const long long *__restrict__ nzoff, int *nrp, int *nci,
                          float2 *nw, int *flag, uint32_t *tkeys, uint32_t *tvals,
                          int *erow) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long r = t >> 3;
  const int lane = threadIdx.x & 31, g8 = lane & 7, grp = lane >> 3;
  if (((t >> 5) << 2) >= rows) return;  // uniform per warp
  const bool have = r < rows;
  const int p0 = have ? __ldg(rp + r) : 0, p1 = have ? __ldg(rp + r + 1) : 0;
  int trips = (p1 - p0 + 7) >> 3;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) trips = max(trips, __shfl_xor_sync(0xffffffffu, trips, o));
  long long o = have ? nzoff[r] : 0;
  const long long lim = have ? nzoff[r + 1] : 0;
  for (int it = 0; it < trips; it++) {
    const int p = p0 + it * 8 + g8;
    const bool on = have && p < p1;
    const double w = on ? __ldg(v + p) : 0.0;
    const bool nz = on && apply_keeps(w);
    const unsigned mg = (__ballot_sync(0xffffffffu, nz) >> (grp * 8)) & 0xffu;
    if (nz) {
      const long long d = o + __popc(mg & ((1u << g8) - 1u));
      if (d < lim) {
        const int c = __ldg(ci + p);
        nci[d] = c;
        nw[d] = df_weight(w, flag);
        tkeys[d] = (uint32_t)c;
        tvals[d] = (uint32_t)d;
        erow[d] = (int)r;
      }
    }
    o += __popc(mg);
  }
  if (have && g8 == 0) nrp[r] = (int)nzoff[r];
  if (have && g8 == 0 && r == rows - 1) nrp[rows] = (int)nzoff[rows];
}

// Transpose support.  Entries are keyed row << 32 | column; the stable
// sort runs on the column bits only, so rows stay ascending inside each
// column (the entries arrive row-major) with a third of the passes a full
// (column, row) key would take.  8 lanes per row write its entries.
__global__ void k_t_keys(long long rows, const int *__restrict__ rowptr,
                         const int *__restrict__ cols, uint32_t *keys, uint32_t *vals,
                         int *erow) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  long long r = t >> 3;
  if (r >= rows) return;
  int lane = (int)(t & 7);
  for (int p = rowptr[r] + lane; p < rowptr[r + 1]; p += 8) {
    keys[p] = (uint32_t)cols[p];
    vals[p] = (uint32_t)p;
    erow[p] = (int)r;
  }
}
__global__ void k_t_fill(long long nnz, const uint32_t *__restrict__ keys,
                         const uint32_t *__restrict__ perm, const int *__restrict__ erow,
                         const float2 *__restrict__ vals, int *tcols, float2 *tvals,
                         int *trowptr) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nnz) return;
  const uint32_t p = perm[i];
  tcols[i] = erow[p];
  tvals[i] = vals[p];
  // column starts: every column in (previous column, this column] begins here
  int c = (int)keys[i];
  int cprev = (i == 0) ? -1 : (int)keys[i - 1];
  for (int j = cprev + 1; j <= c; j++) trowptr[j] = (int)i;
}
__global__ void k_t_tail(long long ncols, long long nnz, const uint32_t *__restrict__ keys,
                         int *trowptr) {
  // columns after the last entry's column are empty
  long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  int clast = nnz ? (int)keys[nnz - 1] : -1;
  if (j > clast && j <= ncols) trowptr[j] = (int)nnz;
}
// Rows ordered by length inside windows of LO_WIN rows (one block per
// window, counting sort on min(length, LO_BUCKETS - 1)); the order inside a
// bucket does not matter, each row's sum is independent of it.
constexpr int LO_WIN = 4096, LO_BUCKETS = 256, LO_THREADS = 256;
// input chunks of a host-buffer transpose apply: the copy of chunk k+1
// overlaps the rows whose inputs lie in chunks <= k
constexpr int TC_CHUNKS = 16;
static_assert(TC_CHUNKS < 32, "k_chunk_bounds runs one warp");
__global__ void __launch_bounds__(LO_THREADS)
    k_len_order(long long rows, const int *__restrict__ rp, const int *__restrict__ list,
                int *perm) {
  __shared__ int s_cnt[LO_BUCKETS], s_off[LO_BUCKETS];
  const long long w0 = (long long)blockIdx.x * LO_WIN;
  for (int i = threadIdx.x; i < LO_BUCKETS; i += LO_THREADS) s_cnt[i] = 0;
  __syncthreads();
  int b[LO_WIN / LO_THREADS];
#pragma unroll
  for (int k = 0; k < LO_WIN / LO_THREADS; k++) {
    const long long r = w0 + threadIdx.x + k * LO_THREADS;
    b[k] = -1;
    if (r < rows) {
      const int row = list ? __ldg(list + r) : (int)r;
      b[k] = min(__ldg(rp + row + 1) - __ldg(rp + row), LO_BUCKETS - 1);
      atomicAdd(&s_cnt[b[k]], 1);
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    int a = 0;
    for (int i = 0; i < LO_BUCKETS; i++) {
      s_off[i] = a;
      a += s_cnt[i];
    }
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < LO_WIN / LO_THREADS; k++)
    if (b[k] >= 0) {
      const long long r = w0 + threadIdx.x + k * LO_THREADS;
      perm[w0 + atomicAdd(&s_off[b[k]], 1)] = list ? __ldg(list + r) : (int)r;
    }
}
void len_order(long long rows, const int *rp, int *perm, cudaStream_t s) {
  launch(k_len_order, blocks_for(rows, LO_WIN), LO_THREADS, 0, s, rows, rp, (const int *)nullptr,
         perm);
}

// P^T rows keyed by the input chunk holding their last (largest) input
// row: chunk = last_row * TC_CHUNKS / n_in, empty rows in chunk 0.
__global__ void k_t_chunk_keys(long long ncols, long long nin, const int *__restrict__ trp,
                               const int *__restrict__ tci, uint64_t *keys, uint32_t *vals) {
  long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncols) return;
  const int p0 = trp[c], p1 = trp[c + 1];
  const long long last = p1 > p0 ? tci[p1 - 1] : 0;
  keys[c] = (uint64_t)((last * TC_CHUNKS) / (nin > 0 ? nin : 1));
  vals[c] = (uint32_t)c;
}
// Start of each chunk's run in the sorted chunk keys: bounds[k] = the first
// position whose key is >= k (lower bound), for k = 0..nk.
__global__ void k_chunk_bounds(long long n, const uint64_t *__restrict__ keys, int nk,
                               long long *bounds) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k > nk) return;
  long long lo = 0, hi = n;
  while (lo < hi) {
    const long long mid = (lo + hi) >> 1;
    if (keys[mid] < (uint64_t)k) lo = mid + 1; else hi = mid;
  }
  bounds[k] = lo;
}
__global__ void k_rowsum(long long rows, const int *__restrict__ rowptr,
                         const float2 *__restrict__ vals, double *sum) {
  long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= rows) return;
  double s = 0.0;
  for (int p = rowptr[r]; p < rowptr[r + 1]; p++) {
    const float2 w = vals[p];
    s = __dadd_rn(s, __dadd_rn((double)w.x, (double)w.y));
  }
  sum[r] = s;
}

// findEnclosing (TMROctForest.cpp:6228-6377) for a batch of nodes: each
// node is an element octant with `info` = its local node index in an
// element of `order` with `knots`; the result is the index of the octant of
// this forest the reference returns, or -1 where it returns NULL.
__global__ void k_find_enclosing_batch(long long n, InterpCtx I, const tmrg_octant *nodes,
                                       long long *out) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const tmrg_octant q = nodes[i];
  const Oct node{q.block, q.x, q.y, q.z, q.level};
  out[i] = find_enclosing(I, node, q.info);
}

void forest_find_enclosing(Forest &f, int order, const double *knots,
                           const tmrg_octant *d_nodes, long long n, long long *d_index) {
  if (!f.have_octs) throw Error(TMRG_ERR_STATE, "findEnclosing: no octants");
  if (order < 2 || order > TMRG_MAX_ORDER)
    throw Error(TMRG_ERR_ARG, "findEnclosing: order out of range");
  if (f.conn->nb >= (1 << 26))
    throw Error(TMRG_ERR_KEY_RANGE, "findEnclosing: more than 2^26 blocks");
  cudaStream_t s = f.s;
  InterpCtx c{};
  c.fo = order;
  for (int k = 0; k < TMRG_MAX_ORDER; k++) c.fk1[k] = k < order ? 1.0 + knots[k] : 0.0;
  c.cn = f.n;
  DBuf<int4> c4(f.n + 1, s);
  launch(k_pack_octs, blocks_for(f.n, 256), 256, 0, s, f.n, (const int *)f.block.p,
         (const int *)f.x.p, (const int *)f.y.p, (const int *)f.z.p,
         (const int16_t *)f.level.p, c4.p);
  c.c4 = c4.p;
  launch(k_find_enclosing_batch, blocks_for(n, 256), 256, 0, s, n, c, d_nodes, d_index);
  TMRG_CUDA(cudaStreamSynchronize(s));
}

void interp_finish(Interp &I, long long nonzeros, cudaStream_t s, const long long *keepoff);

// ---------------------------------------------------------------------
// The general createInterpolation path: any fine and coarse order up to
// TMRG_MAX_ORDER, Lagrange (uniform or Gauss-Lobatto knots) or Bernstein
// elements.  The specialised kernels above cover coarse orders 2-3 with
// Lagrange bases, the multigrid hierarchies that dominate the runtime;
// this path serves the rest (coarse order 4+, the Bernstein element
// hierarchies of the reference's topology-optimisation drivers).
//
// One warp per row, in two passes with the same row construction (count,
// then write at the scanned offsets).  A row is built as computeElemInterp
// builds it (TMROctForest.cpp:6396-6594): the three directions' 1-D weights
// of the enclosing coarse element, the tensor-product entries in (kk, jj,
// ii) order with each dependent coarse node expanded through its CSR row,
// then uniqueSort (TMRBase.h:110-133): a stable sort by column and the
// in-order sum of equal columns.
struct GenInterp {
  int bern;  // Bernstein elements
  // design -> analysis weights (computeWeights): the Bernstein basis is
  // evaluated at u whatever the two orders (evalInterp)
  int topo;
  // eval_bernstein_interp_weights rows (fine order = coarse order + 1):
  // bel[u] are the coarse weights of fine control point u
  double bel[TMRG_MAX_ORDER][TMRG_MAX_ORDER];
  int cnpe;
  const int *conn, *dptr, *dconn;  // coarse element connectivity, dependent CSR
  const double *dw;
  int cap;  // staged entries per warp
};

// The direction's index range of computeElemInterp: [s, e) with the face
// hits that keep a single coarse index.
__device__ __forceinline__ void gen_range(int i, int mo, int co, int32_t nx, int32_t h,
                                          int32_t ox, int32_t hc, int &s, int &e) {
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

// The direction's 1-D weights (N[s] = 1 at a face hit).  Lagrange:
// lagrange_shape_functions (TMRInterpolation.h:40-52) at the coarse knots;
// Bernstein: bernstein_shape_functions (:164-177) when the orders agree,
// else the degree-elevation row of the fine index.  u as the reference
// rounds it: 0.5 h and 2 / hc are powers of two, so those scalings are
// exact.
__device__ void gen_weights(const InterpCtx &I, const GenInterp &G, int i, int s, int e,
                            int32_t nx, int32_t h, int32_t ox, int32_t hc, double *N) {
  const int co = I.co;
  if (e - s == 1) {
    N[s] = 1.0;
    return;
  }
  if (G.bern && !G.topo && I.fo != co) {
    for (int a = 0; a < co; a++) N[a] = G.bel[i][a];
    return;
  }
  const double t = __dadd_rn(exact_double(nx), __dmul_rn(0.5 * (double)h, I.fk1[i]));
  const double u = __dadd_rn(-1.0, __dmul_rn(__dsub_rn(t, exact_double(ox)),
                                             2.0 / (double)hc));
  if (G.bern) {
    const double u1 = __dmul_rn(0.5, __dsub_rn(1.0, u));
    const double u2 = __dmul_rn(0.5, __dadd_rn(u, 1.0));
    N[0] = 1.0;
    for (int j = 1; j < co; j++) {
      double sum = 0.0;
      for (int k = 0; k < j; k++) {
        const double tk = N[k];
        N[k] = __dadd_rn(sum, __dmul_rn(u1, tk));
        sum = __dmul_rn(u2, tk);
      }
      N[j] = sum;
    }
    return;
  }
  for (int a = 0; a < co; a++) {
    double v = 1.0;
    for (int b = 0; b < co; b++)
      if (a != b) v = __dmul_rn(v, __dmul_rn(__dsub_rn(u, I.ck[b]), I.crk[a][b]));
    N[a] = v;
  }
}

// findEnclosing for every row (one thread per row).
__global__ void k_gen_find(long long rows, InterpCtx I, int *trow) {
  const long long row = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (row >= rows) return;
  const unsigned long long rr = I.rep[row];
  const long long e = (long long)(rr >> 8);
  const Oct node{I.fb[e], I.fx[e], I.fy[e], I.fz[e], I.fl[e]};
  const long long t = find_enclosing(I, node, (int)(rr & 255u));
  if (t < 0) atomicExch(I.err, 1);
  trow[row] = (int)t;
}

// Element expansion length bound: the largest sum of dependent row lengths
// over one coarse element's nodes.
__global__ void k_gen_emax(long long n, int cnpe, const int *__restrict__ conn,
                           const int *__restrict__ dptr, int *emax) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const int *c = conn + t * cnpe;
  int e = 0;
  for (int l = 0; l < cnpe; l++) {
    const int cv = __ldg(c + l);
    e += (cv >= 0) ? 1 : (__ldg(dptr - cv) - __ldg(dptr - cv - 1));
  }
  atomicMax(emax, e);
}

// WRITE = false: cnt[row] = merged entries of the row.  WRITE = true: the
// row's entries at off[row] (and nzcount += its apply_keeps entries).
// Dynamic shared memory: per warp, 2 * cap (column, weight) slots.
constexpr int GEN_WARPS = 4;
template <bool WRITE>
__global__ void __launch_bounds__(GEN_WARPS * 32)
    k_gen_rows(long long rows, InterpCtx I, GenInterp G, const int *__restrict__ trow,
               long long *cnt_off, int *cols, double *vals, unsigned long long *nzcount) {
  extern __shared__ unsigned char gen_smem[];
  __shared__ double s_N[GEN_WARPS][3][TMRG_MAX_ORDER];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const long long row = (long long)blockIdx.x * GEN_WARPS + warp;
  if (row >= rows) return;
  const int cap = G.cap;
  int *c0 = (int *)gen_smem + (size_t)warp * 2 * cap;
  int *c1 = c0 + cap;
  double *w0 = (double *)((int *)gen_smem + (size_t)GEN_WARPS * 2 * cap) + (size_t)warp * 2 * cap;
  double *w1 = w0 + cap;
  const int t = trow[row];
  if (t < 0) {
    if (!WRITE && lane == 0) cnt_off[row] = 0;
    return;
  }
  const int mo = I.fo, co = I.co;
  const unsigned long long rr = I.rep[row];
  const long long e = (long long)(rr >> 8);
  const int info = (int)(rr & 255u);
  const int32_t nx[3] = {I.fx[e], I.fy[e], I.fz[e]};
  const int32_t h = side_of(I.fl[e]);
  const int4 cq = __ldg(I.c4 + t);
  const int32_t hc = side_of(cq.x >> 26);
  const int32_t ox[3] = {cq.y, cq.z, cq.w};
  const int idx[3] = {info % mo, (info % (mo * mo)) / mo, info / (mo * mo)};
  int rs[3], re[3];
  for (int d = 0; d < 3; d++) gen_range(idx[d], mo, co, nx[d], h, ox[d], hc, rs[d], re[d]);
  if (lane < 3)
    gen_weights(I, G, idx[lane], rs[lane], re[lane], nx[lane], h, ox[lane], hc,
                s_N[warp][lane]);
  __syncwarp();
  // entries in computeElemInterp's loop order
  const int ni = re[0] - rs[0], nj = re[1] - rs[1], nk = re[2] - rs[2];
  const int npos = ni * nj * nk;
  const int *cc = G.conn + (long long)t * G.cnpe;
  int total = 0;
  for (int q0 = 0; q0 < npos; q0 += 32) {
    const int q = q0 + lane;
    int cv = 0, len = 0, d0 = 0;
    double w = 0.0;
    if (q < npos) {
      const int ii = rs[0] + q % ni, jj = rs[1] + (q / ni) % nj, kk = rs[2] + q / (ni * nj);
      w = __dmul_rn(__dmul_rn(s_N[warp][0][ii], s_N[warp][1][jj]), s_N[warp][2][kk]);
      cv = __ldg(cc + ii + jj * co + kk * co * co);
      if (cv >= 0) {
        len = 1;
      } else {
        d0 = __ldg(G.dptr - cv - 1);
        len = __ldg(G.dptr - cv) - d0;
      }
    }
    int incl = len;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += y;
    }
    const int off = total + incl - len;
    if (off + len <= cap) {
      if (cv >= 0 && len) {
        c0[off] = cv;
        w0[off] = w;
      } else {
        for (int p = 0; p < len; p++) {
          c0[off + p] = __ldg(G.dconn + d0 + p);
          w0[off + p] = __dmul_rn(w, __ldg(G.dw + d0 + p));
        }
      }
    }
    total += __shfl_sync(0xffffffffu, incl, 31);
  }
  if (total > cap) {
    if (lane == 0) atomicExch(I.err, 5);
    if (!WRITE && lane == 0) cnt_off[row] = 0;
    return;
  }
  __syncwarp();
  // stable rank sort by column
  for (int a = lane; a < total; a += 32) {
    const int col = c0[a];
    int rk = 0;
    for (int b = 0; b < total; b++) {
      const int cb = c0[b];
      rk += (cb < col) || (cb == col && b < a);
    }
    c1[rk] = col;
    w1[rk] = w0[a];
  }
  __syncwarp();
  // run heads, their rank among heads, and the in-order run sums
  const long long base = WRITE ? cnt_off[row] : 0;
  int heads = 0, kept = 0;
  for (int a0 = 0; a0 < total; a0 += 32) {
    const int a = a0 + lane;
    const bool head = a < total && (a == 0 || c1[a] != c1[a - 1]);
    const unsigned hb = __ballot_sync(0xffffffffu, head);
    if (WRITE && head) {
      double v = w1[a];
      for (int b = a + 1; b < total && c1[b] == c1[a]; b++) v = __dadd_rn(v, w1[b]);
      const long long o = base + heads + __popc(hb & ((1u << lane) - 1u));
      cols[o] = c1[a];
      vals[o] = v;
      kept += apply_keeps(v);
    }
    heads += __popc(hb);
  }
  if (WRITE) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) kept += __shfl_xor_sync(0xffffffffu, kept, o);
    if (lane == 0 && kept) atomicAdd(nzcount, (unsigned long long)kept);
  } else if (lane == 0) {
    cnt_off[row] = heads;
  }
}

// eval_bernstein_interp_weights (TMRInterpolation.h:441-560) as the
// reference tabulates it, for fine order = coarse order + 1, coarse orders
// 2-5.  The coarse-order-4 rows for u = 2 and u = 3 are reproduced as the
// reference writes them (they are the natural degree-elevation rows of
// u = 3 and u = 2).
static void bernstein_elevation(int mo, int co, double (*N)[TMRG_MAX_ORDER]) {
  for (int u = 0; u < TMRG_MAX_ORDER; u++)
    for (int i = 0; i < TMRG_MAX_ORDER; i++) N[u][i] = 0.0;
  for (int u = 0; u < mo; u++) {
    double *r = N[u];
    if (u == 0) {
      r[0] = 1.0;
    } else if (u == mo - 1) {
      r[co - 1] = 1.0;
    } else if (co == 2) {
      r[0] = 0.5;
      r[1] = 0.5;
    } else if (co == 3) {
      r[u - 1] = (u == 1) ? 1. / 3 : 2. / 3;
      r[u] = (u == 1) ? 2. / 3 : 1. / 3;
    } else if (co == 4) {
      if (u == 1) {
        r[0] = 0.25;
        r[1] = 0.75;
      } else if (u == 2) {
        r[2] = 0.75;
        r[3] = 0.25;
      } else {
        r[1] = 0.5;
        r[2] = 0.5;
      }
    } else {
      const double a[4][2] = {{0.2, 0.8}, {0.4, 0.6}, {0.6, 0.4}, {0.8, 0.2}};
      r[u - 1] = a[u - 1][0];
      r[u] = a[u - 1][1];
    }
  }
}

// Rows of P by the general path: I.rows rows whose (element, local node)
// are in c.rep, the coarse forest's elements in c; G.bern, G.topo and
// G.bel set by the caller.
static void interp_rows_general(Forest &coarse, Interp &I, InterpCtx &c, GenInterp G,
                                DBuf<int> &err, cudaStream_t s) {
  const long long rows = I.rows;
  G.cnpe = coarse.order * coarse.order * coarse.order;
  G.conn = coarse.econn.p;
  G.dptr = coarse.dep_ptr.p;
  G.dconn = coarse.dep_conn.p;
  G.dw = coarse.dep_w.p;
  DBuf<int> emax(1, s);
  emax.zero();
  launch(k_gen_emax, blocks_for(coarse.n, 256), 256, 0, s, coarse.n, G.cnpe,
         (const int *)coarse.econn.p, (const int *)coarse.dep_ptr.p, emax.p);
  const int em = read_scalar(emax.p, s);
  G.cap = std::max(32, (em + 31) / 32 * 32);
  const size_t smem = (size_t)GEN_WARPS * 2 * G.cap * (sizeof(int) + sizeof(double));
  if (smem > 200 * 1024)
    throw Error(TMRG_ERR_UNSUPPORTED,
                "createInterpolation: a coarse element expands to " + std::to_string(em) +
                    " entries, beyond the general path's shared-memory stage");
  TMRG_CUDA(cudaFuncSetAttribute(k_gen_rows<false>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  TMRG_CUDA(cudaFuncSetAttribute(k_gen_rows<true>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  DBuf<int> trow(rows + 1, s);
  DBuf<long long> roff(rows + 1, s);
  launch(k_gen_find, blocks_for(rows, 128), 128, 0, s, rows, c, trow.p);
  launch(k_gen_rows<false>, blocks_for(rows, GEN_WARPS), GEN_WARPS * 32, smem, s, rows, c, G,
         (const int *)trow.p, roff.p, (int *)nullptr, (double *)nullptr,
         (unsigned long long *)nullptr);
  exclusive_scan<long long>(roff.p, roff.p, rows, s);
  const long long nnz = read_scalar(roff.p + rows, s);
  const int e = read_scalar(err.p, s);
  if (e == 5)
    throw Error(TMRG_ERR_INTERNAL, "createInterpolation: a row outgrew its element bound");
  if (e)
    throw Error(TMRG_ERR_INTERNAL,
                "createInterpolation: a fine node has no enclosing coarse octant");
  if (nnz >= (1LL << 31) - 1)
    throw Error(TMRG_ERR_ARG, "createInterpolation: more than 2^31 entries");
  I.nnz = nnz;
  I.rowptr.alloc(rows + 1, s);
  launch(k_ptr32, blocks_for(rows + 1, 256), 256, 0, s, rows, (const long long *)roff.p,
         I.rowptr.p);
  I.colidx.alloc(nnz + 1, s);
  I.vals.alloc(nnz + 1, s);
  DBuf<unsigned long long> nzcount(1, s);
  nzcount.zero();
  prof_bytes(12 * nnz + 20 * rows);
  launch(k_gen_rows<true>, blocks_for(rows, GEN_WARPS), GEN_WARPS * 32, smem, s, rows, c, G,
         (const int *)trow.p, roff.p, I.colidx.p, I.vals.p, nzcount.p);
  const long long nonzeros = (long long)read_scalar(nzcount.p, s);
  trow.release();
  roff.release();
  interp_finish(I, nonzeros, s, nullptr);
}

// Sorted expansion lists of every element of `coarse` (k_elist_*).
struct ElemLists {
  long long total = 0;  // entries of all lists
  DBuf<long long> eoff;
  DBuf<int> lcol;
  DBuf<double> ldw;
  DBuf<uint8_t> lkey, ekind;
};
static void build_elists(Forest &coarse, ElemLists &L, int *err, cudaStream_t s) {
  const int cnpe = coarse.order * coarse.order * coarse.order;
  L.eoff.alloc(coarse.n + 1, s);
  launch(k_elist_count, blocks_for(coarse.n, 256), 256, 0, s, coarse.n, cnpe,
         (const int *)coarse.econn.p, (const int *)coarse.dep_ptr.p, L.eoff.p);
  exclusive_scan<long long>(L.eoff.p, L.eoff.p, coarse.n, s);
  const long long ne = read_scalar(L.eoff.p + coarse.n, s);
  L.total = ne;
  L.lcol.alloc(ne + 1, s);
  L.ldw.alloc(ne + 1, s);
  L.lkey.alloc(ne + 1, s);
  L.ekind.alloc(coarse.n + 1, s);
  launch(k_elist_fill, blocks_for(coarse.n, EL_WARPS), EL_WARPS * 32, 0, s, coarse.n, cnpe,
         (const int *)coarse.econn.p, (const int *)coarse.dep_ptr.p,
         (const int *)coarse.dep_conn.p, (const double *)coarse.dep_w.p,
         (const long long *)L.eoff.p, L.lcol.p, L.ldw.p, L.lkey.p, L.ekind.p, err);
}
void interp_create(Forest &fine, Forest &coarse, Interp &I) {
  Stage st("tmrg_create_interpolation");
  if (&fine == &coarse)
    throw Error(TMRG_ERR_ARG, "Cannot interpolate between the same object");
  if (fine.interp != coarse.interp)
    throw Error(TMRG_ERR_ARG,
                "Interpolation types between meshes are not identical");
  // coarse orders above 3 and Bernstein elements take the general path
  const bool general = coarse.order > IMAX_CO || fine.interp == TMRG_BERNSTEIN_POINTS;
  forest_create_nodes(fine);
  forest_create_nodes(coarse);
  TMRG_CUDA(cudaStreamSynchronize(coarse.s));
  cudaStream_t s = fine.s;
  I.s = s;
  I.have_colsum = false;
  I.colsum.release();
  const int fnpe = fine.order * fine.order * fine.order;
  const int cnpe = coarse.order * coarse.order * coarse.order;
  const long long rows = fine.num_owned;
  I.rows = rows;
  I.cols = coarse.num_owned;
  DBuf<unsigned long long> rep(rows + 1, s);
  rep.fill_bytes(0xff);
  launch(k_first_ref, blocks_for(fine.n, 256), 256, 0, s, fine.n, fnpe, rows,
         (const int *)fine.econn.p, rep.p);
  DBuf<int> err(1, s);
  err.zero();
  InterpCtx c;
  c.fo = fine.order;
  c.co = coarse.order;
  for (int i = 0; i < TMRG_MAX_ORDER; i++) {
    c.fk1[i] = 1.0 + fine.knots[i];
    c.ck[i] = coarse.knots[i];
  }
  c.fb = fine.block.p;
  c.fx = fine.x.p;
  c.fy = fine.y.p;
  c.fz = fine.z.p;
  c.fl = fine.level.p;
  c.cn = coarse.n;
  if (coarse.conn->nb >= (1 << 26))
    throw Error(TMRG_ERR_KEY_RANGE, "createInterpolation: more than 2^26 blocks");
  DBuf<int4> c4(coarse.n, s);
  launch(k_pack_octs, blocks_for(coarse.n, 256), 256, 0, s, coarse.n,
         (const int *)coarse.block.p, (const int *)coarse.x.p,
         (const int *)coarse.y.p, (const int *)coarse.z.p,
         (const int16_t *)coarse.level.p, c4.p);
  c.c4 = c4.p;
  c.rep = rep.p;
  c.err = err.p;
  for (int i = 0; i < TMRG_MAX_ORDER; i++)
    for (int j = 0; j < TMRG_MAX_ORDER; j++)
      c.crk[i][j] = (i != j && i < coarse.order && j < coarse.order)
                        ? 1.0 / (coarse.knots[i] - coarse.knots[j])
                        : 0.0;
  if (general) {
    GenInterp G{};
    G.bern = fine.interp == TMRG_BERNSTEIN_POINTS;
    if (G.bern && fine.order != coarse.order) {
      if (fine.order - coarse.order != 1 || coarse.order > 5)
        throw Error(TMRG_ERR_UNSUPPORTED,
                    "createInterpolation: Bernstein meshes must have equal orders or a "
                    "fine order one above a coarse order of 2-5");
      bernstein_elevation(fine.order, coarse.order, G.bel);
    }
    interp_rows_general(coarse, I, c, G, err, s);
    return;
  }
  // sorted expansion list of every coarse element
  ElemLists EL;
  build_elists(coarse, EL, err.p, s);
  c.eoff = EL.eoff.p;
  c.lcol = EL.lcol.p;
  c.ldw = EL.ldw.p;
  c.lkey = EL.lkey.p;
  c.ekind = EL.ekind.p;
  // direction states (dir_state): fine orders 2 and 3, 1 + each fine knot
  // within 2^-53 of 0, 1 or 2, at most one inexact, and the tie of an
  // inexact knot one level below rounding to -1/2 as on the device
  bool states = fine.order <= 3;
  double fk1odd = 1.0;
  c.fodd = 0;
  for (int i = 0; i < TMRG_MAX_ORDER; i++) {
    const double k1 = c.fk1[i];
    const double r = k1 < 0.5 ? 0.0 : (k1 < 1.5 ? 1.0 : 2.0);
    c.fk1i[i] = (int)r;
    if (i >= fine.order) continue;
    if (std::fabs(k1 - r) > std::ldexp(1.0, -53)) states = false;
    if (k1 != r) {
      c.fodd |= 1 << i;
      fk1odd = k1;
    }
  }
  if (__builtin_popcount((unsigned)c.fodd) > 1) states = false;
  if (c.fodd) {
    volatile double tt = std::ldexp(1.0, TMRG_MAX_LEVEL - 12) * fk1odd;  // lf = 11
    volatile double x = tt * std::ldexp(1.0, 11 - TMRG_MAX_LEVEL);        // lc = 10
    volatile double u = -1.0 + x;
    if (u != -0.5) states = false;
  }
  DBuf<int> wide(1, s);
  wide.zero();
  c.wide = wide.p;
  // enclosing octants and exact row lengths, then the rows: grouped by
  // coarse element where the direction states cover every row, else one
  // warp per 32 consecutive rows
  DBuf<int> trow(rows + 1, s);
  DBuf<long long> roff(rows + 1, s);
  DBuf<unsigned> estart;
  DBuf<int> erows;
  DBuf<unsigned long long> rinfo, einfo;  // per row: box mask | states << 32
  // a warp per coarse element pays off when the elements enclose enough
  // rows to fill it (order 3: about 29 per element; order 2: about 8, where
  // the per-row kernel is faster)
  states = states && rows >= 16LL * coarse.n;
  if (states) {
    estart.alloc(coarse.n + 1, s);
    estart.zero();
    rinfo.alloc(rows + 1, s);
    launch(k_interp_find, blocks_for(rows, 128), 128, 0, s, rows, c, trow.p, estart.p,
           rinfo.p);
    states = read_scalar(wide.p, s) == 0 && read_scalar(err.p, s) == 0;
  }
  if (states) {
    exclusive_scan<unsigned>(estart.p, estart.p, coarse.n, s);
    DBuf<unsigned> ecur(coarse.n + 1, s);
    ecur.zero();
    erows.alloc(rows + 1, s);
    einfo.alloc(rows + 1, s);
    launch(k_group_rows, blocks_for(rows, 256), 256, 0, s, rows, (const int *)trow.p,
           (const unsigned long long *)rinfo.p, (const unsigned *)estart.p, ecur.p, erows.p,
           einfo.p);
    rinfo.release();
    // compulsory traffic of the count pass: per row its group slot, box
    // and count (20 B); per coarse element its row range, list offset and
    // kind (13 B) and its list's columns and keys
    prof_bytes(20 * rows + 13 * coarse.n + 5 * EL.total);
    launch(k_interp_elem<false>, blocks_for(coarse.n, EW_WARPS), EW_WARPS * 32, 0, s, coarse.n,
           c, (const unsigned *)estart.p, (const int *)erows.p,
           (const unsigned long long *)einfo.p, roff.p, (const long long *)nullptr,
           (int *)nullptr, (double *)nullptr);
  } else {
    launch(k_interp_count, blocks_for(rows, 128), 128, 0, s, rows, c, trow.p, roff.p);
  }
  exclusive_scan<long long>(roff.p, roff.p, rows, s);
  const long long nnz = read_scalar(roff.p + rows, s);
  const int e = read_scalar(err.p, s);
  if (e == 2)
    throw Error(TMRG_ERR_INTERNAL,
                "createInterpolation: a coarse element expands to more than 256 entries");
  if (e)
    throw Error(TMRG_ERR_INTERNAL,
                "createInterpolation: a fine node has no enclosing coarse octant");
  if (nnz >= (1LL << 31) - 1)
    throw Error(TMRG_ERR_ARG, "createInterpolation: more than 2^31 entries");
  I.nnz = nnz;
  I.rowptr.alloc(rows + 1, s);
  launch(k_ptr32, blocks_for(rows + 1, 256), 256, 0, s, rows, (const long long *)roff.p,
         I.rowptr.p);
  I.colidx.alloc(nnz + 1, s);
  I.vals.alloc(nnz + 1, s);
  DBuf<unsigned long long> nzcount(1, s);
  nzcount.zero();
  DBuf<double> uvw;
  DBuf<long long> keep;  // per row: entries the applies keep
  if (states) {
    const int nt = UVW_STATES * cnpe;
    uvw.alloc(nt, s);
    launch(k_uvw_table, blocks_for(nt, 128), 128, 0, s, c, fk1odd, uvw.p);
    c.uvw = uvw.p;
    keep.alloc(rows + 1, s);
    // compulsory traffic of the fill: the CSR entries written (12 B each);
    // per row its group slot, box and states, offsets and kept count
    // (36 B); per coarse element 13 B and its list (column, key, dependent
    // weight: 13 B an entry)
    prof_bytes(12 * nnz + 36 * rows + 13 * coarse.n + 13 * EL.total);
    launch(k_interp_elem<true>, blocks_for(coarse.n, EW_WARPS), EW_WARPS * 32, 0, s, coarse.n, c,
           (const unsigned *)estart.p, (const int *)erows.p,
           (const unsigned long long *)einfo.p, keep.p, (const long long *)roff.p, I.colidx.p,
           I.vals.p);
  } else {
    c.uvw = nullptr;
    prof_bytes(12 * nnz + 20 * rows);
    launch(k_interp_rows, blocks_for(rows, IW_WARPS * 32), IW_WARPS * 32, 0, s, rows, c,
           (const int *)trow.p, (const long long *)roff.p, I.colidx.p, I.vals.p, nzcount.p);
  }
  trow.release();
  roff.release();
  estart.release();
  erows.release();
  einfo.release();
  EL = ElemLists();
  c4.release();
  rep.release();
  long long nonzeros;
  if (states) {
    // the per-row counts become the apply copy's offsets
    exclusive_scan<long long>(keep.p, keep.p, rows, s);
    nonzeros = read_scalar(keep.p + rows, s);
  } else {
    nonzeros = (long long)read_scalar(nzcount.p, s);
  }
  const int e2 = read_scalar(err.p, s);
  if (e2 == 4)
    throw Error(TMRG_ERR_INTERNAL, "createInterpolation: a direction state is out of range");
  if (e2)
    throw Error(TMRG_ERR_INTERNAL, "createInterpolation: a row outgrew its counted length");
  interp_finish(I, nonzeros, s, states ? keep.p : nullptr);
}

// The apply structures of a finished P (rows, cols, nnz, rowptr, colidx,
// vals set): the apply copy without numerically-zero entries, the length-ordered
// row permutation and P^T.
void interp_finish(Interp &I, long long nonzeros, cudaStream_t s, const long long *keepoff) {
  const long long rows = I.rows, nnz = I.nnz;
  I.win_maxcol.clear();  // made again by the first host-buffer prolongation
  // the apply copy (apply_keeps entries), worth a second copy only when the
  // dropped entries are a good part of P
  I.nnz_nz = (nnz - nonzeros) * 8 >= nnz ? nonzeros : nnz;
  const long long nnz_nz = I.nnz_nz;
  I.dfflag.alloc(3, s);  // [0] weights, [1] inputs outside the double-float window, [2] TMA wait
  I.dfflag.zero();
  I.ap_w.alloc(nnz_nz + 1, s);
  // transpose sort records (column key, position, row) of every apply entry
  DBuf<uint32_t> tk(nnz_nz + 1, s);
  DBuf<uint32_t> tp(nnz_nz + 1, s);
  DBuf<int> erow(nnz_nz + 1, s);
  if (I.nnz_nz == nnz) {
    launch(k_df_weights, blocks_for(nnz, 256), 256, 0, s, nnz, (const double *)I.vals.p,
           I.ap_w.p, I.dfflag.p);
    launch(k_t_keys, blocks_for(rows * 8, 256), 256, 0, s, rows, (const int *)I.rowptr.p,
           (const int *)I.colidx.p, tk.p, tp.p, erow.p);
  }
  if (I.nnz_nz < nnz) {
    DBuf<long long> nzoff;
    if (!keepoff) {
      nzoff.alloc(rows + 1, s);
      launch(k_nz_count, blocks_for(rows * 8, 256), 256, 0, s, rows, (const int *)I.rowptr.p,
             (const double *)I.vals.p, nzoff.p);
      exclusive_scan<long long>(nzoff.p, nzoff.p, rows, s);
      keepoff = nzoff.p;
    }
    I.nz_rowptr.alloc(rows + 1, s);
    I.nz_colidx.alloc(nnz_nz + 1, s);
    if (rows == 0) TMRG_CUDA(cudaMemsetAsync(I.nz_rowptr.p, 0, sizeof(int), s));
    launch(k_nz_fill, blocks_for(((rows + 3) / 4) * 32, 256), 256, 0, s, rows,
           (const int *)I.rowptr.p, (const int *)I.colidx.p, (const double *)I.vals.p,
           keepoff, I.nz_rowptr.p, I.nz_colidx.p, I.ap_w.p, I.dfflag.p, tk.p, tp.p, erow.p);
  }

  I.perm.alloc(rows + 1, s);
  launch(k_len_order, blocks_for(rows, LO_WIN), LO_THREADS, 0, s, rows, I.ap_rowptr(),
         (const int *)nullptr, I.perm.p);

  // P^T by a stable sort on the column (rows stay ascending per column).
  Stage st_t("tmrg_transpose");
  I.t_colidx.alloc(nnz_nz + 1, s);
  I.t_w.alloc(nnz_nz + 1, s);
  I.t_rowptr.alloc(I.cols + 1, s);
  // the column bits only: a stable LSD sort keeps rows ascending per column
  const int cbits = bits_for(I.cols + 1);
  radix_sort(tk, &tp, nnz_nz, cbits, s);
  launch(k_t_fill, blocks_for(nnz_nz, 256), 256, 0, s, nnz_nz, (const uint32_t *)tk.p,
         (const uint32_t *)tp.p, (const int *)erow.p, (const float2 *)I.ap_w.p, I.t_colidx.p,
         I.t_w.p, I.t_rowptr.p);
  launch(k_t_tail, blocks_for(I.cols + 1, 256), 256, 0, s, I.cols, nnz_nz,
         (const uint32_t *)tk.p, I.t_rowptr.p);
  tk.release();
  tp.release();
  erow.release();
  // P^T rows ordered by the input chunk their last entry needs (stable),
  // then by length inside 4096-row windows of each chunk
  {
    DBuf<uint64_t> ck(I.cols + 1, s);
    DBuf<uint32_t> cv(I.cols + 1, s);
    launch(k_t_chunk_keys, blocks_for(I.cols, 256), 256, 0, s, I.cols, rows,
           (const int *)I.t_rowptr.p, (const int *)I.t_colidx.p, ck.p, cv.p);
    radix_sort(ck, &cv, I.cols, bits_for(TC_CHUNKS), s);
    // the chunk boundaries in the sorted keys, found on the device (only
    // TC_CHUNKS + 1 numbers come back)
    DBuf<long long> cb(TC_CHUNKS + 1, s);
    launch(k_chunk_bounds, 1, 32, 0, s, I.cols, (const uint64_t *)ck.p, TC_CHUNKS, cb.p);
    I.t_chunk.assign(TC_CHUNKS + 1, 0);
    TMRG_CUDA(cudaMemcpyAsync(I.t_chunk.data(), cb.p, sizeof(long long) * (TC_CHUNKS + 1),
                              cudaMemcpyDeviceToHost, s));
    TMRG_CUDA(cudaStreamSynchronize(s));
    I.t_perm.alloc(I.cols + 1, s);
    for (int k = 0; k < TC_CHUNKS; k++) {
      const long long a = I.t_chunk[k], n = I.t_chunk[k + 1] - a;
      launch(k_len_order, blocks_for(n, LO_WIN), LO_THREADS, 0, s, n,
             (const int *)I.t_rowptr.p, (const int *)(cv.p + a), I.t_perm.p + a);
    }
  }
  TMRG_CUDA(cudaStreamSynchronize(s));
}

// ---------------------------------------------------------------------
// Design -> analysis weights (TMROctTACSTopoCreator::computeWeights,
// TMR_TACSTopoCreator.cpp:55-122, called per element at :163-183): the
// centre of every analysis element (an order-3 node with knots -1, 0, 1
// and local index 13) is located in the filter forest with findEnclosing;
// the filter's shape functions at that point, expanded through the filter's
// dependent nodes and merged by column (uniqueSort), are the element's
// row.  The merge follows the filter element's sorted expansion list, in
// the reference's loop order.
__global__ void k_tw_count(long long n, InterpCtx I, const int *__restrict__ ab,
                           const int *__restrict__ ax, const int *__restrict__ ay,
                           const int *__restrict__ az, const int16_t *__restrict__ al,
                           int *trow, long long *cnt) {
  long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  const Oct node{ab[e], ax[e], ay[e], az[e], al[e]};
  const long long t = find_enclosing(I, node, 13);
  trow[e] = (int)t;
  long long m = 0;
  if (t < 0) {
    atomicExch(I.err, 1);
  } else {
    int prev = -1;
    for (long long j = I.eoff[t]; j < I.eoff[t + 1]; j++) {
      const int col = I.lcol[j];
      m += (col != prev);
      prev = col;
    }
  }
  cnt[e] = m;
}
__global__ void k_tw_rows(long long n, InterpCtx I, const int *__restrict__ ax,
                          const int *__restrict__ ay, const int *__restrict__ az,
                          const int16_t *__restrict__ al, const int *__restrict__ trow,
                          const long long *__restrict__ roff, int *cols, double *vals) {
  long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  const int t = trow[e];
  if (t < 0) return;
  const int co = I.co, co2 = co * co;
  const int4 cq = __ldg(I.c4 + t);
  const int32_t hoct = side_of(cq.x >> 26), h = side_of(al[e]);
  const int32_t xyz[3] = {ax[e], ay[e], az[e]};
  double N[3][IMAX_CO];
  for (int a = 0; a < 3; a++) {
    // -1 + 2 ((x mod hoct) + 0.5 h (1 + 0)) / hoct, as the reference rounds it
    const double u = -1.0 + 2.0 * ((double)(xyz[a] % hoct) + 0.5 * (double)h * 1.0) /
                                (double)hoct;
    lagrange3(co, u, I.ck, I.crk, N[a][0], N[a][1], N[a][2]);
  }
  long long o = roff[e];
  const long long lim = roff[e + 1];
  int prev = -1;
  double acc = 0.0;
  bool open = false;
  for (long long j = I.eoff[t]; j < I.eoff[t + 1]; j++) {
    const int key = I.lkey[j], li = key & 31, col = I.lcol[j];
    const int kk = li / co2, jj = (li - kk * co2) / co, ii = li - kk * co2 - jj * co;
    double w = __dmul_rn(__dmul_rn(N[0][ii], N[1][jj]), N[2][kk]);
    if (!(key & KEY_INDEP)) w = __dmul_rn(w, I.ldw[j]);
    if (open && col == prev) {
      acc = __dadd_rn(acc, w);
    } else {
      if (open && o < lim) {
        cols[o] = prev;
        vals[o] = acc;
        o++;
      }
      acc = w;
      prev = col;
      open = true;
    }
  }
  if (open && o < lim) {
    cols[o] = prev;
    vals[o] = acc;
  }
}

// Element centre of every analysis element as (element << 8 | 13): local
// node 13 of an order-3 element with knots -1, 0, 1.
__global__ void k_tw_rep(long long n, unsigned long long *rep) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e < n) rep[e] = ((unsigned long long)e << 8) | 13u;
}

void topo_weights_create(Forest &filter, Forest &analysis, Interp &I) {
  Stage st("tmrg_topo_weights");
  if (!analysis.have_octs) throw Error(TMRG_ERR_STATE, "topo weights: no analysis octants");
  if (filter.order > IMAX_CO || filter.interp == TMRG_BERNSTEIN_POINTS) {
    // filter orders above 3 and Bernstein filters: the general row kernel,
    // with the analysis element centres as the fine nodes (the centre never
    // lies on a filter octant face, so every row takes the full order^3
    // loop of computeWeights)
    forest_create_nodes(filter);
    if (filter.conn->nb >= (1 << 26))
      throw Error(TMRG_ERR_KEY_RANGE, "topo weights: more than 2^26 blocks");
    cudaStream_t s = analysis.s;
    TMRG_CUDA(cudaStreamSynchronize(filter.s));
    I.s = s;
    I.have_colsum = false;
    I.colsum.release();
    I.rows = analysis.n;
    I.cols = filter.num_owned;
    DBuf<int> err(1, s);
    err.zero();
    DBuf<unsigned long long> rep(analysis.n + 1, s);
    launch(k_tw_rep, blocks_for(analysis.n, 256), 256, 0, s, analysis.n, rep.p);
    InterpCtx c{};
    c.fo = 3;
    c.fk1[0] = 0.0;
    c.fk1[1] = 1.0;
    c.fk1[2] = 2.0;
    c.co = filter.order;
    for (int i = 0; i < TMRG_MAX_ORDER; i++) c.ck[i] = filter.knots[i];
    for (int i = 0; i < TMRG_MAX_ORDER; i++)
      for (int j = 0; j < TMRG_MAX_ORDER; j++)
        c.crk[i][j] = (i != j && i < filter.order && j < filter.order)
                          ? 1.0 / (filter.knots[i] - filter.knots[j])
                          : 0.0;
    c.fb = analysis.block.p;
    c.fx = analysis.x.p;
    c.fy = analysis.y.p;
    c.fz = analysis.z.p;
    c.fl = analysis.level.p;
    c.cn = filter.n;
    DBuf<int4> c4(filter.n + 1, s);
    launch(k_pack_octs, blocks_for(filter.n, 256), 256, 0, s, filter.n,
           (const int *)filter.block.p, (const int *)filter.x.p, (const int *)filter.y.p,
           (const int *)filter.z.p, (const int16_t *)filter.level.p, c4.p);
    c.c4 = c4.p;
    c.rep = rep.p;
    c.err = err.p;
    GenInterp G{};
    G.bern = filter.interp == TMRG_BERNSTEIN_POINTS;
    G.topo = 1;
    interp_rows_general(filter, I, c, G, err, s);
    return;
  }
  forest_create_nodes(filter);
  if (filter.conn->nb >= (1 << 26))
    throw Error(TMRG_ERR_KEY_RANGE, "topo weights: more than 2^26 blocks");
  cudaStream_t s = analysis.s;
  TMRG_CUDA(cudaStreamSynchronize(filter.s));
  I.s = s;
  I.have_colsum = false;
  I.colsum.release();
  const long long rows = analysis.n;
  I.rows = rows;
  I.cols = filter.num_owned;
  DBuf<int> err(1, s);
  err.zero();
  InterpCtx c{};
  c.fo = 3;  // the element centre is an order-3 node with knots -1, 0, 1
  c.fk1[0] = 0.0;
  c.fk1[1] = 1.0;
  c.fk1[2] = 2.0;
  c.co = filter.order;
  for (int i = 0; i < TMRG_MAX_ORDER; i++) c.ck[i] = filter.knots[i];
  for (int i = 0; i < TMRG_MAX_ORDER; i++)
    for (int j = 0; j < TMRG_MAX_ORDER; j++)
      c.crk[i][j] = (i != j && i < filter.order && j < filter.order)
                        ? 1.0 / (filter.knots[i] - filter.knots[j])
                        : 0.0;
  c.cn = filter.n;
  DBuf<int4> c4(filter.n + 1, s);
  launch(k_pack_octs, blocks_for(filter.n, 256), 256, 0, s, filter.n,
         (const int *)filter.block.p, (const int *)filter.x.p, (const int *)filter.y.p,
         (const int *)filter.z.p, (const int16_t *)filter.level.p, c4.p);
  c.c4 = c4.p;
  ElemLists EL;
  build_elists(filter, EL, err.p, s);
  c.eoff = EL.eoff.p;
  c.lcol = EL.lcol.p;
  c.ldw = EL.ldw.p;
  c.lkey = EL.lkey.p;
  c.ekind = EL.ekind.p;
  c.err = err.p;
  DBuf<int> trow(rows + 1, s);
  DBuf<long long> roff(rows + 1, s);
  launch(k_tw_count, blocks_for(rows, 128), 128, 0, s, rows, c,
         (const int *)analysis.block.p, (const int *)analysis.x.p, (const int *)analysis.y.p,
         (const int *)analysis.z.p, (const int16_t *)analysis.level.p, trow.p, roff.p);
  exclusive_scan<long long>(roff.p, roff.p, rows, s);
  const long long nnz = read_scalar(roff.p + rows, s);
  const int e = read_scalar(err.p, s);
  if (e == 2)
    throw Error(TMRG_ERR_INTERNAL, "topo weights: a filter element expands to more than 256 entries");
  if (e)
    throw Error(TMRG_ERR_INTERNAL, "topo weights: an element centre has no enclosing filter octant");
  if (nnz >= (1LL << 31) - 1) throw Error(TMRG_ERR_ARG, "topo weights: more than 2^31 entries");
  I.nnz = nnz;
  I.rowptr.alloc(rows + 1, s);
  launch(k_ptr32, blocks_for(rows + 1, 256), 256, 0, s, rows, (const long long *)roff.p,
         I.rowptr.p);
  I.colidx.alloc(nnz + 1, s);
  I.vals.alloc(nnz + 1, s);
  launch(k_tw_rows, blocks_for(rows, 128), 128, 0, s, rows, c, (const int *)analysis.x.p,
         (const int *)analysis.y.p, (const int *)analysis.z.p,
         (const int16_t *)analysis.level.p, (const int *)trow.p, (const long long *)roff.p,
         I.colidx.p, I.vals.p);
  trow.release();
  roff.release();
  EL = ElemLists();
  c4.release();
  interp_finish(I, nnz, s);
}

// Column sums of P for the weight-normalised transpose, on first use.
static void interp_colsum(Interp &I) {
  if (I.have_colsum) return;
  I.colsum.alloc(I.cols + 1, I.s);
  launch(k_rowsum, blocks_for(I.cols, 256), 256, 0, I.s, I.cols,
         (const int *)I.t_rowptr.p, (const float2 *)I.t_w.p, I.colsum.p);
  I.have_colsum = true;
}

// ---------------------------------------------------------------------
// CSR applies over node-major multi-vectors, in double-float arithmetic
// (df_fma; weights and inputs as (hi, lo) pairs), or in FP64 when
// flags[0] | flags[1] says a weight or an input lies outside the
// double-float window (a uniform branch; the FP64 branch reads the FP64
// input and rebuilds each weight as hi + lo).  With `scale` the result is
// divided by scale[row] (weight-normalised transpose).

// G lanes per row, lane v accumulates vectors v, v+G, ... in entry order
// (any number of vectors).
__global__ void __launch_bounds__(256)
    k_df_apply(long long rows, int G, int nvec, const int *__restrict__ rowptr,
               const int *__restrict__ cols, const float2 *__restrict__ w,
               const float2 *__restrict__ xs, const double *__restrict__ x,
               double *__restrict__ y, const double *__restrict__ scale,
               const int *__restrict__ flags) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long r = t / G;
  const int lane = (int)(t - r * G);
  if (r >= rows) return;
  const bool f64 = (__ldg(flags) | __ldg(flags + 1)) != 0;
  const int p0 = __ldg(rowptr + r), p1 = __ldg(rowptr + r + 1);
  for (int v = lane; v < nvec; v += G) {
    double acc = 0.0;
    if (f64) {
      for (int p = p0; p < p1; p++) {
        const float2 wv = __ldg(w + p);
        acc = __fma_rn(__dadd_rn((double)wv.x, (double)wv.y),
                       __ldg(x + (long long)__ldg(cols + p) * nvec + v), acc);
      }
    } else {
      float sh = 0.0f, sl = 0.0f;
      int p = p0;
      for (; p + 4 <= p1; p += 4) {
#pragma unroll
        for (int k = 0; k < 4; k++) {
          const float2 wv = __ldg(w + p + k);
          const float2 xv = __ldg(xs + (long long)__ldg(cols + p + k) * nvec + v);
          df_fma(wv.x, wv.y, xv.x, xv.y, sh, sl);
        }
        df_renorm(sh, sl);
      }
      for (; p < p1; p++) {
        const float2 wv = __ldg(w + p);
        const float2 xv = __ldg(xs + (long long)__ldg(cols + p) * nvec + v);
        df_fma(wv.x, wv.y, xv.x, xv.y, sh, sl);
      }
      df_renorm(sh, sl);
      acc = df_value(sh, sl);
    }
    if (scale) {
      const double sc = scale[r];
      acc = (sc != 0.0) ? __ddiv_rn(acc, sc) : 0.0;
    }
    y[r * nvec + v] = acc;
  }
}

// Vector pairs: LPR lanes per row, lane v holds PPL consecutive vector
// pairs (16-byte loads of (hi, lo, hi, lo) each), and NG groups of LPR
// lanes split a row's entries; the warp runs one trip count with per-entry
// predicates (a masked entry adds an exact 0), and group sums combine in a
// fixed tree order.  With `perm` the rows sharing a warp come from the
// length-ordered permutation, so they have equal trip counts.  Each trip
// group issues the column, weight and input loads of four entries (two
// with four pairs per lane) before their arithmetic, so a warp waits for
// two memory round trips per group; more pairs per lane (PPL) give each
// wait more arithmetic.
template <int LPR, int NG, int PPL>
__global__ void __launch_bounds__(256)
    k_df_apply2(long long rows, int nvec2, const int *__restrict__ rowptr,
                const int *__restrict__ cols, const float2 *__restrict__ w,
                const float4 *__restrict__ xs, const double2 *__restrict__ x,
                double2 *__restrict__ y, const double *__restrict__ scale,
                const int *__restrict__ perm, const int *__restrict__ flags) {
  constexpr int RPW = 32 / (LPR * NG);
  const int lane = threadIdx.x & 31;
  const long long warp = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int sub = lane / (LPR * NG);  // row slot in the warp
  const int g = (lane / LPR) % NG;    // group in the row
  const int v = lane % LPR;           // lane in the group
  const long long slot = warp * RPW + sub;
  if (warp * RPW >= rows) return;     // uniform per warp
  const bool f64 = (__ldg(flags) | __ldg(flags + 1)) != 0;
  const bool have = slot < rows;
  const long long r = (have && perm) ? (long long)__ldg(perm + slot) : slot;
  const int p0 = have ? __ldg(rowptr + r) : 0;
  const int p1 = have ? __ldg(rowptr + r + 1) : 0;
  int trips = (p1 - p0 + NG - 1) / NG;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) trips = max(trips, __shfl_xor_sync(0xffffffffu, trips, o));
  for (int vb = 0; vb < nvec2; vb += LPR * PPL) {
    const int q0 = vb + v * PPL;  // this lane's first pair
    bool act[PPL];
#pragma unroll
    for (int j = 0; j < PPL; j++) act[j] = have && (q0 + j < nvec2);
    double ax[PPL], ay[PPL];
    if (f64) {
#pragma unroll
      for (int j = 0; j < PPL; j++) ax[j] = ay[j] = 0.0;
      for (int t = 0; t < trips; t++) {
        const int p = p0 + g + t * NG;
        const bool on = have && p < p1;
        const int c = on ? __ldg(cols + p) : 0;
        const float2 wv = on ? __ldg(w + p) : make_float2(0.0f, 0.0f);
        const double wd = __dadd_rn((double)wv.x, (double)wv.y);
#pragma unroll
        for (int j = 0; j < PPL; j++) {
          const double2 xv = (on && act[j]) ? __ldg(x + (long long)c * nvec2 + q0 + j)
                                            : make_double2(0.0, 0.0);
          ax[j] = __fma_rn(wd, xv.x, ax[j]);
          ay[j] = __fma_rn(wd, xv.y, ay[j]);
        }
      }
#pragma unroll
      for (int o = (NG / 2) * LPR; o >= LPR; o >>= 1)
#pragma unroll
        for (int j = 0; j < PPL; j++) {
          ax[j] = __dadd_rn(ax[j], __shfl_down_sync(0xffffffffu, ax[j], o));
          ay[j] = __dadd_rn(ay[j], __shfl_down_sync(0xffffffffu, ay[j], o));
        }
    } else {
      float ah[PPL], al[PPL], bh[PPL], bl[PPL];
#pragma unroll
      for (int j = 0; j < PPL; j++) ah[j] = al[j] = bh[j] = bl[j] = 0.0f;
      // entries per batch: four, two with four or more pairs per lane
      // (registers)
      constexpr int UB = PPL >= 4 ? 2 : 4;
      int t = 0;
      for (; t + UB <= trips; t += UB) {
        int c[UB];
        float2 wv[UB];
        float4 xv[UB][PPL];
#pragma unroll
        for (int k = 0; k < UB; k++) {
          const int p = p0 + g + (t + k) * NG;
          const bool on = have && p < p1;
          c[k] = on ? __ldg(cols + p) : -1;
          wv[k] = on ? __ldg(w + p) : make_float2(0.0f, 0.0f);
        }
#pragma unroll
        for (int k = 0; k < UB; k++)
#pragma unroll
          for (int j = 0; j < PPL; j++)
            xv[k][j] = (c[k] >= 0 && act[j]) ? __ldg(xs + (long long)c[k] * nvec2 + q0 + j)
                                             : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
#pragma unroll
        for (int k = 0; k < UB; k++)
#pragma unroll
          for (int j = 0; j < PPL; j++) {
            df_fma(wv[k].x, wv[k].y, xv[k][j].x, xv[k][j].y, ah[j], al[j]);
            df_fma(wv[k].x, wv[k].y, xv[k][j].z, xv[k][j].w, bh[j], bl[j]);
          }
#pragma unroll
        for (int j = 0; j < PPL; j++) {
          df_renorm(ah[j], al[j]);
          df_renorm(bh[j], bl[j]);
        }
      }
      for (; t < trips; t++) {
        const int p = p0 + g + t * NG;
        const bool on = have && p < p1;
        const int c = on ? __ldg(cols + p) : 0;
        const float2 wv = on ? __ldg(w + p) : make_float2(0.0f, 0.0f);
#pragma unroll
        for (int j = 0; j < PPL; j++) {
          const float4 xv = (on && act[j]) ? __ldg(xs + (long long)c * nvec2 + q0 + j)
                                           : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
          df_fma(wv.x, wv.y, xv.x, xv.y, ah[j], al[j]);
          df_fma(wv.x, wv.y, xv.z, xv.w, bh[j], bl[j]);
        }
      }
#pragma unroll
      for (int j = 0; j < PPL; j++) {
        df_renorm(ah[j], al[j]);
        df_renorm(bh[j], bl[j]);
      }
#pragma unroll
      for (int o = (NG / 2) * LPR; o >= LPR; o >>= 1)
#pragma unroll
        for (int j = 0; j < PPL; j++) {
          const float oah = __shfl_down_sync(0xffffffffu, ah[j], o);
          const float oal = __shfl_down_sync(0xffffffffu, al[j], o);
          const float obh = __shfl_down_sync(0xffffffffu, bh[j], o);
          const float obl = __shfl_down_sync(0xffffffffu, bl[j], o);
          df_add(ah[j], al[j], oah, oal);
          df_add(bh[j], bl[j], obh, obl);
        }
#pragma unroll
      for (int j = 0; j < PPL; j++) {
        ax[j] = df_value(ah[j], al[j]);
        ay[j] = df_value(bh[j], bl[j]);
      }
    }
    if (g == 0) {
      const double sc = scale && have ? scale[r] : 1.0;
#pragma unroll
      for (int j = 0; j < PPL; j++) {
        if (!act[j]) continue;
        double a = ax[j], b = ay[j];
        if (scale) {
          a = (sc != 0.0) ? __ddiv_rn(a, sc) : 0.0;
          b = (sc != 0.0) ? __ddiv_rn(b, sc) : 0.0;
        }
        y[r * nvec2 + q0 + j] = make_double2(a, b);
      }
    }
  }
}

// ---------------------------------------------------------------------
// The same apply (2 lanes per row, 4 vector pairs per lane: 16 vectors) with
// the input rows staged in shared memory by the Tensor Memory Accelerator:
// per warp a ring of TG_STAGES batches, a batch being entry b of the warp's
// 16 rows (16 input rows of 128 bytes, four `cp.async.bulk.tensor ...
// tile::gather4` copies of 4 rows each, completion counted on the stage's
// mbarrier).  The warp issues the gathers TG_STAGES - 1 batches ahead of the
// batch it sums, so the input latency is covered without registers; the
// entry order and the renormalisation points are those of k_df_apply2<2, 1,
// 4>, so the results are the same bits.  Every wait is bounded: a stage that
// does not complete sets flags[2] (the host reports it) and the warp drains
// the gathers it issued (bounded again) before it leaves.
constexpr int TG_WARPS = 8, TG_STAGES = 4, TG_ROWB = 128, TG_BATCH = 16 * TG_ROWB;
constexpr int TG_SMEM = TG_WARPS * TG_STAGES * TG_BATCH + TG_WARPS * TG_STAGES * 8;
constexpr long long TG_WAIT_LIMIT = 1LL << 20;  // try_wait rounds before giving up

__device__ __forceinline__ unsigned smem_addr(const void *p) {
  return (unsigned)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t *b, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(b)), "r"(count)
               : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *b, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(b)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *b, unsigned parity) {
  unsigned done;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(done)
      : "r"(smem_addr(b)), "r"(parity)
      : "memory");
  return done != 0;
}
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *b, unsigned parity) {
  for (long long it = 0; it < TG_WAIT_LIMIT; it++)
    if (mbar_try_wait(b, parity)) return true;
  return false;
}
// Rows r0..r3 (columns from c0) of the 2-D tensor `map` to 4 consecutive
// rows of shared memory at dst.
__device__ __forceinline__ void tma_gather4(void *dst, const CUtensorMap *map, int c0, int r0,
                                            int r1, int r2, int r3, uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile::gather4.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4, %5, %6}], [%7];" ::"r"(smem_addr(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(r0), "r"(r1), "r"(r2), "r"(r3),
      "r"(smem_addr(bar))
      : "memory");
}

__global__ void __launch_bounds__(TG_WARPS * 32)
    k_df_apply_tma(const __grid_constant__ CUtensorMap xmap, long long rows,
                   const int *__restrict__ rowptr, const int *__restrict__ cols,
                   const float2 *__restrict__ w, const double2 *__restrict__ x,
                   double2 *__restrict__ y, const double *__restrict__ scale,
                   const int *__restrict__ perm, int *flags) {
  extern __shared__ __align__(128) uint8_t tg_smem[];
  constexpr int PPL = 4, NV2 = 8;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  uint8_t *buf = tg_smem + warp * (TG_STAGES * TG_BATCH);
  uint64_t *bar =
      reinterpret_cast<uint64_t *>(tg_smem + TG_WARPS * TG_STAGES * TG_BATCH) + warp * TG_STAGES;
  const long long slot0 = ((long long)blockIdx.x * TG_WARPS + warp) * 16;
  if (slot0 >= rows) return;  // uniform per warp
  const int i = lane >> 1, half = lane & 1;
  const long long slot = slot0 + i;
  const bool have = slot < rows;
  const long long r = (have && perm) ? (long long)__ldg(perm + slot) : slot;
  const int p0 = have ? __ldg(rowptr + r) : 0;
  const int p1 = have ? __ldg(rowptr + r + 1) : 0;
  int trips = p1 - p0;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) trips = max(trips, __shfl_xor_sync(0xffffffffu, trips, o));
  const int q0 = half * PPL;  // this lane's first pair
  const bool f64 = (__ldg(flags) | __ldg(flags + 1)) != 0;
  double ax[PPL], ay[PPL];
  if (f64) {
    // values outside the double-float window: the FP64 sums of k_df_apply2
#pragma unroll
    for (int j = 0; j < PPL; j++) ax[j] = ay[j] = 0.0;
    for (int t = 0; t < trips; t++) {
      const int p = p0 + t;
      const bool on = have && p < p1;
      const int c = on ? __ldg(cols + p) : 0;
      const float2 wv = on ? __ldg(w + p) : make_float2(0.0f, 0.0f);
      const double wd = __dadd_rn((double)wv.x, (double)wv.y);
#pragma unroll
      for (int j = 0; j < PPL; j++) {
        const double2 xv = on ? __ldg(x + (long long)c * NV2 + q0 + j) : make_double2(0.0, 0.0);
        ax[j] = __fma_rn(wd, xv.x, ax[j]);
        ay[j] = __fma_rn(wd, xv.y, ay[j]);
      }
    }
  } else {
    if (lane < TG_STAGES) mbar_init(&bar[lane], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    __syncwarp();
    // lanes 0..15 hold the entry range of row `lane` for the gathers
    const int g0 = __shfl_sync(0xffffffffu, p0, 2 * (lane & 15));
    const int g1 = __shfl_sync(0xffffffffu, p1, 2 * (lane & 15));
    auto issue = [&](int b) {
      const int st = b % TG_STAGES;
      const int c = (lane < 16 && g0 + b < g1) ? __ldg(cols + g0 + b) : 0;
      const int c1 = __shfl_down_sync(0xffffffffu, c, 1);
      const int c2 = __shfl_down_sync(0xffffffffu, c, 2);
      const int c3 = __shfl_down_sync(0xffffffffu, c, 3);
      if (lane == 0) mbar_expect_tx(&bar[st], TG_BATCH);
      __syncwarp();
      if (lane < 16 && (lane & 3) == 0)
        tma_gather4(buf + st * TG_BATCH + lane * TG_ROWB, &xmap, 0, c, c1, c2, c3, &bar[st]);
    };
    const int pre = min(trips, TG_STAGES);
    for (int b = 0; b < pre; b++) issue(b);
    int issued = pre;
    float ah[PPL], al[PPL], bh[PPL], bl[PPL];
#pragma unroll
    for (int j = 0; j < PPL; j++) ah[j] = al[j] = bh[j] = bl[j] = 0.0f;
    int b = 0;
    for (; b < trips; b++) {
      const int st = b % TG_STAGES;
      if (!mbar_wait_bounded(&bar[st], (unsigned)(b / TG_STAGES) & 1u)) {
        if (lane == 0) atomicExch(flags + 2, 1);
        break;
      }
      const int p = p0 + b;
      const float2 wv = (have && p < p1) ? __ldg(w + p) : make_float2(0.0f, 0.0f);
      const float4 *xr =
          reinterpret_cast<const float4 *>(buf + st * TG_BATCH + i * TG_ROWB + half * 64);
#pragma unroll
      for (int j = 0; j < PPL; j++) {
        const float4 xv = xr[j];
        df_fma(wv.x, wv.y, xv.x, xv.y, ah[j], al[j]);
        df_fma(wv.x, wv.y, xv.z, xv.w, bh[j], bl[j]);
      }
      if (b & 1) {  // k_df_apply2 renormalises after every two entries
#pragma unroll
        for (int j = 0; j < PPL; j++) {
          df_renorm(ah[j], al[j]);
          df_renorm(bh[j], bl[j]);
        }
      }
      // this stage's reads are done before the gathers refill it
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      __syncwarp();
      if (issued < trips) {
        issue(issued);
        issued++;
      }
    }
    if (b < trips) {
      // a stage timed out: wait (bounded) for the other gathers in flight
      for (int bb = b + 1; bb < issued; bb++)
        mbar_wait_bounded(&bar[bb % TG_STAGES], (unsigned)(bb / TG_STAGES) & 1u);
    }
#pragma unroll
    for (int j = 0; j < PPL; j++) {
      df_renorm(ah[j], al[j]);
      df_renorm(bh[j], bl[j]);
      ax[j] = df_value(ah[j], al[j]);
      ay[j] = df_value(bh[j], bl[j]);
    }
  }
  if (have) {
    const double sc = scale ? scale[r] : 1.0;
#pragma unroll
    for (int j = 0; j < PPL; j++) {
      double a = ax[j], bv = ay[j];
      if (scale) {
        a = (sc != 0.0) ? __ddiv_rn(a, sc) : 0.0;
        bv = (sc != 0.0) ? __ddiv_rn(bv, sc) : 0.0;
      }
      y[r * NV2 + q0 + j] = make_double2(a, bv);
    }
  }
}

// The tensor map of the split input (rows of 16 float2 = 128 bytes) for the
// gathers: UINT32 elements, box 32 x 1 (a gather4 box is one row high).
using EncodeTiledFn = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *,
                                   const cuuint64_t *, const cuuint64_t *, const cuuint32_t *,
                                   const cuuint32_t *, CUtensorMapInterleave, CUtensorMapSwizzle,
                                   CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
static EncodeTiledFn encode_tiled() {
  static EncodeTiledFn fn = [] {
    void *f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault,
                                         &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      f = nullptr;
    return reinterpret_cast<EncodeTiledFn>(f);
  }();
  return fn;
}
static bool tma_apply(long long rows, long long nin, const int *rp, const int *ci,
                      const float2 *w, const float2 *xs, const double *x, double *y,
                      const double *scale, const int *perm, int *flags, cudaStream_t s) {
  EncodeTiledFn enc = encode_tiled();
  if (!enc || nin <= 0 || nin >= (1LL << 31) || ((uintptr_t)xs % 16) != 0) return false;
  CUtensorMap map;
  const cuuint64_t dims[2] = {32, (cuuint64_t)nin};
  const cuuint64_t strides[1] = {TG_ROWB};
  const cuuint32_t box[2] = {32, 1};
  const cuuint32_t estr[2] = {1, 1};
  if (enc(&map, CU_TENSOR_MAP_DATA_TYPE_UINT32, 2, const_cast<float2 *>(xs), dims, strides, box,
          estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
          CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
    return false;
  static bool attr = false;
  if (!attr) {
    TMRG_CUDA(cudaFuncSetAttribute(k_df_apply_tma, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   TG_SMEM));
    attr = true;
  }
  const long long rows_per_block = 16LL * TG_WARPS;
  launch(k_df_apply_tma, (unsigned)((rows + rows_per_block - 1) / rows_per_block),
         TG_WARPS * 32, TG_SMEM, s, map, rows, rp, ci, w, (const double2 *)x, (double2 *)y,
         scale, perm, flags);
  return true;
}

// Launch shapes for vector pairs (the autotuner's candidates): LPR lanes per
// row holding PPL pairs each, NG groups of LPR lanes splitting a row's
// entries, 32 / (LPR NG) rows per warp; with `perm` the rows sharing a warp
// come from the length-ordered permutation.
// 8 or more pairs (16+ vectors): {8,1,1} {8,2,1} {8,4,1} {4,1,2} {2,1,4}
// {1,1,8}, and for exactly 8 pairs {2,1,4} with TMA-staged inputs
// (k_df_apply_tma); fewer pairs: LPR = pairs rounded down to a power of
// two, NG 1 or 2
constexpr int DF2_SHAPES_WIDE = 7, DF2_SHAPES_NARROW = 2;
static void df_apply2(int shape, long long rows, int nvec2, const int *rp, const int *ci,
                      const float2 *w, const float2 *xs, const double *x, double *y,
                      const double *scale, const int *perm, int *flags, cudaStream_t s,
                      long long nin) {
  if (shape == 6 && nvec2 == 8 &&
      tma_apply(rows, nin, rp, ci, w, xs, x, y, scale, perm, flags, s))
    return;
  const float4 *x4 = (const float4 *)xs;
  const double2 *x2 = (const double2 *)x;
  double2 *y2 = (double2 *)y;
#define TMRG_DF2(L, N, P)                                                                  \
  launch((k_df_apply2<L, N, P>),                                                           \
         blocks_for(((rows + 32 / ((L) * (N)) - 1) / (32 / ((L) * (N)))) * 32, 256), 256, 0, s, \
         rows, nvec2, rp, ci, w, x4, x2, y2, scale, perm, flags)
  if (nvec2 >= 8) {
    switch (shape) {
      case 0: TMRG_DF2(8, 1, 1); break;
      case 1: TMRG_DF2(8, 2, 1); break;
      case 2: TMRG_DF2(8, 4, 1); break;
      case 3: TMRG_DF2(4, 1, 2); break;
      case 5: TMRG_DF2(1, 1, 8); break;
      default: TMRG_DF2(2, 1, 4);  // 4, and 6 where the staged kernel does not apply
    }
  } else if (nvec2 >= 4) {
    if (shape == 0)
      TMRG_DF2(4, 1, 1);
    else
      TMRG_DF2(4, 2, 1);
  } else if (nvec2 >= 2) {
    if (shape == 0)
      TMRG_DF2(2, 1, 1);
    else
      TMRG_DF2(2, 2, 1);
  } else {
    if (shape == 0)
      TMRG_DF2(1, 1, 1);
    else
      TMRG_DF2(1, 2, 1);
  }
#undef TMRG_DF2
}
// Size class of an apply: direction, vector pairs (8 = 8 or more), log2 of
// the rows, mean row length in quarters (capped).
static TuneKey df_key(int which, long long rows, long long nnz, int nvec2) {
  int lr = 0;
  while ((1LL << (lr + 1)) <= rows) lr++;
  const int q = rows ? (int)std::min(4096LL, (4 * nnz) / rows) : 0;
  return TuneKey{which == 0 ? TUNE_P : TUNE_PT, std::min(nvec2, 8), lr, q, 0, 0};
}

// The input as (hi, lo) pairs in pool memory, with its window flag.
static void df_split_input(Interp &I, const double *x, long long n, DBuf<float2> &xs,
                           cudaStream_t s) {
  if (n <= 0) return;
  prof_bytes(16 * n);
  launch(k_df_split_x, blocks_for(n, 256), 256, 0, s, n, x, xs.p, I.dfflag.p + 1);
}

// Transpose apply with the input in host memory: the input rows are copied
// in TC_CHUNKS pieces on a second stream, and after piece k arrives (and is
// split into (hi, lo) pairs) the output rows whose inputs all lie in pieces
// <= k are computed (t_perm holds the rows grouped that way), so the copy
// of the next piece overlaps them.  Same kernel, rows and summation order
// as the single apply; a piece with a value outside the double-float window
// sends that piece's rows and every later piece's rows to FP64 (each row
// only reads pieces already split, so a row never runs in double-float on
// an input that was not represented).
// Returns false (nothing done) where the grouped kernel does not apply.
// Reports (and clears) a TMA input stage of k_df_apply_tma that did not
// complete within its wait limit; read where the host already waits.
void interp_check_apply(Interp &I) {
  if (read_scalar(I.dfflag.p + 2, I.s)) {
    TMRG_CUDA(cudaMemsetAsync(I.dfflag.p + 2, 0, sizeof(int), I.s));
    throw Error(TMRG_ERR_INTERNAL, "P apply: a staged input batch did not arrive");
  }
}

bool interp_apply_transpose_staged(Interp &I, int which, const double *xh, double *dx,
                                   double *y, int nvec) {
  if ((which != 1 && which != 2) || nvec % 2 != 0 || nvec / 2 < 8 ||
      ((uintptr_t)dx % 16) != 0 || ((uintptr_t)y % 16) != 0 ||
      (long long)I.t_chunk.size() != TC_CHUNKS + 1)
    return false;
  Stage st("tmrg_interp_mult_transpose_staged");
  cudaStream_t s = I.s;
  if (which == 2) interp_colsum(I);
  const long long nin = I.rows;
  DBuf<float2> xs(nin * nvec + 1, s);
  TMRG_CUDA(cudaMemsetAsync(I.dfflag.p + 1, 0, sizeof(int), s));
  cudaStream_t cs;
  TMRG_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
  cudaEvent_t ev[TC_CHUNKS + 1];
  for (int k = 0; k <= TC_CHUNKS; k++)
    TMRG_CUDA(cudaEventCreateWithFlags(&ev[k], cudaEventDisableTiming));
  // the copies start after the work already queued on the forest stream
  TMRG_CUDA(cudaEventRecord(ev[TC_CHUNKS], s));
  TMRG_CUDA(cudaStreamWaitEvent(cs, ev[TC_CHUNKS], 0));
  long long r0s[TC_CHUNKS + 1];
  for (int k = 0; k <= TC_CHUNKS; k++) r0s[k] = (k * nin + TC_CHUNKS - 1) / TC_CHUNKS;
  for (int k = 0; k < TC_CHUNKS; k++) {
    const long long r0 = r0s[k], r1 = r0s[k + 1];
    if (r1 > r0)
      TMRG_CUDA(cudaMemcpyAsync(dx + r0 * nvec, xh + r0 * nvec, sizeof(double) * (r1 - r0) * nvec,
                                cudaMemcpyHostToDevice, cs));
    TMRG_CUDA(cudaEventRecord(ev[k], cs));
  }
  const double *sc = which == 2 ? (const double *)I.colsum.p : (const double *)nullptr;
  // the tuned shape of the whole apply's class (the pieces are not tuned)
  const int shape = tune_lookup(df_key(1, I.cols, I.nnz_nz, nvec / 2));
  for (int k = 0; k < TC_CHUNKS; k++) {
    TMRG_CUDA(cudaStreamWaitEvent(s, ev[k], 0));
    const long long r0 = r0s[k], r1 = r0s[k + 1];
    if (r1 > r0)
      launch(k_df_split_x, blocks_for((r1 - r0) * nvec, 256), 256, 0, s, (r1 - r0) * nvec,
             (const double *)(dx + r0 * nvec), xs.p + r0 * nvec, I.dfflag.p + 1);
    const long long a = I.t_chunk[k], n = I.t_chunk[k + 1] - a;
    if (n > 0)
      df_apply2(shape, n, nvec / 2, I.t_rowptr.p, I.t_colidx.p, I.t_w.p, xs.p, dx, y, sc,
                I.t_perm.p + a, I.dfflag.p, s, nin);
  }
  TMRG_CUDA(cudaStreamSynchronize(s));
  for (int k = 0; k <= TC_CHUNKS; k++) cudaEventDestroy(ev[k]);
  cudaStreamDestroy(cs);
  interp_check_apply(I);
  return true;
}

// Largest column of each LO_WIN-row window of a column-sorted CSR (the last
// entry of each row), -1 for a window of empty rows; wmax starts at -1.
__global__ void k_win_maxcol(long long rows, const int *__restrict__ rp,
                             const int *__restrict__ ci, int *wmax) {
  const long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  int m = -1;
  if (r < rows) {
    const int a = rp[r], b = rp[r + 1];
    if (b > a) m = ci[b - 1];
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
  // a warp's 32 rows lie in one window (LO_WIN is a multiple of 32)
  if ((threadIdx.x & 31) == 0 && r < rows && m >= 0) atomicMax(wmax + r / LO_WIN, m);
}

// Prolongation with the input and the output in host memory: the input
// (coarse values) is copied in FC_CHUNKS column ranges on a second stream,
// and the rows are computed in FC_CHUNKS pieces of whole 4096-row windows
// (the length-ordered permutation stays inside a window, so a piece of
// slots is exactly a piece of rows) into device memory, each piece as soon
// as the input range holding its largest column has arrived and been split
// (rows and columns follow the same node order, so piece k mostly needs
// the first ranges), and each piece is copied to the host on a third
// stream while the next piece computes.  One bulk copy per piece runs the
// host link at its copy rate (the kernel writing host memory directly ran
// it at less than half).  Same kernel, rows and summation order as the
// single apply; as in the transpose, a range with a value outside the
// double-float window sends the rows computed after its split to FP64.
// Returns false (nothing done) where the pair kernel does not apply.
constexpr int FC_CHUNKS = 16;
bool interp_apply_forward_staged(Interp &I, const double *xh, double *dx, double *yh,
                                 int nvec) {
  if (nvec % 2 != 0 || ((uintptr_t)dx % 16) != 0 || I.rows < (long long)LO_WIN * FC_CHUNKS)
    return false;
  Stage st("tmrg_interp_mult_staged");
  cudaStream_t s = I.s;
  const long long nin = I.cols, rows = I.rows;
  const long long nwin = (rows + LO_WIN - 1) / LO_WIN;
  if ((long long)I.win_maxcol.size() != nwin) {
    DBuf<int> wm(nwin, s);
    TMRG_CUDA(cudaMemsetAsync(wm.p, 0xff, sizeof(int) * nwin, s));
    launch(k_win_maxcol, blocks_for(rows, 256), 256, 0, s, rows, I.ap_rowptr(), I.ap_colidx(),
           wm.p);
    I.win_maxcol.resize(nwin);
    TMRG_CUDA(cudaMemcpyAsync(I.win_maxcol.data(), wm.p, sizeof(int) * nwin,
                              cudaMemcpyDeviceToHost, s));
    TMRG_CUDA(cudaStreamSynchronize(s));
    g_host_syncs.fetch_add(1, std::memory_order_relaxed);
  }
  DBuf<float2> xs(nin * nvec + 1, s);
  TMRG_CUDA(cudaMemsetAsync(I.dfflag.p + 1, 0, sizeof(int), s));
  DBuf<double> dy(rows * nvec + 2, s);
  double *y = dy.p;
  if ((uintptr_t)y % 16) y++;
  const int n2 = nvec / 2;
  const int shape = tune_lookup(df_key(0, rows, I.nnz_nz, n2));
  cudaStream_t is, cs;
  TMRG_CUDA(cudaStreamCreateWithFlags(&is, cudaStreamNonBlocking));
  TMRG_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
  cudaEvent_t iev[FC_CHUNKS + 1], ev[FC_CHUNKS];
  for (int k = 0; k <= FC_CHUNKS; k++)
    TMRG_CUDA(cudaEventCreateWithFlags(&iev[k], cudaEventDisableTiming));
  for (int k = 0; k < FC_CHUNKS; k++)
    TMRG_CUDA(cudaEventCreateWithFlags(&ev[k], cudaEventDisableTiming));
  // input ranges: columns [c0[j], c0[j + 1]), copied in order after the work
  // already queued on the forest stream
  long long c0[FC_CHUNKS + 1];
  for (int j = 0; j <= FC_CHUNKS; j++) c0[j] = nin * j / FC_CHUNKS;
  TMRG_CUDA(cudaEventRecord(iev[FC_CHUNKS], s));
  TMRG_CUDA(cudaStreamWaitEvent(is, iev[FC_CHUNKS], 0));
  for (int j = 0; j < FC_CHUNKS; j++) {
    if (c0[j + 1] > c0[j])
      TMRG_CUDA(cudaMemcpyAsync(dx + c0[j] * nvec, xh + c0[j] * nvec,
                                sizeof(double) * (c0[j + 1] - c0[j]) * nvec,
                                cudaMemcpyHostToDevice, is));
    TMRG_CUDA(cudaEventRecord(iev[j], is));
  }
  int split = 0;  // input ranges [0, split) are on the device and split
  for (int k = 0; k < FC_CHUNKS; k++) {
    const long long w0 = nwin * k / FC_CHUNKS, w1 = nwin * (k + 1) / FC_CHUNKS;
    const long long r0 = std::min(rows, w0 * LO_WIN), r1 = std::min(rows, w1 * LO_WIN);
    int need = -1;  // largest column the piece reads
    for (long long w = w0; w < w1; w++) need = std::max(need, I.win_maxcol[w]);
    // ranges up to the one holding `need` (all of them if a column were
    // out of range)
    int upto = need < 0 ? 0 : FC_CHUNKS;
    for (int j = 0; j < FC_CHUNKS && need >= 0; j++)
      if (need < c0[j + 1]) {
        upto = j + 1;
        break;
      }
    for (; split < upto; split++) {
      TMRG_CUDA(cudaStreamWaitEvent(s, iev[split], 0));
      const long long a = c0[split], b = c0[split + 1];
      if (b > a) {
        prof_bytes(16 * (b - a) * nvec);
        launch(k_df_split_x, blocks_for((b - a) * nvec, 256), 256, 0, s, (b - a) * nvec,
               (const double *)(dx + a * nvec), xs.p + a * nvec, I.dfflag.p + 1);
      }
    }
    if (r1 > r0) {
      prof_bytes(12 * I.nnz_nz * (r1 - r0) / rows + 4 * (r1 - r0) + 8LL * nvec * (r1 - r0));
      df_apply2(shape, r1 - r0, n2, I.ap_rowptr(), I.ap_colidx(), I.ap_w.p, xs.p, dx, y,
                nullptr, I.perm.p + r0, I.dfflag.p, s, nin);
    }
    TMRG_CUDA(cudaEventRecord(ev[k], s));
    TMRG_CUDA(cudaStreamWaitEvent(cs, ev[k], 0));
    if (r1 > r0)
      TMRG_CUDA(cudaMemcpyAsync(yh + r0 * nvec, y + r0 * nvec, sizeof(double) * (r1 - r0) * nvec,
                                cudaMemcpyDeviceToHost, cs));
  }
  // every input range is waited for before the call returns
  for (; split < FC_CHUNKS; split++) TMRG_CUDA(cudaStreamWaitEvent(s, iev[split], 0));
  TMRG_CUDA(cudaStreamSynchronize(cs));
  TMRG_CUDA(cudaStreamSynchronize(s));
  for (int k = 0; k <= FC_CHUNKS; k++) cudaEventDestroy(iev[k]);
  for (int k = 0; k < FC_CHUNKS; k++) cudaEventDestroy(ev[k]);
  cudaStreamDestroy(is);
  cudaStreamDestroy(cs);
  interp_check_apply(I);
  return true;
}

void interp_apply(Interp &I, int which, const double *x, double *y, int nvec) {
  Stage st(which == 0 ? "tmrg_interp_mult" : "tmrg_interp_mult_transpose");
  if (nvec <= 0) throw Error(TMRG_ERR_ARG, "interp apply: nvec <= 0");
  cudaStream_t s = I.s;
  if (which == 2) interp_colsum(I);
  const long long nin = (which == 0) ? I.cols : I.rows;
  const long long nout = (which == 0) ? I.rows : I.cols;
  const int *rp = which == 0 ? I.ap_rowptr() : I.t_rowptr.p;
  const int *ci = which == 0 ? I.ap_colidx() : I.t_colidx.p;
  const float2 *w = which == 0 ? (const float2 *)I.ap_w.p : (const float2 *)I.t_w.p;
  const double *sc = which == 2 ? (const double *)I.colsum.p : (const double *)nullptr;
  const int *perm = which == 0 ? (const int *)I.perm.p : (const int *)I.t_perm.p;
  DBuf<float2> xs(nin * nvec + 1, s);
  TMRG_CUDA(cudaMemsetAsync(I.dfflag.p + 1, 0, sizeof(int), s));
  df_split_input(I, x, nin * nvec, xs, s);
  // compulsory traffic: 12 B per nonzero entry, the row pointers, one read
  // of the input (its (hi, lo) copy) and one write of the output vectors
  const long long bytes = 12 * I.nnz_nz + 4 * (nout + 1) + 8LL * nvec * (nin + nout) +
                          (which == 2 ? 8 * nout : 0);
  prof_bytes(bytes);
  if (nvec % 2 == 0 && ((uintptr_t)x % 16) == 0 && ((uintptr_t)y % 16) == 0) {
    const int n2 = nvec / 2;
    tune_run(df_key(which, nout, I.nnz_nz, n2), n2 >= 8 ? DF2_SHAPES_WIDE : DF2_SHAPES_NARROW,
             [&](int shape) {
               df_apply2(shape, nout, n2, rp, ci, w, xs.p, x, y, sc, perm, I.dfflag.p, s, nin);
             },
             s);
    return;
  }
  int G = 1;
  while (G < nvec && G < 32) G <<= 1;
  launch(k_df_apply, blocks_for(nout * G, 256), 256, 0, s, nout, G, nvec, rp, ci, w,
         (const float2 *)xs.p, x, y, sc, (const int *)I.dfflag.p);
}

}  // namespace tmrg
