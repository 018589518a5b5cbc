// createInterpolation and the P / P^T applies on the GPU.
//
// P (coarse -> fine) has one row per owned fine node.  A node is handled
// through the first (element, local node) that references it in element
// order (TMROctForest.cpp:6654-6688): the reference's findEnclosing search
// over the sorted coarse octants, computeElemInterp's tensor-product
// Lagrange weights with the coarse dependent-node expansion, and a sort and
// merge of the entries by column (TMRIndexWeight::uniqueSort), one warp per
// row.  Rows are made in two passes (count, then write at the scanned
// offsets).  P^T is the same matrix re-sorted by
// (column, row), so transpose applies gather without atomics and sum in a
// fixed order.
#include "tmrg_tree.cuh"

namespace tmrg {

constexpr int IMAX_CO = 3;  // coarse orders built for createInterpolation
constexpr int IMAX_W = IMAX_CO * IMAX_CO * IMAX_CO * IMAX_CO * IMAX_CO;

struct InterpCtx {
  int fo, co;  // fine / coarse order
  double fk[TMRG_MAX_ORDER], ck[TMRG_MAX_ORDER];
  double crk[TMRG_MAX_ORDER][TMRG_MAX_ORDER];  // 1/(ck_i - ck_j)
  // fine octants
  const int *fb, *fx, *fy, *fz;
  const int16_t *fl;
  // coarse octants {block | level << 26, x, y, z}, connectivity and
  // dependent CSR
  long long cn;
  const int4 *c4;
  const int *cconn;
  const int *cdptr, *cdconn;
  const double *cdw;
  const unsigned long long *rep;  // fine node -> element*npe + local index
  int *err;
};

__global__ void k_pack_octs(long long n, const int *__restrict__ b,
                            const int *__restrict__ x, const int *__restrict__ y,
                            const int *__restrict__ z,
                            const int16_t *__restrict__ l, int4 *out) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = make_int4(b[i] | ((int)l[i] << 26), x[i], y[i], z[i]);
}

__global__ void k_first_ref(long long m, int npe, long long nowned,
                            const int *__restrict__ conn,
                            unsigned long long *rep) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= m) return;
  int c = conn[t];
  if (c >= 0 && c < nowned) atomicMin(rep + c, (unsigned long long)t);
}

// 1-D Lagrange basis (TMRInterpolation.h:40-52).  rk[i][j] holds
// 1/(k_i - k_j), rounded once on the host exactly as the reference rounds
// it, so no FP64 division runs here (FP64 is a scarce pipe on GB300).
__device__ __forceinline__ void lagrange_w(int order, double u, const double *kn,
                                           const double (*rk)[TMRG_MAX_ORDER],
                                           double *N) {
  for (int i = 0; i < order; i++) {
    double v = 1.0;
    for (int j = 0; j < order; j++) {
      if (i != j) v = __dmul_rn(v, __dmul_rn(__dsub_rn(u, kn[j]), rk[i][j]));
    }
    N[i] = v;
  }
}
// 1/2^e for an octant side 2^e, exact (same value as 1.0/h).
__device__ __forceinline__ double inv_side(int level) {
  return __hiloint2double((1023 - (TMRG_MAX_LEVEL - level)) << 20, 0);
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
  double hd = (double)h;
  double xd = __dadd_rn((double)node.x, __dmul_rn(__dmul_rn(0.5, hd), __dadd_rn(1.0, I.fk[ii])));
  double yd = __dadd_rn((double)node.y, __dmul_rn(__dmul_rn(0.5, hd), __dadd_rn(1.0, I.fk[jj])));
  double zd = __dadd_rn((double)node.z, __dmul_rn(__dmul_rn(0.5, hd), __dadd_rn(1.0, I.fk[kk])));
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
      bool xin = (xi >= 0) ? (ax <= xi && xi <= ax + hm)
                           : ((double)ax <= xd && xd <= (double)(ax + hm));
      bool yin = (yi >= 0) ? (ay <= yi && yi <= ay + hm)
                           : ((double)ay <= yd && yd <= (double)(ay + hm));
      bool zin = (zi >= 0) ? (az <= zi && zi <= az + hm)
                           : ((double)az <= zd && zd <= (double)(az + hm));
      if (xin && yin && zin) return mid;
    }
    mid++;
  }
  return -1;
}

// One coordinate direction of computeElemInterp (TMROctForest.cpp:
// 6497-6548, Lagrange branch): exact face hits short-circuit to one weight.
__device__ __forceinline__ void dir_weights(const InterpCtx &I, int i, int32_t nx,
                                            int32_t h, int32_t ox, int32_t hc,
                                            double ihc, int &s, int &e, double *N) {
  const int mo = I.fo, co = I.co;
  if ((i == 0 && ox == nx) || (i == mo - 1 && ox == nx + h)) {
    s = 0;
    e = 1;
    N[0] = 1.0;
  } else if ((i == 0 && ox + hc == nx) || (i == mo - 1 && ox + hc == nx + h)) {
    s = co - 1;
    e = co;
    N[s] = 1.0;
  } else {
    s = 0;
    e = co;
    double t = __dadd_rn((double)nx,
                         __dmul_rn(__dmul_rn(0.5, (double)h), __dadd_rn(1.0, I.fk[i])));
    // division by the power of two hc is an exact scaling
    double u = __dadd_rn(-1.0, __dmul_rn(__dmul_rn(2.0, __dsub_rn(t, (double)ox)), ihc));
    lagrange_w(co, u, I.ck, I.crk, N);
  }
}

// Rows of P, one warp per row, 32 rows per warp.  Phase A: each lane runs
// findEnclosing and the per-direction weights of one row.  Phase B, row by
// row: lane i expands box node i (ii fastest, as computeElemInterp loops)
// through the coarse dependent CSR into shared memory; a stable rank sort
// orders the entries by column and the first entry of each column run sums
// the run in order (TMRIndexWeight::uniqueSort, TMRBase.h:103-130).
constexpr int IW_WARPS = 4;

// Pass 1 (bound): findEnclosing per row, kept in `trow`, and an upper bound
// of the row's entries (sum of the box nodes' expansions) in `bound`.
__global__ void k_interp_bound(long long rows, InterpCtx I, int *trow,
                               long long *bound) {
  long long row = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (row >= rows) return;
  const int mo = I.fo, co = I.co, fnpe = mo * mo * mo;
  unsigned long long r = I.rep[row];
  long long e = (long long)(r / fnpe);
  int info = (int)(r - (unsigned long long)e * fnpe);
  Oct node{I.fb[e], I.fx[e], I.fy[e], I.fz[e], I.fl[e]};
  long long t = find_enclosing(I, node, info);
  trow[row] = (int)t;
  long long ne = 0;
  if (t < 0) {
    atomicExch(I.err, 1);
  } else {
    // the box of coarse nodes the row touches (computeElemInterp's
    // istart..iend per direction), expanded through the dependent rows
    int4 cq = __ldg(I.c4 + t);
    int32_t h = side_of(node.level), hc = side_of(cq.x >> 26);
    int i = info % mo, j = (info % (mo * mo)) / mo, k = info / (mo * mo);
    int rs[3], re[3];
    const int ijk[3] = {i, j, k};
    const int32_t nx[3] = {node.x, node.y, node.z}, ox[3] = {cq.y, cq.z, cq.w};
    for (int d = 0; d < 3; d++) {
      int a = ijk[d];
      if ((a == 0 && ox[d] == nx[d]) || (a == mo - 1 && ox[d] == nx[d] + h)) {
        rs[d] = 0;
        re[d] = 1;
      } else if ((a == 0 && ox[d] + hc == nx[d]) || (a == mo - 1 && ox[d] + hc == nx[d] + h)) {
        rs[d] = co - 1;
        re[d] = co;
      } else {
        rs[d] = 0;
        re[d] = co;
      }
    }
    const int *c = I.cconn + t * (long long)(co * co * co);
    for (int kk = rs[2]; kk < re[2]; kk++)
      for (int jj = rs[1]; jj < re[1]; jj++)
        for (int ii = rs[0]; ii < re[0]; ii++) {
          int cv = __ldg(c + ii + jj * co + kk * co * co);
          ne += (cv >= 0) ? 1 : (__ldg(I.cdptr - cv) - __ldg(I.cdptr - cv - 1));
        }
  }
  bound[row] = ne;
}

// Pass 2: the rows, written merged at the bound offsets of a scratch
// buffer; cnt[row] = merged length.
__global__ void __launch_bounds__(IW_WARPS * 32)
    k_interp_rows(long long rows, InterpCtx I, const int *__restrict__ trow,
                  const long long *__restrict__ toff, int *cnt, int *cols,
                  double *vals) {
  __shared__ int s_col[IW_WARPS][IMAX_W];
  __shared__ double s_w[IW_WARPS][IMAX_W];
  __shared__ short s_ord[IW_WARPS][IMAX_W];
  const bool WRITE = true;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const unsigned lt = (1u << lane) - 1u;
  const long long base = ((long long)blockIdx.x * IW_WARPS + warp) * 32;
  if (base >= rows) return;
  const int mo = I.fo, co = I.co, fnpe = mo * mo * mo;
  // phase A
  long long t = -1;
  int box = 0;  // is | ie<<2 | js<<4 | je<<6 | ks<<8 | ke<<10
  double Nu[IMAX_CO] = {0, 0, 0}, Nv[IMAX_CO] = {0, 0, 0}, Nw[IMAX_CO] = {0, 0, 0};
  {
    long long row = base + lane;
    if (row < rows) {
      unsigned long long r = I.rep[row];
      long long e = (long long)(r / fnpe);
      int info = (int)(r - (unsigned long long)e * fnpe);
      Oct node{I.fb[e], I.fx[e], I.fy[e], I.fz[e], I.fl[e]};
      t = trow[row];
      if (t >= 0) {
        int i = info % mo, j = (info % (mo * mo)) / mo, k = info / (mo * mo);
        int4 cq = __ldg(I.c4 + t);
        int cl = cq.x >> 26;
        int32_t h = side_of(node.level), hc = side_of(cl);
        double ihc = inv_side(cl);
        int is, ie, js, je, ks, ke;
        dir_weights(I, i, node.x, h, cq.y, hc, ihc, is, ie, Nu);
        dir_weights(I, j, node.y, h, cq.z, hc, ihc, js, je, Nv);
        dir_weights(I, k, node.z, h, cq.w, hc, ihc, ks, ke, Nw);
        box = is | (ie << 2) | (js << 4) | (je << 6) | (ks << 8) | (ke << 10);
      } else {
        atomicExch(I.err, 1);
      }
    }
  }
  // phase B
  for (int q = 0; q < 32; q++) {
    long long row = base + q;
    if (row >= rows) break;
    long long tq = __shfl_sync(0xffffffffu, t, q);
    int bq = __shfl_sync(0xffffffffu, box, q);
    double nu[IMAX_CO], nv[IMAX_CO], nw[IMAX_CO];
#pragma unroll
    for (int a = 0; a < IMAX_CO; a++) {
      nu[a] = __shfl_sync(0xffffffffu, Nu[a], q);
      nv[a] = __shfl_sync(0xffffffffu, Nv[a], q);
      nw[a] = __shfl_sync(0xffffffffu, Nw[a], q);
    }
    if (tq < 0) {
      if (lane == 0) cnt[row] = 0;
      continue;
    }
    int is = bq & 3, ie = (bq >> 2) & 3, js = (bq >> 4) & 3, je = (bq >> 6) & 3,
        ks = (bq >> 8) & 3, ke = (bq >> 10) & 3;
    int di = ie - is, dj = je - js, nb = di * dj * (ke - ks);
    int cv = 0, myn = 0, dp0 = 0;
    double wt = 0.0;
    if (lane < nb) {
      int ii = is + lane % di, jj = js + (lane / di) % dj, kk = ks + lane / (di * dj);
      cv = __ldg(I.cconn + tq * (long long)(co * co * co) + ii + jj * co + kk * co * co);
      wt = __dmul_rn(__dmul_rn(nu[ii], nv[jj]), nw[kk]);
      if (cv >= 0) {
        myn = 1;
      } else {
        int d = -cv - 1;
        dp0 = __ldg(I.cdptr + d);
        myn = __ldg(I.cdptr + d + 1) - dp0;
      }
    }
    int incl = myn;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int y = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += y;
    }
    const int ne = __shfl_sync(0xffffffffu, incl, 31);
    int off = incl - myn;
    if (myn == 1 && cv >= 0) {
      s_col[warp][off] = cv;
      s_w[warp][off] = wt;
    } else {
      for (int p = 0; p < myn; p++) {
        s_col[warp][off + p] = __ldg(I.cdconn + dp0 + p);
        s_w[warp][off + p] = __dmul_rn(wt, __ldg(I.cdw + dp0 + p));
      }
    }
    __syncwarp();
    // stable ranks
    for (int a = lane; a < ne; a += 32) {
      int col = s_col[warp][a];
      int rk = 0;
      for (int b = 0; b < ne; b++) {
        int cb = s_col[warp][b];
        rk += (cb < col) || (cb == col && b < a);
      }
      s_ord[warp][rk] = (short)a;
    }
    __syncwarp();
    // merge runs of equal columns
    int run = 0;
    long long rp = toff[row];
    for (int c0 = 0; c0 < ne; c0 += 32) {
      int sidx = c0 + lane;
      bool head = false;
      int col = 0;
      if (sidx < ne) {
        col = s_col[warp][s_ord[warp][sidx]];
        head = (sidx == 0) || (s_col[warp][s_ord[warp][sidx - 1]] != col);
      }
      unsigned hm = __ballot_sync(0xffffffffu, head);
      if (WRITE && head) {
        double acc = s_w[warp][s_ord[warp][sidx]];
        for (int n2 = sidx + 1; n2 < ne && s_col[warp][s_ord[warp][n2]] == col; n2++)
          acc = __dadd_rn(acc, s_w[warp][s_ord[warp][n2]]);
        long long o = rp + run + __popc(hm & lt);
        cols[o] = col;
        vals[o] = acc;
      }
      run += __popc(hm);
    }
    if (lane == 0) cnt[row] = run;
    __syncwarp();
  }
}

// 8 lanes per row copy a merged row from scratch into the CSR.
__global__ void k_interp_compact(long long rows, const long long *__restrict__ toff,
                                 const long long *__restrict__ rp,
                                 const int *__restrict__ tc, const double *__restrict__ tv,
                                 int *cols, double *vals) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  long long r = t >> 3;
  if (r >= rows) return;
  int lane = (int)(t & 7);
  long long s0 = toff[r], d0 = rp[r], n = rp[r + 1] - d0;
  for (long long k = lane; k < n; k += 8) {
    cols[d0 + k] = tc[s0 + k];
    vals[d0 + k] = tv[s0 + k];
  }
}
__global__ void k_ptr32(long long n, const long long *__restrict__ in, int *out) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i <= n) out[i] = (int)in[i];
}
__global__ void k_widen(long long n, const int *__restrict__ in, long long *out) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = in[i];
}

// Transpose support.  Entries are keyed row << 32 | column; the stable
// sort runs on the column bits only, so rows stay ascending inside each
// column (the entries arrive row-major) with a third of the passes a full
// (column, row) key would take.  8 lanes per row write its entries.
__global__ void k_t_keys(long long rows, const int *__restrict__ rowptr,
                         const int *__restrict__ cols, uint64_t *keys,
                         uint32_t *vals) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  long long r = t >> 3;
  if (r >= rows) return;
  int lane = (int)(t & 7);
  for (int p = rowptr[r] + lane; p < rowptr[r + 1]; p += 8) {
    keys[p] = ((uint64_t)r << 32) | (uint64_t)(uint32_t)cols[p];
    vals[p] = (uint32_t)p;
  }
}
__global__ void k_t_fill(long long nnz, const uint64_t *__restrict__ keys,
                         const uint32_t *__restrict__ perm,
                         const double *__restrict__ vals, int *tcols,
                         double *tvals, int *trowptr) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nnz) return;
  uint64_t k = keys[i];
  tcols[i] = (int)(k >> 32);
  tvals[i] = vals[perm[i]];
  // column starts: every column in (previous column, this column] begins here
  int c = (int)(k & 0xffffffffu);
  int cprev = (i == 0) ? -1 : (int)(keys[i - 1] & 0xffffffffu);
  for (int j = cprev + 1; j <= c; j++) trowptr[j] = (int)i;
}
__global__ void k_t_tail(long long ncols, long long nnz, const uint64_t *__restrict__ keys,
                         int *trowptr) {
  // columns after the last entry's column are empty
  long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  int clast = nnz ? (int)(keys[nnz - 1] & 0xffffffffu) : -1;
  if (j > clast && j <= ncols) trowptr[j] = (int)nnz;
}
__global__ void k_rowsum(long long rows, const int *__restrict__ rowptr,
                         const double *__restrict__ vals, double *sum) {
  long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= rows) return;
  double s = 0.0;
  for (int p = rowptr[r]; p < rowptr[r + 1]; p++) s = __dadd_rn(s, vals[p]);
  sum[r] = s;
}

void interp_create(Forest &fine, Forest &coarse, Interp &I) {
  Stage st("tmrg_create_interpolation");
  if (&fine == &coarse)
    throw Error(TMRG_ERR_ARG, "Cannot interpolate between the same object");
  if (fine.interp != coarse.interp)
    throw Error(TMRG_ERR_ARG,
                "Interpolation types between meshes are not identical");
  if (coarse.order > IMAX_CO)
    throw Error(TMRG_ERR_UNSUPPORTED,
                "createInterpolation: coarse order > 3 is not built");
  forest_create_nodes(fine);
  forest_create_nodes(coarse);
  TMRG_CUDA(cudaStreamSynchronize(coarse.s));
  cudaStream_t s = fine.s;
  I.s = s;
  const int fnpe = fine.order * fine.order * fine.order;
  const long long rows = fine.num_owned;
  I.rows = rows;
  I.cols = coarse.num_owned;
  DBuf<unsigned long long> rep(rows + 1, s);
  rep.fill_bytes(0xff);
  long long m = fine.n * fnpe;
  launch(k_first_ref, blocks_for(m, 256), 256, 0, s, m, fnpe, rows,
         (const int *)fine.econn.p, rep.p);
  DBuf<int> err(1, s);
  err.zero();
  InterpCtx c;
  c.fo = fine.order;
  c.co = coarse.order;
  for (int i = 0; i < TMRG_MAX_ORDER; i++) {
    c.fk[i] = fine.knots[i];
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
  c.cconn = coarse.econn.p;
  c.cdptr = coarse.dep_ptr.p;
  c.cdconn = coarse.dep_conn.p;
  c.cdw = coarse.dep_w.p;
  c.rep = rep.p;
  c.err = err.p;
  for (int i = 0; i < TMRG_MAX_ORDER; i++)
    for (int j = 0; j < TMRG_MAX_ORDER; j++)
      c.crk[i][j] = (i != j && i < coarse.order && j < coarse.order)
                        ? 1.0 / (coarse.knots[i] - coarse.knots[j])
                        : 0.0;
  const unsigned rblocks = blocks_for(rows, IW_WARPS * 32);
  // pass 1: enclosing octants and entry bounds; pass 2: merged rows into
  // scratch at the bound offsets; pass 3: compact into the CSR
  DBuf<int> trow(rows + 1, s);
  DBuf<long long> toff(rows + 1, s);
  launch(k_interp_bound, blocks_for(rows, 128), 128, 0, s, rows, c, trow.p, toff.p);
  exclusive_scan<long long>(toff.p, toff.p, rows, s);
  const long long nbound = read_scalar(toff.p + rows, s);
  DBuf<int> tcols(nbound + 1, s);
  DBuf<double> tvals(nbound + 1, s);
  DBuf<int> cnt(rows + 1, s);
  launch(k_interp_rows, rblocks, IW_WARPS * 32, 0, s, rows, c, (const int *)trow.p,
         (const long long *)toff.p, cnt.p, tcols.p, tvals.p);
  DBuf<long long> rp64(rows + 1, s);
  launch(k_widen, blocks_for(rows, 256), 256, 0, s, rows, (const int *)cnt.p,
         rp64.p);
  exclusive_scan<long long>(rp64.p, rp64.p, rows, s);
  const long long nnz = read_scalar(rp64.p + rows, s);
  if (nnz >= (1LL << 31) - 1)
    throw Error(TMRG_ERR_ARG, "createInterpolation: more than 2^31 entries");
  I.nnz = nnz;
  I.rowptr.alloc(rows + 1, s);
  launch(k_ptr32, blocks_for(rows + 1, 256), 256, 0, s, rows,
         (const long long *)rp64.p, I.rowptr.p);
  I.colidx.alloc(nnz + 1, s);
  I.vals.alloc(nnz + 1, s);
  launch(k_interp_compact, blocks_for(rows * 8, 256), 256, 0, s, rows,
         (const long long *)toff.p, (const long long *)rp64.p, (const int *)tcols.p,
         (const double *)tvals.p, I.colidx.p, I.vals.p);
  if (read_scalar(err.p, s))
    throw Error(TMRG_ERR_INTERNAL,
                "createInterpolation: a fine node has no enclosing coarse octant");

  // P^T by a stable sort on the column (rows stay ascending per column).
  Stage st_t("tmrg_transpose");
  const int cbits = bits_for(I.cols + 1);
  DBuf<uint64_t> tk(nnz, s);
  DBuf<uint32_t> tp(nnz, s);
  launch(k_t_keys, blocks_for(rows * 8, 256), 256, 0, s, rows,
         (const int *)I.rowptr.p, (const int *)I.colidx.p, tk.p, tp.p);
  radix_sort(tk, &tp, nnz, cbits, s);
  I.t_colidx.alloc(nnz + 1, s);
  I.t_vals.alloc(nnz + 1, s);
  I.t_rowptr.alloc(I.cols + 1, s);
  launch(k_t_fill, blocks_for(nnz, 256), 256, 0, s, nnz, (const uint64_t *)tk.p,
         (const uint32_t *)tp.p, (const double *)I.vals.p, I.t_colidx.p, I.t_vals.p,
         I.t_rowptr.p);
  launch(k_t_tail, blocks_for(I.cols + 1, 256), 256, 0, s, I.cols, nnz,
         (const uint64_t *)tk.p, I.t_rowptr.p);
  I.colsum.alloc(I.cols + 1, s);
  launch(k_rowsum, blocks_for(I.cols, 256), 256, 0, s, I.cols,
         (const int *)I.t_rowptr.p, (const double *)I.t_vals.p, I.colsum.p);
  TMRG_CUDA(cudaStreamSynchronize(s));
}

// ---------------------------------------------------------------------
// CSR apply over node-major multi-vectors: G lanes per row, lane v
// accumulates vectors v, v+G, ... in entry order.  With `scale` the
// result is divided by scale[row] (weight-normalised transpose).
__global__ void __launch_bounds__(256)
    k_csr_apply(long long rows, int G, int nvec, const int *__restrict__ rowptr,
                const int *__restrict__ cols, const double *__restrict__ vals,
                const double *__restrict__ x, double *__restrict__ y,
                const double *__restrict__ scale) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  long long r = t / G;
  int lane = (int)(t - r * G);
  if (r >= rows) return;
  int p0 = rowptr[r], p1 = rowptr[r + 1];
  for (int v = lane; v < nvec; v += G) {
    double acc = 0.0;
    for (int p = p0; p < p1; p++)
      acc = __fma_rn(__ldg(vals + p), __ldg(x + (long long)__ldg(cols + p) * nvec + v), acc);
    if (scale) {
      double sc = scale[r];
      acc = (sc != 0.0) ? __ddiv_rn(acc, sc) : 0.0;
    }
    y[r * nvec + v] = acc;
  }
}

// Paired-vector form for an even number of vectors: lane l of a row owns
// vectors 2l, 2l+1 (16-byte loads), LPR lanes per row.  Column indices and
// weights of 8 entries are loaded ahead of their 8 independent gathers;
// the accumulation still runs entry by entry in CSR order.
template <int LPR>
__global__ void __launch_bounds__(256)
    k_csr_apply2(long long rows, int nvec2, const int *__restrict__ rowptr,
                 const int *__restrict__ cols, const double *__restrict__ vals,
                 const double2 *__restrict__ x, double2 *__restrict__ y,
                 const double *__restrict__ scale) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  long long r = t / LPR;
  int lane = (int)(t & (LPR - 1));
  if (r >= rows) return;
  const int p0 = __ldg(rowptr + r), p1 = __ldg(rowptr + r + 1);
  for (int v = lane; v < nvec2; v += LPR) {
    double ax = 0.0, ay = 0.0;
    int p = p0;
    for (; p + 8 <= p1; p += 8) {
      int c[8];
      double w[8];
      double2 xv[8];
#pragma unroll
      for (int k = 0; k < 8; k++) {
        c[k] = __ldg(cols + p + k);
        w[k] = __ldg(vals + p + k);
      }
#pragma unroll
      for (int k = 0; k < 8; k++) xv[k] = __ldg(x + (long long)c[k] * nvec2 + v);
#pragma unroll
      for (int k = 0; k < 8; k++) {
        ax = __fma_rn(w[k], xv[k].x, ax);
        ay = __fma_rn(w[k], xv[k].y, ay);
      }
    }
    for (; p < p1; p++) {
      double2 xv = __ldg(x + (long long)__ldg(cols + p) * nvec2 + v);
      double w = __ldg(vals + p);
      ax = __fma_rn(w, xv.x, ax);
      ay = __fma_rn(w, xv.y, ay);
    }
    if (scale) {
      double sc = scale[r];
      ax = (sc != 0.0) ? __ddiv_rn(ax, sc) : 0.0;
      ay = (sc != 0.0) ? __ddiv_rn(ay, sc) : 0.0;
    }
    y[r * nvec2 + v] = make_double2(ax, ay);
  }
}

// Split-row form: NG groups of LPR lanes share one row (RPW = 32/(LPR*NG)
// rows per warp); group g takes entries g, g+NG, ...  The warp runs one
// trip count (the longest row it holds) with per-entry predicates, so no
// lane diverges: on GB300 the FP64 pipe is the bound and a diverged or
// half-masked warp instruction costs the pipe as much as a full one.
// Group partial sums are combined in a fixed tree order.
template <int LPR, int NG>
__global__ void __launch_bounds__(256)
    k_csr_apply_split(long long rows, int nvec2, const int *__restrict__ rowptr,
                      const int *__restrict__ cols, const double *__restrict__ vals,
                      const double2 *__restrict__ x, double2 *__restrict__ y,
                      const double *__restrict__ scale) {
  constexpr int RPW = 32 / (LPR * NG);
  const int lane = threadIdx.x & 31;
  const long long warp = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int sub = lane / (LPR * NG);       // row slot in the warp
  const int g = (lane / LPR) % NG;         // group in the row
  const int v = lane % LPR;                // vector pair
  const long long r = warp * RPW + sub;
  if (warp * RPW >= rows) return;          // uniform per warp
  const bool have = r < rows;
  const int p0 = have ? __ldg(rowptr + r) : 0;
  const int p1 = have ? __ldg(rowptr + r + 1) : 0;
  int trips = (p1 - p0 + NG - 1) / NG;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) trips = max(trips, __shfl_xor_sync(0xffffffffu, trips, o));
  for (int vb = 0; vb < nvec2; vb += LPR) {
    const bool act = have && (vb + v < nvec2);
    double ax = 0.0, ay = 0.0;
#pragma unroll 4
    for (int t = 0; t < trips; t++) {
      int p = p0 + g + t * NG;
      bool on = act && p < p1;
      int c = on ? __ldg(cols + p) : 0;
      double w = on ? __ldg(vals + p) : 0.0;
      double2 xv = on ? __ldg(x + (long long)c * nvec2 + vb + v) : make_double2(0.0, 0.0);
      ax = __fma_rn(w, xv.x, ax);
      ay = __fma_rn(w, xv.y, ay);
    }
#pragma unroll
    for (int o = (NG / 2) * LPR; o >= LPR; o >>= 1) {
      ax = __dadd_rn(ax, __shfl_down_sync(0xffffffffu, ax, o));
      ay = __dadd_rn(ay, __shfl_down_sync(0xffffffffu, ay, o));
    }
    if (act && g == 0) {
      if (scale) {
        double sc = scale[r];
        ax = (sc != 0.0) ? __ddiv_rn(ax, sc) : 0.0;
        ay = (sc != 0.0) ? __ddiv_rn(ay, sc) : 0.0;
      }
      y[r * nvec2 + vb + v] = make_double2(ax, ay);
    }
  }
}

template <int LPR>
static void apply2(long long rows, long long nnz, int nvec2, const int *rp,
                   const int *ci, const double *v, const double *x, double *y,
                   const double *scale, cudaStream_t s) {
  // long rows (P^T): the whole warp on one row; short rows (P): two rows
  // per warp when the lanes allow
  double avg = rows ? (double)nnz / (double)rows : 0.0;
  if (LPR == 8) {
    if (avg >= 48)
      launch((k_csr_apply_split<8, 4>), blocks_for(rows * 32, 256), 256, 0, s, rows,
             nvec2, rp, ci, v, (const double2 *)x, (double2 *)y, scale);
    else
      launch((k_csr_apply_split<8, 2>), blocks_for((rows + 1) / 2 * 32, 256), 256, 0, s,
             rows, nvec2, rp, ci, v, (const double2 *)x, (double2 *)y, scale);
    return;
  }
  launch(k_csr_apply2<LPR>, blocks_for(rows * LPR, 256), 256, 0, s, rows, nvec2,
         rp, ci, v, (const double2 *)x, (double2 *)y, scale);
}

void interp_apply(Interp &I, int which, const double *x, double *y, int nvec) {
  Stage st(which == 0 ? "tmrg_interp_mult" : "tmrg_interp_mult_transpose");
  if (nvec <= 0) throw Error(TMRG_ERR_ARG, "interp apply: nvec <= 0");
  cudaStream_t s = I.s;
  if (nvec % 2 == 0 && ((uintptr_t)x % 16) == 0 && ((uintptr_t)y % 16) == 0) {
    long long nin = (which == 0) ? I.cols : I.rows;
    long long nout = (which == 0) ? I.rows : I.cols;
    prof_bytes(12 * I.nnz + 4 * (nout + 1) + 8LL * nvec * (nin + nout) +
               (which == 2 ? 8 * nout : 0));
    prof_flops(2LL * nvec * I.nnz);
    const int *rp = which == 0 ? I.rowptr.p : I.t_rowptr.p;
    const int *ci = which == 0 ? I.colidx.p : I.t_colidx.p;
    const double *v = which == 0 ? I.vals.p : I.t_vals.p;
    const double *sc = which == 2 ? I.colsum.p : nullptr;
    int n2 = nvec / 2;
    if (n2 >= 8)
      apply2<8>(nout, I.nnz, n2, rp, ci, v, x, y, sc, s);
    else if (n2 >= 4)
      apply2<4>(nout, I.nnz, n2, rp, ci, v, x, y, sc, s);
    else if (n2 >= 2)
      apply2<2>(nout, I.nnz, n2, rp, ci, v, x, y, sc, s);
    else
      apply2<1>(nout, I.nnz, n2, rp, ci, v, x, y, sc, s);
    return;
  }
  int G = 1;
  while (G < nvec && G < 32) G <<= 1;
  // compulsory traffic: 12 B per entry, the row pointers, one read of the
  // input and one write of the output vectors
  long long nin = (which == 0) ? I.cols : I.rows;
  long long nout = (which == 0) ? I.rows : I.cols;
  prof_bytes(12 * I.nnz + 4 * (nout + 1) + 8LL * nvec * (nin + nout) +
             (which == 2 ? 8 * nout : 0));
  prof_flops(2LL * nvec * I.nnz);
  if (which == 0) {
    long long threads = I.rows * G;
    launch(k_csr_apply, blocks_for(threads, 256), 256, 0, s, I.rows, G, nvec,
           (const int *)I.rowptr.p, (const int *)I.colidx.p,
           (const double *)I.vals.p, x, y, (const double *)nullptr);
  } else {
    long long threads = I.cols * G;
    launch(k_csr_apply, blocks_for(threads, 256), 256, 0, s, I.cols, G, nvec,
           (const int *)I.t_rowptr.p, (const int *)I.t_colidx.p,
           (const double *)I.t_vals.p, x, y,
           which == 2 ? (const double *)I.colsum.p : (const double *)nullptr);
  }
}

}  // namespace tmrg
