// createInterpolation and the P / P^T applies on the GPU.
//
// P (coarse -> fine) has one row per owned fine node.  A node is handled
// through the first (element, local node) that references it in element
// order (TMROctForest.cpp:6654-6688); one thread per row runs the
// reference's findEnclosing search over the sorted coarse octants and
// computeElemInterp's tensor-product Lagrange weights with the coarse
// dependent-node expansion, then sorts and merges its entries by column
// (TMRIndexWeight::uniqueSort).  Rows are made in two passes (count, then
// write at the scanned offsets).  P^T is the same matrix re-sorted by
// (column, row), so transpose applies gather without atomics and sum in a
// fixed order.
#include "tmrg_tree.cuh"

namespace tmrg {

constexpr int IMAX_CO = 3;  // coarse orders built for createInterpolation
constexpr int IMAX_W = IMAX_CO * IMAX_CO * IMAX_CO * IMAX_CO * IMAX_CO;

struct InterpCtx {
  int fo, co;  // fine / coarse order
  double fk[TMRG_MAX_ORDER], ck[TMRG_MAX_ORDER];
  // fine octants
  const int *fb, *fx, *fy, *fz;
  const int16_t *fl;
  // coarse octants, connectivity and dependent CSR
  long long cn;
  const int *cb, *cx, *cy, *cz;
  const int16_t *cl;
  const int *cconn;
  const int *cdptr, *cdconn;
  const double *cdw;
  const unsigned long long *rep;  // fine node -> element*npe + local index
  int *err;
};

__global__ void k_first_ref(long long m, int npe, long long nowned,
                            const int *__restrict__ conn,
                            unsigned long long *rep) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= m) return;
  int c = conn[t];
  if (c >= 0 && c < nowned) atomicMin(rep + c, (unsigned long long)t);
}

__device__ __forceinline__ void lagrange_w(int order, double u, const double *kn,
                                           double *N) {
  for (int i = 0; i < order; i++) {
    double v = 1.0;
    for (int j = 0; j < order; j++) {
      if (i != j) {
        double dd = 1.0 / __dsub_rn(kn[i], kn[j]);
        v = __dmul_rn(v, __dmul_rn(__dsub_rn(u, kn[j]), dd));
      }
    }
    N[i] = v;
  }
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
    int32_t hm = side_of(I.cl[mid]);
    int32_t ab = I.cb[mid], ax = I.cx[mid], ay = I.cy[mid], az = I.cz[mid];
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
  while (mid < I.cn &&
         cmp_position(I.cb[mid], I.cx[mid], I.cy[mid], I.cz[mid], node.block, bx,
                      by, bz) <= 0) {
    if (I.cb[mid] == node.block) {
      int32_t hm = side_of(I.cl[mid]);
      int32_t ax = I.cx[mid], ay = I.cy[mid], az = I.cz[mid];
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
                                            int &s, int &e, double *N) {
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
    double u = __dadd_rn(-1.0, __ddiv_rn(__dmul_rn(2.0, __dsub_rn(t, (double)ox)),
                                          (double)hc));
    lagrange_w(co, u, I.ck, N);
  }
}

// Row of P for fine node `row`; returns the entry count, writes entries
// when cols/vals are given.
__device__ int interp_row(const InterpCtx &I, long long row, int *cols,
                          double *vals) {
  unsigned long long r = I.rep[row];
  const int fnpe = I.fo * I.fo * I.fo;
  long long e = (long long)(r / fnpe);
  int info = (int)(r - (unsigned long long)e * fnpe);
  Oct node{I.fb[e], I.fx[e], I.fy[e], I.fz[e], I.fl[e]};
  long long t = find_enclosing(I, node, info);
  if (t < 0) {
    atomicExch(I.err, 1);
    return 0;
  }
  const int mo = I.fo, co = I.co;
  int i = info % mo, j = (info % (mo * mo)) / mo, k = info / (mo * mo);
  int32_t h = side_of(node.level), hc = side_of(I.cl[t]);
  double Nu[IMAX_CO], Nv[IMAX_CO], Nw[IMAX_CO];
  int is, ie, js, je, ks, ke;
  dir_weights(I, i, node.x, h, I.cx[t], hc, is, ie, Nu);
  dir_weights(I, j, node.y, h, I.cy[t], hc, js, je, Nv);
  dir_weights(I, k, node.z, h, I.cz[t], hc, ks, ke, Nw);
  int idx[IMAX_W];
  double w[IMAX_W];
  int n = 0;
  const int *c = I.cconn + t * (long long)(co * co * co);
  for (int kk = ks; kk < ke; kk++)
    for (int jj = js; jj < je; jj++)
      for (int ii = is; ii < ie; ii++) {
        int cv = c[ii + jj * co + kk * co * co];
        double wt = __dmul_rn(__dmul_rn(Nu[ii], Nv[jj]), Nw[kk]);
        if (cv >= 0) {
          idx[n] = cv;
          w[n] = wt;
          n++;
        } else {
          int d = -cv - 1;
          for (int p = I.cdptr[d]; p < I.cdptr[d + 1]; p++) {
            idx[n] = I.cdconn[p];
            w[n] = __dmul_rn(wt, I.cdw[p]);
            n++;
          }
        }
      }
  // stable insertion sort by column, then merge equal columns in order
  for (int a = 1; a < n; a++) {
    int ti = idx[a];
    double tw = w[a];
    int b = a - 1;
    while (b >= 0 && idx[b] > ti) {
      idx[b + 1] = idx[b];
      w[b + 1] = w[b];
      b--;
    }
    idx[b + 1] = ti;
    w[b + 1] = tw;
  }
  int m = 0;
  for (int a = 0; a < n; a++, m++) {
    double acc = w[a];
    int col = idx[a];
    while (a < n - 1 && idx[a + 1] == col) {
      acc = __dadd_rn(acc, w[a + 1]);
      a++;
    }
    if (cols) {
      cols[m] = col;
      vals[m] = acc;
    }
  }
  return m;
}

__global__ void k_interp_count(long long rows, InterpCtx I, int *cnt) {
  long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (r < rows) cnt[r] = interp_row(I, r, nullptr, nullptr);
}
__global__ void k_interp_write(long long rows, InterpCtx I,
                               const long long *__restrict__ rowptr64,
                               int *cols, double *vals) {
  long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (r < rows) interp_row(I, r, cols + rowptr64[r], vals + rowptr64[r]);
}
__global__ void k_ptr32(long long n, const long long *__restrict__ in, int *out) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i <= n) out[i] = (int)in[i];
}
__global__ void k_widen(long long n, const int *__restrict__ in, long long *out) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = in[i];
}

// Transpose support: (col, row) keys for every entry.
__global__ void k_t_keys(long long rows, const int *__restrict__ rowptr,
                         const int *__restrict__ cols, int rbits,
                         uint64_t *keys, uint32_t *vals) {
  long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= rows) return;
  for (int p = rowptr[r]; p < rowptr[r + 1]; p++) {
    keys[p] = ((uint64_t)(uint32_t)cols[p] << rbits) | (uint64_t)r;
    vals[p] = (uint32_t)p;
  }
}
__global__ void k_t_fill(long long nnz, int rbits, const uint64_t *__restrict__ keys,
                         const uint32_t *__restrict__ perm,
                         const double *__restrict__ vals, int *tcols,
                         double *tvals, int *tcount) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nnz) return;
  uint64_t k = keys[i];
  tcols[i] = (int)(k & ((1ULL << rbits) - 1));
  tvals[i] = vals[perm[i]];
  atomicAdd(tcount + (k >> rbits), 1);
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
  c.cb = coarse.block.p;
  c.cx = coarse.x.p;
  c.cy = coarse.y.p;
  c.cz = coarse.z.p;
  c.cl = coarse.level.p;
  c.cconn = coarse.econn.p;
  c.cdptr = coarse.dep_ptr.p;
  c.cdconn = coarse.dep_conn.p;
  c.cdw = coarse.dep_w.p;
  c.rep = rep.p;
  c.err = err.p;
  DBuf<int> cnt(rows + 1, s);
  launch(k_interp_count, blocks_for(rows, 128), 128, 0, s, rows, c, cnt.p);
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
  launch(k_interp_write, blocks_for(rows, 128), 128, 0, s, rows, c,
         (const long long *)rp64.p, I.colidx.p, I.vals.p);
  if (read_scalar(err.p, s))
    throw Error(TMRG_ERR_INTERNAL,
                "createInterpolation: a fine node has no enclosing coarse octant");

  // P^T by a stable sort on (column, row).
  const int rbits = bits_for(rows + 1);
  const int cbits = bits_for(I.cols + 1);
  if (rbits + cbits > 64) throw Error(TMRG_ERR_KEY_RANGE, "transpose key range");
  DBuf<uint64_t> tk(nnz, s);
  DBuf<uint32_t> tp(nnz, s);
  launch(k_t_keys, blocks_for(rows, 256), 256, 0, s, rows,
         (const int *)I.rowptr.p, (const int *)I.colidx.p, rbits, tk.p, tp.p);
  radix_sort(tk, &tp, nnz, rbits + cbits, s);
  I.t_colidx.alloc(nnz + 1, s);
  I.t_vals.alloc(nnz + 1, s);
  I.t_rowptr.alloc(I.cols + 1, s);
  I.t_rowptr.zero();
  launch(k_t_fill, blocks_for(nnz, 256), 256, 0, s, nnz, rbits,
         (const uint64_t *)tk.p, (const uint32_t *)tp.p, (const double *)I.vals.p,
         I.t_colidx.p, I.t_vals.p, I.t_rowptr.p);
  exclusive_scan<int>(I.t_rowptr.p, I.t_rowptr.p, I.cols, s);
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
      acc = __dadd_rn(acc, __dmul_rn(__ldg(vals + p), __ldg(x + (long long)__ldg(cols + p) * nvec + v)));
    if (scale) {
      double sc = scale[r];
      acc = (sc != 0.0) ? __ddiv_rn(acc, sc) : 0.0;
    }
    y[r * nvec + v] = acc;
  }
}

void interp_apply(Interp &I, int which, const double *x, double *y, int nvec) {
  if (nvec <= 0) throw Error(TMRG_ERR_ARG, "interp apply: nvec <= 0");
  int G = 1;
  while (G < nvec && G < 32) G <<= 1;
  cudaStream_t s = I.s;
  // compulsory traffic: 12 B per entry, the row pointers, one read of the
  // input and one write of the output vectors
  long long nin = (which == 0) ? I.cols : I.rows;
  long long nout = (which == 0) ? I.rows : I.cols;
  prof_bytes(12 * I.nnz + 4 * (nout + 1) + 8LL * nvec * (nin + nout) +
             (which == 2 ? 8 * nout : 0));
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
