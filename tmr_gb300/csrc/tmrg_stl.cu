// Iso-surface triangles of a design field on a forest
// (TMR_GenerateSTLTriangles, TMR_STLTools.cpp:639-852) on the GPU.
//
// Every element of the forest is split into (order-1)^3 cells whose corners
// are element nodes; a cell's corner values are the design values of its
// nodes (dependent nodes through their weights, TMR_STLTools.cpp:733-744)
// and its corner positions the forest's node points.  Each cell contributes
// the marching-cubes triangles of the level set value = cutoff and, where
// all four corners of a cell face lie on the domain boundary, the part of
// that face where value >= cutoff (so that the solid is closed).
// Triangles are written in element order, cells in (z, y, x) order inside
// an element, a cell's iso-surface triangles before its boundary-face
// triangles (faces in the order -x, +x, -y, +y, -z, +z): the reference's
// output order.  Two passes: a count per element, a scan, then each element
// writes its triangles at its offset (staged in shared memory, so that
// the output is stored block by block in full lines).
//
// Case tables are built here, on the host, by one construction rule rather
// than taken from a published table:
// * a cube face whose corners alternate inside/outside (inside = value <
//   cutoff) separates its inside corners (the solid is connected across
//   the face), every other face has at most one crossing segment;
// * the segments of the six faces, each directed from the crossing where
//   the counter-clockwise face boundary leaves the inside region to the
//   crossing where it re-enters it, chain into closed loops;
// * each loop, started at its lowest edge number, is split into a fan of
//   triangles (normals point to the inside, lower-valued, side);
// * a boundary face's polygon is its solid corners and crossings in
//   counter-clockwise order seen from outside, split into a fan.
// The crossing points themselves are computed exactly as the reference
// computes them (vertex_interp, TMR_STLTools.cpp:339-356, with the same
// endpoint order per edge), so every triangle vertex is bit-equal to a
// reference vertex; loops equal the reference's wherever its table makes
// the same face choice, and fans may split a loop differently.
#include <cstdio>
#include <mutex>
#include <string>

#include "tmrg_internal.h"

namespace tmrg {

// Marching-cubes corner positions (x, y, z bits), edges as (from, to)
// corner pairs, and cube faces as corner lists counter-clockwise seen from
// outside: the corner and edge numbering of TMR_STLTools.cpp:385-427 and
// its face_vertex table (:465-466), which fix the interpolation order.
static const int MC_CORNER[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0},
                                    {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};
static const int MC_EDGE[12][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 0}, {4, 5}, {5, 6},
                                   {6, 7}, {7, 4}, {0, 4}, {1, 5}, {2, 6}, {3, 7}};
static const int MC_FACE[6][4] = {{0, 4, 7, 3}, {1, 2, 6, 5}, {0, 1, 5, 4},
                                  {3, 7, 6, 2}, {0, 3, 2, 1}, {4, 5, 6, 7}};
constexpr int MC_MAXTRI = 12;

struct StlTables {
  // volume cases: triangle count and edge triples
  int vn[256];
  signed char vt[256][MC_MAXTRI][3];
  // boundary-face cases: vertex ids 0-3 corners, 4-7 crossings on the face
  // edges (i, i+1)
  int fn[16];
  signed char ft[16][4][3];
  // cube faces (corner lists), corner offsets and edges, as MC_*
  int fe[6][4];
  int corner[8][3];
  int edge[12][2];
};

static int edge_of(int a, int b) {
  for (int e = 0; e < 12; e++)
    if ((MC_EDGE[e][0] == a && MC_EDGE[e][1] == b) || (MC_EDGE[e][0] == b && MC_EDGE[e][1] == a))
      return e;
  return -1;
}

static void build_tables(StlTables &T) {
  for (int c = 0; c < 256; c++) {
    int next[12];
    for (int e = 0; e < 12; e++) next[e] = -1;
    for (int f = 0; f < 6; f++) {
      const int *q = MC_FACE[f];
      // exits (inside -> outside) and entries (outside -> inside) along
      // the counter-clockwise boundary, with the position k of their edge
      int ex[2], en[2], exk[2], enk[2], nex = 0, nen = 0;
      for (int k = 0; k < 4; k++) {
        int a = q[k], b = q[(k + 1) & 3];
        int ia = (c >> a) & 1, ib = (c >> b) & 1;
        if (ia && !ib) {
          exk[nex] = k;
          ex[nex++] = edge_of(a, b);
        } else if (!ia && ib) {
          enk[nen] = k;
          en[nen++] = edge_of(a, b);
        }
      }
      // each inside arc runs from an entry to the next exit; its segment
      // goes from that exit back to that entry
      for (int i = 0; i < nen; i++) {
        // the first exit after entry i, counter-clockwise
        int best = -1, bd = 5;
        for (int j = 0; j < nex; j++) {
          int d = (exk[j] - enk[i] + 4) & 3;
          if (d < bd) {
            bd = d;
            best = j;
          }
        }
        next[ex[best]] = en[i];
      }
    }
    int n = 0;
    bool seen[12] = {false};
    for (int e0 = 0; e0 < 12; e0++) {
      if (next[e0] < 0 || seen[e0]) continue;
      int loop[12], k = 0;
      for (int e = e0; !seen[e]; e = next[e]) {
        seen[e] = true;
        loop[k++] = e;
      }
      for (int i = 1; i + 1 < k; i++) {
        T.vt[c][n][0] = (signed char)loop[0];
        T.vt[c][n][1] = (signed char)loop[i];
        T.vt[c][n][2] = (signed char)loop[i + 1];
        n++;
      }
    }
    T.vn[c] = n;
  }
  for (int c = 0; c < 16; c++) {
    int poly[8], k = 0;
    for (int i = 0; i < 4; i++) {
      int in_i = (c >> i) & 1, in_j = (c >> ((i + 1) & 3)) & 1;
      if (!in_i) poly[k++] = i;
      if (in_i != in_j) poly[k++] = 4 + i;
    }
    int n = 0;
    for (int i = 1; i + 1 < k; i++) {
      T.ft[c][n][0] = (signed char)poly[0];
      T.ft[c][n][1] = (signed char)poly[i];
      T.ft[c][n][2] = (signed char)poly[i + 1];
      n++;
    }
    T.fn[c] = n;
  }
  for (int f = 0; f < 6; f++)
    for (int i = 0; i < 4; i++) T.fe[f][i] = MC_FACE[f][i];
  for (int m = 0; m < 8; m++)
    for (int a = 0; a < 3; a++) T.corner[m][a] = MC_CORNER[m][a];
  for (int e = 0; e < 12; e++)
    for (int a = 0; a < 2; a++) T.edge[e][a] = MC_EDGE[e][a];
}

static const StlTables &tables() {
  static StlTables T;
  static std::once_flag once;
  std::call_once(once, [] {
    build_tables(T);
    for (int c = 0; c < 256; c++)
      if (T.vn[c] > MC_MAXTRI) throw Error(TMRG_ERR_INTERNAL, "stl: case table overflow");
  });
  return T;
}

struct StlCtx {
  long long n;
  int o;                    // mesh order
  long long num_dep;        // local index of node g is g + num_dep
  const int *econn;
  const int *dptr, *dconn;
  const double *dw;
  const double *X;          // node points (num_local x 3)
  const double *x;          // design values, vpn interleaved
  int vpn, off;
  double cutoff;
  const int *block, *ox, *oy, *oz;
  const int16_t *level;
  const int *bface;         // 6 per block: block face on the domain boundary
  int bern;                 // Bernstein interpolation (order 2): values by the basis
  const double *NB;         // npe x npe corner weights when bern
};

__constant__ StlTables c_stl;

// vertex_interp (TMR_STLTools.cpp:339-356): the point where the value
// reaches iso on the segment p1 -> p2, with the reference's exact-hit rules.
__device__ __forceinline__ void vinterp(double iso, const double *p1, const double *p2,
                                        double v1, double v2, double *p) {
  const double *q = nullptr;
  if (fabs(iso - v1) <= 0.0)
    q = p1;
  else if (fabs(iso - v2) <= 0.0)
    q = p2;
  else if (fabs(v1 - v2) <= 0.0)
    q = p1;
  if (q) {
    p[0] = q[0];
    p[1] = q[1];
    p[2] = q[2];
    return;
  }
  double mu = __ddiv_rn(iso - v1, v2 - v1);
  for (int a = 0; a < 3; a++) p[a] = p1[a] + mu * (p2[a] - p1[a]);
}

// Per element: node values and points, then every cell; count only, or
// write the triangles from `out` (9 doubles each).
template <int O>
__device__ long long stl_element(const StlCtx &c, long long e, double *out) {
  constexpr int N = O * O * O;
  const int *ec = c.econn + e * N;
  double lv[N];
  int li[N];
  for (int a = 0; a < N; a++) {
    int g = ec[a];
    li[a] = (int)(g + c.num_dep);
    if (g >= 0) {
      lv[a] = c.x[(long long)g * c.vpn + c.off];
    } else {
      int d = -g - 1;
      double s = 0.0;
      for (int p = c.dptr[d]; p < c.dptr[d + 1]; p++)
        s = __dadd_rn(s, __dmul_rn(c.dw[p], c.x[(long long)c.dconn[p] * c.vpn + c.off]));
      lv[a] = s;
    }
  }
  // element faces on the domain boundary (TMR_STLTools.cpp:707-722)
  const int b = c.block[e];
  const int h = 1 << (TMRG_MAX_LEVEL - c.level[e]);
  const int hmax = TMRG_HMAX;
  bool fb[6];
  fb[0] = c.bface[6 * b + 0] && c.ox[e] == 0;
  fb[1] = c.bface[6 * b + 1] && c.ox[e] + h == hmax;
  fb[2] = c.bface[6 * b + 2] && c.oy[e] == 0;
  fb[3] = c.bface[6 * b + 3] && c.oy[e] + h == hmax;
  fb[4] = c.bface[6 * b + 4] && c.oz[e] == 0;
  fb[5] = c.bface[6 * b + 5] && c.oz[e] + h == hmax;
  long long cnt = 0;
  for (int iz = 0; iz < O - 1; iz++)
    for (int iy = 0; iy < O - 1; iy++)
      for (int ix = 0; ix < O - 1; ix++) {
        double val[8];
        int off[8];
        int onb = 0, any = 0;
        for (int m = 0; m < 8; m++) {
          const int ii = c_stl.corner[m][0], jj = c_stl.corner[m][1], kk = c_stl.corner[m][2];
          const int o = (ix + ii) + (iy + jj) * O + (iz + kk) * O * O;
          off[m] = o;
          if (c.bern) {
            double s = 0.0;
            for (int q = 0; q < N; q++) s = __dadd_rn(s, __dmul_rn(c.NB[o * N + q], lv[q]));
            val[m] = s;
          } else {
            val[m] = lv[o];
          }
          int bnd = (fb[0] && ix == 0 && ii == 0) || (fb[1] && ix == O - 2 && ii == 1) ||
                    (fb[2] && iy == 0 && jj == 0) || (fb[3] && iy == O - 2 && jj == 1) ||
                    (fb[4] && iz == 0 && kk == 0) || (fb[5] && iz == O - 2 && kk == 1);
          onb |= bnd << m;
          any |= bnd;
        }
        int ci = 0;
        for (int m = 0; m < 8; m++) ci |= (val[m] < c.cutoff) << m;
        const int nv = c_stl.vn[ci];
        if (out) {
          double vp[12][3];
          // crossing points of the edges the level set cuts
          for (int ed = 0; ed < 12 && nv; ed++) {
            const int a = c_stl.edge[ed][0], bb = c_stl.edge[ed][1];
            if (((ci >> a) ^ (ci >> bb)) & 1)
              vinterp(c.cutoff, c.X + 3LL * li[off[a]], c.X + 3LL * li[off[bb]], val[a], val[bb],
                      vp[ed]);
          }
          for (int t = 0; t < nv; t++) {
            double *w = out + 9 * (cnt + t);
            for (int k = 0; k < 3; k++)
              for (int a = 0; a < 3; a++) w[3 * k + a] = vp[c_stl.vt[ci][t][k]][a];
          }
        }
        cnt += nv;
        if (!any) continue;
        for (int f = 0; f < 6; f++) {
          int fc[4];
          bool all = true;
          for (int i = 0; i < 4; i++) {
            fc[i] = c_stl.fe[f][i];
            all = all && ((onb >> fc[i]) & 1);
          }
          if (!all) continue;
          int fi = 0;
          for (int i = 0; i < 4; i++) fi |= (val[fc[i]] < c.cutoff) << i;
          const int nf = c_stl.fn[fi];
          if (out && nf) {
            double vp[8][3];
            for (int i = 0; i < 4; i++)
              for (int a = 0; a < 3; a++) vp[i][a] = c.X[3LL * li[off[fc[i]]] + a];
            for (int i = 0; i < 4; i++) {
              const int j = (i + 1) & 3;
              if (((fi >> i) & 1) != ((fi >> j) & 1))
                vinterp(c.cutoff, vp[i], vp[j], val[fc[i]], val[fc[j]], vp[4 + i]);
            }
            for (int t = 0; t < nf; t++) {
              double *w = out + 9 * (cnt + t);
              for (int k = 0; k < 3; k++)
                for (int a = 0; a < 3; a++) w[3 * k + a] = vp[c_stl.ft[fi][t][k]][a];
            }
          }
          cnt += nf;
        }
      }
  return cnt;
}

template <int O>
__global__ void k_stl_count(StlCtx c, long long *cnt) {
  long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= c.n) return;
  cnt[e] = stl_element<O>(c, e, nullptr);
}
// The block's triangles are one contiguous run of the output: each thread
// writes its element's triangles into a shared-memory copy of that run,
// then the block stores the run with consecutive threads on consecutive
// doubles.  A block whose run exceeds the staging area writes directly.
constexpr int STL_THREADS = 128;
constexpr int STL_STAGE = 640;  // triangles (46 KB)
template <int O>
__global__ void __launch_bounds__(STL_THREADS)
    k_stl_write(StlCtx c, const long long *__restrict__ off, double *tris) {
  extern __shared__ double st[];
  const long long e0 = (long long)blockIdx.x * blockDim.x;
  const long long e = e0 + threadIdx.x;
  const long long e1 = min(e0 + (long long)blockDim.x, c.n);
  const long long base = off[e0], end = off[e1];
  const bool staged = end - base <= STL_STAGE;
  if (e < c.n) stl_element<O>(c, e, staged ? st + 9 * (off[e] - base) : tris + 9 * off[e]);
  if (staged) {
    __syncthreads();
    double *dst = tris + 9 * base;
    for (long long i = threadIdx.x; i < 9 * (end - base); i += blockDim.x) dst[i] = st[i];
  }
}


// Bernstein polynomials of degree o-1 at u in [-1, 1], by the recurrence
// of bernstein_shape_functions (TMRInterpolation.h:164-178).
static void bernstein(int o, double u, double *N) {
  const double a = 0.5 * (1.0 - u), b = 0.5 * (u + 1.0);
  N[0] = 1.0;
  for (int j = 1; j < o; j++) {
    double carry = 0.0;
    for (int k = 0; k < j; k++) {
      const double t = N[k];
      N[k] = carry + a * t;
      carry = b * t;
    }
    N[j] = carry;
  }
}

// Triangles of the level set x[offset] = cutoff on forest f (x: device,
// vpn interleaved values per independent node).  Returns the count and
// leaves 9 doubles per triangle in `tris`.
long long stl_triangles(Forest &f, const double *d_x, int vpn, int offset, double cutoff,
                        DBuf<double> &tris) {
  Stage st("tmrg_stl_triangles");
  if (!f.have_nodes) forest_create_nodes(f);
  if (f.order < 2 || f.order > 3)
    throw Error(TMRG_ERR_UNSUPPORTED, "STL triangles: forest order must be 2 or 3");
  if (vpn < 1 || offset < 0 || offset >= vpn)
    throw Error(TMRG_ERR_ARG, "STL triangles: offset outside the values per node");
  cudaStream_t s = f.s;
  static std::mutex mu;
  static bool uploaded[256] = {false};
  {
    int dev = 0;
    TMRG_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lk(mu);
    if (dev >= 0 && dev < 256 && !uploaded[dev]) {
      const StlTables &T = tables();
      TMRG_CUDA(cudaMemcpyToSymbol(c_stl, &T, sizeof(StlTables)));
      uploaded[dev] = true;
    }
  }
  const Conn &C = *f.conn;
  // node points (zero without geometry, as getPoints)
  DBuf<double> X(3 * std::max(1LL, f.num_local), s);
  if (C.boxes.empty())
    X.zero();
  else
    forest_get_points(f, C.d_boxes.p, X.p);
  // block faces on the domain boundary: faces shared by one block
  std::vector<int> hb(6 * std::max(1, C.nb), 0);
  for (int b = 0; b < C.nb; b++)
    for (int k = 0; k < 6; k++) {
      int fc = C.block_face[6 * b + k];
      hb[6 * b + k] = (C.face_ptr[fc + 1] - C.face_ptr[fc]) == 1;
    }
  DBuf<int> bface(hb.size(), s);
  TMRG_CUDA(cudaMemcpyAsync(bface.p, hb.data(), sizeof(int) * hb.size(),
                            cudaMemcpyHostToDevice, s));
  const int o = f.order, npe = o * o * o;
  // Bernstein values at the cell corners (order 2: the corner weights are
  // 0 and 1), the reference's evalInterp sum (TMR_STLTools.cpp:769-786)
  DBuf<double> NB;
  const bool bern = f.interp == TMRG_BERNSTEIN_POINTS;
  if (bern) {
    std::vector<double> hn((size_t)npe * npe);
    for (int q = 0; q < npe; q++) {
      int uu = q % o, vv = (q / o) % o, ww = q / (o * o);
      double pt[3] = {-1.0 + 2.0 / (o - 1.0) * uu, -1.0 + 2.0 / (o - 1.0) * vv,
                      -1.0 + 2.0 / (o - 1.0) * ww};
      double B[3][TMRG_MAX_ORDER];
      for (int a = 0; a < 3; a++) bernstein(o, pt[a], B[a]);
      for (int k = 0; k < o; k++)
        for (int j = 0; j < o; j++)
          for (int i = 0; i < o; i++) hn[(size_t)q * npe + i + o * j + o * o * k] =
                                          B[0][i] * B[1][j] * B[2][k];
    }
    NB.alloc(hn.size(), s);
    TMRG_CUDA(cudaMemcpyAsync(NB.p, hn.data(), sizeof(double) * hn.size(),
                              cudaMemcpyHostToDevice, s));
  }
  StlCtx c{f.n, o, f.num_dep, f.econn.p, f.dep_ptr.p, f.dep_conn.p, f.dep_w.p, X.p, d_x,
           vpn, offset, cutoff, f.block.p, f.x.p, f.y.p, f.z.p, f.level.p, bface.p,
           bern ? 1 : 0, NB.p};
  const long long n = f.n;
  DBuf<long long> cnt(n + 1, s);
  // compulsory traffic of a pass: element connectivity and octant fields,
  // the design values and dependent weights once, the per-element count
  const long long base = (4LL * npe + 18) * n + 8LL * f.num_owned * vpn +
                         16LL * f.dep_nnz + 4 * (f.num_dep + 1);
  prof_bytes(base + 8 * n);
  if (o == 2)
    launch(k_stl_count<2>, blocks_for(n, 128), 128, 0, s, c, cnt.p);
  else
    launch(k_stl_count<3>, blocks_for(n, 128), 128, 0, s, c, cnt.p);
  exclusive_scan<long long>(cnt.p, cnt.p, n, s);
  const long long ntri = read_scalar(cnt.p + n, s);
  tris.alloc(9 * std::max(1LL, ntri), s);
  if (ntri) {
    // plus the node points once and the triangles written
    prof_bytes(base + 8 * n + 24LL * f.num_local + 72LL * ntri);
    const size_t sm = sizeof(double) * 9 * STL_STAGE;
    if (o == 2)
      launch(k_stl_write<2>, blocks_for(n, STL_THREADS), STL_THREADS, sm, s, c,
             (const long long *)cnt.p, tris.p);
    else
      launch(k_stl_write<3>, blocks_for(n, STL_THREADS), STL_THREADS, sm, s, c,
             (const long long *)cnt.p, tris.p);
  }
  TMRG_CUDA(cudaStreamSynchronize(s));
  return ntri;
}

}  // namespace tmrg
