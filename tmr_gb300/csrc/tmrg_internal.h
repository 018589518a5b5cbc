// Internal object layouts shared by the library's translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <functional>
#include <memory>
#include <vector>

#include "tmrg_common.cuh"
#include "tmrg_prims.cuh"

namespace tmrg {

// The autotuner's interface (TuneKey, tune_run, tune_lookup) is declared
// in tmrg_prims.cuh, beside the radix sort that uses it.

// Device view of the block connectivity tables.  CSR entries hold
// 8*block+corner, 12*block+edge, 6*block+face; the first entry of each
// list is the lowest-numbered block, which owns the shared entity
// (TMROctForest.cpp:1090-1143).
struct ConnDev {
  int nb;
  const int *block_conn;  // 8 per block
  const int *block_edge;  // 12 per block: global edge number
  const int *block_face;  // 6 per block: global face number
  const int *face_ids;    // 6 per block: orientation relative to owner
  const int *node_ptr, *node_ent;
  const int *edge_ptr, *edge_ent;
  const int *face_ptr, *face_ent;
};

// Block connectivity: built on the host (O(blocks)) and mirrored on the
// device.  Shared by a forest and the forests derived from it.
struct Conn {
  int num_nodes = 0, num_edges = 0, num_faces = 0, nb = 0;
  std::vector<int> block_conn, block_edge, block_face, face_ids;
  std::vector<int> node_ptr, node_ent, edge_ptr, edge_ent, face_ptr, face_ent;
  int max_node_val = 1, max_edge_val = 1, max_face_val = 1;
  DBuf<int> d_all;
  ConnDev dev{};
  int block_bits = 1;
  // optional axis-aligned box of every block (origin xyz, extent xyz): the
  // geometry getPoints maps nodes through; empty = no geometry
  std::vector<double> boxes;
  DBuf<double> d_boxes;
};
std::shared_ptr<Conn> build_conn(int num_nodes, const int *block_conn,
                                 int num_blocks, cudaStream_t s, int num_edges = 0,
                                 const int *block_edge = nullptr, int num_faces = 0,
                                 const int *block_face = nullptr);

struct Forest {
  cudaStream_t s = 0;
  int order = 2, interp = 1;
  double knots[TMRG_MAX_ORDER] = {0};
  std::shared_ptr<Conn> conn;

  // Octants, structure of arrays, sorted in TMR element order.
  bool have_octs = false;
  long long n = 0;
  int maxlev = 0;  // finest level present (key width)
  DBuf<int> block, x, y, z;
  DBuf<int16_t> level, info;

  // createNodes products.
  bool have_nodes = false;
  long long num_local = 0, num_owned = 0, num_dep = 0, dep_nnz = 0,
            ext_pre = 0;
  DBuf<int> econn;  // n * order^3 global node numbers
  DBuf<int> dep_ptr, dep_conn;
  DBuf<double> dep_w;

  void free_nodes() {
    have_nodes = false;
    econn.release();
    dep_ptr.release();
    dep_conn.release();
    dep_w.release();
    num_local = num_owned = num_dep = dep_nnz = ext_pre = 0;
  }
  void set_order(int o, int it);
  OctKey oct_key() const;
};

// An entry the P / P^T applies keep: |w| >= 2^-49 (and Inf / NaN), from the
// exponent bits (no FP64 compare).
#ifdef __CUDACC__
__device__ __forceinline__ int apply_keeps(double w) {
  return (int)((__double_as_longlong(w) >> 52) & 0x7ff) >= 1023 - 49;
}
#endif

struct Interp {
  cudaStream_t s = 0;
  long long rows = 0, cols = 0, nnz = 0;
  DBuf<int> rowptr, colidx;  // P, row-sorted CSR, every entry the reference keeps
  DBuf<double> vals;
  // The applies run on P without its numerically-zero entries, |w| < 2^-49
  // (apply_keeps): a fine node on a coarse knot plane has zero weights for
  // the other knots of that direction, exactly 0 with exact knots and
  // rounding residue below 4e-17 with the Gauss-Lobatto middle knot
  // -cos(pi/2) = -6.1e-17 (about half of an order-3 P).  Leaving them out
  // changes y_i = sum_j P_ij x_j by at most (dropped entries of row i)
  // * 2^-49 * max |x_j|, below 1e-13 of max |x| for the row lengths of P;
  // P itself (getCSR) keeps every entry.  Without such entries
  // (nnz_nz == nnz) the applies use P's structure.
  long long nnz_nz = 0;
  DBuf<int> nz_rowptr, nz_colidx;
  const int *ap_rowptr() const { return nnz_nz < nnz ? nz_rowptr.p : rowptr.p; }
  const int *ap_colidx() const { return nnz_nz < nnz ? nz_colidx.p : colidx.p; }
  // The apply copy's weights as double-float pairs (hi, lo): w = hi + lo to
  // 2^-48 |w| (df_split).  The applies run in double-float arithmetic on the
  // FP32 pipe (GB300 issues FP64 at 1/64 of its FP32 rate), same 8 bytes
  // per weight as an FP64 copy.
  DBuf<float2> ap_w;
  DBuf<int> perm;  // apply rows ordered by length inside windows
  DBuf<int> t_rowptr, t_colidx;  // P^T (zero-free) as CSR, rows = coarse nodes
  DBuf<int> t_perm;  // P^T rows by input chunk of their last entry, then length
  std::vector<long long> t_chunk;  // t_perm range of each input chunk
  // largest column read by each LO_WIN-row window of the apply copy (host
  // copy, made by the first host-buffer prolongation)
  std::vector<int> win_maxcol;
  DBuf<float2> t_w;  // P^T weights (hi, lo)
  // dfflag[0]: a weight outside the double-float window (the applies then
  // run in FP64); dfflag[1]: the same for the input vector of one apply
  DBuf<int> dfflag;
  bool have_colsum = false;
  DBuf<double> colsum;  // P^T 1 (column sums of P), made on first use
};

struct Filter {
  cudaStream_t s = 0;
  long long n = 0, nnz = 0;
  int N = 10;
  double r = 0.0;
  DBuf<int> rowptr, colidx;
  DBuf<double> vals;
  DBuf<double> Ainv, B, Tinv;
  DBuf<float> Ainv32, B32, Tinv32;
  // M as sliced ELL for the Horner steps: rows in length order inside
  // 4096-row windows (sperm, with each position's row length in srl),
  // slices of 32 positions stored entry-major from soff[slice], so a warp
  // reads its rows' k-th entries as one contiguous run
  long long npos = 0, nsell = 0;
  DBuf<int> sperm, srl, scol;
  DBuf<long long> soff;
  DBuf<double> sval;
  DBuf<float> sval32;
};

// Operations (tmrg_forest.cu, tmrg_nodes.cu, tmrg_interp.cu,
// tmrg_filter.cu).
void forest_create_trees(Forest &f, int level);
void forest_refine(Forest &f, const int *d_ref, long long nref, int min_level,
                   int max_level);
void forest_coarsen(Forest &f, Forest &out);
void forest_duplicate(Forest &f, Forest &out);
void forest_balance(Forest &f, int corner);
void forest_create_nodes(Forest &f);
void interp_create(Forest &fine, Forest &coarse, Interp &I);
void interp_apply(Interp &I, int which, const double *x, double *y, int nvec);
// The apply structures of a finished P with `nonzeros` apply_keeps entries;
// keepoff (optional, device) holds their exclusive per-row offsets.
void interp_finish(Interp &I, long long nonzeros, cudaStream_t s,
                   const long long *keepoff = nullptr);
void interp_check_apply(Interp &I);
bool interp_apply_transpose_staged(Interp &I, int which, const double *xh, double *dx,
                                   double *y, int nvec);
bool interp_apply_forward_staged(Interp &I, const double *xh, double *dx, double *yh,
                                 int nvec);
void topo_weights_create(Forest &filter, Forest &analysis, Interp &I);
void filter_create(Forest &f, double len, double r, int N, Filter &F);
struct QForest;
void filter_create_quad(QForest &f, double len, double r, int N, Filter &F);
// Rows in length order inside 4096-row windows (perm[position] = row).
void len_order(long long rows, const int *rp, int *perm, cudaStream_t s);
void filter_apply(Filter &F, bool transpose, int vpn, const double *in,
                  double *out);
void filter_apply_f32(Filter &F, bool transpose, int vpn, const float *in,
                      float *out);
void filter_apply_static(Filter &F, bool transpose, int vpn, const double *in,
                         double *out);
void random_refinement(uint64_t seed, uint64_t stream, double prob, int *out,
                       long long n, cudaStream_t s);
void forest_create_random_trees(Forest &f, int nrand, int min_level, int max_level,
                                uint64_t seed);
void batch_refinement(Forest &f, int nforests, const int *d_first_block,
                      const int *d_block_forest, const double *d_prob, const int *d_active,
                      uint64_t seed, uint64_t pass, long long *d_start, int *d_out);
void bump_indicator(Forest &f, const double *d_centres, int K, const double sigma[3],
                    double t_refine, double t_coarsen, int min_level, int max_level,
                    int *d_out);
void forest_transform_nodes(Forest &f, tmrg_octant *d_octs, long long n, int edge_dir,
                            int *d_rev, int *d_fid);
void forest_find_enclosing(Forest &f, int order, const double *knots,
                           const tmrg_octant *d_nodes, long long n, long long *d_index);
void forest_get_points(Forest &f, const double *boxes, double *d_X);
long long stl_triangles(Forest &f, const double *d_x, int vpn, int offset, double cutoff,
                        DBuf<double> &tris);

}  // namespace tmrg
