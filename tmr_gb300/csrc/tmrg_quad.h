// Quadtree forest objects (tmrg_quad.cu).
#pragma once

#include <memory>
#include <vector>

#include "tmrg_internal.h"

namespace tmrg {

template <typename Key>
struct QKeyT;
using QKey = QKeyT<uint64_t>;

// Device view of the face connectivity: CSR entries hold 4*face+corner and
// 4*face+edge; the first entry of each list is the lowest-numbered face,
// the owner of the shared node or edge (TMRQuadForest.cpp:388-650).
struct QConnDev {
  int nf;
  const int *face_conn;  // 4 per face
  const int *face_edge;  // 4 per face
  const int *node_ptr, *node_ent;
  const int *edge_ptr, *edge_ent;
};

struct QConn {
  int num_nodes = 0, num_edges = 0, nf = 0;
  std::vector<int> face_conn, face_edge, node_ptr, node_ent, edge_ptr, edge_ent;
  DBuf<int> d_all;
  QConnDev dev{};
  int block_bits = 1;
  // optional box of every face (origin x, y, extent x, y) for getPoints
  std::vector<double> boxes;
  DBuf<double> d_boxes;
};
std::shared_ptr<QConn> qconn_build(int num_nodes, const int *face_conn, int nf,
                                   const int *face_edge, int num_edges, cudaStream_t s);

struct QForest {
  cudaStream_t s = 0;
  int order = 2, interp = 1;
  double knots[3] = {-1.0, 1.0, 0.0};
  std::shared_ptr<QConn> conn;
  bool have_quads = false;
  long long n = 0;
  int maxlev = 0;
  DBuf<int> block, x, y;
  DBuf<int16_t> level, info;
  bool have_nodes = false;
  long long num_local = 0, num_owned = 0, num_dep = 0, dep_nnz = 0;
  DBuf<int> econn, dep_ptr, dep_conn;
  DBuf<double> dep_w;
  DBuf<int> node_num;        // node number of each local node
  void free_nodes() {
    have_nodes = false;
    econn.release();
    dep_ptr.release();
    dep_conn.release();
    dep_w.release();
    node_num.release();
    num_local = num_owned = num_dep = dep_nnz = 0;
  }
  void set_order(int o, int it);
  QKey key() const;
};

void qforest_create_trees(QForest &f, int level);
void qforest_create_random_trees(QForest &f, int nrand, int min_level, int max_level,
                                 uint64_t seed);
void qforest_refine(QForest &f, const int *d_ref, long long nref, int min_level, int max_level);
void qforest_coarsen(QForest &f, QForest &out);
void qforest_duplicate(QForest &f, QForest &out);
void qforest_balance(QForest &f, int corner);
void qforest_create_nodes(QForest &f);
void qinterp_create(QForest &fine, QForest &coarse, Interp &I);
void qforest_get_points(QForest &f, double *d_X);

}  // namespace tmrg
