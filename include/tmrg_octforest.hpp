/*
  tmrg_octforest.hpp — C++ host facade with the TMROctForest interface,
  implemented over the tmrg C ABI (tmrg.h).  Header only.

  A TMR user swaps `#include "TMROctForest.h"` for this header and links
  libtmrg.so: the same class and method names (TMROctForest.h:46-411,
  TMROctant.h:36-81), the same intrusive reference counting
  (TMREntity::incref/decref, TMRBase.cpp:145-156) and the same error
  behaviour (a message on stderr and an early return,
  TMROctForest.cpp:2919-2922), while the octants, nodes and operators live
  on the GPU.  MPI_Comm arguments are accepted as `int` and ignored: one
  GPU holds the whole forest.  createInterpolation fills a TMRGVecInterp,
  which provides the TACSBVecInterp applies used by TMR's filters
  (mult / multTranspose / multWeightTranspose).
*/
#ifndef TMRG_OCTFOREST_HPP
#define TMRG_OCTFOREST_HPP

#include <stdint.h>
#include <stdio.h>

#include <vector>

#include "tmrg.h"

enum TMRInterpolationType {
  TMR_UNIFORM_POINTS = TMRG_UNIFORM_POINTS,
  TMR_GAUSS_LOBATTO_POINTS = TMRG_GAUSS_LOBATTO_POINTS,
  TMR_BERNSTEIN_POINTS = TMRG_BERNSTEIN_POINTS
};
static const int TMR_MAX_LEVEL = 30;

// Same field layout as TMROctant (TMROctant.h:47-52).
class TMROctant {
 public:
  int32_t block, x, y, z, tag;
  int16_t level, info;
};

static_assert(sizeof(TMROctant) == sizeof(tmrg_octant), "TMROctant layout");

// The octants (TMROctantArray, TMROctant.h:65-81): a view of the forest's
// page-locked host octants, which the forest owns, valid until the forest
// changes (the reference's getOctants hands out its own array the same
// way).
class TMROctantArray {
 public:
  void getArray(TMROctant **a, int *size) {
    if (a) *a = ptr;
    if (size) *size = (int)n;
  }
  TMROctant *ptr = nullptr;
  int64_t n = 0;
};

// Node location (TMRPoint, TMRBase.h).
class TMRPoint {
 public:
  double x, y, z;
};

class TMRGEntity {
 public:
  TMRGEntity() : ref_count(0) {}
  virtual ~TMRGEntity() {}
  void incref() { ref_count++; }
  void decref() {
    if (--ref_count == 0) delete this;
  }

 private:
  int ref_count;
};

inline bool tmrg_report(int status, const char *where) {
  if (status != TMRG_OK) {
    fprintf(stderr, "TMROctForest Error: %s: %s\n", where, tmrg_last_error());
    return false;
  }
  return true;
}

class TMRGVecInterp : public TMRGEntity {
 public:
  TMRGVecInterp() : I(nullptr) {}
  ~TMRGVecInterp() { tmrg_interp_destroy(I); }
  // y = P x ; y = P^T x ; y = (P^T x) / (P^T 1), host vectors node-major
  void mult(const double *x, double *y, int nvec = 1) {
    tmrg_report(tmrg_interp_mult(I, x, y, nvec), "mult");
  }
  void multTranspose(const double *x, double *y, int nvec = 1) {
    tmrg_report(tmrg_interp_mult_transpose(I, x, y, nvec), "multTranspose");
  }
  void multWeightTranspose(const double *x, double *y, int nvec = 1) {
    tmrg_report(tmrg_interp_mult_weight_transpose(I, x, y, nvec),
                "multWeightTranspose");
  }
  void getSizes(int64_t *rows, int64_t *cols, int64_t *nnz) {
    int64_t s[3] = {0, 0, 0};
    tmrg_interp_sizes(I, s);
    if (rows) *rows = s[0];
    if (cols) *cols = s[1];
    if (nnz) *nnz = s[2];
  }
  tmrg_interp *I;
};

class TMROctForest : public TMRGEntity {
 public:
  static const int MAX_ORDER = 16;

  explicit TMROctForest(int comm = 0, int mesh_order = 2,
                        TMRInterpolationType interp_type =
                            TMR_GAUSS_LOBATTO_POINTS,
                        void *cuda_stream = nullptr)
      : f(nullptr), stream(cuda_stream) {
    (void)comm;
    tmrg_report(tmrg_forest_create(mesh_order, interp_type, stream, &f),
                "TMROctForest");
  }
  ~TMROctForest() { tmrg_forest_destroy(f); }

  void setConnectivity(int num_nodes, const int *block_conn, int num_blocks) {
    tmrg_report(tmrg_forest_set_connectivity(f, num_nodes, block_conn,
                                             num_blocks),
                "setConnectivity");
  }
  void setFullConnectivity(int num_nodes, int num_edges, int num_faces, int num_blocks,
                           const int *block_conn, const int *block_edge_conn,
                           const int *block_face_conn) {
    tmrg_report(tmrg_forest_set_full_connectivity(f, num_nodes, num_edges, num_faces,
                                                  num_blocks, block_conn, block_edge_conn,
                                                  block_face_conn),
                "setFullConnectivity");
  }
  void getConnectivity(int *nblocks, int *nfaces, int *nedges, int *nnodes,
                       const int **block_conn, const int **block_face_conn,
                       const int **block_edge_conn, const int **block_face_ids) {
    tmrg_report(tmrg_forest_get_connectivity(f, nblocks, nfaces, nedges, nnodes, block_conn,
                                             block_face_conn, block_edge_conn,
                                             block_face_ids),
                "getConnectivity");
  }
  void getInverseConnectivity(const int **node_block_conn, const int **node_block_ptr,
                              const int **edge_block_conn, const int **edge_block_ptr,
                              const int **face_block_conn, const int **face_block_ptr) {
    tmrg_report(tmrg_forest_get_inverse_connectivity(f, node_block_conn, node_block_ptr,
                                                     edge_block_conn, edge_block_ptr,
                                                     face_block_conn, face_block_ptr),
                "getInverseConnectivity");
  }
  void setMeshOrder(int order,
                    TMRInterpolationType t = TMR_GAUSS_LOBATTO_POINTS) {
    tmrg_report(tmrg_forest_set_mesh_order(f, order, t), "setMeshOrder");
  }
  int getMeshOrder() {
    int o = 0;
    tmrg_forest_get_mesh_order(f, &o, nullptr);
    return o;
  }
  TMRInterpolationType getInterpType() {
    int t = 0;
    tmrg_forest_get_mesh_order(f, nullptr, &t);
    return (TMRInterpolationType)t;
  }
  int getInterpKnots(const double **knots) {
    int o = getMeshOrder();
    knots_.resize(o);
    tmrg_forest_get_interp_knots(f, knots_.data());
    if (knots) *knots = knots_.data();
    return o;
  }
  void createTrees(int refine_level) {
    tmrg_report(tmrg_forest_create_trees(f, refine_level), "createTrees");
  }
  // The reference draws from libc rand(); this draws from a seeded
  // generator (tmrg_forest_create_random_trees).
  void createRandomTrees(int nrand = 10, int min_level = 0, int max_level = 8,
                         uint64_t seed = 0) {
    tmrg_report(tmrg_forest_create_random_trees(f, nrand, min_level, max_level, seed),
                "createRandomTrees");
  }
  void repartition(int max_rank = -1) {
    tmrg_report(tmrg_forest_repartition(f, max_rank), "repartition");
  }
  void refine(const int refinement[] = nullptr, int min_level = 0,
              int max_level = TMR_MAX_LEVEL) {
    int64_t n = 0;
    tmrg_forest_num_octants(f, &n);
    tmrg_report(tmrg_forest_refine(f, refinement, n, min_level, max_level),
                "refine");
  }
  TMROctForest *duplicate() { return derived(tmrg_forest_duplicate, "duplicate"); }
  TMROctForest *coarsen() { return derived(tmrg_forest_coarsen, "coarsen"); }
  void balance(int balance_corner = 0) {
    tmrg_report(tmrg_forest_balance(f, balance_corner), "balance");
  }
  void createNodes() { tmrg_report(tmrg_forest_create_nodes(f), "createNodes"); }

  void getOctants(TMROctantArray **octs) {
    const tmrg_octant *p = nullptr;
    int64_t n = 0;
    if (!tmrg_report(tmrg_forest_octants_host(f, &p, &n), "getOctants")) {
      p = nullptr;
      n = 0;
    }
    octants_.ptr = reinterpret_cast<TMROctant *>(const_cast<tmrg_octant *>(p));
    octants_.n = n;
    if (octs) *octs = &octants_;
  }
  void getNodeConn(const int **conn = nullptr, int *num_elements = nullptr,
                   int *num_owned_nodes = nullptr,
                   int *num_local_nodes = nullptr) {
    int64_t s[6] = {0};
    tmrg_forest_node_sizes(f, s);
    if (conn) {
      const int *p = nullptr;
      *conn = tmrg_report(tmrg_forest_node_conn_host(f, &p, nullptr), "getNodeConn")
                  ? p
                  : nullptr;
    }
    if (num_elements) *num_elements = (int)s[4];
    if (num_owned_nodes) *num_owned_nodes = (int)s[1];
    if (num_local_nodes) *num_local_nodes = (int)s[0];
  }
  int getDepNodeConn(const int **ptr = nullptr, const int **conn = nullptr,
                     const double **weights = nullptr) {
    const int *p = nullptr, *c = nullptr;
    const double *w = nullptr;
    int64_t nd = 0;
    if (!tmrg_report(tmrg_forest_dep_node_conn_host(f, &p, &c, &w, &nd), "getDepNodeConn"))
      nd = 0;
    if (ptr) *ptr = p;
    if (conn) *conn = c;
    if (weights) *weights = w;
    return (int)nd;
  }
  int getOwnedNodeRange(const int **node_range) {
    int64_t s[6] = {0};
    tmrg_forest_node_sizes(f, s);
    range_[0] = 0;
    range_[1] = (int)s[1];
    if (node_range) *node_range = range_;
    return 1;
  }
  int getNodeNumbers(const int **node_numbers) {
    int64_t s[6] = {0};
    tmrg_forest_node_sizes(f, s);
    nn_.resize((size_t)s[0]);
    if (!nn_.empty()) tmrg_forest_get_node_numbers(f, nn_.data(), (int64_t)nn_.size());
    if (node_numbers) *node_numbers = nn_.data();
    return (int)s[0];
  }
  int getLocalNodeNumber(int node) {
    int li = -1;
    if (!tmrg_report(tmrg_forest_get_local_node_number(f, node, &li), "getLocalNodeNumber"))
      return -1;
    return li;
  }
  // Node locations (zeros unless block boxes were set with
  // tmrg_forest_set_block_boxes, as the reference without a topology).
  int getPoints(TMRPoint **X) {
    int64_t s[6] = {0};
    tmrg_forest_node_sizes(f, s);
    points_.resize((size_t)s[0]);
    if (!points_.empty() &&
        !tmrg_report(tmrg_forest_get_points(f, &points_[0].x, s[0]), "getPoints"))
      points_.clear();
    if (X) *X = points_.data();
    return (int)points_.size();
  }
  void evalInterp(const double pt[], double N[]) {
    tmrg_report(tmrg_forest_eval_interp(f, pt, N, nullptr, nullptr, nullptr), "evalInterp");
  }
  void evalInterp(const double pt[], double N[], double Nxi[], double Neta[],
                  double Nzeta[]) {
    tmrg_report(tmrg_forest_eval_interp(f, pt, N, Nxi, Neta, Nzeta), "evalInterp");
  }
  void evalInterp(const double pt[], double N[], double N1[], double N2[], double N3[],
                  double N11[], double N22[], double N33[], double N23[], double N13[],
                  double N12[]) {
    tmrg_report(tmrg_forest_eval_interp2(f, pt, N, N1, N2, N3, N11, N22, N33, N23, N13, N12),
                "evalInterp");
  }
  // Returns the enclosing octant inside the borrowed host octants
  // (getOctants), or nullptr.
  TMROctant *findEnclosing(const int order, const double *knots, TMROctant *node,
                           int *mpi_owner = nullptr) {
    if (mpi_owner) *mpi_owner = 0;
    int64_t idx = -1;
    if (!tmrg_report(tmrg_forest_find_enclosing(f, order, knots,
                                                reinterpret_cast<const tmrg_octant *>(node),
                                                1, &idx),
                     "findEnclosing") ||
        idx < 0)
      return nullptr;
    TMROctantArray *a = nullptr;
    getOctants(&a);
    return (a && idx < a->n) ? a->ptr + idx : nullptr;
  }
  void transformNode(TMROctant *oct, int edge_dir = -1, int *edge_reversed = nullptr,
                     int *src_face_id = nullptr) {
    tmrg_report(tmrg_forest_transform_nodes(f, reinterpret_cast<tmrg_octant *>(oct), 1,
                                            edge_dir, edge_reversed, src_face_id),
                "transformNode");
  }
  // writeToVTK (TMROctForest.cpp:1149-1228): the block mesh as VTK
  // hexahedra, each connectivity node at its owner block's corner through
  // the block boxes (the reference evaluates the topology's volumes), the
  // block index as the cell scalar entity_index.  Nothing is written when no
  // block boxes are set (the reference needs a topology).
  void writeToVTK(const char *filename) {
    int nb = 0, nn = 0;
    const int *bc = nullptr;
    std::vector<double> X;
    if (!blockNodePoints(&nb, &nn, &bc, X)) return;
    FILE *fp = filename ? fopen(filename, "w") : nullptr;
    if (!fp) return;
    fprintf(fp, "# vtk DataFile Version 3.0\nvtk output\nASCII\n");
    fprintf(fp, "DATASET UNSTRUCTURED_GRID\nPOINTS %d float\n", nn);
    for (int k = 0; k < nn; k++) fprintf(fp, "%e %e %e\n", X[3 * k], X[3 * k + 1], X[3 * k + 2]);
    fprintf(fp, "\nCELLS %d %d\n", nb, 9 * nb);
    for (int k = 0; k < nb; k++) {
      const int *c = bc + 8 * k;
      fprintf(fp, "8 %d %d %d %d %d %d %d %d\n", c[0], c[1], c[3], c[2], c[4], c[5], c[7], c[6]);
    }
    fprintf(fp, "\nCELL_TYPES %d\n", nb);
    for (int k = 0; k < nb; k++) fprintf(fp, "12\n");
    fprintf(fp, "CELL_DATA %d\nSCALARS entity_index float 1\nLOOKUP_TABLE default\n", nb);
    for (int k = 0; k < nb; k++) fprintf(fp, "%e\n", 1.0 * k);
    fclose(fp);
  }
  // Axis-aligned box (origin xyz, extent xyz) of every block: the stand-in
  // for the topology's volumes that getPoints and writeForestToVTK map
  // through (tmrg_forest_set_block_boxes).
  void setBlockBoxes(const double *boxes, int nblocks) {
    if (tmrg_report(tmrg_forest_set_block_boxes(f, boxes, nblocks), "setBlockBoxes"))
      boxes_.assign(boxes, boxes + (size_t)(boxes ? 6 * nblocks : 0));
  }
  // writeToTecplot (TMROctForest.cpp:1233-1311): the block mesh as one
  // Tecplot FEBRICK zone, each connectivity node at its owner block's
  // corner (the lowest-numbered block touching it) mapped through the
  // block's box, and the block index as a cell-centred variable.  Nothing
  // is written when no block boxes are set (the reference needs a topology).
  void writeToTecplot(const char *filename) {
    int nb = 0, nn = 0;
    const int *bc = nullptr;
    std::vector<double> X;
    if (!blockNodePoints(&nb, &nn, &bc, X)) return;
    FILE *fp = filename ? fopen(filename, "w") : nullptr;
    if (!fp) return;
    fprintf(fp, "Variables = X,Y,Z,block\n");
    fprintf(fp, "Zone N = %d E = %d ", nn, nb);
    fprintf(fp, "DATAPACKING=BLOCK, ZONETYPE=FEBRICK\n");
    fprintf(fp, "VARLOCATION = ([4]=CELLCENTERED)\n");
    for (int d = 0; d < 3; d++)
      for (int k = 0; k < nn; k++) fprintf(fp, "%e\n", X[3 * k + d]);
    for (int k = 0; k < nb; k++) fprintf(fp, "%e\n", 1.0 * k);
    for (int k = 0; k < nb; k++) {
      const int *c = bc + 8 * k;
      fprintf(fp, "%d %d %d %d %d %d %d %d\n", c[0] + 1, c[1] + 1, c[3] + 1, c[2] + 1,
              c[4] + 1, c[5] + 1, c[7] + 1, c[6] + 1);
    }
    fclose(fp);
  }
  // Each block connectivity node at its owner block's corner (the
  // lowest-numbered block touching it, node_block_owners) through the
  // block boxes; false without boxes.
  bool blockNodePoints(int *nb, int *nn, const int **bc, std::vector<double> &X) {
    if (boxes_.empty()) return false;
    int nf = 0, ne = 0;
    const int *bf = nullptr, *be = nullptr, *fid = nullptr;
    getConnectivity(nb, &nf, &ne, nn, bc, &bf, &be, &fid);
    if (!*bc) return false;
    std::vector<int> owner(*nn, *nb);
    for (int b = 0; b < *nb; b++)
      for (int c = 0; c < 8; c++)
        if (b < owner[(*bc)[8 * b + c]]) owner[(*bc)[8 * b + c]] = b;
    X.assign(3 * (size_t)*nn, 0.0);
    for (int k = 0; k < *nn; k++) {
      const int b = owner[k];
      if (b >= *nb) continue;
      int corner = 0;
      while (corner < 8 && (*bc)[8 * b + corner] != k) corner++;
      const double uvw[3] = {1.0 * (corner & 1), 1.0 * ((corner >> 1) & 1),
                             1.0 * (corner >> 2)};
      for (int d = 0; d < 3; d++)
        X[3 * k + d] = boxes_[6 * b + d] + boxes_[6 * b + 3 + d] * uvw[d];
    }
    return true;
  }
  // writeForestToVTK (TMROctForest.cpp:1317-1384): every octant as a
  // hexahedron with its own eight corners (x fastest) mapped through its
  // block's box, and the block index as the cell scalar entity_index.
  // Like the reference without a topology, nothing is written when no
  // block boxes are set.
  void writeForestToVTK(const char *filename) {
    if (boxes_.empty()) return;
    TMROctantArray *arr = nullptr;
    getOctants(&arr);
    if (!arr) return;
    FILE *fp = filename ? fopen(filename, "w") : nullptr;
    if (!fp) return;
    const int n = (int)arr->n;
    const TMROctant *o = arr->ptr;
    const double hmax = (double)(1 << 30);
    fprintf(fp, "# vtk DataFile Version 3.0\nvtk output\nASCII\n");
    fprintf(fp, "DATASET UNSTRUCTURED_GRID\nPOINTS %d float\n", 8 * n);
    for (int k = 0; k < n; k++) {
      const int32_t h = 1 << (30 - o[k].level);
      const double *b = &boxes_[6 * (size_t)o[k].block];
      for (int kk = 0; kk < 2; kk++)
        for (int jj = 0; jj < 2; jj++)
          for (int ii = 0; ii < 2; ii++) {
            const double u = 1.0 * (o[k].x + ii * h) / hmax;
            const double v = 1.0 * (o[k].y + jj * h) / hmax;
            const double w = 1.0 * (o[k].z + kk * h) / hmax;
            fprintf(fp, "%e %e %e\n", b[0] + b[3] * u, b[1] + b[4] * v, b[2] + b[5] * w);
          }
    }
    fprintf(fp, "\nCELLS %d %d\n", n, 9 * n);
    for (int k = 0; k < n; k++)
      fprintf(fp, "8 %d %d %d %d %d %d %d %d\n", 8 * k, 8 * k + 1, 8 * k + 3, 8 * k + 2,
              8 * k + 4, 8 * k + 5, 8 * k + 7, 8 * k + 6);
    fprintf(fp, "\nCELL_TYPES %d\n", n);
    for (int k = 0; k < n; k++) fprintf(fp, "12\n");
    fprintf(fp, "CELL_DATA %d\nSCALARS entity_index float 1\nLOOKUP_TABLE default\n", n);
    for (int k = 0; k < n; k++) fprintf(fp, "%e\n", 1.0 * o[k].block);
    fclose(fp);
  }
  int getExtPreOffset() {
    int64_t s[6] = {0};
    tmrg_forest_node_sizes(f, s);
    return (int)s[3];
  }
  void createInterpolation(TMROctForest *coarse, TMRGVecInterp *interp) {
    if (coarse == this) {
      fprintf(stderr, "TMROctForest Error: Cannot interpolate between the same object\n");
      return;
    }
    tmrg_interp_destroy(interp->I);
    interp->I = nullptr;
    tmrg_report(tmrg_interp_create(f, coarse->f, &interp->I), "createInterpolation");
  }

  tmrg_forest *handle() { return f; }

 private:
  TMROctForest *derived(int (*fn)(tmrg_forest *, tmrg_forest **), const char *w) {
    TMROctForest *d = new TMROctForest(0, getMeshOrder(), getInterpType(), stream);
    tmrg_forest_destroy(d->f);
    d->f = nullptr;
    if (!tmrg_report(fn(f, &d->f), w)) {
      tmrg_forest_create(getMeshOrder(), getInterpType(), stream, &d->f);
    }
    return d;
  }
  tmrg_forest *f;
  void *stream;
  TMROctantArray octants_;
  std::vector<int> nn_;
  std::vector<TMRPoint> points_;
  std::vector<double> knots_;
  std::vector<double> boxes_;
  int range_[2];
};

#endif
