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
  std::vector<double> knots_;
  int range_[2];
};

#endif
