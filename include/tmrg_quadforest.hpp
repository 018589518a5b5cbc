/*
  tmrg_quadforest.hpp — C++ host facade with the TMRQuadForest interface
  (TMRQuadForest.h:43-161, TMRQuadrant.h:36-52), the STL tools
  (TMR_STLTools.h:44-77) and TMRHelmholtzFilter (TMRHelmholtzFilter.h:31-61)
  over the tmrg C ABI.  Header only; include after (or instead of)
  tmrg_octforest.hpp, whose TMRGEntity, TMRGVecInterp, TMRPoint and error
  reporting it shares.  TMRMatrixFilter (TMRMatrixFilter.h:63-110) for
  either forest type is here too.
*/
#ifndef TMRG_QUADFOREST_HPP
#define TMRG_QUADFOREST_HPP

#include <stdint.h>
#include <stdio.h>

#include <vector>

#include "tmrg.h"
#include "tmrg_octforest.hpp"

// Same field layout as TMRQuadrant (TMRQuadrant.h:46-51).
class TMRQuadrant {
 public:
  int32_t face, x, y, tag;
  int16_t level, info;
};

// The quadrants (TMRQuadrantArray): a copy owned by the forest, valid until
// the forest changes.
class TMRQuadrantArray {
 public:
  void getArray(TMRQuadrant **a, int *size) {
    if (a) *a = quads.data();
    if (size) *size = (int)quads.size();
  }
  std::vector<TMRQuadrant> quads;
};

class TMRQuadForest : public TMRGEntity {
 public:
  explicit TMRQuadForest(int comm = 0, int mesh_order = 2,
                         TMRInterpolationType interp_type = TMR_GAUSS_LOBATTO_POINTS,
                         void *cuda_stream = nullptr)
      : f(nullptr), stream(cuda_stream) {
    (void)comm;
    tmrg_report(tmrg_qforest_create(mesh_order, interp_type, stream, &f), "TMRQuadForest");
  }
  ~TMRQuadForest() { tmrg_qforest_destroy(f); }

  void setConnectivity(int num_nodes, const int *face_conn, int num_faces) {
    tmrg_report(tmrg_qforest_set_connectivity(f, num_nodes, face_conn, num_faces),
                "setConnectivity");
  }
  void setFullConnectivity(int num_nodes, int num_edges, int num_faces, const int *face_conn,
                           const int *face_edge_conn) {
    tmrg_report(tmrg_qforest_set_full_connectivity(f, num_nodes, num_edges, num_faces,
                                                   face_conn, face_edge_conn),
                "setFullConnectivity");
  }
  void getConnectivity(int *nfaces, int *nedges, int *nnodes, const int **face_conn,
                       const int **face_edge_conn) {
    int sz[3] = {0, 0, 0};
    tmrg_qforest_get_connectivity(f, sz, nullptr, nullptr);
    fc_.assign(4 * (size_t)sz[0], 0);
    fe_.assign(4 * (size_t)sz[0], 0);
    tmrg_report(tmrg_qforest_get_connectivity(f, sz, fc_.data(), fe_.data()), "getConnectivity");
    if (nfaces) *nfaces = sz[0];
    if (nedges) *nedges = sz[1];
    if (nnodes) *nnodes = sz[2];
    if (face_conn) *face_conn = fc_.data();
    if (face_edge_conn) *face_edge_conn = fe_.data();
  }
  void setMeshOrder(int mesh_order, TMRInterpolationType interp = TMR_GAUSS_LOBATTO_POINTS) {
    tmrg_report(tmrg_qforest_set_mesh_order(f, mesh_order, interp), "setMeshOrder");
  }
  int getMeshOrder() {
    int o = 2;
    tmrg_qforest_get_mesh_order(f, &o, nullptr, nullptr);
    return o;
  }
  TMRInterpolationType getInterpType() {
    int t = 1;
    tmrg_qforest_get_mesh_order(f, nullptr, &t, nullptr);
    return (TMRInterpolationType)t;
  }
  int getInterpKnots(const double **knots) {
    knots_.assign(3, 0.0);
    int o = 2;
    tmrg_qforest_get_mesh_order(f, &o, nullptr, knots_.data());
    if (knots) *knots = knots_.data();
    return o;
  }
  void createTrees(int refine_level) {
    tmrg_report(tmrg_qforest_create_trees(f, refine_level), "createTrees");
  }
  // createRandomTrees (TMRQuadForest.cpp:1327-1407) with the seeded
  // generator U(seed, face, 3i + k) in place of libc rand().
  void createRandomTrees(int nrand = 10, int min_level = 0, int max_level = 8,
                         uint64_t seed = 0) {
    tmrg_report(tmrg_qforest_create_random_trees(f, nrand, min_level, max_level, seed),
                "createRandomTrees");
  }
  // repartition: the forest lives on one GPU, nothing to redistribute.
  void repartition() {}
  void refine(const int refinement[] = nullptr, int min_level = 0,
              int max_level = TMR_MAX_LEVEL) {
    int64_t n = 0;
    tmrg_qforest_num_quadrants(f, &n);
    tmrg_report(tmrg_qforest_refine(f, refinement, refinement ? n : 0, min_level, max_level),
                "refine");
  }
  TMRQuadForest *duplicate() { return derived(tmrg_qforest_duplicate, "duplicate"); }
  TMRQuadForest *coarsen() { return derived(tmrg_qforest_coarsen, "coarsen"); }
  void balance(int balance_corner = 0) {
    tmrg_report(tmrg_qforest_balance(f, balance_corner), "balance");
  }
  void createNodes() { tmrg_report(tmrg_qforest_create_nodes(f), "createNodes"); }

  void getQuadrants(TMRQuadrantArray **quads) {
    int64_t n = 0;
    tmrg_qforest_num_quadrants(f, &n);
    std::vector<int> raw(6 * (size_t)n);
    if (n && !tmrg_report(tmrg_qforest_get_quadrants(f, raw.data()), "getQuadrants")) n = 0;
    quads_.quads.resize((size_t)n);
    for (int64_t i = 0; i < n; i++) {
      TMRQuadrant &q = quads_.quads[i];
      q.face = raw[6 * i];
      q.x = raw[6 * i + 1];
      q.y = raw[6 * i + 2];
      q.tag = raw[6 * i + 3];
      q.level = (int16_t)raw[6 * i + 4];
      q.info = (int16_t)raw[6 * i + 5];
    }
    if (quads) *quads = &quads_;
  }
  void getNodeConn(const int **conn = nullptr, int *num_elements = nullptr,
                   int *num_owned_nodes = nullptr, int *num_local_nodes = nullptr) {
    int64_t s[6] = {0};
    tmrg_qforest_sizes(f, s);
    const int o = getMeshOrder();
    conn_.assign((size_t)s[4] * o * o, 0);
    if (conn) {
      *conn = (s[4] && tmrg_report(tmrg_qforest_get_node_conn(f, conn_.data()), "getNodeConn"))
                  ? conn_.data()
                  : nullptr;
    }
    if (num_elements) *num_elements = (int)s[4];
    if (num_owned_nodes) *num_owned_nodes = (int)s[1];
    if (num_local_nodes) *num_local_nodes = (int)s[0];
  }
  int getDepNodeConn(const int **ptr = nullptr, const int **conn = nullptr,
                     const double **weights = nullptr) {
    int64_t s[6] = {0};
    tmrg_qforest_sizes(f, s);
    dptr_.assign((size_t)s[2] + 1, 0);
    dconn_.assign((size_t)s[5] + 1, 0);
    dw_.assign((size_t)s[5] + 1, 0.0);
    if (!tmrg_report(tmrg_qforest_get_dep_node_conn(f, dptr_.data(), dconn_.data(), dw_.data()),
                     "getDepNodeConn"))
      return 0;
    if (ptr) *ptr = dptr_.data();
    if (conn) *conn = dconn_.data();
    if (weights) *weights = dw_.data();
    return (int)s[2];
  }
  int getOwnedNodeRange(const int **node_range) {
    int64_t s[6] = {0};
    tmrg_qforest_sizes(f, s);
    range_[0] = 0;
    range_[1] = (int)s[1];
    if (node_range) *node_range = range_;
    return 1;
  }
  void createInterpolation(TMRQuadForest *coarse, TMRGVecInterp *interp) {
    if (coarse == this) {
      fprintf(stderr, "TMRQuadForest Error: Cannot interpolate between the same object\n");
      return;
    }
    tmrg_interp_destroy(interp->I);
    interp->I = nullptr;
    tmrg_report(tmrg_qforest_create_interpolation(f, coarse->f, &interp->I),
                "createInterpolation");
  }
  tmrg_qforest *handle() { return f; }
  // A box (origin x, y, extent x, y) per face: the stand-in for the
  // topology's surfaces that getPoints and the VTK writers map through
  // (tmrg_qforest_set_face_boxes).
  void setFaceBoxes(const double *boxes, int nfaces) {
    if (tmrg_report(tmrg_qforest_set_face_boxes(f, boxes, nfaces), "setFaceBoxes"))
      boxes_.assign(boxes, boxes + (size_t)(boxes ? 4 * nfaces : 0));
  }
  // writeToVTK (TMRQuadForest.cpp:651-720): the face mesh as VTK
  // quadrilaterals, each connectivity node at its owner face's corner (the
  // lowest-numbered face touching it) through the face boxes, the face
  // index as the cell scalar entity_index; nothing without face boxes.
  void writeToVTK(const char *filename) {
    if (boxes_.empty()) return;
    int nf = 0, ne = 0, nn = 0;
    const int *fc = nullptr, *fe = nullptr;
    getConnectivity(&nf, &ne, &nn, &fc, &fe);
    FILE *fp = filename ? fopen(filename, "w") : nullptr;
    if (!fp) return;
    std::vector<int> owner(nn, nf);
    for (int q = 0; q < nf; q++)
      for (int c = 0; c < 4; c++)
        if (q < owner[fc[4 * q + c]]) owner[fc[4 * q + c]] = q;
    fprintf(fp, "# vtk DataFile Version 3.0\nvtk output\nASCII\n");
    fprintf(fp, "DATASET UNSTRUCTURED_GRID\nPOINTS %d float\n", nn);
    for (int k = 0; k < nn; k++) {
      const int q = owner[k];
      double x = 0.0, y = 0.0;
      if (q < nf) {
        int corner = 0;
        while (corner < 4 && fc[4 * q + corner] != k) corner++;
        x = boxes_[4 * q] + boxes_[4 * q + 2] * (1.0 * (corner & 1));
        y = boxes_[4 * q + 1] + boxes_[4 * q + 3] * (1.0 * (corner >> 1));
      }
      fprintf(fp, "%e %e %e\n", x, y, 0.0);
    }
    fprintf(fp, "\nCELLS %d %d\n", nf, 5 * nf);
    for (int q = 0; q < nf; q++)
      fprintf(fp, "4 %d %d %d %d\n", fc[4 * q], fc[4 * q + 1], fc[4 * q + 3], fc[4 * q + 2]);
    fprintf(fp, "\nCELL_TYPES %d\n", nf);
    for (int q = 0; q < nf; q++) fprintf(fp, "9\n");
    fprintf(fp, "CELL_DATA %d\nSCALARS entity_index float 1\nLOOKUP_TABLE default\n", nf);
    for (int q = 0; q < nf; q++) fprintf(fp, "%e\n", 1.0 * q);
    fclose(fp);
  }
  // writeToTecplot (TMRQuadForest.cpp:729-804): the face mesh as one
  // Tecplot FEQUADRILATERAL zone, nodes at their owner face's corner through
  // the face boxes, the face index cell-centred; nothing without face boxes.
  void writeToTecplot(const char *filename) {
    if (boxes_.empty()) return;
    int nf = 0, ne = 0, nn = 0;
    const int *fc = nullptr, *fe = nullptr;
    getConnectivity(&nf, &ne, &nn, &fc, &fe);
    FILE *fp = filename ? fopen(filename, "w") : nullptr;
    if (!fp) return;
    std::vector<int> owner(nn, nf);
    for (int q = 0; q < nf; q++)
      for (int c = 0; c < 4; c++)
        if (q < owner[fc[4 * q + c]]) owner[fc[4 * q + c]] = q;
    std::vector<double> X(3 * (size_t)nn, 0.0);
    for (int k = 0; k < nn; k++) {
      const int q = owner[k];
      if (q >= nf) continue;
      int corner = 0;
      while (corner < 4 && fc[4 * q + corner] != k) corner++;
      X[3 * k] = boxes_[4 * q] + boxes_[4 * q + 2] * (1.0 * (corner & 1));
      X[3 * k + 1] = boxes_[4 * q + 1] + boxes_[4 * q + 3] * (1.0 * (corner >> 1));
    }
    fprintf(fp, "Variables = X,Y,Z,face\n");
    fprintf(fp, "Zone N = %d E = %d ", nn, nf);
    fprintf(fp, "DATAPACKING=BLOCK, ZONETYPE=FEQUADRILATERAL\n");
    fprintf(fp, "VARLOCATION = ([4]=CELLCENTERED)\n");
    for (int d = 0; d < 3; d++)
      for (int k = 0; k < nn; k++) fprintf(fp, "%e\n", X[3 * k + d]);
    for (int q = 0; q < nf; q++) fprintf(fp, "%e\n", 1.0 * q);
    for (int q = 0; q < nf; q++)
      fprintf(fp, "%d %d %d %d\n", fc[4 * q] + 1, fc[4 * q + 1] + 1, fc[4 * q + 3] + 1,
              fc[4 * q + 2] + 1);
    fclose(fp);
  }
  // getNodeNumbers / getLocalNodeNumber / getExtPreOffset (TMRQuadForest.h):
  // the local nodes are numbered -num_dep .. -1, then the owned nodes.
  int getNodeNumbers(const int **nodes) {
    int64_t sz[6] = {0};
    tmrg_qforest_sizes(f, sz);
    nums_.resize((size_t)(sz[1] + sz[2]));
    for (int64_t i = 0; i < sz[1] + sz[2]; i++) nums_[i] = (int)(i - sz[2]);
    if (nodes) *nodes = nums_.data();
    return (int)(sz[1] + sz[2]);
  }
  int getLocalNodeNumber(int node) {
    int64_t sz[6] = {0};
    tmrg_qforest_sizes(f, sz);
    return (node >= -sz[2] && node < sz[1]) ? (int)(node + sz[2]) : -1;
  }
  int getExtPreOffset() {
    int64_t sz[6] = {0};
    tmrg_qforest_sizes(f, sz);
    return (int)sz[3];
  }
  // writeForestToVTK (TMRQuadForest.cpp:809-870): every quadrant as a
  // quadrilateral with its own four corners (x fastest) through its face's
  // box, the face index as entity_index; nothing without face boxes.
  void writeForestToVTK(const char *filename) {
    if (boxes_.empty()) return;
    TMRQuadrantArray *arr = nullptr;
    getQuadrants(&arr);
    FILE *fp = filename ? fopen(filename, "w") : nullptr;
    if (!fp) return;
    const int n = (int)arr->quads.size();
    const double hmax = (double)(1 << 30);
    fprintf(fp, "# vtk DataFile Version 3.0\nvtk output\nASCII\n");
    fprintf(fp, "DATASET UNSTRUCTURED_GRID\nPOINTS %d float\n", 4 * n);
    for (int k = 0; k < n; k++) {
      const TMRQuadrant &q = arr->quads[k];
      const int32_t h = 1 << (30 - q.level);
      const double *b = &boxes_[4 * (size_t)q.face];
      for (int jj = 0; jj < 2; jj++)
        for (int ii = 0; ii < 2; ii++) {
          const double u = 1.0 * (q.x + ii * h) / hmax;
          const double v = 1.0 * (q.y + jj * h) / hmax;
          fprintf(fp, "%e %e %e\n", b[0] + b[2] * u, b[1] + b[3] * v, 0.0);
        }
    }
    fprintf(fp, "\nCELLS %d %d\n", n, 5 * n);
    for (int k = 0; k < n; k++)
      fprintf(fp, "4 %d %d %d %d\n", 4 * k, 4 * k + 1, 4 * k + 3, 4 * k + 2);
    fprintf(fp, "\nCELL_TYPES %d\n", n);
    for (int k = 0; k < n; k++) fprintf(fp, "9\n");
    fprintf(fp, "CELL_DATA %d\nSCALARS entity_index float 1\nLOOKUP_TABLE default\n", n);
    for (int k = 0; k < n; k++) fprintf(fp, "%e\n", 1.0 * arr->quads[k].face);
    fclose(fp);
  }

 private:
  TMRQuadForest *derived(int (*fn)(tmrg_qforest *, tmrg_qforest **), const char *w) {
    TMRQuadForest *d = new TMRQuadForest(0, getMeshOrder(), getInterpType(), stream);
    tmrg_qforest_destroy(d->f);
    d->f = nullptr;
    if (!tmrg_report(fn(f, &d->f), w)) tmrg_qforest_create(getMeshOrder(), getInterpType(), stream, &d->f);
    return d;
  }
  tmrg_qforest *f;
  void *stream;
  TMRQuadrantArray quads_;
  std::vector<int> fc_, fe_, conn_, dptr_, dconn_, nums_;
  std::vector<double> dw_, knots_, boxes_;
  int range_[2];
};

// STL triangle (TMR_STLTriangle, TMRBase.h:79-82).
class TMR_STLTriangle {
 public:
  TMRPoint p[3];
};

// TMR_GenerateSTLTriangles (TMR_STLTools.h:44-46) with the design vector
// given as `vpn` interleaved values per independent node (host pointer)
// in place of a TACSBVec; *tris is allocated with new[] (delete[] it).
inline int TMR_GenerateSTLTriangles(int root, TMROctForest *filter, const double *x, int vpn,
                                    int x_offset, double cutoff, int *ntris,
                                    TMR_STLTriangle **tris) {
  (void)root;
  int64_t n = 0;
  *ntris = 0;
  *tris = nullptr;
  if (!tmrg_report(tmrg_stl_triangles(filter->handle(), x, vpn, x_offset, cutoff, &n, nullptr, 0),
                   "TMR_GenerateSTLTriangles"))
    return 1;
  *tris = new TMR_STLTriangle[n > 0 ? n : 1];
  if (!tmrg_report(tmrg_stl_triangles(filter->handle(), x, vpn, x_offset, cutoff, &n,
                                      reinterpret_cast<double *>(*tris), n),
                   "TMR_GenerateSTLTriangles")) {
    delete[] * tris;
    *tris = nullptr;
    return 1;
  }
  *ntris = (int)n;
  return 0;
}
inline int TMR_GenerateBinFile(const char *filename, TMROctForest *filter, const double *x,
                               int vpn, int x_offset, double cutoff) {
  return tmrg_report(tmrg_generate_bin_file(filename, filter->handle(), x, vpn, x_offset, cutoff),
                     "TMR_GenerateBinFile")
             ? 0
             : 1;
}
inline int TMR_ConvertBinToSTL(const char *binfile, const char *stlfile) {
  return tmrg_report(tmrg_convert_bin_to_stl(binfile, stlfile), "TMR_ConvertBinToSTL") ? 0 : 1;
}

// TMRHelmholtzFilter over octree or quadtree filter forests (finest first, boxes
// set); applyFilter / applyTranspose on host vectors of vpn interleaved
// components.  The TACS assemblers of the reference's constructor have no
// counterpart here.
class TMRHelmholtzFilter : public TMRGEntity {
 public:
  TMRHelmholtzFilter(double helmholtz_radius, int nlevels, TMROctForest *filter[])
      : H(nullptr) {
    std::vector<tmrg_forest *> fs(nlevels);
    for (int k = 0; k < nlevels; k++) fs[k] = filter[k]->handle();
    tmrg_report(tmrg_helmholtz_create(fs.data(), nlevels, helmholtz_radius, &H),
                "TMRHelmholtzFilter");
  }
  // The 2-D filter (TMRHelmholtzFilter.cpp:35-40): quadtree forests with
  // face boxes.
  TMRHelmholtzFilter(double helmholtz_radius, int nlevels, TMRQuadForest *filter[])
      : H(nullptr) {
    std::vector<tmrg_qforest *> fs(nlevels);
    for (int k = 0; k < nlevels; k++) fs[k] = filter[k]->handle();
    tmrg_report(tmrg_helmholtz_create_quad(fs.data(), nlevels, helmholtz_radius, &H),
                "TMRHelmholtzFilter");
  }
  ~TMRHelmholtzFilter() { tmrg_helmholtz_destroy(H); }
  void applyFilter(const double *in, double *out, int vpn = 1) {
    tmrg_report(tmrg_helmholtz_apply(H, vpn, in, out), "applyFilter");
  }
  void applyTranspose(const double *in, double *out, int vpn = 1) {
    tmrg_report(tmrg_helmholtz_apply_transpose(H, vpn, in, out), "applyTranspose");
  }
  tmrg_helmholtz *handle() { return H; }

 private:
  tmrg_helmholtz *H;
};

// TMRMatrixFilter (TMRMatrixFilter.h:63-110) over octree or quadtree filter
// forests: the filter is built on filter[0] (order 2; blocks / faces are
// cubes / squares of side block_len in place of the TACS assemblers'
// geometry); applyFilter / applyTranspose on host vectors of vpn
// interleaved components.  The restriction down the remaining forests
// (setDesignVars) is the interpolation objects' multWeightTranspose.
class TMRMatrixFilter : public TMRGEntity {
 public:
  TMRMatrixFilter(double r, int N, int nlevels, TMROctForest *filter[], double block_len = 1.0)
      : F(nullptr) {
    (void)nlevels;
    tmrg_report(tmrg_filter_create(filter[0]->handle(), block_len, r, N, &F), "TMRMatrixFilter");
  }
  TMRMatrixFilter(double r, int N, int nlevels, TMRQuadForest *filter[], double block_len = 1.0)
      : F(nullptr) {
    (void)nlevels;
    tmrg_report(tmrg_filter_create_quad(filter[0]->handle(), block_len, r, N, &F),
                "TMRMatrixFilter");
  }
  ~TMRMatrixFilter() { tmrg_filter_destroy(F); }
  void applyFilter(const double *in, double *out, int vpn = 1) {
    tmrg_report(tmrg_filter_apply(F, vpn, in, out), "applyFilter");
  }
  void applyTranspose(const double *in, double *out, int vpn = 1) {
    tmrg_report(tmrg_filter_apply_transpose(F, vpn, in, out), "applyTranspose");
  }
  tmrg_filter *handle() { return F; }

 private:
  tmrg_filter *F;
};

#endif
