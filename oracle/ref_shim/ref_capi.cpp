/*
  C entry points over the reference TMR octree core, compiled from the
  reference's own sources (TMROctant.cpp, TMROctForest.cpp, TMRBase.cpp)
  with the single-rank shims in this folder.  Test infrastructure only:
  it produces golden vectors and pins the C restatement in oracle/.

  Every function mirrors one public TMROctForest method
  (TMROctForest.h:46-411); the copy-out helpers flatten the reference's
  borrowed pointers into caller buffers.
*/
#include <stdio.h>

#include "TMROctForest.h"

// The reference's TMROctForest.cpp reaches these only with a topology
// attached or with Bernstein interpolation plus a topology; the checker
// never attaches one.
void TMRTopology::getConnectivity(int *, int *, int *, int *, const int **,
                                  const int **, const int **) {
  fprintf(stderr, "ref checker: topology not available\n");
  abort();
}
void TMRTopology::getVolume(int, TMRVolume **) { abort(); }
void TMRTopology::getFace(int, TMRFace **) { abort(); }
void TMRTopology::getEdge(int, TMREdge **) { abort(); }
void TMRTopology::getVertex(int, TMRVertex **) { abort(); }
extern "C" void dgetrf_(int *, int *, double *, int *, int *, int *) {
  abort();
}
extern "C" void dgetrs_(const char *, int *, int *, double *, int *, int *,
                        double *, int *, int *) {
  abort();
}

extern "C" {

void *tmrref_forest_create(int order, int interp) {
  TMROctForest *f =
      new TMROctForest(0, order, (TMRInterpolationType)interp);
  f->incref();
  return f;
}
void tmrref_forest_destroy(void *f) { ((TMROctForest *)f)->decref(); }
void tmrref_set_connectivity(void *f, int nnodes, const int *conn,
                             int nblocks) {
  ((TMROctForest *)f)->setConnectivity(nnodes, conn, nblocks);
}
void tmrref_set_mesh_order(void *f, int order, int interp) {
  ((TMROctForest *)f)->setMeshOrder(order, (TMRInterpolationType)interp);
}
void tmrref_create_trees(void *f, int level) {
  ((TMROctForest *)f)->createTrees(level);
}
void tmrref_refine(void *f, const int *refine, int min_level, int max_level) {
  ((TMROctForest *)f)->refine(refine, min_level, max_level);
}
void *tmrref_coarsen(void *f) {
  TMROctForest *c = ((TMROctForest *)f)->coarsen();
  c->incref();
  return c;
}
void *tmrref_duplicate(void *f) {
  TMROctForest *c = ((TMROctForest *)f)->duplicate();
  c->incref();
  return c;
}
void tmrref_balance(void *f, int corner) {
  ((TMROctForest *)f)->balance(corner);
}
void tmrref_create_nodes(void *f) { ((TMROctForest *)f)->createNodes(); }

int tmrref_num_octants(void *f) {
  TMROctantArray *a;
  ((TMROctForest *)f)->getOctants(&a);
  int n = 0;
  if (a) a->getArray(NULL, &n);
  return n;
}
// out: 7 ints per octant {block, x, y, z, tag, level, info}
void tmrref_get_octants(void *f, int *out) {
  TMROctantArray *a;
  ((TMROctForest *)f)->getOctants(&a);
  int n = 0;
  TMROctant *o;
  a->getArray(&o, &n);
  for (int i = 0; i < n; i++) {
    out[7 * i + 0] = o[i].block;
    out[7 * i + 1] = o[i].x;
    out[7 * i + 2] = o[i].y;
    out[7 * i + 3] = o[i].z;
    out[7 * i + 4] = o[i].tag;
    out[7 * i + 5] = o[i].level;
    out[7 * i + 6] = o[i].info;
  }
}
// out: {num_local_nodes, owned nodes (node_range[1]), num_dep, ext_pre,
//       num_elements, dep nnz}
void tmrref_node_sizes(void *f, int *out) {
  TMROctForest *F = (TMROctForest *)f;
  const int *conn;
  int nelems = 0;
  F->getNodeConn(&conn, &nelems);
  const int *range;
  F->getOwnedNodeRange(&range);
  const int *ptr, *dconn;
  const double *w;
  int nd = F->getDepNodeConn(&ptr, &dconn, &w);
  out[0] = F->getNodeNumbers(NULL);
  out[1] = range ? range[1] : 0;
  out[2] = nd;
  out[3] = F->getExtPreOffset();
  out[4] = nelems;
  out[5] = (ptr && nd > 0) ? ptr[nd] : 0;
}
void tmrref_get_conn(void *f, int *out) {
  TMROctForest *F = (TMROctForest *)f;
  const int *conn;
  int nelems = 0;
  F->getNodeConn(&conn, &nelems);
  int o = F->getMeshOrder();
  memcpy(out, conn, sizeof(int) * (size_t)nelems * o * o * o);
}
void tmrref_get_node_numbers(void *f, int *out) {
  TMROctForest *F = (TMROctForest *)f;
  const int *nn;
  int n = F->getNodeNumbers(&nn);
  memcpy(out, nn, sizeof(int) * (size_t)n);
}
void tmrref_get_dep(void *f, int *ptr_out, int *conn_out, double *w_out) {
  TMROctForest *F = (TMROctForest *)f;
  const int *ptr, *dconn;
  const double *w;
  int nd = F->getDepNodeConn(&ptr, &dconn, &w);
  if (!ptr) {
    ptr_out[0] = 0;
    return;
  }
  memcpy(ptr_out, ptr, sizeof(int) * (size_t)(nd + 1));
  memcpy(conn_out, dconn, sizeof(int) * (size_t)ptr[nd]);
  memcpy(w_out, w, sizeof(double) * (size_t)ptr[nd]);
}

void *tmrref_create_interp(void *fine, void *coarse) {
  TACSBVecInterp *interp = new TACSBVecInterp();
  ((TMROctForest *)fine)->createInterpolation((TMROctForest *)coarse, interp);
  return interp;
}
// out: {number of addInterp calls, total entries}
void tmrref_interp_sizes(void *h, int *out) {
  TACSBVecInterp *I = (TACSBVecInterp *)h;
  out[0] = (int)I->rows.size();
  out[1] = (int)I->cols_.size();
}
void tmrref_interp_get(void *h, int *rows, int *end_ptr, int *cols,
                       double *w) {
  TACSBVecInterp *I = (TACSBVecInterp *)h;
  memcpy(rows, I->rows.data(), sizeof(int) * I->rows.size());
  memcpy(end_ptr, I->ptr.data(), sizeof(int) * I->ptr.size());
  memcpy(cols, I->cols_.data(), sizeof(int) * I->cols_.size());
  memcpy(w, I->weights.data(), sizeof(double) * I->weights.size());
}
void tmrref_interp_destroy(void *h) { delete (TACSBVecInterp *)h; }

}  // extern "C"
