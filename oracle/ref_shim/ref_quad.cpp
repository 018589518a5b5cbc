/*
  C entry points over the reference TMR quadtree core (TMRQuadrant.cpp,
  TMRQuadForest.cpp), compiled from the reference's own sources with the
  single-rank shims in this folder.  Test infrastructure only: it produces
  golden vectors for the quadtree twin.

  Every function mirrors one public TMRQuadForest method
  (TMRQuadForest.h:43-161); the copy-out helpers flatten the reference's
  borrowed pointers into caller buffers.
*/
#include <string.h>

#include "TACSBVecInterp.h"
#include "TMRQuadForest.h"
#include "TMRTopology.h"

// TMRQuadForest.cpp reaches the topology only when one is attached; the
// checker never attaches one.
void TMRTopology::getConnectivity(int *, int *, int *, const int **, const int **) {
  abort();
}

extern "C" {

void *tmrref_qforest_create(int order, int interp) {
  TMRQuadForest *f = new TMRQuadForest(0, order, (TMRInterpolationType)interp);
  f->incref();
  return f;
}
void tmrref_qforest_destroy(void *f) { ((TMRQuadForest *)f)->decref(); }
void tmrref_qset_connectivity(void *f, int nnodes, const int *conn, int nfaces) {
  ((TMRQuadForest *)f)->setConnectivity(nnodes, conn, nfaces);
}
void tmrref_qset_mesh_order(void *f, int order, int interp) {
  ((TMRQuadForest *)f)->setMeshOrder(order, (TMRInterpolationType)interp);
}
void tmrref_qcreate_trees(void *f, int level) { ((TMRQuadForest *)f)->createTrees(level); }
void tmrref_qrefine(void *f, const int *refine, int min_level, int max_level) {
  ((TMRQuadForest *)f)->refine(refine, min_level, max_level);
}
void *tmrref_qcoarsen(void *f) {
  TMRQuadForest *c = ((TMRQuadForest *)f)->coarsen();
  c->incref();
  return c;
}
void *tmrref_qduplicate(void *f) {
  TMRQuadForest *c = ((TMRQuadForest *)f)->duplicate();
  c->incref();
  return c;
}
void tmrref_qbalance(void *f, int corner) { ((TMRQuadForest *)f)->balance(corner); }
void tmrref_qcreate_nodes(void *f) { ((TMRQuadForest *)f)->createNodes(); }
int tmrref_qnum_quads(void *f) {
  TMRQuadrantArray *a;
  ((TMRQuadForest *)f)->getQuadrants(&a);
  int n = 0;
  if (a) a->getArray(NULL, &n);
  return n;
}
// out: 6 ints per quadrant {face, x, y, tag, level, info}
void tmrref_qget_quads(void *f, int *out) {
  TMRQuadrantArray *a;
  ((TMRQuadForest *)f)->getQuadrants(&a);
  int n = 0;
  TMRQuadrant *q;
  a->getArray(&q, &n);
  for (int i = 0; i < n; i++) {
    out[6 * i + 0] = q[i].face;
    out[6 * i + 1] = q[i].x;
    out[6 * i + 2] = q[i].y;
    out[6 * i + 3] = q[i].tag;
    out[6 * i + 4] = q[i].level;
    out[6 * i + 5] = q[i].info;
  }
}
// out: {num_local_nodes, owned nodes, num_dep, ext_pre, num_elements, dep nnz}
void tmrref_qnode_sizes(void *f, int *out) {
  TMRQuadForest *F = (TMRQuadForest *)f;
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
void tmrref_qget_conn(void *f, int *out) {
  TMRQuadForest *F = (TMRQuadForest *)f;
  const int *conn;
  int nelems = 0;
  F->getNodeConn(&conn, &nelems);
  int o = F->getMeshOrder();
  memcpy(out, conn, sizeof(int) * (size_t)nelems * o * o);
}
void tmrref_qget_node_numbers(void *f, int *out) {
  TMRQuadForest *F = (TMRQuadForest *)f;
  const int *nn;
  int n = F->getNodeNumbers(&nn);
  memcpy(out, nn, sizeof(int) * (size_t)n);
}
void tmrref_qget_dep(void *f, int *ptr_out, int *conn_out, double *w_out) {
  TMRQuadForest *F = (TMRQuadForest *)f;
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
void *tmrref_qcreate_interp(void *fine, void *coarse) {
  TACSBVecInterp *interp = new TACSBVecInterp();
  ((TMRQuadForest *)fine)->createInterpolation((TMRQuadForest *)coarse, interp);
  return interp;
}
// sizes = {faces, edges, nodes}; face_conn 4, face_edge 4 per face
void tmrref_qget_connectivity(void *f, int *sizes, int *face_conn, int *face_edge) {
  int nf, ne, nn;
  const int *fc, *fe;
  ((TMRQuadForest *)f)->getConnectivity(&nf, &ne, &nn, &fc, &fe);
  sizes[0] = nf;
  sizes[1] = ne;
  sizes[2] = nn;
  if (face_conn) memcpy(face_conn, fc, sizeof(int) * 4 * nf);
  if (face_edge) memcpy(face_edge, fe, sizeof(int) * 4 * nf);
}
// evalInterp (TMRQuadForest.cpp:1069-1160), N1 == NULL: values only
void tmrref_qeval_interp(void *f, const double *pt, double *N, double *N1, double *N2) {
  if (N1)
    ((TMRQuadForest *)f)->evalInterp(pt, N, N1, N2);
  else
    ((TMRQuadForest *)f)->evalInterp(pt, N);
}

}  // extern "C"
