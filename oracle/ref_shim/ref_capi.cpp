/*
  C entry points over the reference TMR octree core, compiled from the
  reference's own sources (TMROctant.cpp, TMROctForest.cpp, TMRBase.cpp,
  TMR_STLTools.cpp) with the single-rank shims in this folder.  Test infrastructure only:
  it produces golden vectors and pins the C restatement in oracle/.

  Every function mirrors one public TMROctForest method
  (TMROctForest.h:46-411); the copy-out helpers flatten the reference's
  borrowed pointers into caller buffers.
*/
#include <stdio.h>

#include <vector>

#include "TMROctForest.h"
#include "TMR_STLTools.h"

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

// evalInterp (TMROctForest.cpp:1510-1631); N1 == NULL selects the
// values-only form.
void tmrref_eval_interp(void *f, const double *pt, double *N, double *N1,
                        double *N2, double *N3) {
  if (N1)
    ((TMROctForest *)f)->evalInterp(pt, N, N1, N2, N3);
  else
    ((TMROctForest *)f)->evalInterp(pt, N);
}
void tmrref_eval_interp2(void *f, const double *pt, double *N, double *N1,
                         double *N2, double *N3, double *N11, double *N22,
                         double *N33, double *N23, double *N13, double *N12) {
  ((TMROctForest *)f)->evalInterp(pt, N, N1, N2, N3, N11, N22, N33, N23, N13,
                                  N12);
}
// getConnectivity (TMROctForest.cpp:1633-1692): sizes[4] = blocks, faces,
// edges, nodes; arrays copied out when the buffers are given.
void tmrref_get_connectivity(void *f, int *sizes, int *block_conn,
                             int *block_face, int *block_edge, int *face_ids) {
  int nb, nf, ne, nn;
  const int *bc, *bf, *be, *fi;
  ((TMROctForest *)f)->getConnectivity(&nb, &nf, &ne, &nn, &bc, &bf, &be, &fi);
  sizes[0] = nb;
  sizes[1] = nf;
  sizes[2] = ne;
  sizes[3] = nn;
  if (block_conn) memcpy(block_conn, bc, sizeof(int) * 8 * nb);
  if (block_face) memcpy(block_face, bf, sizeof(int) * 6 * nb);
  if (block_edge) memcpy(block_edge, be, sizeof(int) * 12 * nb);
  if (face_ids) memcpy(face_ids, fi, sizeof(int) * 6 * nb);
}
// getInverseConnectivity (TMROctForest.cpp:1694-1740) copied out; the
// pointer arrays have nodes+1, edges+1, faces+1 entries.
void tmrref_get_inverse_connectivity(void *f, int *node_conn, int *node_ptr,
                                     int *edge_conn, int *edge_ptr,
                                     int *face_conn, int *face_ptr) {
  int nb, nf, ne, nn;
  ((TMROctForest *)f)->getConnectivity(&nb, &nf, &ne, &nn, NULL, NULL, NULL,
                                       NULL);
  const int *a, *b, *c, *d, *e, *g;
  ((TMROctForest *)f)->getInverseConnectivity(&a, &b, &c, &d, &e, &g);
  memcpy(node_ptr, b, sizeof(int) * (nn + 1));
  memcpy(node_conn, a, sizeof(int) * b[nn]);
  memcpy(edge_ptr, d, sizeof(int) * (ne + 1));
  memcpy(edge_conn, c, sizeof(int) * d[ne]);
  memcpy(face_ptr, g, sizeof(int) * (nf + 1));
  memcpy(face_conn, e, sizeof(int) * g[nf]);
}
// findEnclosing (TMROctForest.cpp:6228-6377) for nodes given as 7 ints
// {block, x, y, z, tag, level, info}: index of the returned octant, or -1.
void tmrref_find_enclosing(void *f, int order, const double *knots, int n,
                           const int *nodes7, long *out) {
  TMROctForest *F = (TMROctForest *)f;
  TMROctantArray *arr;
  F->getOctants(&arr);
  TMROctant *base;
  int size;
  arr->getArray(&base, &size);
  for (int i = 0; i < n; i++) {
    TMROctant q;
    q.block = nodes7[7 * i];
    q.x = nodes7[7 * i + 1];
    q.y = nodes7[7 * i + 2];
    q.z = nodes7[7 * i + 3];
    q.tag = nodes7[7 * i + 4];
    q.level = (int16_t)nodes7[7 * i + 5];
    q.info = (int16_t)nodes7[7 * i + 6];
    TMROctant *t = F->findEnclosing(order, knots, &q);
    out[i] = t ? (long)(t - base) : -1;
  }
}
// transformNode (TMROctForest.cpp:3847-4039) in place on 7-int nodes.
void tmrref_transform_nodes(void *f, int n, int *nodes7, int edge_dir,
                            int *rev, int *fid) {
  TMROctForest *F = (TMROctForest *)f;
  for (int i = 0; i < n; i++) {
    TMROctant q;
    q.block = nodes7[7 * i];
    q.x = nodes7[7 * i + 1];
    q.y = nodes7[7 * i + 2];
    q.z = nodes7[7 * i + 3];
    q.tag = nodes7[7 * i + 4];
    q.level = (int16_t)nodes7[7 * i + 5];
    q.info = (int16_t)nodes7[7 * i + 6];
    int r = 0, id = 0;
    F->transformNode(&q, edge_dir, rev ? &r : NULL, fid ? &id : NULL);
    nodes7[7 * i] = q.block;
    nodes7[7 * i + 1] = q.x;
    nodes7[7 * i + 2] = q.y;
    nodes7[7 * i + 3] = q.z;
    if (rev) rev[i] = r;
    if (fid) fid[i] = id;
  }
}
void tmrref_get_knots(void *f, double *out) {
  const double *k;
  int n = ((TMROctForest *)f)->getInterpKnots(&k);
  memcpy(out, k, sizeof(double) * n);
}
// TMROctTACSTopoCreator::computeWeights (TMR_TACSTopoCreator.cpp:55-122) as
// createElements calls it per element (:163-183), written out over the
// reference's own forest methods (the creator itself needs TACS): rows of
// merged (index, weight) pairs per analysis element.  With cols == NULL
// only the number of entries is returned.
long tmrref_topo_weights(void *filt, void *ana, int *rowptr, int *cols,
                         double *w) {
  TMROctForest *filter = (TMROctForest *)filt, *forest = (TMROctForest *)ana;
  TMROctantArray *arr;
  forest->getOctants(&arr);
  TMROctant *octs;
  int n;
  arr->getArray(&octs, &n);
  const int order = filter->getMeshOrder(), np = order * order * order;
  const int *dep_ptr, *dep_conn;
  const double *dep_w;
  filter->getDepNodeConn(&dep_ptr, &dep_conn, &dep_w);
  const int *conn;
  filter->getNodeConn(&conn);
  const double node_knots[] = {-1.0, 0.0, 1.0};
  std::vector<TMRIndexWeight> wt(np * order * order + 8);
  std::vector<double> N(np);
  long nnz = 0;
  if (rowptr) rowptr[0] = 0;
  for (int i = 0; i < n; i++) {
    TMROctant node = octs[i];
    node.info = 13;
    TMROctant *oct = filter->findEnclosing(3, node_knots, &node);
    if (oct) {
      const int32_t h = 1 << (TMR_MAX_LEVEL - node.level);
      const int32_t hoct = 1 << (TMR_MAX_LEVEL - oct->level);
      double pt[3];
      pt[0] = -1.0 + 2.0 * ((node.x % hoct) + 0.5 * h * (1.0 + node_knots[1])) / hoct;
      pt[1] = -1.0 + 2.0 * ((node.y % hoct) + 0.5 * h * (1.0 + node_knots[1])) / hoct;
      pt[2] = -1.0 + 2.0 * ((node.z % hoct) + 0.5 * h * (1.0 + node_knots[1])) / hoct;
      filter->evalInterp(pt, N.data());
      const int *c = &conn[np * oct->tag];
      int m = 0;
      for (int off = 0; off < np; off++) {
        if (c[off] >= 0) {
          wt[m].index = c[off];
          wt[m].weight = N[off];
          m++;
        } else {
          int d = -c[off] - 1;
          for (int jp = dep_ptr[d]; jp < dep_ptr[d + 1]; jp++) {
            wt[m].index = dep_conn[jp];
            wt[m].weight = N[off] * dep_w[jp];
            m++;
          }
        }
      }
      m = TMRIndexWeight::uniqueSort(wt.data(), m);
      if (cols)
        for (int k = 0; k < m; k++) {
          cols[nnz + k] = wt[k].index;
          w[nnz + k] = wt[k].weight;
        }
      nnz += m;
    }
    if (rowptr) rowptr[i + 1] = (int)nnz;
  }
  return nnz;
}
int tmrref_get_local_node_number(void *f, int node) {
  return ((TMROctForest *)f)->getLocalNodeNumber(node);
}

// TMR_GenerateSTLTriangles (TMR_STLTools.cpp:854-902) with the forest's
// node points set to X (num_local x 3; the checker attaches no topology,
// so the reference's own points are zero) and the design values x
// (vpn per independent node).  The triangles are kept until
// tmrref_stl_get copies them out.
static std::vector<double> g_stl;
int tmrref_stl_triangles(void *f, const double *X, const double *x, int vpn, int offset,
                         double cutoff) {
  if (!TMRIsInitialized()) TMRInitialize();
  TMROctForest *F = (TMROctForest *)f;
  TMRPoint *P;
  int nl = F->getPoints(&P);
  for (int i = 0; i < nl; i++) {
    P[i].x = X[3 * i];
    P[i].y = X[3 * i + 1];
    P[i].z = X[3 * i + 2];
  }
  TACSBVec vec(x, vpn);
  int ntris = 0;
  TMR_STLTriangle *tris = NULL;
  TMR_GenerateSTLTriangles(0, F, &vec, offset, cutoff, &ntris, &tris);
  g_stl.assign((size_t)ntris * 9, 0.0);
  for (int i = 0; i < ntris; i++)
    for (int k = 0; k < 3; k++) {
      g_stl[9 * i + 3 * k] = tris[i].p[k].x;
      g_stl[9 * i + 3 * k + 1] = tris[i].p[k].y;
      g_stl[9 * i + 3 * k + 2] = tris[i].p[k].z;
    }
  delete[] tris;
  return ntris;
}
void tmrref_stl_get(double *out) {
  for (size_t i = 0; i < g_stl.size(); i++) out[i] = g_stl[i];
}
int tmrref_convert_bin_to_stl(const char *binfile, const char *stlfile) {
  return TMR_ConvertBinToSTL(binfile, stlfile);
}
// TMR_GenerateBinFile + TMR_ConvertBinToSTL (TMR_STLTools.cpp:904-993).
int tmrref_stl_files(void *f, const double *X, const double *x, int vpn, int offset,
                     double cutoff, const char *binfile, const char *stlfile) {
  if (!TMRIsInitialized()) TMRInitialize();
  TMROctForest *F = (TMROctForest *)f;
  TMRPoint *P;
  int nl = F->getPoints(&P);
  for (int i = 0; i < nl; i++) {
    P[i].x = X[3 * i];
    P[i].y = X[3 * i + 1];
    P[i].z = X[3 * i + 2];
  }
  TACSBVec vec(x, vpn);
  int fail = TMR_GenerateBinFile(binfile, F, &vec, offset, cutoff);
  if (!fail && stlfile) fail = TMR_ConvertBinToSTL(binfile, stlfile);
  return fail;
}

}  // extern "C"
