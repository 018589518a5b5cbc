// Drives the C++ TMRQuadForest facade (include/tmrg_quadforest.hpp) the
// way TMR code drives TMRQuadForest, then the STL tools on a small octree
// forest.  Prints counts and checksums for the test to compare with the
// Python binding on the same input.
#include <stdio.h>

#include <vector>

#include "tmrg_quadforest.hpp"

int main(int argc, char **argv) {
  const int nx = 3, ny = 2;
  std::vector<int> conn;
  for (int j = 0; j < ny; j++)
    for (int i = 0; i < nx; i++) {
      int n0 = i + (nx + 1) * j;
      conn.insert(conn.end(), {n0, n0 + 1, n0 + nx + 1, n0 + nx + 2});
    }
  TMRQuadForest *f = new TMRQuadForest(0, 3, TMR_GAUSS_LOBATTO_POINTS);
  f->incref();
  f->setConnectivity((nx + 1) * (ny + 1), conn.data(), nx * ny);
  f->createTrees(1);
  for (int pass = 0; pass < 3; pass++) {
    TMRQuadrantArray *quads;
    f->getQuadrants(&quads);
    int n;
    TMRQuadrant *a;
    quads->getArray(&a, &n);
    std::vector<int> ref(n);
    for (int i = 0; i < n; i++) ref[i] = ((a[i].x >> 20) + (a[i].y >> 21) + a[i].face + pass) % 3 == 0;
    f->refine(ref.data(), 0, 6);
    f->balance(1);
  }
  f->createNodes();
  TMRQuadForest *c = f->coarsen();
  c->incref();
  c->balance(1);
  c->createNodes();
  TMRGVecInterp *I = new TMRGVecInterp();
  I->incref();
  f->createInterpolation(c, I);
  int64_t rows, cols, nnz;
  I->getSizes(&rows, &cols, &nnz);
  std::vector<double> x(cols, 1.0), y(rows, 0.0);
  I->mult(x.data(), y.data());
  double s = 0.0;
  for (double v : y) s += v;
  const int *ec;
  int ne, nown;
  f->getNodeConn(&ec, &ne, &nown);
  long long csum = 0;
  for (long long i = 0; i < (long long)ne * 9; i++) csum += ec[i];
  const int *dp, *dc;
  const double *dw;
  int nd = f->getDepNodeConn(&dp, &dc, &dw);
  int nfaces, nedges, nnodes;
  const int *fc, *fe;
  f->getConnectivity(&nfaces, &nedges, &nnodes, &fc, &fe);
  printf("elements %d owned %d dep %d conn_sum %lld P_rows %lld P_nnz %lld P1_sum %.17g "
         "faces %d edges %d nodes %d\n",
         ne, nown, nd, csum, (long long)rows, (long long)nnz, s, nfaces, nedges, nnodes);
  // the face mesh and the quadrants through face boxes (x offset = face)
  std::vector<double> boxes(4 * nfaces);
  for (int k = 0; k < nfaces; k++) {
    boxes[4 * k] = k, boxes[4 * k + 1] = 0.0;
    boxes[4 * k + 2] = boxes[4 * k + 3] = 1.0;
  }
  f->setFaceBoxes(boxes.data(), nfaces);
  f->writeToVTK(argc > 1 ? argv[1] : "/dev/null");
  f->writeForestToVTK(argc > 2 ? argv[2] : "/dev/null");
  f->writeToTecplot(argc > 3 ? argv[3] : "/dev/null");
  const int *qnums = nullptr;
  const int nnum = f->getNodeNumbers(&qnums);
  printf("node_numbers %d first %d local_of_first %d ext_pre %d\n", nnum, nnum ? qnums[0] : 0,
         nnum ? f->getLocalNodeNumber(qnums[0]) : -1, f->getExtPreOffset());
  // seeded random trees
  TMRQuadForest *r = new TMRQuadForest(0, 2, TMR_GAUSS_LOBATTO_POINTS);
  r->incref();
  r->setConnectivity((nx + 1) * (ny + 1), conn.data(), nx * ny);
  r->createRandomTrees(25, 1, 6, 5);
  r->repartition();
  TMRQuadrantArray *rq;
  r->getQuadrants(&rq);
  int nr;
  TMRQuadrant *ra;
  rq->getArray(&ra, &nr);
  long long rsum = 0;
  for (int i = 0; i < nr; i++) rsum += (long long)ra[i].x + 3LL * ra[i].y + ra[i].level;
  printf("rand_quads %d rand_sum %lld\n", nr, rsum);
  r->decref();
  // STL tools on a one-block octree forest with a linear field in x
  std::vector<int> bconn = {0, 1, 2, 3, 4, 5, 6, 7};
  TMROctForest *o = new TMROctForest(0, 2, TMR_GAUSS_LOBATTO_POINTS);
  o->incref();
  o->setConnectivity(8, bconn.data(), 1);
  o->createTrees(2);
  o->createNodes();
  int nl;
  const int *nums;
  nl = o->getNodeNumbers(&nums);
  int no;
  o->getNodeConn(nullptr, nullptr, &no);
  std::vector<double> xv(no);
  // value = node number parity: a ragged level set, enough to produce
  // triangles
  for (int i = 0; i < no; i++) xv[i] = (i % 3) * 0.5;
  int ntris = 0;
  TMR_STLTriangle *tris = nullptr;
  TMR_GenerateSTLTriangles(0, o, xv.data(), 1, 0, 0.4, &ntris, &tris);
  double tsum = 0.0;
  for (int i = 0; i < ntris; i++)
    for (int k = 0; k < 3; k++) tsum += tris[i].p[k].x + tris[i].p[k].y + tris[i].p[k].z;
  delete[] tris;
  printf("stl_tris %d stl_sum %.17g local %d\n", ntris, tsum, nl);
  // the matrix filter on an order-2 quadtree forest of the same faces
  TMRQuadForest *q2 = new TMRQuadForest(0, 2, TMR_GAUSS_LOBATTO_POINTS);
  q2->incref();
  q2->setConnectivity((nx + 1) * (ny + 1), conn.data(), nx * ny);
  q2->createTrees(3);
  q2->createNodes();
  int n2;
  q2->getNodeConn(nullptr, nullptr, &n2);
  TMRMatrixFilter *mf = new TMRMatrixFilter(0.1, 10, 1, &q2);
  mf->incref();
  std::vector<double> fx(n2), fy(n2);
  for (int i = 0; i < n2; i++) fx[i] = (i % 5) * 0.25;
  mf->applyFilter(fx.data(), fy.data());
  double fsum = 0.0;
  for (int i = 0; i < n2; i++) fsum += fy[i];
  printf("filter_nodes %d filter_sum %.17g\n", n2, fsum);
  mf->decref();
  q2->decref();
  I->decref();
  c->decref();
  f->decref();
  o->decref();
  return 0;
}
