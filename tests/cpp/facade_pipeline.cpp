// Drives the C++ TMROctForest facade (include/tmrg_octforest.hpp) the way
// TMR code drives TMROctForest: setConnectivity, createTrees, refine,
// balance, createNodes, coarsen, createInterpolation, the P applies.
// Prints one line of counts and checksums for the test to compare with
// the Python binding on the same input.
#include <stdio.h>

#include <vector>

#include "tmrg_octforest.hpp"

int main() {
  const int nx = 3, ny = 2, nz = 2;
  std::vector<int> conn;
  for (int k = 0; k < nz; k++)
    for (int j = 0; j < ny; j++)
      for (int i = 0; i < nx; i++)
        for (int c = 0; c < 8; c++) {
          int ii = i + (c & 1), jj = j + ((c >> 1) & 1), kk = k + (c >> 2);
          conn.push_back(ii + (nx + 1) * (jj + (ny + 1) * kk));
        }
  TMROctForest *f = new TMROctForest(0, 3, TMR_GAUSS_LOBATTO_POINTS);
  f->incref();
  f->setConnectivity((nx + 1) * (ny + 1) * (nz + 1), conn.data(), nx * ny * nz);
  f->createTrees(1);
  for (int pass = 0; pass < 3; pass++) {
    TMROctantArray *octs;
    f->getOctants(&octs);
    int n;
    TMROctant *a;
    octs->getArray(&a, &n);
    std::vector<int> ref(n);
    for (int i = 0; i < n; i++) ref[i] = ((a[i].x >> 20) + (a[i].y >> 21) + a[i].block + pass) % 3 == 0;
    f->refine(ref.data(), 0, 5);
    f->balance(1);
  }
  f->createNodes();
  TMROctForest *c = f->coarsen();
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
  for (long long i = 0; i < (long long)ne * 27; i++) csum += ec[i];
  const int *dp, *dc;
  const double *dw;
  int nd = f->getDepNodeConn(&dp, &dc, &dw);
  printf("elements %d owned %d dep %d conn_sum %lld P_rows %lld P_nnz %lld P1_sum %.12f\n",
         ne, nown, nd, csum, (long long)rows, (long long)nnz, s);
  I->decref();
  c->decref();
  f->decref();
  return 0;
}
