// Drives the C++ TMROctForest facade (include/tmrg_octforest.hpp) the way
// TMR code drives TMROctForest: setConnectivity, createTrees, refine,
// balance, createNodes, coarsen, createInterpolation, the P applies.
// Prints one line of counts and checksums for the test to compare with
// the Python binding on the same input.
#include <stdio.h>

#include <vector>

#include "tmrg_octforest.hpp"

int main(int argc, char **argv) {
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
  // the rest of the surface: connectivity getters, local numbers, shape
  // functions (partition of unity), findEnclosing, transformNode
  int nb, nf, ned, nn;
  const int *bc, *bf, *be, *fi;
  f->getConnectivity(&nb, &nf, &ned, &nn, &bc, &bf, &be, &fi);
  const int *npt, *nco, *ept, *eco, *fpt, *fco;
  f->getInverseConnectivity(&nco, &npt, &eco, &ept, &fco, &fpt);
  const int *nums;
  int nl = f->getNodeNumbers(&nums);
  int local_ok = f->getLocalNodeNumber(nums[nl / 2]) == nl / 2;
  double pt[3] = {0.25, -0.5, 0.75}, N[27], N1[27], N2[27], N3[27];
  f->evalInterp(pt, N, N1, N2, N3);
  double pu = 0.0, du = 0.0;
  for (int i = 0; i < 27; i++) {
    pu += N[i];
    du += N1[i];
  }
  TMROctantArray *octs;
  f->getOctants(&octs);
  TMROctant *a;
  int na;
  octs->getArray(&a, &na);
  TMROctant node = a[na / 2];
  node.info = 13;  // element centre: enclosed by the element itself
  const double *kn;
  f->getInterpKnots(&kn);
  TMROctant *enc = f->findEnclosing(3, kn, &node);
  TMROctant corner = a[0];
  corner.x = corner.y = corner.z = 0;
  int rev = -1, fid = -1;
  f->transformNode(&corner, -1, &rev, &fid);
  // the forest outline through unit block boxes (writeForestToVTK)
  std::vector<double> boxes(6 * nb);
  for (int b = 0; b < nb; b++) {
    boxes[6 * b + 0] = b, boxes[6 * b + 1] = 0.0, boxes[6 * b + 2] = 0.0;
    boxes[6 * b + 3] = boxes[6 * b + 4] = boxes[6 * b + 5] = 1.0;
  }
  f->setBlockBoxes(boxes.data(), nb);
  f->writeForestToVTK(argc > 1 ? argv[1] : "/dev/null");
  f->writeToTecplot(argc > 2 ? argv[2] : "/dev/null");
  f->writeToVTK(argc > 3 ? argv[3] : "/dev/null");
  printf("elements %d owned %d dep %d conn_sum %lld P_rows %lld P_nnz %lld P1_sum %.12f "
         "blocks %d faces %d edges %d nodes %d node_refs %d local_ok %d pu %.15f du %.15f "
         "enclosed_self %d corner_block %d\n",
         ne, nown, nd, csum, (long long)rows, (long long)nnz, s, nb, nf, ned, nn, npt[nn],
         local_ok, pu, du, enc == &a[na / 2], corner.block);
  I->decref();
  c->decref();
  f->decref();
  return 0;
}
