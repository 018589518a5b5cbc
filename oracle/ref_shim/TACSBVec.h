/*
  Read-only stand-in for TACS's TACSBVec, used only to compile the
  reference TMR_STLTools.cpp as a CPU checker (test infrastructure).

  TMR_GenerateSTLTriangles (TMR_STLTools.cpp:639-852) distributes the
  vector, asks its block size and reads one node's block of values at a
  time; this class serves those calls from a caller-owned array of
  `bsize` interleaved values per independent node.
*/
#ifndef TMRG_REF_SHIM_TACSBVEC_H
#define TMRG_REF_SHIM_TACSBVEC_H

#include <string.h>

typedef double TacsScalar;

class TACSBVec {
 public:
  TACSBVec(const double *v, int b) : vals(v), bsize(b) {}
  void beginDistributeValues() {}
  void endDistributeValues() {}
  int getBlockSize() { return bsize; }
  void getValues(int n, const int *index, TacsScalar *out) {
    for (int i = 0; i < n; i++)
      memcpy(out + (size_t)i * bsize, vals + (size_t)index[i] * bsize,
             sizeof(double) * bsize);
  }

 private:
  const double *vals;
  int bsize;
};

#endif
