/*
  Recording stand-in for TACS's TACSBVecInterp, used only to compile the
  reference TMR octree core as a CPU checker (test infrastructure).

  TMROctForest::createInterpolation (TMROctForest.cpp:6611-6793) calls
  addInterp(row, weights, cols, n) once per fine owned node.  This class
  keeps those calls, in call order, so the checker can return the
  prolongation operator as (row, cols[], weights[]) records.
*/
#ifndef TMRG_REF_SHIM_TACSBVECINTERP_H
#define TMRG_REF_SHIM_TACSBVECINTERP_H

#include <vector>

class TACSBVecInterp {
 public:
  void addInterp(int row, const double w[], const int cols[], int n) {
    rows.push_back(row);
    ptr.push_back((int)cols_.size() + n);
    for (int i = 0; i < n; i++) {
      cols_.push_back(cols[i]);
      weights.push_back(w[i]);
    }
  }
  std::vector<int> rows;
  std::vector<int> ptr;  // end offset of each recorded call
  std::vector<int> cols_;
  std::vector<double> weights;
};

#endif
