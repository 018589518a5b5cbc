// Helmholtz PDE filter objects (tmrg_helmholtz.cu).
#pragma once

#include <memory>
#include <vector>

#include "tmrg_internal.h"

namespace tmrg {

// Coarsest levels up to this many nodes are solved with a dense inverse.
constexpr long long HM_DENSE_MAX = 2048;

// Per-element factors: x = V (Jacobian determinant), y, z, w = r^2 / s_d^2
// for the half sides s_d.
template <typename T>
struct alignas(4 * sizeof(T)) HGeoT {
  T x, y, z, w;
};

// 1-D reference mass and stiffness matrices of the element basis on
// [-1, 1] (o = 2 linear, o = 3 quadratic Bernstein).
template <typename T>
struct HBasisT {
  int o;
  T M[3][3], K[3][3];
};

// Work vectors of one level in one precision.
template <typename T>
struct HWork {
  int cap = 0;  // components the vectors hold
  DBuf<T> x, b, r, d, t, xd, yE;
};

// One level of the filter hierarchy: the forest's element connectivity
// and dependent weights, per-element factors, the node-ordered scatter
// list of element slots, the inverse Jacobi diagonal and the largest
// eigenvalue estimate the Chebyshev smoother scales its interval by.  The operator data is held in FP64 (the
// Krylov iteration, the filter's mass products) and FP32 (the multigrid
// preconditioner).
struct HLevel {
  long long ne = 0, nn = 0, ndep = 0, dnnz = 0, snnz = 0;
  int dim = 3, o = 2, npe = 8;
  HBasisT<double> bas{};
  HBasisT<float> bas32{};
  DBuf<int> econn, dptr, dconn, srp, sslot;
  DBuf<double> dw, geo, sw, dinv;
  DBuf<float> dw32, geo32, sw32, dinv32;
  double lam = 0.0;  // Lanczos estimate of the largest eigenvalue of D^-1 K
  HWork<double> w64;
  HWork<float> w32;
};

// FP32 copies of one createInterpolation operator's values (P and P^T).
struct HInterp32 {
  DBuf<float> p, pt;
};

struct Helmholtz {
  cudaStream_t s = 0;
  double r = 0.0;
  int nlevels = 0;
  std::vector<std::unique_ptr<HLevel>> L;
  std::vector<std::unique_ptr<Interp>> P;  // P[k]: level k+1 -> level k
  std::vector<std::unique_ptr<HInterp32>> P32;
  bool dense = false;
  long long nc = 0;
  DBuf<float> Ainv32;  // coarsest level's dense inverse
  // solver settings (the reference's GMRES tolerances,
  // TMRHelmholtzFilter.cpp:95-101)
  double rtol = 1e-12, atol = 1e-30;
  int max_iters = 300;
  // Chebyshev smoother: interval [lower, upper] x lam; degree and lower
  // bound by level order
  double cheb_lower2 = 0.05, cheb_lower3 = 0.1, cheb_upper = 1.1;
  int cheb_degree2 = 5, cheb_degree3 = 6;
  int lanczos_steps = 16;
  int coarse_sweeps = 4;
  // last solve
  int last_iters = 0;
  std::vector<double> last_res;
  // finest-level Krylov vectors
  DBuf<double> cg_r, cg_p, cg_q, cg_z, cg_zo, rhs, psi, part, dots, sc;
};

void helmholtz_create(Forest *const *forests, int nlevels, double r, Helmholtz &H);
struct QForest;
void helmholtz_create_quad(QForest *const *forests, int nlevels, double r, Helmholtz &H);
void helmholtz_apply(Helmholtz &H, bool transpose, int vpn, const double *in, double *out);
void helmholtz_operator(Helmholtz &H, int level, bool stiff, int nvec, const double *in,
                        double *out);

}  // namespace tmrg
