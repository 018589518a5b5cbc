/*
  tmr_oracle — CPU restatement of TMR's octree-forest adaptation path.

  TEST INFRASTRUCTURE ONLY.  This is the checker the GPU library is
  compared against: plain sequential C that follows the reference's
  algorithms step by step (TMROctForest.cpp, TMROctant.cpp, TMRBase.h,
  TMRMatrixFilter.cpp).  Only the test-suite, the smoke check and the
  CPU-baseline leg of the benchmark may load it; the product never does.

  Parity of this restatement is pinned against the reference itself:
  tests/golden/ holds vectors produced by the reference's own
  TMROctant.cpp/TMROctForest.cpp/TMRBase.cpp compiled for one rank
  (oracle/ref_shim/, built by oracle/build.py into oracle/_ref/), and
  tests/test_oracle_golden.py checks this code against them.  The
  TACS-side pieces (P/P^T apply, mass matrix, filter) have no reference
  implementation in the reference tree; they are restated here from the
  call sites and marked "parity unpinned".
*/
#ifndef TMR_ORACLE_H
#define TMR_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Same field layout as TMROctant (TMROctant.h:47-52), 24 bytes. */
typedef struct {
  int32_t block, x, y, z, tag;
  int16_t level, info;
} oo_oct;

typedef struct oo_forest oo_forest;
typedef struct oo_interp oo_interp;

oo_forest *oo_forest_create(int order, int interp_type);
void oo_forest_destroy(oo_forest *f);
int oo_set_connectivity(oo_forest *f, int num_nodes, const int *block_conn,
                        int num_blocks);
void oo_set_mesh_order(oo_forest *f, int order, int interp_type);
void oo_create_trees(oo_forest *f, int level);
void oo_refine(oo_forest *f, const int *refinement, int min_level,
               int max_level);
oo_forest *oo_coarsen(oo_forest *f);
oo_forest *oo_duplicate(oo_forest *f);
void oo_balance(oo_forest *f, int balance_corner);
void oo_create_nodes(oo_forest *f);

int oo_num_octants(oo_forest *f);
void oo_get_octants(oo_forest *f, int *out7);
/* out: {num_local_nodes, num_owned, num_dep, ext_pre_offset, num_elements,
          dep_nnz} */
void oo_node_sizes(oo_forest *f, int *out6);
void oo_get_conn(oo_forest *f, int *out);
void oo_get_node_numbers(oo_forest *f, int *out);
void oo_get_dep(oo_forest *f, int *ptr, int *conn, double *weights);
void oo_get_knots(oo_forest *f, double *knots);

/* Prolongation P (coarse -> fine), recorded in the order rows are made. */
oo_interp *oo_create_interp(oo_forest *fine, oo_forest *coarse);
void oo_interp_sizes(oo_interp *I, int *out2); /* {rows, nnz} */
void oo_interp_get(oo_interp *I, int *rows, int *end_ptr, int *cols,
                   double *w);
void oo_interp_destroy(oo_interp *I);

/* CSR applies over row-sorted P (parity unpinned: TACS is absent).
   rowptr/cols/vals describe P with n_fine rows and n_coarse columns; X
   holds k vectors stored node-major (x[node*k + v]). */
void oo_csr_mult(int n_rows, const int *rowptr, const int *cols,
                 const double *vals, int k, const double *x, double *y);
void oo_csr_mult_t(int n_rows, int n_cols, const int *rowptr,
                   const int *cols, const double *vals, int k,
                   const double *x, double *y);
void oo_csr_mult_wt(int n_rows, int n_cols, const int *rowptr,
                    const int *cols, const double *vals, int k,
                    const double *x, double *y);

/* Matrix density filter (TMRMatrixFilter.cpp:30-235), restated. */
typedef struct oo_filter oo_filter;
oo_filter *oo_filter_create(oo_forest *f, double block_len, double r, int N);
void oo_filter_sizes(oo_filter *F, int *out2); /* {n, nnz} */
void oo_filter_get_matrix(oo_filter *F, int *rowptr, int *cols, double *vals,
                          double *Ainv, double *B, double *Tinv);
void oo_filter_apply(oo_filter *F, int vpn, const double *in, double *out);
void oo_filter_apply_t(oo_filter *F, int vpn, const double *in, double *out);
void oo_filter_destroy(oo_filter *F);

/* Seeded synthetic inputs shared by the GPU path and the oracle. */
uint64_t oo_splitmix64(uint64_t x);
double oo_uniform(uint64_t seed, uint64_t stream, uint64_t index);

#ifdef __cplusplus
}
#endif
#endif
