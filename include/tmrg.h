/*
  tmrg.h — C ABI of the GB300 octree-forest adaptation library.

  One opaque forest handle stands for one TMROctForest (TMROctForest.h:46);
  the octants, nodes and operators live in GPU memory as structure-of-arrays
  and are produced by CUDA kernels for sm_103a.  Every entry point returns
  a tmrg_status (0 = success) and never aborts; host pointers are copied
  in/out with explicit sizes, and *_device variants take device pointers.

  Each declaration names the reference interface it replaces
  (file:line in the TMR sources).  The reference reports errors by printing
  to stderr and returning; tmrg returns the status instead and
  tmrg_last_error() gives the message.
*/
#ifndef TMRG_H
#define TMRG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  TMRG_OK = 0,
  TMRG_ERR_ARG = 1,         /* bad argument (null, size mismatch, range) */
  TMRG_ERR_STATE = 2,       /* call out of order (e.g. no octants yet) */
  TMRG_ERR_CUDA = 3,        /* CUDA runtime error */
  TMRG_ERR_NOMEM = 4,       /* device allocation failed */
  TMRG_ERR_KEY_RANGE = 5,   /* blocks x levels exceed the 64-bit sort key */
  TMRG_ERR_UNSUPPORTED = 6, /* order/interpolation not built */
  TMRG_ERR_INTERNAL = 7     /* a device-side consistency check failed */
} tmrg_status;

/* Interpolation types, same values as TMRInterpolationType
   (TMRBase.h:39-43). */
enum { TMRG_UNIFORM_POINTS = 0, TMRG_GAUSS_LOBATTO_POINTS = 1,
       TMRG_BERNSTEIN_POINTS = 2 };

typedef struct tmrg_forest tmrg_forest;
typedef struct tmrg_interp tmrg_interp;
typedef struct tmrg_filter tmrg_filter;
typedef struct tmrg_helmholtz tmrg_helmholtz;
typedef struct tmrg_qforest tmrg_qforest;

/* Message of the last failed call on this thread ("" if none). */
const char *tmrg_last_error(void);
/* Library version string. */
const char *tmrg_version(void);

/* ---- forest ---------------------------------------------------------- */
/* TMROctForest::TMROctForest(MPI_Comm, int order, TMRInterpolationType)
   (TMROctForest.h:51-52).  `stream` is a cudaStream_t (NULL = default);
   all work of this forest is ordered on it. */
int tmrg_forest_create(int order, int interp_type, void *stream,
                       tmrg_forest **out);
/* TMREntity::decref reaching zero (TMRBase.cpp:145-156). */
int tmrg_forest_destroy(tmrg_forest *f);
/* TMROctForest::setConnectivity (TMROctForest.h:64-65;
   TMROctForest.cpp:558-590).  block_conn: host, 8 ints per block. */
int tmrg_forest_set_connectivity(tmrg_forest *f, int num_nodes,
                                 const int *block_conn, int num_blocks);
/* TMROctForest::setFullConnectivity (TMROctForest.h:66-69;
   TMROctForest.cpp:596-637): corners, edges and faces of every block given
   (8, 12 and 6 ints per block, host); adjacency follows the given edge and
   face numbers. */
int tmrg_forest_set_full_connectivity(tmrg_forest *f, int num_nodes,
                                      int num_edges, int num_faces,
                                      int num_blocks, const int *block_conn,
                                      const int *block_edge_conn,
                                      const int *block_face_conn);
/* TMROctForest::getConnectivity (TMROctForest.h:142-145;
   TMROctForest.cpp:1633-1692): borrowed host arrays, 8 / 6 / 12 / 6 ints
   per block; edges and faces numbered in order of first use as the
   reference numbers them.  Valid until the connectivity is replaced. */
int tmrg_forest_get_connectivity(tmrg_forest *f, int *nblocks, int *nfaces,
                                 int *nedges, int *nnodes,
                                 const int **block_conn,
                                 const int **block_face_conn,
                                 const int **block_edge_conn,
                                 const int **block_face_ids);
/* TMROctForest::getInverseConnectivity (TMROctForest.h:146-151;
   TMROctForest.cpp:1694-1740): CSR lists of 8*block+corner,
   12*block+edge and 6*block+face entries in block order (borrowed). */
int tmrg_forest_get_inverse_connectivity(
    tmrg_forest *f, const int **node_block_conn, const int **node_block_ptr,
    const int **edge_block_conn, const int **edge_block_ptr,
    const int **face_block_conn, const int **face_block_ptr);
/* TMROctForest::createRandomTrees (TMROctForest.h:81;
   TMROctForest.cpp:1838-1917): nrand octants per block at random levels in
   [min_level, max_level] and random anchors, sorted and unique by position
   (finest kept).  The reference draws from libc rand(); here octant i of
   block b draws a seeded splitmix64 uniform U(seed, b, 4i+k). */
int tmrg_forest_create_random_trees(tmrg_forest *f, int nrand, int min_level,
                                    int max_level, uint64_t seed);
/* TMROctForest::setMeshOrder / getMeshOrder / getInterpType
   (TMROctForest.h:72-75; TMROctForest.cpp:1389-1440). */
int tmrg_forest_set_mesh_order(tmrg_forest *f, int order, int interp_type);
int tmrg_forest_get_mesh_order(tmrg_forest *f, int *order, int *interp_type);
/* TMROctForest::getInterpKnots (TMROctForest.cpp:1492-1497). */
int tmrg_forest_get_interp_knots(tmrg_forest *f, double *knots);
/* TMROctForest::createTrees (TMROctForest.h:79; TMROctForest.cpp:1744). */
int tmrg_forest_create_trees(tmrg_forest *f, int level);
/* TMROctForest::refine(const int refinement[], int min, int max)
   (TMROctForest.h:87; TMROctForest.cpp:2169-2329).  `refinement` is a
   host array of n = number of octants, or NULL to refine every octant. */
int tmrg_forest_refine(tmrg_forest *f, const int *refinement, int64_t n,
                       int min_level, int max_level);
/* Same, with `refinement` in device memory. */
int tmrg_forest_refine_device(tmrg_forest *f, const int *d_refinement,
                              int64_t n, int min_level, int max_level);
/* TMROctForest::coarsen / duplicate (TMROctForest.h:83-84;
   TMROctForest.cpp:2097-2164): a new forest owned by the caller. */
int tmrg_forest_coarsen(tmrg_forest *f, tmrg_forest **out);
int tmrg_forest_duplicate(tmrg_forest *f, tmrg_forest **out);
/* TMROctForest::balance(int balance_corner) (TMROctForest.h:91;
   TMROctForest.cpp:2917-3089). */
int tmrg_forest_balance(tmrg_forest *f, int balance_corner);
/* TMROctForest::repartition (TMROctForest.h:80): one GPU holds the whole
   forest, so this only validates the handle. */
int tmrg_forest_repartition(tmrg_forest *f, int max_rank);
/* TMROctForest::createNodes (TMROctForest.h:95; TMROctForest.cpp:4064). */
int tmrg_forest_create_nodes(tmrg_forest *f);

/* TMROctForest::getOctants (TMROctForest.h:125).  Number of octants, then
   a host copy: 7 ints per octant {block, x, y, z, tag, level, info}. */
int tmrg_forest_num_octants(tmrg_forest *f, int64_t *n);
int tmrg_forest_get_octants(tmrg_forest *f, int *out7, int64_t n);
/* Device view of the octant arrays (borrowed, valid until the next
   mutating call): block, x, y, z as int32, level and info as int16. */
int tmrg_forest_octants_device(tmrg_forest *f, const int **block,
                               const int **x, const int **y, const int **z,
                               const int16_t **level, const int16_t **info);
/* Sizes after createNodes: out[0] num_local_nodes, [1] owned nodes
   (getOwnedNodeRange, TMROctForest.cpp:1445), [2] dependent nodes
   (getDepNodeConn return), [3] getExtPreOffset, [4] elements,
   [5] dependent-CSR entries. */
int tmrg_forest_node_sizes(tmrg_forest *f, int64_t out6[6]);
/* TMROctForest::getNodeConn (TMROctForest.cpp:5686): elements x order^3
   global node numbers, dependent nodes as -k-1.  Host copy. */
int tmrg_forest_get_node_conn(tmrg_forest *f, int *conn, int64_t n);
/* TMROctForest::getNodeNumbers (TMROctForest.cpp:1461): sorted. */
int tmrg_forest_get_node_numbers(tmrg_forest *f, int *out, int64_t n);
/* TMROctForest::getDepNodeConn (TMROctForest.cpp:5717): host copies of
   ptr[num_dep+1], conn[nnz], weights[nnz]. */
int tmrg_forest_get_dep_node_conn(tmrg_forest *f, int *ptr, int *conn,
                                  double *weights);
/* Device views of conn and the dependent CSR (borrowed). */
int tmrg_forest_node_conn_device(tmrg_forest *f, const int **conn);
int tmrg_forest_dep_node_conn_device(tmrg_forest *f, const int **ptr,
                                     const int **conn, const double **w);

/* Borrowed host views, the reference getters' own semantics: pointers into
   page-locked host memory owned by the forest, valid until the next call
   that changes the forest (setConnectivity, setMeshOrder, createTrees,
   refine, balance, createNodes) or its destruction.  Built on first
   request after a change.
   TMROctForest::getOctants (TMROctForest.h:128; TMROctForest.cpp:1452):
   octants in TMROctant layout, tag = index. */
typedef struct {
  int32_t block, x, y, z, tag;
  int16_t level, info;
} tmrg_octant; /* TMROctant field layout (TMROctant.h:47-52), 24 bytes */
int tmrg_forest_octants_host(tmrg_forest *f, const tmrg_octant **octs,
                             int64_t *n);
/* TMROctForest::getNodeConn (TMROctForest.h:108; TMROctForest.cpp:5686). */
int tmrg_forest_node_conn_host(tmrg_forest *f, const int **conn,
                               int64_t *num_elements);
/* TMROctForest::getDepNodeConn (TMROctForest.h:110;
   TMROctForest.cpp:5717); *num_dep is the reference's return value. */
int tmrg_forest_dep_node_conn_host(tmrg_forest *f, const int **ptr,
                                   const int **conn, const double **weights,
                                   int64_t *num_dep);
/* Returns the page-locked blocks kept for reuse by host views to the
   system (no reference counterpart). */
int tmrg_host_pool_trim(void);

/* TMROctForest::getLocalNodeNumber (TMROctForest.cpp:1486-1496): index of
   global node number `node` in getNodeNumbers, or -1. */
int tmrg_forest_get_local_node_number(tmrg_forest *f, int node, int *local);
/* TMROctForest::getPoints (TMROctForest.cpp:1476-1482) with the node
   locations of evaluateNodeLocations (:5524-5680): X[3*num_local_nodes],
   each node placed by the first element (in element order) that uses it.
   The reference evaluates a TMRTopology volume and leaves every point at 0
   without one; here the geometry is an optional axis-aligned box per block
   (tmrg_forest_set_block_boxes: origin xyz, extent xyz), mapping the
   block's parameter cube linearly; without boxes every point is 0. */
int tmrg_forest_set_block_boxes(tmrg_forest *f, const double *boxes,
                                int num_blocks);
int tmrg_forest_get_points(tmrg_forest *f, double *X, int64_t n);
/* TMROctForest::evalInterp (TMROctForest.h:131-138;
   TMROctForest.cpp:1510-1631): tensor-product shape functions of the
   forest's order and interpolation at a parametric point pt[3] in
   [-1,1]^3, ii fastest; N1..N3 (all or none) the first derivatives.  The
   *_eval_interp forms take the order, type and knots explicitly. */
int tmrg_eval_interp(int order, int interp_type, const double *knots,
                     const double *pt, double *N, double *N1, double *N2,
                     double *N3);
int tmrg_forest_eval_interp(tmrg_forest *f, const double *pt, double *N,
                            double *N1, double *N2, double *N3);
/* Second-derivative form.  Reproduces the reference: N33 ends holding the
   mixed (1,2) derivative and N12 is not written
   (TMROctForest.cpp:1614-1615). */
int tmrg_eval_interp2(int order, int interp_type, const double *knots,
                      const double *pt, double *N, double *N1, double *N2,
                      double *N3, double *N11, double *N22, double *N33,
                      double *N23, double *N13, double *N12);
int tmrg_forest_eval_interp2(tmrg_forest *f, const double *pt, double *N,
                             double *N1, double *N2, double *N3, double *N11,
                             double *N22, double *N33, double *N23,
                             double *N13, double *N12);
/* TMROctForest::findEnclosing (TMROctForest.h:155-156;
   TMROctForest.cpp:6228-6377) for n nodes (host): each node is an element
   octant whose `info` is the local node index in an element of `order`
   with `knots`; index[i] = the octant of this forest the reference
   returns, or -1 where it returns NULL.  Single rank: mpi_owner is 0. */
int tmrg_forest_find_enclosing(tmrg_forest *f, int order, const double *knots,
                               const tmrg_octant *nodes, int64_t n,
                               int64_t *index);
/* TMROctForest::transformNode (TMROctForest.h:160-161;
   TMROctForest.cpp:3847-4039) on n nodes in place (host); edge_reversed and
   src_face_id (optional, n ints each) as the reference reports them. */
int tmrg_forest_transform_nodes(tmrg_forest *f, tmrg_octant *octs, int64_t n,
                                int edge_dir, int *edge_reversed,
                                int *src_face_id);

/* ---- interpolation (prolongation P: coarse -> fine) ------------------- */
/* TMROctForest::createInterpolation(TMROctForest *coarse, TACSBVecInterp*)
   (TMROctForest.h:115; TMROctForest.cpp:6611-6793).  Rows are the fine
   forest's owned nodes, columns the coarse forest's owned nodes. */
int tmrg_interp_create(tmrg_forest *fine, tmrg_forest *coarse,
                       tmrg_interp **out);
int tmrg_interp_destroy(tmrg_interp *I);
/* Design -> analysis weights (TMROctTACSTopoCreator::computeWeights,
   TMR_TACSTopoCreator.cpp:55-122, per element as createElements calls it,
   :163-183): one row per analysis-forest element, one column per owned
   filter node; the row holds the filter's shape functions at the element
   centre (located with findEnclosing), expanded through the filter's
   dependent nodes and merged by column.  The result is an interpolation
   object: tmrg_interp_mult maps filter design values to element values.
   The reference copies a fixed filter_order^3 slots per element; rows here
   hold every merged entry. */
int tmrg_topo_weights_create(tmrg_forest *filter, tmrg_forest *analysis,
                             tmrg_interp **out);
/* out: {rows, cols, nnz} */
int tmrg_interp_sizes(tmrg_interp *I, int64_t out3[3]);
/* Entries the applies use: P without its numerically-zero weights
   (|w| < 2^-49; for Gauss-Lobatto order 3 the rounding residue of the
   middle knot -cos(pi/2)).  Equal to nnz when P has none. */
int tmrg_interp_apply_nnz(tmrg_interp *I, int64_t *out);
/* Row-sorted CSR of P, host copies. */
int tmrg_interp_get_csr(tmrg_interp *I, int *rowptr, int *cols, double *w);
/* The TACSBVecInterp applies used at TMRConformFilter.cpp:163 and
   TMRMatrixFilter.cpp:315 (TACS is not in the reference tree):
     mult:            y = P x                 (x: cols x nvec, y: rows x nvec)
     mult_transpose:  y = P^T x               (x: rows x nvec, y: cols x nvec)
     mult_weight_transpose: y_j = (P^T x)_j / (P^T 1)_j
   Vectors are node-major (v[node*nvec + k]).  Host pointers; the *_device
   forms take device pointers and run on the interpolation's stream. */
int tmrg_interp_mult(tmrg_interp *I, const double *x, double *y, int nvec);
int tmrg_interp_mult_transpose(tmrg_interp *I, const double *x, double *y,
                               int nvec);
int tmrg_interp_mult_weight_transpose(tmrg_interp *I, const double *x,
                                      double *y, int nvec);
int tmrg_interp_mult_device(tmrg_interp *I, const double *x, double *y,
                            int nvec);
int tmrg_interp_mult_transpose_device(tmrg_interp *I, const double *x,
                                      double *y, int nvec);
int tmrg_interp_mult_weight_transpose_device(tmrg_interp *I, const double *x,
                                             double *y, int nvec);

/* ---- matrix density filter ------------------------------------------ */
/* TMRMatrixFilter::TMRMatrixFilter(r, N, ...) / initialize_matrix
   (TMRMatrixFilter.cpp:30-166), on the nodes of `f` (order 2, trilinear
   elements as TMRMatrixCreator.h:79-80 selects).  The reference takes node
   coordinates from a TMRTopology; here every block is a cube of side
   `block_len`, so an element of level l is a cube of side
   block_len * 2^-l and its consistent mass matrix is exact.  M is
   assembled with dependent nodes condensed onto their independent nodes. */
int tmrg_filter_create(tmrg_forest *f, double block_len, double r, int N,
                       tmrg_filter **out);
/* The same filter on a quadtree forest (the TMRQuadForest constructor,
   TMRMatrixFilter.cpp:39-46, and its 2-D scalings :133-137): bilinear
   elements, every face a square of side `block_len`.  The applies and the
   rest of the tmrg_filter_* calls are shared. */
int tmrg_filter_create_quad(tmrg_qforest *f, double block_len, double r, int N,
                            tmrg_filter **out);
int tmrg_filter_destroy(tmrg_filter *F);
/* out: {n (owned nodes), nnz of M} */
int tmrg_filter_sizes(tmrg_filter *F, int64_t out2[2]);
/* Host copies of M (CSR) and the diagonal scalings Ainv, B, Tinv. */
int tmrg_filter_get_matrix(tmrg_filter *F, int *rowptr, int *cols,
                           double *vals, double *Ainv, double *B,
                           double *Tinv);
/* TMRMatrixFilter::applyFilter / applyTranspose over `vpn` interleaved
   components (setDesignVars/addValues, TMRMatrixFilter.cpp:272-368).
   Host pointers; *_device forms take device pointers. */
int tmrg_filter_apply(tmrg_filter *F, int vpn, const double *in, double *out);
int tmrg_filter_apply_transpose(tmrg_filter *F, int vpn, const double *in,
                                double *out);
int tmrg_filter_apply_device(tmrg_filter *F, int vpn, const double *in,
                             double *out);
int tmrg_filter_apply_transpose_device(tmrg_filter *F, int vpn,
                                       const double *in, double *out);
/* FP32 variant of the filter apply (device pointers, float vectors). */
int tmrg_filter_apply_f32_device(tmrg_filter *F, int vpn, const float *in,
                                 float *out);
int tmrg_filter_apply_transpose_f32_device(tmrg_filter *F, int vpn,
                                           const float *in, float *out);

/* Allocation-free form of tmrg_filter_apply_device (transpose != 0 gives
   the applyTranspose form).  No counterpart in the reference: it exists
   for callers that cannot allocate device memory where they filter (a
   framework whose allocator owns the GPU's memory, or code that must not
   call cudaMalloc/cudaFree because they can synchronise the device).  Its
   work vectors live in a static 16 MiB device array, so nodes x vpn must
   not exceed 1048576 (TMRG_ERR_ARG otherwise).  The first call on a device
   looks the array up (call it before any stream capture); calls that
   overlap on the GPU race on the shared array.  Device pointers; runs on
   the filter's stream; allocates nothing. */
int tmrg_filter_apply_static_device(tmrg_filter *F, int transpose, int vpn,
                                    const double *in, double *out);

/* ---- quadtree forest (the 2-D twin) ------------------------------------ */
/* TMRQuadForest (TMRQuadForest.h:43-161) on the GPU: orders 2 and 3 with
   Gauss-Lobatto or uniform knots (TMRG_ERR_UNSUPPORTED otherwise). */
int tmrg_qforest_create(int order, int interp, void *cuda_stream, tmrg_qforest **out);
int tmrg_qforest_destroy(tmrg_qforest *f);
/* setConnectivity (TMRQuadForest.cpp:318-349): 4 nodes per face, corners
   x fastest; edges numbered from the nodes. */
int tmrg_qforest_set_connectivity(tmrg_qforest *f, int num_nodes, const int *face_conn,
                                  int num_faces);
/* setFullConnectivity (:351-386): edge numbers given (4 per face). */
int tmrg_qforest_set_full_connectivity(tmrg_qforest *f, int num_nodes, int num_edges,
                                       int num_faces, const int *face_conn,
                                       const int *face_edge_conn);
/* getConnectivity (:1162-1201): sizes3 = {faces, edges, nodes}. */
int tmrg_qforest_get_connectivity(tmrg_qforest *f, int *sizes3, int *face_conn,
                                  int *face_edge_conn);
/* setMeshOrder / getMeshOrder / getInterpType / getInterpKnots
   (:948-1067). */
int tmrg_qforest_set_mesh_order(tmrg_qforest *f, int order, int interp);
int tmrg_qforest_get_mesh_order(tmrg_qforest *f, int *order, int *interp, double *knots);
/* createTrees (:1239-1325), refine (:1644-1800; host or device array, NULL
   refines every quadrant by one level), coarsen (:1594-1640), duplicate
   (:1572-1592), balance (:2237-2410), createNodes (:2996-3216). */
int tmrg_qforest_create_trees(tmrg_qforest *f, int level);
/* createRandomTrees (TMRQuadForest.cpp:1327-1407): nrand quadrants per face
   at random levels in [min_level, max_level] and random anchors, sorted and
   made unique on position (finest kept), with the seeded generator
   U(seed, face, 3i + k) in place of libc rand(). */
int tmrg_qforest_create_random_trees(tmrg_qforest *f, int nrand, int min_level, int max_level,
                                     uint64_t seed);
int tmrg_qforest_refine(tmrg_qforest *f, const int *refine, int64_t n, int min_level,
                        int max_level);
int tmrg_qforest_refine_device(tmrg_qforest *f, const int *d_refine, int64_t n, int min_level,
                               int max_level);
int tmrg_qforest_coarsen(tmrg_qforest *f, tmrg_qforest **out);
int tmrg_qforest_duplicate(tmrg_qforest *f, tmrg_qforest **out);
int tmrg_qforest_balance(tmrg_qforest *f, int corner);
int tmrg_qforest_create_nodes(tmrg_qforest *f);
/* getQuadrants (:1011-1018): 6 ints per quadrant {face, x, y, tag, level,
   info}, in element order. */
int tmrg_qforest_num_quadrants(tmrg_qforest *f, int64_t *n);
int tmrg_qforest_get_quadrants(tmrg_qforest *f, int *out);
/* out6 = {local nodes, owned nodes, dependent nodes, ext_pre_offset,
   elements, dependent-weight entries}. */
int tmrg_qforest_sizes(tmrg_qforest *f, int64_t *out6);
/* getNodeConn (:4005-4032): order^2 nodes per element; getDepNodeConn
   (:4034-4063): `order` entries per dependent node. */
int tmrg_qforest_get_node_conn(tmrg_qforest *f, int *conn);
int tmrg_qforest_get_dep_node_conn(tmrg_qforest *f, int *ptr, int *conn, double *w);
/* createInterpolation (:4660-4845): P from `coarse` to `fine`, applied with
   the tmrg_interp_* functions. */
int tmrg_qforest_create_interpolation(tmrg_qforest *fine, tmrg_qforest *coarse,
                                      tmrg_interp **out);
/* Geometry stand-in for the topology: a box per face (origin x, y,
   extent x, y); getPoints (:1035-1043) then gives num_local x 3 points
   (z = 0), zero without boxes. */
int tmrg_qforest_set_face_boxes(tmrg_qforest *f, const double *boxes, int nboxes);
int tmrg_qforest_get_points(tmrg_qforest *f, double *X);

/* ---- iso-surface STL ----------------------------------------------------- */
/* TMR_GenerateSTLTriangles(root, filter, x, x_offset, cutoff, &ntris,
   &tris) (TMR_STLTools.h:44-46, TMR_STLTools.cpp:639-902): the
   triangles of the level set x[x_offset] = cutoff over every element of
   `f` (marching cubes on the (order-1)^3 cells of each element, plus the
   part of every domain-boundary cell face where x >= cutoff), in the
   reference's element / cell / face order.  x holds `vpn` interleaved
   values per independent node (host pointer; the _device form takes a
   device pointer and writes device memory).  *ntris is always set; the
   triangles (9 doubles each: three points x, y, z) are written only when
   `tris` is non-NULL and max_tris >= *ntris.  Node positions are the
   forest's points (tmrg_forest_get_points; zero without block boxes, as
   the reference without a topology).  Crossing points are bit-equal to
   the reference's; each cell's polygon loops are the reference's, split
   into triangles from each loop's lowest edge. */
int tmrg_stl_triangles(tmrg_forest *f, const double *x, int vpn, int x_offset, double cutoff,
                       int64_t *ntris, double *tris, int64_t max_tris);
int tmrg_stl_triangles_device(tmrg_forest *f, const double *x, int vpn, int x_offset,
                              double cutoff, int64_t *ntris, double *tris, int64_t max_tris);
/* TMR_GenerateBinFile (TMR_STLTools.cpp:904-966): int32 triangle count,
   then 9 doubles per triangle, native byte order. */
int tmrg_generate_bin_file(const char *filename, tmrg_forest *f, const double *x, int vpn,
                           int x_offset, double cutoff);
/* TMR_ConvertBinToSTL (TMR_STLTools.cpp:968-993): the ASCII STL of a
   binary triangle file ("solid topology", one facet per triangle with
   its unit normal, "%e" fields). */
int tmrg_convert_bin_to_stl(const char *binfile, const char *stlfile);

/* ---- Helmholtz PDE filter ------------------------------------------- */
/* TMRHelmholtzFilter::TMRHelmholtzFilter(r, nlevels, assemblers, filters)
   (TMRHelmholtzFilter.cpp:29-33, initialize_helmholtz :48-111): the
   Helmholtz operator K = int(r^2 grad N . grad N + N N) and mass M on each
   forest of `filters` (finest first; each nested in the previous one,
   nodes created, block boxes set; order 2 or 3 with the element bases of
   TMRMatrixCreator.h:76-92), the createInterpolation operators between
   consecutive forests, and the multigrid-preconditioned solver.  The
   reference's TACS assemblers have no counterpart: the geometry is the
   forests' block boxes (tmrg_forest_set_block_boxes). */
int tmrg_helmholtz_create(tmrg_forest *const *filters, int nlevels, double r,
                          tmrg_helmholtz **out);
/* The same filter over quadtree forests (TMRHelmholtzFilter.cpp:35-40,
   TMRQuadHelmholtzModel :23-59): bilinear (order 2) or quadratic Bernstein
   (order 3) quadrilaterals, face boxes from tmrg_qforest_set_face_boxes. */
int tmrg_helmholtz_create_quad(tmrg_qforest *const *filters, int nlevels, double r,
                               tmrg_helmholtz **out);
int tmrg_helmholtz_destroy(tmrg_helmholtz *H);
/* out4[4 * k + {0, 1, 2, 3}] = independent nodes, elements, dependent
   nodes and scatter-list entries (element slots expanded through the
   dependent weights) of level k, for k < nlevels. */
int tmrg_helmholtz_sizes(tmrg_helmholtz *H, int *nlevels, int64_t *out4);
/* applyFilter (TMRHelmholtzFilter.cpp:126-196): out = K^-1 M in, and
   applyTranspose (:199-247): out = M K^-1 in, for `vpn` (1..16)
   interleaved components over the finest forest's independent nodes.
   Host pointers; *_device forms take device pointers on the filter's
   stream. */
int tmrg_helmholtz_apply(tmrg_helmholtz *H, int vpn, const double *in, double *out);
int tmrg_helmholtz_apply_transpose(tmrg_helmholtz *H, int vpn, const double *in,
                                   double *out);
int tmrg_helmholtz_apply_device(tmrg_helmholtz *H, int vpn, const double *in,
                                double *out);
int tmrg_helmholtz_apply_transpose_device(tmrg_helmholtz *H, int vpn,
                                          const double *in, double *out);
/* Solver tolerances (the reference's KSM setTolerances(1e-12, 1e-30) with
   at most 300 iterations, TMRHelmholtzFilter.cpp:91-101, are the
   defaults): a component stops when |r| <= max(rtol |b|, atol). */
int tmrg_helmholtz_set_tolerances(tmrg_helmholtz *H, double rtol, double atol,
                                  int max_iters);
/* Multigrid smoother of the preconditioner: Chebyshev polynomials of
   degree `degree_order2` over [lower_order2, upper] x lam on order-2
   levels and `degree_order3` over [lower_order3, upper] x lam on order-3
   levels, lam the Lanczos estimate of the largest eigenvalue of D^-1 K.
   Defaults 5, 6, 0.05, 0.1, 1.1.  The reference's TACS multigrid uses
   symmetric SOR or, optionally, degree-3 Chebyshev over [1/30, 1.1]
   (TMR_RefinementTools.cpp:44-50); the smoother changes only the iteration
   count, not the converged result. */
int tmrg_helmholtz_set_smoother(tmrg_helmholtz *H, int degree_order2, int degree_order3,
                                double lower_order2, double lower_order3, double upper);
/* Iterations and final residual norms (one per component, at most `n`)
   of the last solve. */
int tmrg_helmholtz_last_solve(tmrg_helmholtz *H, int *iters, double *res, int n);
/* out = K in (which = 0) or M in (which = 1) on level `level`, the
   assembled operators with dependent nodes condensed (device pointers,
   nvec interleaved components). */
int tmrg_helmholtz_mult_device(tmrg_helmholtz *H, int level, int which, int nvec,
                               const double *in, double *out);

/* ---- utilities -------------------------------------------------------- */
/* Seeded refinement indicator used by the synthetic workloads:
   out[i] = (U(seed, stream, i) < prob) ? 1 : 0, with U the splitmix64
   uniform shared with the CPU oracle.  Device pointer. */
int tmrg_random_refinement_device(uint64_t seed, uint64_t stream, double prob,
                                  int *d_out, int64_t n, void *cuda_stream);
/* Refinement array of a batch of independent forests held as one forest
   over the disjoint union of their blocks (no reference counterpart):
   forest k owns blocks [d_first_block[k], d_first_block[k+1]) (num_forests
   + 1 entries), d_block_forest maps a block to its forest; d_start
   (num_forests + 1, device) receives each forest's first octant; octant j
   of forest k gets U(seed, k * 1024 + pass, j) < d_prob[k] when
   d_active[k] is nonzero, else 0 -- the draws that forest alone gets from
   tmrg_random_refinement_device(seed, k * 1024 + pass, prob). */
int tmrg_batch_refinement_device(tmrg_forest *f, int num_forests,
                                 const int *d_first_block,
                                 const int *d_block_forest, const double *d_prob,
                                 const int *d_active, uint64_t seed,
                                 uint64_t pass, int64_t *d_start, int *d_out);
/* Refinement array of the large adaptive workload (no reference
   counterpart): per octant the sum of Gaussian bumps
   exp(-|(p - c_k) / sigma|^2 / 2) at its centre p (physical, through the
   block boxes of tmrg_forest_set_block_boxes); +1 where the sum exceeds
   t_refine and the level is below max_level, -1 where it is under
   t_coarsen and the level is above min_level, else 0.  d_centres: device,
   3 doubles per bump; d_out: device, one int per octant. */
int tmrg_bump_indicator_device(tmrg_forest *f, const double *d_centres,
                               int num_bumps, const double *sigma,
                               double t_refine, double t_coarsen,
                               int min_level, int max_level, int *d_out);
/* Number of kernels this library has launched in this process. */
int64_t tmrg_kernel_launch_count(void);
/* Number of device-to-host scalar reads that waited for a stream (sizes
   the host needs before its next allocation). */
int64_t tmrg_host_sync_count(void);
/* Number of device buffers this library has allocated in this process (its
   stream-ordered pool allocations); no counterpart in the reference.  An
   entry point that must not allocate leaves it unchanged. */
int64_t tmrg_device_alloc_count(void);
/* Per-kernel timing for benchmarks (no counterpart in the reference, which
   has no GPU code): between begin and end every launch is bracketed by
   CUDA events on its stream.  end() writes a JSON object
   {"kernel": [launches, total_ms, algorithmic_bytes, flops], ...} into
   json[cap]. */
int tmrg_profile_begin(void);
int tmrg_profile_end(char *json, int64_t cap);
/* Autotuner of the applies' launch shapes, the filter's layout and the
   radix scatter's shape (no counterpart in the reference): the first
   operation of each size class on a device times every candidate shape
   once and the fastest is used from then on.  reset clears the choices and
   any forced candidate (enabled = 0 turns tuning off: fixed default
   shapes); report writes a JSON list of the tuned classes {"device",
   "kind", "key", "choice", "ms"} into json[cap]; force makes every
   operation of `kind` (1 P apply, 2 P^T apply, 3/4 three-component filter
   FP32/FP64, 5 radix scatter) run candidate `choice` (< 0: tuned again),
   for tests that check each candidate. */
int tmrg_tune_reset(int enabled);
int tmrg_tune_report(char *json, int64_t cap);
int tmrg_tune_force(int kind, int choice);
/* FP64 FMA throughput of the current GPU in TFLOP/s (independent FMA
   chains, ~20 ms): the roofline denominator for FP64-pipe-bound kernels.
   No counterpart in the reference. */
int tmrg_measure_fp64_peak(double *tflops);

#ifdef __cplusplus
}
#endif
#endif /* TMRG_H */
