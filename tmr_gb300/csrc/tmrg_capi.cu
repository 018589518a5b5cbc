// The C ABI (include/tmrg.h): status codes in, exceptions never out.
#include <stdio.h>
#include <string.h>

#include <unistd.h>

#include <algorithm>
#include <atomic>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "tmrg_internal.h"
#include "tmrg_helmholtz.h"
#include "tmrg_quad.h"

using namespace tmrg;

// ---------------------------------------------------------------------
// Pinned host memory, pooled.  Borrowed host views of a forest (octants,
// connectivity, dependent CSR) live in page-locked memory so that the
// device writes them at the host link's full rate; a fresh pageable buffer
// is first touched page by page during the copy, an order of magnitude
// slower.  Blocks come in power-of-two sizes from 1 MiB and go back to the
// pool when a forest is destroyed or its views are rebuilt;
// tmrg_host_pool_trim() returns them to the system.
namespace {
struct PinnedBlock {
  void *p = nullptr;
  size_t cap = 0;
};
std::mutex g_pin_mu;
std::multimap<size_t, void *> g_pin_free;

PinnedBlock pin_get(size_t bytes) {
  size_t cap = size_t(1) << 20;
  while (cap < bytes) cap <<= 1;
  {
    std::lock_guard<std::mutex> g(g_pin_mu);
    auto it = g_pin_free.find(cap);
    if (it != g_pin_free.end()) {
      PinnedBlock b{it->second, cap};
      g_pin_free.erase(it);
      return b;
    }
  }
  void *p = nullptr;
  if (cudaMallocHost(&p, cap) != cudaSuccess) {
    cudaGetLastError();
    throw Error(TMRG_ERR_NOMEM,
                "pinned host allocation of " + std::to_string(cap) + " bytes failed");
  }
  return PinnedBlock{p, cap};
}
void pin_put(PinnedBlock &b) {
  if (!b.p) return;
  std::lock_guard<std::mutex> g(g_pin_mu);
  g_pin_free.emplace(b.cap, b.p);
  b = PinnedBlock{};
}
void pin_ensure(PinnedBlock &b, size_t bytes) {
  if (b.p && b.cap >= bytes) return;
  pin_put(b);
  b = pin_get(bytes);
}

// Host views of one forest and the forest generation they were made from.
struct HostMirror {
  uint64_t oct_gen = ~0ULL, conn_gen = ~0ULL, dep_gen = ~0ULL;
  PinnedBlock octs, conn, dptr, dconn, dw;
  void release() {
    pin_put(octs);
    pin_put(conn);
    pin_put(dptr);
    pin_put(dconn);
    pin_put(dw);
    oct_gen = conn_gen = dep_gen = ~0ULL;
  }
};
}  // namespace

struct tmrg_forest {
  Forest f;
  // bumped by every call that changes the octants or nodes; a host view
  // made from an older generation is rebuilt on request
  uint64_t gen = 0;
  HostMirror m;
  ~tmrg_forest() { m.release(); }
};
struct tmrg_interp {
  Interp I;
};
struct tmrg_filter {
  Filter F;
};
struct tmrg_helmholtz {
  Helmholtz H;
};
struct tmrg_qforest {
  QForest f;
};

static thread_local std::string g_last_error;

// Per-kernel event timing (tmrg_profile_begin / tmrg_profile_end).
namespace tmrg {
struct ProfRec {
  const char *name;
  cudaEvent_t a, b;
  long long bytes, flops;
};
static std::mutex g_prof_mu;
static std::vector<ProfRec> g_prof_recs;
static std::vector<cudaEvent_t> g_prof_pool;
static size_t g_prof_next = 0;
cudaEvent_t prof_event() {
  std::lock_guard<std::mutex> lk(g_prof_mu);
  if (g_prof_next == g_prof_pool.size()) {
    cudaEvent_t e;
    TMRG_CUDA(cudaEventCreate(&e));
    g_prof_pool.push_back(e);
  }
  return g_prof_pool[g_prof_next++];
}
void prof_push(const char *name, cudaEvent_t a, cudaEvent_t b, long long bytes,
               long long flops) {
  std::lock_guard<std::mutex> lk(g_prof_mu);
  g_prof_recs.push_back({name, a, b, bytes, flops});
}
}  // namespace tmrg

template <typename Fn>
static int guarded(Fn &&fn) {
  try {
    fn();
    g_last_error.clear();
    return TMRG_OK;
  } catch (const Error &e) {
    g_last_error = e.what();
    return e.status;
  } catch (const std::bad_alloc &) {
    g_last_error = "host allocation failed";
    return TMRG_ERR_NOMEM;
  } catch (const std::exception &e) {
    g_last_error = e.what();
    return TMRG_ERR_INTERNAL;
  }
}
#define ARG(cond, msg)                                     \
  do {                                                     \
    if (!(cond)) throw Error(TMRG_ERR_ARG, std::string(msg)); \
  } while (0)

// Device-usable address of page-locked host memory (cudaMallocHost,
// cudaHostAlloc, registered), or null for any other pointer.
static std::atomic<unsigned> g_warm_sink{0};
static void *host_mapped(void *p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return (a.type == cudaMemoryTypeHost) ? a.devicePointer : nullptr;
}
// One read per OS page of a large page-locked host buffer, on a few host
// threads, before the copy engine moves it.  On guests whose kernel samples
// page accesses in the background (clearing the pages' accessed state),
// page-locked memory last touched by the CPU some seconds earlier was
// measured to copy at 31-91 GB/s instead of the link's 210, and a CPU read
// pass over it restored the full rate; the pass costs a few milliseconds
// against the ~36 ms a 7.7 GB copy takes.  Pageable memory is skipped (the
// driver stages it through the CPU anyway).
static void host_warm(const void *p, size_t bytes) {
  if (!p || bytes < ((size_t)16 << 20) || !host_mapped(const_cast<void *>(p))) return;
  static const size_t pg = [] {
    long v = sysconf(_SC_PAGESIZE);
    return v > 0 ? (size_t)v : (size_t)4096;
  }();
  const volatile unsigned char *c = (const volatile unsigned char *)p;
  const size_t npg = (bytes + pg - 1) / pg;
  const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
  const unsigned nt = bytes >= ((size_t)256 << 20) ? std::min(8u, hw) : 1u;
  std::vector<unsigned> sums(nt, 0u);
  auto run = [&](unsigned t) {
    unsigned acc = 0;
    for (size_t i = t; i < npg; i += nt) acc += c[std::min(i * pg, bytes - 1)];
    sums[t] = acc;
  };
  std::vector<std::thread> th;
  for (unsigned t = 1; t < nt; t++) th.emplace_back(run, t);
  run(0);
  for (auto &x : th) x.join();
  unsigned tot = 0;
  for (unsigned v : sums) tot += v;
  g_warm_sink.fetch_add(tot, std::memory_order_relaxed);
}
static void copy_d2h(void *dst, const void *src, size_t bytes, cudaStream_t s) {
  if (!bytes) return;
  host_warm(dst, bytes);
  TMRG_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, s));
  TMRG_CUDA(cudaStreamSynchronize(s));
}

// ---------------------------------------------------------------------
// 1-D bases of evalInterp (host; TMRInterpolation.h).  Each evaluates in
// the reference's operation order so the values agree bit for bit.
namespace {
// Lagrange values, and first derivatives when Nd is given
// (lagrange_shape_functions :40-52, lagrange_shape_func_derivative :66-93).
void basis_lagrange(int o, double u, const double *kn, double *N, double *Nd) {
  for (int i = 0; i < o; i++) {
    double v = 1.0, dv = 0.0;
    for (int j = 0; j < o; j++) {
      if (j == i) continue;
      double t = 1.0 / (kn[i] - kn[j]);
      v *= (u - kn[j]) * t;
      if (Nd) {
        for (int m = 0; m < o; m++)
          if (m != i && m != j) t *= (u - kn[m]) / (kn[i] - kn[m]);
        dv += t;
      }
    }
    N[i] = v;
    if (Nd) Nd[i] = dv;
  }
}
// Lagrange values, first and second derivatives
// (lagrange_shape_func_second_derivative :107-148); note the value product
// associates as (N (u - k_j)) d_j here.
void basis_lagrange2(int o, double u, const double *kn, double *N, double *Nd,
                     double *Ndd) {
  for (int i = 0; i < o; i++) {
    double v = 1.0, dv = 0.0, ddv = 0.0;
    for (int j = 0; j < o; j++) {
      if (j == i) continue;
      const double rj = 1.0 / (kn[i] - kn[j]);
      double a = rj;
      v = v * (u - kn[j]) * a;
      for (int k = 0; k < o; k++) {
        if (k == i || k == j) continue;
        double b = 1.0 / (kn[i] - kn[k]);
        a *= (u - kn[k]) * b;
        b *= rj;
        for (int m = 0; m < o; m++)
          if (m != i && m != j && m != k) b *= (u - kn[m]) / (kn[i] - kn[m]);
        ddv += b;
      }
      dv += a;
    }
    N[i] = v;
    Nd[i] = dv;
    Ndd[i] = ddv;
  }
}
// Bernstein values of degree o-1 by the de Casteljau-style recurrence
// (bernstein_shape_functions :164-178).
void basis_bernstein(int o, double u, double *N) {
  const double a = 0.5 * (1.0 - u), b = 0.5 * (u + 1.0);
  N[0] = 1.0;
  for (int j = 1; j < o; j++) {
    double carry = 0.0;
    for (int k = 0; k < j; k++) {
      const double t = N[k];
      N[k] = carry + a * t;
      carry = b * t;
    }
    N[j] = carry;
  }
}
// Derivative from the degree o-2 basis (bernstein_shape_func_derivative
// :194-223).
void basis_bernstein_d1(int o, double u, double *N, double *Nd) {
  basis_bernstein(o - 1, u, N);
  const double c = 0.5 * (o - 1);
  for (int j = 0; j < o; j++) {
    double v = 0.0;
    if (j > 0) v += c * N[j - 1];
    if (j < o - 1) v -= c * N[j];
    Nd[j] = v;
  }
  basis_bernstein(o, u, N);
}
// Second derivative from the degree o-3 basis
// (bernstein_shape_func_second_derivative :240-275).
void basis_bernstein_d2(int o, double u, double *N, double *Nd, double *Ndd) {
  basis_bernstein(o - 2, u, N);
  const double c2 = 0.5 * (o - 2), c1 = 0.5 * (o - 1);
  for (int j = 0; j < o - 1; j++) {
    double v = 0.0;
    if (j > 0) v += c2 * N[j - 1];
    if (j < o - 2) v -= c2 * N[j];
    Nd[j] = v;
  }
  for (int j = 0; j < o; j++) {
    double v = 0.0;
    if (j > 0) v += c1 * Nd[j - 1];
    if (j < o - 1) v -= c1 * Nd[j];
    Ndd[j] = v;
  }
  basis_bernstein_d1(o, u, N, Nd);
}
}  // namespace

extern "C" {

const char *tmrg_last_error(void) { return g_last_error.c_str(); }
const char *tmrg_version(void) { return "tmr_gb300 0.1 (sm_103a)"; }
int64_t tmrg_kernel_launch_count(void) { return g_kernel_launches.load(); }
int64_t tmrg_host_sync_count(void) { return g_host_syncs.load(); }
int64_t tmrg_device_alloc_count(void) { return g_device_allocs.load(); }

// FP64 FMA throughput of the current device: 8 independent FMA chains per
// thread over a grid of 8 blocks per SM; the denominator of the roofline of
// FP64-pipe-bound kernels (no measured FP64 figure exists).
__global__ void k_fp64_peak(double *out, int iters, double a, double b) {
  double x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4,
         x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
  for (int i = 0; i < iters; i++) {
    x0 = __fma_rn(x0, a, b);
    x1 = __fma_rn(x1, a, b);
    x2 = __fma_rn(x2, a, b);
    x3 = __fma_rn(x3, a, b);
    x4 = __fma_rn(x4, a, b);
    x5 = __fma_rn(x5, a, b);
    x6 = __fma_rn(x6, a, b);
    x7 = __fma_rn(x7, a, b);
  }
  out[(long long)blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

int tmrg_measure_fp64_peak(double *tflops) {
  return guarded([&] {
    ARG(tflops, "NULL argument");
    int dev = 0, sms = 0;
    TMRG_CUDA(cudaGetDevice(&dev));
    TMRG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const int blocks = sms * 8, threads = 256, iters = 4096;
    DBuf<double> out((size_t)blocks * threads, 0);
    cudaEvent_t e0, e1;
    TMRG_CUDA(cudaEventCreate(&e0));
    TMRG_CUDA(cudaEventCreate(&e1));
    launch(k_fp64_peak, blocks, threads, 0, 0, out.p, 16, 0.999, 0.001);
    TMRG_CUDA(cudaEventRecord(e0, 0));
    launch(k_fp64_peak, blocks, threads, 0, 0, out.p, iters, 0.999, 0.001);
    TMRG_CUDA(cudaEventRecord(e1, 0));
    TMRG_CUDA(cudaEventSynchronize(e1));
    float ms = 0;
    TMRG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    *tflops = 2.0 * 8 * iters * (double)blocks * threads / (ms * 1e-3) / 1e12;
  });
}

int tmrg_profile_begin(void) {
  return guarded([&] {
    std::lock_guard<std::mutex> lk(g_prof_mu);
    g_prof_recs.clear();
    g_prof_next = 0;
    g_profile_on = true;
  });
}
int tmrg_profile_end(char *json, int64_t cap) {
  return guarded([&] {
    g_profile_on = false;
    TMRG_CUDA(cudaDeviceSynchronize());
    std::lock_guard<std::mutex> lk(g_prof_mu);
    struct Agg {
      long long n = 0, bytes = 0, flops = 0;
      double ms = 0;
    };
    std::map<std::string, Agg> agg;
    for (auto &r : g_prof_recs) {
      float ms = 0;
      TMRG_CUDA(cudaEventElapsedTime(&ms, r.a, r.b));
      Agg &a = agg[r.name];
      a.n++;
      a.ms += ms;
      a.bytes += r.bytes;
      a.flops += r.flops;
    }
    std::string s = "{";
    bool first = true;
    for (auto &kv : agg) {
      char buf[512];
      snprintf(buf, sizeof buf, "%s\"%s\": [%lld, %.6f, %lld, %lld]", first ? "" : ", ",
               kv.first.c_str(), kv.second.n, kv.second.ms, kv.second.bytes,
               kv.second.flops);
      s += buf;
      first = false;
    }
    s += "}";
    g_prof_recs.clear();
    g_prof_next = 0;
    if (json && cap > 0) {
      snprintf(json, (size_t)cap, "%s", s.c_str());
      if ((int64_t)s.size() >= cap) throw Error(TMRG_ERR_ARG, "profile buffer too small");
    }
  });
}

// Keep freed stream-ordered allocations in the device's default pool
// instead of returning them at every synchronisation: the pipeline
// allocates and frees GB-sized sort buffers at every step.
static void keep_pool() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return;
  static thread_local int done_dev = -1;
  if (done_dev == dev) return;
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
    uint64_t thr = UINT64_MAX;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
  }
  done_dev = dev;
}

int tmrg_forest_create(int order, int interp_type, void *stream,
                       tmrg_forest **out) {
  return guarded([&] {
    ARG(out, "out is NULL");
    keep_pool();
    ARG(interp_type >= 0 && interp_type <= 2, "bad interpolation type");
    auto *h = new tmrg_forest;
    h->f.s = (cudaStream_t)stream;
    h->f.set_order(order, interp_type);
    *out = h;
  });
}
int tmrg_forest_destroy(tmrg_forest *f) {
  return guarded([&] {
    if (!f) return;
    cudaStreamSynchronize(f->f.s);
    delete f;
  });
}
int tmrg_forest_set_connectivity(tmrg_forest *f, int num_nodes,
                                 const int *block_conn, int num_blocks) {
  return guarded([&] {
    ARG(f && block_conn, "NULL argument");
    f->gen++;
    // validate and build first: a rejected connectivity leaves the forest
    // as it was
    auto c = build_conn(num_nodes, block_conn, num_blocks, f->f.s);
    f->f.free_nodes();
    f->f.have_octs = false;
    f->f.n = 0;
    f->f.conn = c;
  });
}
int tmrg_forest_set_full_connectivity(tmrg_forest *f, int num_nodes, int num_edges,
                                      int num_faces, int num_blocks, const int *block_conn,
                                      const int *block_edge_conn,
                                      const int *block_face_conn) {
  return guarded([&] {
    ARG(f && block_conn && block_edge_conn && block_face_conn, "NULL argument");
    f->gen++;
    auto c = build_conn(num_nodes, block_conn, num_blocks, f->f.s, num_edges,
                        block_edge_conn, num_faces, block_face_conn);
    f->f.free_nodes();
    f->f.have_octs = false;
    f->f.n = 0;
    f->f.conn = c;
  });
}
int tmrg_forest_get_connectivity(tmrg_forest *f, int *nblocks, int *nfaces, int *nedges,
                                 int *nnodes, const int **block_conn,
                                 const int **block_face_conn, const int **block_edge_conn,
                                 const int **block_face_ids) {
  return guarded([&] {
    ARG(f, "NULL forest");
    const Conn *c = f->f.conn.get();
    if (nblocks) *nblocks = c ? c->nb : 0;
    if (nfaces) *nfaces = c ? c->num_faces : 0;
    if (nedges) *nedges = c ? c->num_edges : 0;
    if (nnodes) *nnodes = c ? c->num_nodes : 0;
    if (block_conn) *block_conn = c ? c->block_conn.data() : nullptr;
    if (block_face_conn) *block_face_conn = c ? c->block_face.data() : nullptr;
    if (block_edge_conn) *block_edge_conn = c ? c->block_edge.data() : nullptr;
    if (block_face_ids) *block_face_ids = c ? c->face_ids.data() : nullptr;
  });
}
int tmrg_forest_get_inverse_connectivity(tmrg_forest *f, const int **node_block_conn,
                                         const int **node_block_ptr,
                                         const int **edge_block_conn,
                                         const int **edge_block_ptr,
                                         const int **face_block_conn,
                                         const int **face_block_ptr) {
  return guarded([&] {
    ARG(f, "NULL forest");
    const Conn *c = f->f.conn.get();
    if (node_block_conn) *node_block_conn = c ? c->node_ent.data() : nullptr;
    if (node_block_ptr) *node_block_ptr = c ? c->node_ptr.data() : nullptr;
    if (edge_block_conn) *edge_block_conn = c ? c->edge_ent.data() : nullptr;
    if (edge_block_ptr) *edge_block_ptr = c ? c->edge_ptr.data() : nullptr;
    if (face_block_conn) *face_block_conn = c ? c->face_ent.data() : nullptr;
    if (face_block_ptr) *face_block_ptr = c ? c->face_ptr.data() : nullptr;
  });
}
int tmrg_forest_create_random_trees(tmrg_forest *f, int nrand, int min_level,
                                    int max_level, uint64_t seed) {
  return guarded([&] {
    ARG(f, "NULL forest");
    f->gen++;
    forest_create_random_trees(f->f, nrand, min_level, max_level, seed);
  });
}
int tmrg_forest_get_local_node_number(tmrg_forest *f, int node, int *local) {
  return guarded([&] {
    ARG(f && local, "NULL argument");
    const Forest &F = f->f;
    if (!F.have_nodes) throw Error(TMRG_ERR_STATE, "getLocalNodeNumber: no nodes");
    // node numbers are -num_dep .. -1, 0 .. num_owned-1, sorted
    long long li = (long long)node + F.num_dep;
    *local = (li >= 0 && li < F.num_local) ? (int)li : -1;
  });
}
int tmrg_forest_find_enclosing(tmrg_forest *f, int order, const double *knots,
                               const tmrg_octant *nodes, int64_t n, int64_t *index) {
  return guarded([&] {
    ARG(f && knots && (n == 0 || (nodes && index)), "NULL argument");
    ARG(n >= 0, "findEnclosing: n < 0");
    if (!n) return;
    Forest &F = f->f;
    DBuf<tmrg_octant> d(n, F.s);
    DBuf<long long> r(n, F.s);
    TMRG_CUDA(cudaMemcpyAsync(d.p, nodes, sizeof(tmrg_octant) * n, cudaMemcpyHostToDevice, F.s));
    forest_find_enclosing(F, order, knots, d.p, n, r.p);
    static_assert(sizeof(long long) == sizeof(int64_t), "int64");
    copy_d2h(index, r.p, sizeof(int64_t) * n, F.s);
  });
}
int tmrg_forest_transform_nodes(tmrg_forest *f, tmrg_octant *octs, int64_t n, int edge_dir,
                                int *edge_reversed, int *src_face_id) {
  return guarded([&] {
    ARG(f && (n == 0 || octs), "NULL argument");
    ARG(n >= 0 && edge_dir >= -1 && edge_dir <= 2, "transformNode: bad argument");
    if (!n) return;
    Forest &F = f->f;
    DBuf<tmrg_octant> d(n, F.s);
    DBuf<int> r(edge_reversed ? n : 0, F.s), id(src_face_id ? n : 0, F.s);
    TMRG_CUDA(cudaMemcpyAsync(d.p, octs, sizeof(tmrg_octant) * n, cudaMemcpyHostToDevice, F.s));
    forest_transform_nodes(F, d.p, n, edge_dir, edge_reversed ? r.p : nullptr,
                           src_face_id ? id.p : nullptr);
    if (edge_reversed)
      TMRG_CUDA(cudaMemcpyAsync(edge_reversed, r.p, sizeof(int) * n, cudaMemcpyDeviceToHost, F.s));
    if (src_face_id)
      TMRG_CUDA(cudaMemcpyAsync(src_face_id, id.p, sizeof(int) * n, cudaMemcpyDeviceToHost, F.s));
    copy_d2h(octs, d.p, sizeof(tmrg_octant) * n, F.s);
  });
}
int tmrg_forest_set_block_boxes(tmrg_forest *f, const double *boxes, int num_blocks) {
  return guarded([&] {
    ARG(f, "NULL forest");
    Conn *c = f->f.conn.get();
    if (!c) throw Error(TMRG_ERR_STATE, "setBlockBoxes: no connectivity");
    if (!boxes) {
      c->boxes.clear();
      c->d_boxes.release();
      return;
    }
    ARG(num_blocks == c->nb, "setBlockBoxes: one box per block");
    c->boxes.assign(boxes, boxes + 6LL * num_blocks);
    c->d_boxes.alloc(6LL * num_blocks, f->f.s);
    TMRG_CUDA(cudaMemcpyAsync(c->d_boxes.p, c->boxes.data(), sizeof(double) * 6 * num_blocks,
                              cudaMemcpyHostToDevice, f->f.s));
    TMRG_CUDA(cudaStreamSynchronize(f->f.s));
  });
}
int tmrg_forest_get_points(tmrg_forest *f, double *X, int64_t n) {
  return guarded([&] {
    ARG(f && X, "NULL argument");
    Forest &F = f->f;
    if (!F.have_nodes) throw Error(TMRG_ERR_STATE, "getPoints: no nodes");
    ARG(n == F.num_local, "getPoints: buffer length != number of local nodes");
    DBuf<double> d(3 * (size_t)n + 1, F.s);
    forest_get_points(F, F.conn->boxes.empty() ? nullptr : (const double *)F.conn->d_boxes.p,
                      d.p);
    copy_d2h(X, d.p, sizeof(double) * 3 * (size_t)n, F.s);
  });
}

int tmrg_forest_set_mesh_order(tmrg_forest *f, int order, int interp_type) {
  return guarded([&] {
    ARG(f, "NULL forest");
    f->gen++;
    ARG(interp_type >= 0 && interp_type <= 2, "bad interpolation type");
    f->f.set_order(order, interp_type);
  });
}
int tmrg_forest_get_mesh_order(tmrg_forest *f, int *order, int *interp_type) {
  return guarded([&] {
    ARG(f, "NULL forest");
    if (order) *order = f->f.order;
    if (interp_type) *interp_type = f->f.interp;
  });
}
int tmrg_forest_get_interp_knots(tmrg_forest *f, double *knots) {
  return guarded([&] {
    ARG(f && knots, "NULL argument");
    memcpy(knots, f->f.knots, sizeof(double) * f->f.order);
  });
}
int tmrg_forest_create_trees(tmrg_forest *f, int level) {
  return guarded([&] {
    ARG(f, "NULL forest");
    f->gen++;
    forest_create_trees(f->f, level);
  });
}
int tmrg_forest_refine(tmrg_forest *f, const int *refinement, int64_t n,
                       int min_level, int max_level) {
  return guarded([&] {
    ARG(f, "NULL forest");
    f->gen++;
    if (!refinement) {
      forest_refine(f->f, nullptr, 0, min_level, max_level);
      return;
    }
    if (!f->f.have_octs) throw Error(TMRG_ERR_STATE, "refine: no octants");
    ARG(n == f->f.n, "refine: refinement array length != number of octants");
    DBuf<int> d(n, f->f.s);
    if (n)
      TMRG_CUDA(cudaMemcpyAsync(d.p, refinement, n * sizeof(int),
                                cudaMemcpyHostToDevice, f->f.s));
    forest_refine(f->f, d.p, n, min_level, max_level);
  });
}
int tmrg_forest_refine_device(tmrg_forest *f, const int *d_refinement,
                              int64_t n, int min_level, int max_level) {
  return guarded([&] {
    ARG(f, "NULL forest");
    f->gen++;
    forest_refine(f->f, d_refinement, d_refinement ? n : 0, min_level,
                  max_level);
  });
}
int tmrg_forest_coarsen(tmrg_forest *f, tmrg_forest **out) {
  return guarded([&] {
    ARG(f && out, "NULL argument");
    auto *h = new tmrg_forest;
    h->f.s = f->f.s;
    try {
      forest_coarsen(f->f, h->f);
    } catch (...) {
      delete h;
      throw;
    }
    *out = h;
  });
}
int tmrg_forest_duplicate(tmrg_forest *f, tmrg_forest **out) {
  return guarded([&] {
    ARG(f && out, "NULL argument");
    auto *h = new tmrg_forest;
    h->f.s = f->f.s;
    try {
      forest_duplicate(f->f, h->f);
    } catch (...) {
      delete h;
      throw;
    }
    *out = h;
  });
}
int tmrg_forest_balance(tmrg_forest *f, int balance_corner) {
  return guarded([&] {
    ARG(f, "NULL forest");
    f->gen++;
    forest_balance(f->f, balance_corner ? 1 : 0);
  });
}
int tmrg_forest_repartition(tmrg_forest *f, int) {
  return guarded([&] { ARG(f, "NULL forest"); });
}
int tmrg_forest_create_nodes(tmrg_forest *f) {
  return guarded([&] {
    ARG(f, "NULL forest");
    f->gen++;
    forest_create_nodes(f->f);
  });
}
int tmrg_forest_num_octants(tmrg_forest *f, int64_t *n) {
  return guarded([&] {
    ARG(f && n, "NULL argument");
    *n = f->f.have_octs ? f->f.n : 0;
  });
}

__global__ void k_pack_octants(long long n, const int *b, const int *x,
                               const int *y, const int *z, const int16_t *l,
                               const int16_t *info, int *out) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int *o = out + 7 * i;
  o[0] = b[i];
  o[1] = x[i];
  o[2] = y[i];
  o[3] = z[i];
  o[4] = (int)i;
  o[5] = l[i];
  o[6] = info[i];
}

int tmrg_forest_get_octants(tmrg_forest *f, int *out7, int64_t n) {
  return guarded([&] {
    ARG(f && out7, "NULL argument");
    Forest &F = f->f;
    if (!F.have_octs) throw Error(TMRG_ERR_STATE, "getOctants: no octants");
    ARG(n == F.n, "getOctants: buffer length != number of octants");
    DBuf<int> d(7 * (size_t)n, F.s);
    launch(k_pack_octants, blocks_for(n, 256), 256, 0, F.s, (long long)n,
           (const int *)F.block.p, (const int *)F.x.p, (const int *)F.y.p,
           (const int *)F.z.p, (const int16_t *)F.level.p,
           (const int16_t *)F.info.p, d.p);
    copy_d2h(out7, d.p, 7 * sizeof(int) * (size_t)n, F.s);
  });
}
int tmrg_forest_octants_device(tmrg_forest *f, const int **block, const int **x,
                               const int **y, const int **z,
                               const int16_t **level, const int16_t **info) {
  return guarded([&] {
    ARG(f, "NULL forest");
    Forest &F = f->f;
    if (block) *block = F.block.p;
    if (x) *x = F.x.p;
    if (y) *y = F.y.p;
    if (z) *z = F.z.p;
    if (level) *level = F.level.p;
    if (info) *info = F.info.p;
  });
}
__global__ void k_pack_octants24(long long n, const int *__restrict__ b,
                                 const int *__restrict__ x, const int *__restrict__ y,
                                 const int *__restrict__ z, const int16_t *__restrict__ l,
                                 const int16_t *__restrict__ info, tmrg_octant *out) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  tmrg_octant o;
  o.block = b[i];
  o.x = x[i];
  o.y = y[i];
  o.z = z[i];
  o.tag = (int32_t)i;
  o.level = l[i];
  o.info = info[i];
  out[i] = o;
}
static_assert(sizeof(tmrg_octant) == 24, "TMROctant layout");

int tmrg_forest_octants_host(tmrg_forest *f, const tmrg_octant **octs, int64_t *n) {
  return guarded([&] {
    ARG(f && octs, "NULL argument");
    Forest &F = f->f;
    if (!F.have_octs) throw Error(TMRG_ERR_STATE, "getOctants: no octants");
    if (f->m.oct_gen != f->gen) {
      f->m.oct_gen = ~0ULL;
      pin_ensure(f->m.octs, sizeof(tmrg_octant) * (size_t)F.n);
      // packed in HBM, then one bulk copy (24-byte stores straight over the
      // host link run at a fraction of the copy rate)
      DBuf<tmrg_octant> d(F.n, F.s);
      launch(k_pack_octants24, blocks_for(F.n, 256), 256, 0, F.s, F.n,
             (const int *)F.block.p, (const int *)F.x.p, (const int *)F.y.p,
             (const int *)F.z.p, (const int16_t *)F.level.p, (const int16_t *)F.info.p,
             d.p);
      host_warm(f->m.octs.p, sizeof(tmrg_octant) * (size_t)F.n);
      if (F.n)
        TMRG_CUDA(cudaMemcpyAsync(f->m.octs.p, d.p, sizeof(tmrg_octant) * (size_t)F.n,
                                  cudaMemcpyDeviceToHost, F.s));
      TMRG_CUDA(cudaStreamSynchronize(F.s));
      f->m.oct_gen = f->gen;
    }
    *octs = (const tmrg_octant *)f->m.octs.p;
    if (n) *n = F.n;
  });
}
static void conn_mirror(tmrg_forest *f) {
  Forest &F = f->f;
  if (!F.have_nodes) throw Error(TMRG_ERR_STATE, "no nodes: call createNodes first");
  if (f->m.conn_gen == f->gen) return;
  f->m.conn_gen = ~0ULL;
  const size_t nconn = (size_t)F.n * F.order * F.order * F.order;
  pin_ensure(f->m.conn, sizeof(int) * nconn);
  host_warm(f->m.conn.p, sizeof(int) * nconn);
  if (nconn)
    TMRG_CUDA(cudaMemcpyAsync(f->m.conn.p, F.econn.p, sizeof(int) * nconn,
                              cudaMemcpyDeviceToHost, F.s));
  TMRG_CUDA(cudaStreamSynchronize(F.s));
  f->m.conn_gen = f->gen;
}
static void dep_mirror(tmrg_forest *f) {
  Forest &F = f->f;
  if (!F.have_nodes) throw Error(TMRG_ERR_STATE, "no nodes: call createNodes first");
  if (f->m.dep_gen == f->gen) return;
  f->m.dep_gen = ~0ULL;
  pin_ensure(f->m.dptr, sizeof(int) * ((size_t)F.num_dep + 1));
  pin_ensure(f->m.dconn, sizeof(int) * (size_t)F.dep_nnz + 1);
  pin_ensure(f->m.dw, sizeof(double) * (size_t)F.dep_nnz + 1);
  TMRG_CUDA(cudaMemcpyAsync(f->m.dptr.p, F.dep_ptr.p, sizeof(int) * ((size_t)F.num_dep + 1),
                            cudaMemcpyDeviceToHost, F.s));
  if (F.dep_nnz) {
    host_warm(f->m.dconn.p, sizeof(int) * (size_t)F.dep_nnz);
    host_warm(f->m.dw.p, sizeof(double) * (size_t)F.dep_nnz);
    TMRG_CUDA(cudaMemcpyAsync(f->m.dconn.p, F.dep_conn.p, sizeof(int) * (size_t)F.dep_nnz,
                              cudaMemcpyDeviceToHost, F.s));
    TMRG_CUDA(cudaMemcpyAsync(f->m.dw.p, F.dep_w.p, sizeof(double) * (size_t)F.dep_nnz,
                              cudaMemcpyDeviceToHost, F.s));
  }
  TMRG_CUDA(cudaStreamSynchronize(F.s));
  f->m.dep_gen = f->gen;
}
int tmrg_forest_node_conn_host(tmrg_forest *f, const int **conn, int64_t *num_elements) {
  return guarded([&] {
    ARG(f && conn, "NULL argument");
    conn_mirror(f);
    *conn = (const int *)f->m.conn.p;
    if (num_elements) *num_elements = f->f.n;
  });
}
int tmrg_forest_dep_node_conn_host(tmrg_forest *f, const int **ptr, const int **conn,
                                   const double **weights, int64_t *num_dep) {
  return guarded([&] {
    ARG(f, "NULL forest");
    dep_mirror(f);
    if (ptr) *ptr = (const int *)f->m.dptr.p;
    if (conn) *conn = (const int *)f->m.dconn.p;
    if (weights) *weights = (const double *)f->m.dw.p;
    if (num_dep) *num_dep = f->f.num_dep;
  });
}
// evalInterp (TMROctForest.cpp:1510-1631): tensor-product shape functions
// at a parametric point, ii fastest, with optional first derivatives.
int tmrg_eval_interp(int order, int interp_type, const double *knots, const double *pt,
                     double *N, double *N1, double *N2, double *N3) {
  return guarded([&] {
    ARG(pt && N && order >= 2 && order <= TMRG_MAX_ORDER, "bad argument");
    ARG(interp_type == TMRG_BERNSTEIN_POINTS || knots, "knots are NULL");
    const bool d1 = N1 && N2 && N3;
    double B[3][TMRG_MAX_ORDER], D[3][TMRG_MAX_ORDER];
    for (int a = 0; a < 3; a++) {
      if (interp_type == TMRG_BERNSTEIN_POINTS) {
        if (d1)
          basis_bernstein_d1(order, pt[a], B[a], D[a]);
        else
          basis_bernstein(order, pt[a], B[a]);
      } else {
        basis_lagrange(order, pt[a], knots, B[a], d1 ? D[a] : nullptr);
      }
    }
    int p = 0;
    for (int k = 0; k < order; k++)
      for (int j = 0; j < order; j++)
        for (int i = 0; i < order; i++, p++) {
          N[p] = B[0][i] * B[1][j] * B[2][k];
          if (d1) {
            N1[p] = D[0][i] * B[1][j] * B[2][k];
            N2[p] = B[0][i] * D[1][j] * B[2][k];
            N3[p] = B[0][i] * B[1][j] * D[2][k];
          }
        }
  });
}
// The second-derivative form (TMROctForest.cpp:1572-1631).  As in the
// reference, N33 receives the mixed (1,2) derivative after the (3,3) one
// and N12 is not written (TMROctForest.cpp:1614-1615).
int tmrg_eval_interp2(int order, int interp_type, const double *knots, const double *pt,
                      double *N, double *N1, double *N2, double *N3, double *N11,
                      double *N22, double *N33, double *N23, double *N13, double *N12) {
  return guarded([&] {
    ARG(pt && N && N1 && N2 && N3 && N11 && N22 && N33 && N23 && N13 && order >= 2 &&
            order <= TMRG_MAX_ORDER,
        "bad argument");
    ARG(interp_type == TMRG_BERNSTEIN_POINTS || knots, "knots are NULL");
    (void)N12;
    double B[3][TMRG_MAX_ORDER], D[3][TMRG_MAX_ORDER], DD[3][TMRG_MAX_ORDER];
    for (int a = 0; a < 3; a++) {
      if (interp_type == TMRG_BERNSTEIN_POINTS)
        basis_bernstein_d2(order, pt[a], B[a], D[a], DD[a]);
      else
        basis_lagrange2(order, pt[a], knots, B[a], D[a], DD[a]);
    }
    int p = 0;
    for (int k = 0; k < order; k++)
      for (int j = 0; j < order; j++)
        for (int i = 0; i < order; i++, p++) {
          const double u = B[0][i], v = B[1][j], w = B[2][k];
          const double du = D[0][i], dv = D[1][j], dw = D[2][k];
          N[p] = u * v * w;
          N1[p] = du * v * w;
          N2[p] = u * dv * w;
          N3[p] = u * v * dw;
          N11[p] = DD[0][i] * v * w;
          N22[p] = u * DD[1][j] * w;
          N33[p] = u * v * DD[2][k];
          N23[p] = u * dv * dw;
          N13[p] = du * v * dw;
          N33[p] = du * dv * w;
        }
  });
}
int tmrg_forest_eval_interp(tmrg_forest *f, const double *pt, double *N, double *N1,
                            double *N2, double *N3) {
  if (!f) {
    g_last_error = "NULL forest";
    return TMRG_ERR_ARG;
  }
  return tmrg_eval_interp(f->f.order, f->f.interp, f->f.knots, pt, N, N1, N2, N3);
}
int tmrg_forest_eval_interp2(tmrg_forest *f, const double *pt, double *N, double *N1,
                             double *N2, double *N3, double *N11, double *N22, double *N33,
                             double *N23, double *N13, double *N12) {
  if (!f) {
    g_last_error = "NULL forest";
    return TMRG_ERR_ARG;
  }
  return tmrg_eval_interp2(f->f.order, f->f.interp, f->f.knots, pt, N, N1, N2, N3, N11, N22,
                           N33, N23, N13, N12);
}

int tmrg_host_pool_trim(void) {
  return guarded([&] {
    std::lock_guard<std::mutex> g(g_pin_mu);
    for (auto &kv : g_pin_free) cudaFreeHost(kv.second);
    g_pin_free.clear();
  });
}

int tmrg_forest_node_sizes(tmrg_forest *f, int64_t out6[6]) {
  return guarded([&] {
    ARG(f && out6, "NULL argument");
    Forest &F = f->f;
    out6[0] = F.num_local;
    out6[1] = F.num_owned;
    out6[2] = F.num_dep;
    out6[3] = F.ext_pre;
    out6[4] = F.have_octs ? F.n : 0;
    out6[5] = F.dep_nnz;
  });
}
int tmrg_forest_get_node_conn(tmrg_forest *f, int *conn, int64_t n) {
  return guarded([&] {
    ARG(f && conn, "NULL argument");
    Forest &F = f->f;
    if (!F.have_nodes) throw Error(TMRG_ERR_STATE, "getNodeConn: no nodes");
    long long m = F.n * (long long)F.order * F.order * F.order;
    ARG(n == m, "getNodeConn: buffer length mismatch");
    copy_d2h(conn, F.econn.p, sizeof(int) * (size_t)m, F.s);
  });
}
int tmrg_forest_get_node_numbers(tmrg_forest *f, int *out, int64_t n) {
  return guarded([&] {
    ARG(f && out, "NULL argument");
    Forest &F = f->f;
    if (!F.have_nodes) throw Error(TMRG_ERR_STATE, "getNodeNumbers: no nodes");
    ARG(n == F.num_local, "getNodeNumbers: buffer length mismatch");
    // sorted: -num_dep .. -1, then 0 .. num_owned-1
    for (long long i = 0; i < F.num_dep; i++) out[i] = (int)(i - F.num_dep);
    for (long long i = 0; i < F.num_owned; i++) out[F.num_dep + i] = (int)i;
  });
}
int tmrg_forest_get_dep_node_conn(tmrg_forest *f, int *ptr, int *conn,
                                  double *weights) {
  return guarded([&] {
    ARG(f, "NULL forest");
    Forest &F = f->f;
    if (!F.have_nodes) throw Error(TMRG_ERR_STATE, "getDepNodeConn: no nodes");
    if (ptr) copy_d2h(ptr, F.dep_ptr.p, sizeof(int) * (F.num_dep + 1), F.s);
    if (conn) copy_d2h(conn, F.dep_conn.p, sizeof(int) * F.dep_nnz, F.s);
    if (weights) copy_d2h(weights, F.dep_w.p, sizeof(double) * F.dep_nnz, F.s);
  });
}
int tmrg_forest_node_conn_device(tmrg_forest *f, const int **conn) {
  return guarded([&] {
    ARG(f && conn, "NULL argument");
    *conn = f->f.econn.p;
  });
}
int tmrg_forest_dep_node_conn_device(tmrg_forest *f, const int **ptr,
                                     const int **conn, const double **w) {
  return guarded([&] {
    ARG(f, "NULL forest");
    if (ptr) *ptr = f->f.dep_ptr.p;
    if (conn) *conn = f->f.dep_conn.p;
    if (w) *w = f->f.dep_w.p;
  });
}

// ---- interpolation ----------------------------------------------------
int tmrg_interp_create(tmrg_forest *fine, tmrg_forest *coarse,
                       tmrg_interp **out) {
  return guarded([&] {
    ARG(fine && coarse && out, "NULL argument");
    auto *h = new tmrg_interp;
    try {
      interp_create(fine->f, coarse->f, h->I);
    } catch (...) {
      delete h;
      throw;
    }
    *out = h;
  });
}
int tmrg_topo_weights_create(tmrg_forest *filter, tmrg_forest *analysis, tmrg_interp **out) {
  return guarded([&] {
    ARG(filter && analysis && out, "NULL argument");
    auto *h = new tmrg_interp;
    try {
      topo_weights_create(filter->f, analysis->f, h->I);
    } catch (...) {
      delete h;
      throw;
    }
    *out = h;
  });
}
int tmrg_interp_destroy(tmrg_interp *I) {
  return guarded([&] {
    if (!I) return;
    cudaStreamSynchronize(I->I.s);
    delete I;
  });
}
int tmrg_interp_sizes(tmrg_interp *I, int64_t out3[3]) {
  return guarded([&] {
    ARG(I && out3, "NULL argument");
    out3[0] = I->I.rows;
    out3[1] = I->I.cols;
    out3[2] = I->I.nnz;
  });
}
int tmrg_interp_apply_nnz(tmrg_interp *I, int64_t *out) {
  return guarded([&] {
    ARG(I && out, "NULL argument");
    *out = I->I.nnz_nz;
  });
}
int tmrg_interp_get_csr(tmrg_interp *I, int *rowptr, int *cols, double *w) {
  return guarded([&] {
    ARG(I, "NULL interp");
    Interp &P = I->I;
    if (rowptr) copy_d2h(rowptr, P.rowptr.p, sizeof(int) * (P.rows + 1), P.s);
    if (cols) copy_d2h(cols, P.colidx.p, sizeof(int) * P.nnz, P.s);
    if (w) copy_d2h(w, P.vals.p, sizeof(double) * P.nnz, P.s);
  });
}
static int interp_host(tmrg_interp *I, int which, const double *x, double *y,
                       int nvec) {
  return guarded([&] {
    ARG(I && x && y && nvec > 0, "bad argument");
    Interp &P = I->I;
    long long nin = (which == 0 ? P.cols : P.rows) * nvec;
    long long nout = (which == 0 ? P.rows : P.cols) * nvec;
    DBuf<double> dx(nin, P.s);
    double *ym = (double *)host_mapped(y);
    host_warm(x, sizeof(double) * nin);
    host_warm(y, sizeof(double) * nout);
    if (which != 0) {
      // restriction: copy the input in pieces overlapped with the rows
      // they complete
      DBuf<double> dy;
      if (!ym) dy.alloc(nout, P.s);
      if (interp_apply_transpose_staged(P, which, x, dx.p, ym ? ym : dy.p, nvec)) {
        if (!ym) copy_d2h(y, dy.p, sizeof(double) * nout, P.s);
        return;
      }
    }
    // prolongation: rows computed in pieces, each piece copied back while
    // the next one computes
    if (which == 0 && interp_apply_forward_staged(P, x, dx.p, y, nvec)) return;
    TMRG_CUDA(cudaMemcpyAsync(dx.p, x, sizeof(double) * nin,
                              cudaMemcpyHostToDevice, P.s));
    if (ym) {
      // page-locked output: the apply writes it over the host link while
      // it computes, instead of a copy after it
      interp_apply(P, which, dx.p, ym, nvec);
      TMRG_CUDA(cudaStreamSynchronize(P.s));
      interp_check_apply(P);
      return;
    }
    DBuf<double> dy(nout, P.s);
    interp_apply(P, which, dx.p, dy.p, nvec);
    copy_d2h(y, dy.p, sizeof(double) * nout, P.s);
    interp_check_apply(P);
  });
}
static int interp_dev(tmrg_interp *I, int which, const double *x, double *y,
                      int nvec) {
  return guarded([&] {
    ARG(I && x && y && nvec > 0, "bad argument");
    interp_apply(I->I, which, x, y, nvec);
  });
}
int tmrg_interp_mult(tmrg_interp *I, const double *x, double *y, int nvec) {
  return interp_host(I, 0, x, y, nvec);
}
int tmrg_interp_mult_transpose(tmrg_interp *I, const double *x, double *y,
                               int nvec) {
  return interp_host(I, 1, x, y, nvec);
}
int tmrg_interp_mult_weight_transpose(tmrg_interp *I, const double *x,
                                      double *y, int nvec) {
  return interp_host(I, 2, x, y, nvec);
}
int tmrg_interp_mult_device(tmrg_interp *I, const double *x, double *y,
                            int nvec) {
  return interp_dev(I, 0, x, y, nvec);
}
int tmrg_interp_mult_transpose_device(tmrg_interp *I, const double *x,
                                      double *y, int nvec) {
  return interp_dev(I, 1, x, y, nvec);
}
int tmrg_interp_mult_weight_transpose_device(tmrg_interp *I, const double *x,
                                             double *y, int nvec) {
  return interp_dev(I, 2, x, y, nvec);
}

// ---- matrix filter ----------------------------------------------------
int tmrg_filter_create(tmrg_forest *f, double block_len, double r, int N,
                       tmrg_filter **out) {
  return guarded([&] {
    ARG(f && out, "NULL argument");
    ARG(block_len > 0.0 && r >= 0.0 && N >= 0, "bad filter parameters");
    auto *h = new tmrg_filter;
    try {
      filter_create(f->f, block_len, r, N, h->F);
    } catch (...) {
      delete h;
      throw;
    }
    *out = h;
  });
}
int tmrg_filter_create_quad(tmrg_qforest *f, double block_len, double r, int N,
                            tmrg_filter **out) {
  return guarded([&] {
    ARG(f && out, "NULL argument");
    ARG(block_len > 0.0 && r >= 0.0 && N >= 0, "bad filter parameters");
    auto *h = new tmrg_filter;
    try {
      filter_create_quad(f->f, block_len, r, N, h->F);
    } catch (...) {
      delete h;
      throw;
    }
    *out = h;
  });
}
int tmrg_filter_destroy(tmrg_filter *F) {
  return guarded([&] {
    if (!F) return;
    cudaStreamSynchronize(F->F.s);
    delete F;
  });
}
int tmrg_filter_sizes(tmrg_filter *F, int64_t out2[2]) {
  return guarded([&] {
    ARG(F && out2, "NULL argument");
    out2[0] = F->F.n;
    out2[1] = F->F.nnz;
  });
}
int tmrg_filter_get_matrix(tmrg_filter *F, int *rowptr, int *cols,
                           double *vals, double *Ainv, double *B,
                           double *Tinv) {
  return guarded([&] {
    ARG(F, "NULL filter");
    Filter &M = F->F;
    if (rowptr) copy_d2h(rowptr, M.rowptr.p, sizeof(int) * (M.n + 1), M.s);
    if (cols) copy_d2h(cols, M.colidx.p, sizeof(int) * M.nnz, M.s);
    if (vals) copy_d2h(vals, M.vals.p, sizeof(double) * M.nnz, M.s);
    if (Ainv) copy_d2h(Ainv, M.Ainv.p, sizeof(double) * M.n, M.s);
    if (B) copy_d2h(B, M.B.p, sizeof(double) * M.n, M.s);
    if (Tinv) copy_d2h(Tinv, M.Tinv.p, sizeof(double) * M.n, M.s);
  });
}
static int filter_host(tmrg_filter *F, bool tr, int vpn, const double *in,
                       double *out) {
  return guarded([&] {
    ARG(F && in && out && vpn > 0, "bad argument");
    Filter &M = F->F;
    long long len = M.n * vpn;
    DBuf<double> a(len, M.s), b(len, M.s);
    host_warm(in, sizeof(double) * len);
    TMRG_CUDA(cudaMemcpyAsync(a.p, in, sizeof(double) * len,
                              cudaMemcpyHostToDevice, M.s));
    filter_apply(M, tr, vpn, a.p, b.p);
    copy_d2h(out, b.p, sizeof(double) * len, M.s);
  });
}
int tmrg_filter_apply(tmrg_filter *F, int vpn, const double *in, double *out) {
  return filter_host(F, false, vpn, in, out);
}
int tmrg_filter_apply_transpose(tmrg_filter *F, int vpn, const double *in,
                                double *out) {
  return filter_host(F, true, vpn, in, out);
}
int tmrg_filter_apply_device(tmrg_filter *F, int vpn, const double *in,
                             double *out) {
  return guarded([&] {
    ARG(F && in && out && vpn > 0, "bad argument");
    filter_apply(F->F, false, vpn, in, out);
  });
}
int tmrg_filter_apply_transpose_device(tmrg_filter *F, int vpn,
                                       const double *in, double *out) {
  return guarded([&] {
    ARG(F && in && out && vpn > 0, "bad argument");
    filter_apply(F->F, true, vpn, in, out);
  });
}
int tmrg_filter_apply_f32_device(tmrg_filter *F, int vpn, const float *in,
                                 float *out) {
  return guarded([&] {
    ARG(F && in && out && vpn > 0, "bad argument");
    filter_apply_f32(F->F, false, vpn, in, out);
  });
}
int tmrg_filter_apply_transpose_f32_device(tmrg_filter *F, int vpn,
                                           const float *in, float *out) {
  return guarded([&] {
    ARG(F && in && out && vpn > 0, "bad argument");
    filter_apply_f32(F->F, true, vpn, in, out);
  });
}

int tmrg_filter_apply_static_device(tmrg_filter *F, int transpose, int vpn,
                                    const double *in, double *out) {
  return guarded([&] {
    ARG(F && in && out && vpn > 0, "bad argument");
    filter_apply_static(F->F, transpose != 0, vpn, in, out);
  });
}

// ---- quadtree forest ----------------------------------------------------
static QForest &QF(tmrg_qforest *f) {
  if (!f) throw Error(TMRG_ERR_ARG, "NULL quadtree forest");
  return f->f;
}
int tmrg_qforest_create(int order, int interp, void *cuda_stream, tmrg_qforest **out) {
  return guarded([&] {
    ARG(out, "NULL argument");
    auto *h = new tmrg_qforest;
    h->f.s = (cudaStream_t)cuda_stream;
    try {
      h->f.set_order(order, interp);
    } catch (...) {
      delete h;
      throw;
    }
    *out = h;
  });
}
int tmrg_qforest_destroy(tmrg_qforest *f) {
  return guarded([&] {
    if (!f) return;
    cudaStreamSynchronize(f->f.s);
    delete f;
  });
}
int tmrg_qforest_set_connectivity(tmrg_qforest *f, int num_nodes, const int *face_conn,
                                  int num_faces) {
  return guarded([&] {
    ARG(face_conn, "NULL connectivity");
    QForest &F = QF(f);
    F.free_nodes();
    F.have_quads = false;
    F.n = 0;
    F.conn = qconn_build(num_nodes, face_conn, num_faces, nullptr, 0, F.s);
  });
}
int tmrg_qforest_set_full_connectivity(tmrg_qforest *f, int num_nodes, int num_edges,
                                       int num_faces, const int *face_conn,
                                       const int *face_edge_conn) {
  return guarded([&] {
    ARG(face_conn && face_edge_conn && num_edges > 0, "bad argument");
    QForest &F = QF(f);
    F.free_nodes();
    F.have_quads = false;
    F.n = 0;
    F.conn = qconn_build(num_nodes, face_conn, num_faces, face_edge_conn, num_edges, F.s);
  });
}
int tmrg_qforest_get_connectivity(tmrg_qforest *f, int *sizes3, int *face_conn,
                                  int *face_edge_conn) {
  return guarded([&] {
    QForest &F = QF(f);
    ARG(F.conn, "no connectivity");
    const QConn &C = *F.conn;
    if (sizes3) {
      sizes3[0] = C.nf;
      sizes3[1] = C.num_edges;
      sizes3[2] = C.num_nodes;
    }
    if (face_conn) memcpy(face_conn, C.face_conn.data(), sizeof(int) * C.face_conn.size());
    if (face_edge_conn)
      memcpy(face_edge_conn, C.face_edge.data(), sizeof(int) * C.face_edge.size());
  });
}
int tmrg_qforest_set_mesh_order(tmrg_qforest *f, int order, int interp) {
  return guarded([&] { QF(f).set_order(order, interp); });
}
int tmrg_qforest_get_mesh_order(tmrg_qforest *f, int *order, int *interp, double *knots) {
  return guarded([&] {
    QForest &F = QF(f);
    if (order) *order = F.order;
    if (interp) *interp = F.interp;
    if (knots)
      for (int i = 0; i < F.order; i++) knots[i] = F.knots[i];
  });
}
int tmrg_qforest_create_trees(tmrg_qforest *f, int level) {
  return guarded([&] { qforest_create_trees(QF(f), level); });
}
int tmrg_qforest_create_random_trees(tmrg_qforest *f, int nrand, int min_level, int max_level,
                                     uint64_t seed) {
  return guarded([&] { qforest_create_random_trees(QF(f), nrand, min_level, max_level, seed); });
}
int tmrg_qforest_refine(tmrg_qforest *f, const int *refine, int64_t n, int min_level,
                        int max_level) {
  return guarded([&] {
    QForest &F = QF(f);
    if (!refine) {
      qforest_refine(F, nullptr, 0, min_level, max_level);
      return;
    }
    DBuf<int> d(std::max<int64_t>(n, 1), F.s);
    if (n)
      host_warm(refine, sizeof(int) * n);
      TMRG_CUDA(cudaMemcpyAsync(d.p, refine, sizeof(int) * n, cudaMemcpyHostToDevice, F.s));
    qforest_refine(F, d.p, n, min_level, max_level);
  });
}
int tmrg_qforest_refine_device(tmrg_qforest *f, const int *d_refine, int64_t n,
                               int min_level, int max_level) {
  return guarded([&] { qforest_refine(QF(f), d_refine, d_refine ? n : 0, min_level, max_level); });
}
int tmrg_qforest_coarsen(tmrg_qforest *f, tmrg_qforest **out) {
  return guarded([&] {
    ARG(out, "NULL argument");
    QForest &F = QF(f);
    auto *h = new tmrg_qforest;
    h->f.s = F.s;
    try {
      qforest_coarsen(F, h->f);
    } catch (...) {
      delete h;
      throw;
    }
    *out = h;
  });
}
int tmrg_qforest_duplicate(tmrg_qforest *f, tmrg_qforest **out) {
  return guarded([&] {
    ARG(out, "NULL argument");
    QForest &F = QF(f);
    auto *h = new tmrg_qforest;
    h->f.s = F.s;
    try {
      qforest_duplicate(F, h->f);
    } catch (...) {
      delete h;
      throw;
    }
    *out = h;
  });
}
int tmrg_qforest_balance(tmrg_qforest *f, int corner) {
  return guarded([&] { qforest_balance(QF(f), corner); });
}
int tmrg_qforest_create_nodes(tmrg_qforest *f) {
  return guarded([&] {
    QForest &F = QF(f);
    if (!F.have_quads)
      throw Error(TMRG_ERR_STATE, "Cannot call createNodes(), no quadrants have been created");
    qforest_create_nodes(F);
  });
}
int tmrg_qforest_num_quadrants(tmrg_qforest *f, int64_t *n) {
  return guarded([&] {
    ARG(n, "NULL argument");
    *n = QF(f).have_quads ? QF(f).n : 0;
  });
}
// out: 6 ints per quadrant {face, x, y, tag, level, info}
int tmrg_qforest_get_quadrants(tmrg_qforest *f, int *out) {
  return guarded([&] {
    QForest &F = QF(f);
    ARG(out, "NULL argument");
    const long long n = F.n;
    std::vector<int> b(n), x(n), y(n);
    std::vector<int16_t> l(n), in(n);
    copy_d2h(b.data(), F.block.p, 4 * n, F.s);
    copy_d2h(x.data(), F.x.p, 4 * n, F.s);
    copy_d2h(y.data(), F.y.p, 4 * n, F.s);
    copy_d2h(l.data(), F.level.p, 2 * n, F.s);
    copy_d2h(in.data(), F.info.p, 2 * n, F.s);
    for (long long i = 0; i < n; i++) {
      int *o = out + 6 * i;
      o[0] = b[i];
      o[1] = x[i];
      o[2] = y[i];
      o[3] = (int)i;
      o[4] = l[i];
      o[5] = in[i];
    }
  });
}
// out6: {local nodes, owned nodes, dependent nodes, ext_pre, elements, dep nnz}
int tmrg_qforest_sizes(tmrg_qforest *f, int64_t *out6) {
  return guarded([&] {
    QForest &F = QF(f);
    ARG(out6, "NULL argument");
    out6[0] = F.num_local;
    out6[1] = F.num_owned;
    out6[2] = F.num_dep;
    out6[3] = F.num_dep;
    out6[4] = F.have_quads ? F.n : 0;
    out6[5] = F.dep_nnz;
  });
}
int tmrg_qforest_get_node_conn(tmrg_qforest *f, int *conn) {
  return guarded([&] {
    QForest &F = QF(f);
    ARG(conn && F.have_nodes, "no nodes (call createNodes)");
    copy_d2h(conn, F.econn.p, sizeof(int) * F.n * F.order * F.order, F.s);
  });
}
int tmrg_qforest_get_dep_node_conn(tmrg_qforest *f, int *ptr, int *conn, double *w) {
  return guarded([&] {
    QForest &F = QF(f);
    ARG(F.have_nodes, "no nodes (call createNodes)");
    if (ptr) copy_d2h(ptr, F.dep_ptr.p, sizeof(int) * (F.num_dep + 1), F.s);
    if (conn) copy_d2h(conn, F.dep_conn.p, sizeof(int) * F.dep_nnz, F.s);
    if (w) copy_d2h(w, F.dep_w.p, sizeof(double) * F.dep_nnz, F.s);
  });
}
int tmrg_qforest_create_interpolation(tmrg_qforest *fine, tmrg_qforest *coarse,
                                      tmrg_interp **out) {
  return guarded([&] {
    ARG(fine && coarse && out, "NULL argument");
    auto *h = new tmrg_interp;
    try {
      qinterp_create(fine->f, coarse->f, h->I);
    } catch (...) {
      delete h;
      throw;
    }
    *out = h;
  });
}
int tmrg_qforest_set_face_boxes(tmrg_qforest *f, const double *boxes, int nboxes) {
  return guarded([&] {
    QForest &F = QF(f);
    ARG(F.conn, "no connectivity");
    QConn &C = *F.conn;
    if (!boxes) {
      C.boxes.clear();
      C.d_boxes.release();
      return;
    }
    ARG(nboxes == C.nf, "one box per face expected");
    C.boxes.assign(boxes, boxes + 4 * (size_t)nboxes);
    C.d_boxes.alloc(C.boxes.size(), F.s);
    TMRG_CUDA(cudaMemcpyAsync(C.d_boxes.p, C.boxes.data(), sizeof(double) * C.boxes.size(),
                              cudaMemcpyHostToDevice, F.s));
    TMRG_CUDA(cudaStreamSynchronize(F.s));
  });
}
int tmrg_qforest_get_points(tmrg_qforest *f, double *X) {
  return guarded([&] {
    QForest &F = QF(f);
    ARG(X && F.have_nodes, "no nodes (call createNodes)");
    DBuf<double> d(3 * std::max(1LL, F.num_local), F.s);
    qforest_get_points(F, d.p);
    copy_d2h(X, d.p, sizeof(double) * 3 * F.num_local, F.s);
  });
}

// ---- iso-surface STL ----------------------------------------------------
static long long stl_run(tmrg_forest *f, const double *x, bool device, int vpn,
                         int x_offset, double cutoff, DBuf<double> &tris) {
  Forest &F = f->f;
  if (!F.have_nodes) forest_create_nodes(F);
  const long long len = F.num_owned * vpn;
  if (device) return stl_triangles(F, x, vpn, x_offset, cutoff, tris);
  DBuf<double> dx(std::max(1LL, len), F.s);
  if (len)
    TMRG_CUDA(cudaMemcpyAsync(dx.p, x, sizeof(double) * len, cudaMemcpyHostToDevice, F.s));
  return stl_triangles(F, dx.p, vpn, x_offset, cutoff, tris);
}
static int stl_entry(tmrg_forest *f, const double *x, bool device, int vpn, int x_offset,
                     double cutoff, int64_t *ntris, double *tris, int64_t max_tris) {
  return guarded([&] {
    ARG(f && x && ntris && vpn > 0, "bad argument");
    DBuf<double> d;
    const long long n = stl_run(f, x, device, vpn, x_offset, cutoff, d);
    *ntris = n;
    if (tris && max_tris >= n && n) {
      if (device) {
        TMRG_CUDA(cudaMemcpyAsync(tris, d.p, sizeof(double) * 9 * n, cudaMemcpyDeviceToDevice,
                                  f->f.s));
        TMRG_CUDA(cudaStreamSynchronize(f->f.s));
      } else {
        copy_d2h(tris, d.p, sizeof(double) * 9 * n, f->f.s);
      }
    }
  });
}
int tmrg_stl_triangles(tmrg_forest *f, const double *x, int vpn, int x_offset, double cutoff,
                       int64_t *ntris, double *tris, int64_t max_tris) {
  return stl_entry(f, x, false, vpn, x_offset, cutoff, ntris, tris, max_tris);
}
int tmrg_stl_triangles_device(tmrg_forest *f, const double *x, int vpn, int x_offset,
                              double cutoff, int64_t *ntris, double *tris, int64_t max_tris) {
  return stl_entry(f, x, true, vpn, x_offset, cutoff, ntris, tris, max_tris);
}
int tmrg_generate_bin_file(const char *filename, tmrg_forest *f, const double *x, int vpn,
                           int x_offset, double cutoff) {
  return guarded([&] {
    ARG(filename && f && x && vpn > 0, "bad argument");
    DBuf<double> d;
    const long long n = stl_run(f, x, false, vpn, x_offset, cutoff, d);
    ARG(n < (1LL << 31), "more triangles than the binary format's int count holds");
    std::vector<double> h((size_t)9 * n);
    copy_d2h(h.data(), d.p, sizeof(double) * h.size(), f->f.s);
    FILE *fp = fopen(filename, "wb");
    if (!fp) throw Error(TMRG_ERR_ARG, std::string("cannot open ") + filename);
    int32_t cnt = (int32_t)n;
    bool ok = fwrite(&cnt, sizeof(cnt), 1, fp) == 1 &&
              (n == 0 || fwrite(h.data(), sizeof(double), h.size(), fp) == h.size());
    ok = (fclose(fp) == 0) && ok;
    if (!ok) throw Error(TMRG_ERR_ARG, std::string("write failed: ") + filename);
  });
}
int tmrg_convert_bin_to_stl(const char *binfile, const char *stlfile) {
  return guarded([&] {
    ARG(binfile && stlfile, "NULL file name");
    FILE *fp = fopen(binfile, "rb");
    if (!fp) throw Error(TMRG_ERR_ARG, std::string("cannot open ") + binfile);
    int32_t n = 0;
    std::vector<double> t;
    bool ok = fread(&n, sizeof(n), 1, fp) == 1 && n >= 0;
    if (ok) {
      t.resize((size_t)9 * n);
      ok = n == 0 || fread(t.data(), sizeof(double), t.size(), fp) == t.size();
    }
    fclose(fp);
    if (!ok) throw Error(TMRG_ERR_ARG, std::string("bad STL binary file: ") + binfile);
    FILE *out = fopen(stlfile, "w");
    if (!out) throw Error(TMRG_ERR_ARG, std::string("cannot open ") + stlfile);
    // the reference's text layout and facet normal (writeSTLFile and
    // compute_normal, TMR_STLTools.cpp:440-461, 544-574)
    fprintf(out, "solid topology\n");
    for (int32_t i = 0; i < n; i++) {
      const double *p = t.data() + 9 * (size_t)i;
      double a[3] = {p[3] - p[0], p[4] - p[1], p[5] - p[2]};
      double b[3] = {p[6] - p[0], p[7] - p[1], p[8] - p[2]};
      double nn[3] = {a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2],
                      a[0] * b[1] - a[1] * b[0]};
      double norm = sqrt(nn[0] * nn[0] + nn[1] * nn[1] + nn[2] * nn[2]);
      nn[0] /= norm;
      nn[1] /= norm;
      nn[2] /= norm;
      fprintf(out, "facet normal %e %e %e\n", nn[0], nn[1], nn[2]);
      fprintf(out, "outer loop\n");
      for (int k = 0; k < 3; k++)
        fprintf(out, "vertex %e %e %e\n", p[3 * k], p[3 * k + 1], p[3 * k + 2]);
      fprintf(out, "endloop\nendfacet\n");
    }
    fprintf(out, "endsolid topology\n");
    if (fclose(out) != 0) throw Error(TMRG_ERR_ARG, std::string("write failed: ") + stlfile);
  });
}

// ---- Helmholtz filter ---------------------------------------------------
int tmrg_helmholtz_create(tmrg_forest *const *filters, int nlevels, double r,
                          tmrg_helmholtz **out) {
  return guarded([&] {
    ARG(filters && out && nlevels > 0, "bad argument");
    ARG(r >= 0.0, "Helmholtz radius must be >= 0");
    std::vector<Forest *> fs(nlevels);
    for (int k = 0; k < nlevels; k++) {
      ARG(filters[k], "NULL forest");
      fs[k] = &filters[k]->f;
    }
    auto *h = new tmrg_helmholtz;
    try {
      helmholtz_create(fs.data(), nlevels, r, h->H);
    } catch (...) {
      delete h;
      throw;
    }
    *out = h;
  });
}
int tmrg_helmholtz_create_quad(tmrg_qforest *const *filters, int nlevels, double r,
                               tmrg_helmholtz **out) {
  return guarded([&] {
    ARG(filters && out && nlevels > 0, "bad argument");
    ARG(r >= 0.0, "Helmholtz radius must be >= 0");
    std::vector<QForest *> fs(nlevels);
    for (int k = 0; k < nlevels; k++) {
      ARG(filters[k], "NULL forest");
      fs[k] = &filters[k]->f;
    }
    auto *h = new tmrg_helmholtz;
    try {
      helmholtz_create_quad(fs.data(), nlevels, r, h->H);
    } catch (...) {
      delete h;
      throw;
    }
    *out = h;
  });
}
int tmrg_helmholtz_destroy(tmrg_helmholtz *H) {
  return guarded([&] {
    if (!H) return;
    cudaStreamSynchronize(H->H.s);
    delete H;
  });
}
int tmrg_helmholtz_sizes(tmrg_helmholtz *H, int *nlevels, int64_t *out4) {
  return guarded([&] {
    ARG(H, "NULL filter");
    if (nlevels) *nlevels = H->H.nlevels;
    if (out4)
      for (int k = 0; k < H->H.nlevels; k++) {
        out4[4 * k] = H->H.L[k]->nn;
        out4[4 * k + 1] = H->H.L[k]->ne;
        out4[4 * k + 2] = H->H.L[k]->ndep;
        out4[4 * k + 3] = H->H.L[k]->snnz;
      }
  });
}
static int helmholtz_host(tmrg_helmholtz *H, bool tr, int vpn, const double *in,
                          double *out) {
  return guarded([&] {
    ARG(H && in && out && vpn > 0, "bad argument");
    Helmholtz &M = H->H;
    long long len = M.L[0]->nn * vpn;
    DBuf<double> a(std::max(1LL, len), M.s), b(std::max(1LL, len), M.s);
    if (len)
      TMRG_CUDA(cudaMemcpyAsync(a.p, in, sizeof(double) * len, cudaMemcpyHostToDevice, M.s));
    helmholtz_apply(M, tr, vpn, a.p, b.p);
    copy_d2h(out, b.p, sizeof(double) * len, M.s);
  });
}
int tmrg_helmholtz_apply(tmrg_helmholtz *H, int vpn, const double *in, double *out) {
  return helmholtz_host(H, false, vpn, in, out);
}
int tmrg_helmholtz_apply_transpose(tmrg_helmholtz *H, int vpn, const double *in,
                                   double *out) {
  return helmholtz_host(H, true, vpn, in, out);
}
int tmrg_helmholtz_apply_device(tmrg_helmholtz *H, int vpn, const double *in,
                                double *out) {
  return guarded([&] {
    ARG(H && in && out && vpn > 0, "bad argument");
    helmholtz_apply(H->H, false, vpn, in, out);
  });
}
int tmrg_helmholtz_apply_transpose_device(tmrg_helmholtz *H, int vpn,
                                          const double *in, double *out) {
  return guarded([&] {
    ARG(H && in && out && vpn > 0, "bad argument");
    helmholtz_apply(H->H, true, vpn, in, out);
  });
}
int tmrg_helmholtz_set_tolerances(tmrg_helmholtz *H, double rtol, double atol,
                                  int max_iters) {
  return guarded([&] {
    ARG(H && rtol >= 0.0 && atol >= 0.0 && max_iters > 0, "bad argument");
    H->H.rtol = rtol;
    H->H.atol = atol;
    H->H.max_iters = max_iters;
  });
}
int tmrg_helmholtz_set_smoother(tmrg_helmholtz *H, int degree_order2, int degree_order3,
                                double lower_order2, double lower_order3, double upper) {
  return guarded([&] {
    ARG(H && degree_order2 >= 1 && degree_order3 >= 1 && degree_order2 <= 64 &&
            degree_order3 <= 64,
        "bad smoother degree");
    ARG(lower_order2 > 0.0 && lower_order3 > 0.0 && upper > lower_order2 &&
            upper > lower_order3,
        "bad smoother interval");
    H->H.cheb_degree2 = degree_order2;
    H->H.cheb_degree3 = degree_order3;
    H->H.cheb_lower2 = lower_order2;
    H->H.cheb_lower3 = lower_order3;
    H->H.cheb_upper = upper;
  });
}
int tmrg_helmholtz_last_solve(tmrg_helmholtz *H, int *iters, double *res, int n) {
  return guarded([&] {
    ARG(H, "NULL filter");
    if (iters) *iters = H->H.last_iters;
    if (res)
      for (int k = 0; k < n && k < (int)H->H.last_res.size(); k++) res[k] = H->H.last_res[k];
  });
}
int tmrg_helmholtz_mult_device(tmrg_helmholtz *H, int level, int which, int nvec,
                               const double *in, double *out) {
  return guarded([&] {
    ARG(H && in && out && nvec > 0 && (which == 0 || which == 1), "bad argument");
    helmholtz_operator(H->H, level, which == 0, nvec, in, out);
  });
}

int tmrg_batch_refinement_device(tmrg_forest *f, int num_forests, const int *d_first_block,
                                 const int *d_block_forest, const double *d_prob,
                                 const int *d_active, uint64_t seed, uint64_t pass,
                                 int64_t *d_start, int *d_out) {
  return guarded([&] {
    ARG(f && num_forests > 0 && d_first_block && d_block_forest && d_prob && d_active &&
            d_start && (d_out || f->f.n == 0),
        "NULL argument");
    static_assert(sizeof(long long) == sizeof(int64_t), "int64");
    batch_refinement(f->f, num_forests, d_first_block, d_block_forest, d_prob, d_active, seed,
                     pass, (long long *)d_start, d_out);
  });
}
int tmrg_bump_indicator_device(tmrg_forest *f, const double *d_centres, int num_bumps,
                               const double *sigma, double t_refine, double t_coarsen,
                               int min_level, int max_level, int *d_out) {
  return guarded([&] {
    ARG(f && sigma && (d_out || f->f.n == 0) && (d_centres || num_bumps == 0),
        "NULL argument");
    bump_indicator(f->f, d_centres, num_bumps, sigma, t_refine, t_coarsen, min_level,
                   max_level, d_out);
  });
}
int tmrg_random_refinement_device(uint64_t seed, uint64_t stream, double prob,
                                  int *d_out, int64_t n, void *cuda_stream) {
  return guarded([&] {
    ARG(d_out || n == 0, "NULL output");
    random_refinement(seed, stream, prob, d_out, n, (cudaStream_t)cuda_stream);
  });
}

}  // extern "C"
