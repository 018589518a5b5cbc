// Block connectivity for a forest of hexahedral trees: from the 8 corner
// nodes of every block derive the unique edges and faces, the relative
// orientation of every shared face and the block lists of every corner,
// edge and face (TMROctForest.cpp:558-1143).  Host work, O(blocks), done
// once per setConnectivity and uploaded to the device in one allocation.
#include <algorithm>
#include <map>
#include <tuple>

#include "tmrg_internal.h"

namespace tmrg {

// The 8 symmetries of a square as corner permutations
// (face_orientations, TMROctForest.cpp:69-72).
static const int kFaceOrient[8][4] = {{0, 1, 2, 3}, {2, 0, 3, 1}, {3, 2, 1, 0},
                                      {1, 3, 0, 2}, {0, 2, 1, 3}, {2, 3, 0, 1},
                                      {3, 1, 2, 0}, {1, 0, 3, 2}};

static void make_csr(int nitems, const std::vector<int> &item_of,
                     std::vector<int> &ptr, std::vector<int> &ent) {
  ptr.assign(nitems + 1, 0);
  for (int it : item_of) ptr[it + 1]++;
  for (int i = 0; i < nitems; i++) ptr[i + 1] += ptr[i];
  ent.assign(item_of.size(), 0);
  std::vector<int> fill(ptr.begin(), ptr.end() - 1);
  // entries are visited in block order: the first one is the owner
  for (size_t e = 0; e < item_of.size(); e++) ent[fill[item_of[e]]++] = (int)e;
}

std::shared_ptr<Conn> build_conn(int num_nodes, const int *bc, int nb,
                                 cudaStream_t s, int num_edges, const int *be,
                                 int num_faces, const int *bf) {
  if (nb <= 0 || num_nodes <= 0 || !bc)
    throw Error(TMRG_ERR_ARG, "setConnectivity: empty connectivity");
  for (long long i = 0; i < 8LL * nb; i++)
    if (bc[i] < 0 || bc[i] >= num_nodes)
      throw Error(TMRG_ERR_ARG, "setConnectivity: node index out of range");
  auto c = std::make_shared<Conn>();
  c->num_nodes = num_nodes;
  c->nb = nb;
  c->block_conn.assign(bc, bc + 8LL * nb);
  c->block_bits = bits_for(nb);

  // Corner -> blocks.
  make_csr(num_nodes, c->block_conn, c->node_ptr, c->node_ent);

  // Edges: keyed by their unordered node pair, numbered by first use
  // (computeEdgesFromNodes, TMROctForest.cpp:791-862), or as given
  // (setFullConnectivity, :596-637).
  std::map<std::pair<int, int>, int> edges;
  c->block_edge.assign(12LL * nb, 0);
  if (be) {
    for (long long i = 0; i < 12LL * nb; i++)
      if (be[i] < 0 || be[i] >= num_edges)
        throw Error(TMRG_ERR_ARG, "setFullConnectivity: edge index out of range");
    c->block_edge.assign(be, be + 12LL * nb);
  }
  for (int b = 0; b < nb && !be; b++)
    for (int e = 0; e < 12; e++) {
      int a1, a2;
      edge_corners(e, a1, a2);
      int n1 = bc[8 * b + a1], n2 = bc[8 * b + a2];
      auto key = std::make_pair(std::min(n1, n2), std::max(n1, n2));
      auto it = edges.find(key);
      int id;
      if (it == edges.end()) {
        id = (int)edges.size();
        edges.emplace(key, id);
      } else {
        id = it->second;
      }
      c->block_edge[12 * b + e] = id;
    }
  c->num_edges = be ? num_edges : (int)edges.size();
  make_csr(c->num_edges, c->block_edge, c->edge_ptr, c->edge_ent);

  // Faces: keyed by their sorted node 4-tuple; orientation is checked
  // against the owner's corner order below.
  std::map<std::tuple<int, int, int, int>, int> faces;
  c->block_face.assign(6LL * nb, 0);
  if (bf) {
    for (long long i = 0; i < 6LL * nb; i++)
      if (bf[i] < 0 || bf[i] >= num_faces)
        throw Error(TMRG_ERR_ARG, "setFullConnectivity: face index out of range");
    c->block_face.assign(bf, bf + 6LL * nb);
  }
  for (int b = 0; b < nb && !bf; b++)
    for (int f = 0; f < 6; f++) {
      int q[4];
      for (int k = 0; k < 4; k++) q[k] = bc[8 * b + face_corner(f, k)];
      std::sort(q, q + 4);
      auto key = std::make_tuple(q[0], q[1], q[2], q[3]);
      auto it = faces.find(key);
      int id;
      if (it == faces.end()) {
        id = (int)faces.size();
        faces.emplace(key, id);
      } else {
        id = it->second;
      }
      c->block_face[6 * b + f] = id;
    }
  c->num_faces = bf ? num_faces : (int)faces.size();
  make_csr(c->num_faces, c->block_face, c->face_ptr, c->face_ent);

  // Orientation of each block face relative to the face owner: the first
  // of the 8 square symmetries mapping the owner's corners onto it.
  c->face_ids.assign(6LL * nb, 0);
  for (int face = 0; face < c->num_faces; face++) {
    int own = c->face_ent[c->face_ptr[face]];
    int ob = own / 6, of = own % 6;
    int on[4];
    for (int k = 0; k < 4; k++) on[k] = bc[8 * ob + face_corner(of, k)];
    for (int p = c->face_ptr[face]; p < c->face_ptr[face + 1]; p++) {
      int b = c->face_ent[p] / 6, f = c->face_ent[p] % 6;
      int an[4];
      for (int k = 0; k < 4; k++) an[k] = bc[8 * b + face_corner(f, k)];
      int found = -1;
      for (int o = 0; o < 8 && found < 0; o++)
        if (on[0] == an[kFaceOrient[o][0]] && on[1] == an[kFaceOrient[o][1]] &&
            on[2] == an[kFaceOrient[o][2]] && on[3] == an[kFaceOrient[o][3]])
          found = o;
      if (found < 0)
        throw Error(TMRG_ERR_ARG, "setConnectivity: inconsistent face");
      c->face_ids[6 * b + f] = found;
    }
  }
  auto maxval = [](const std::vector<int> &ptr) {
    int m = 1;
    for (size_t i = 0; i + 1 < ptr.size(); i++) m = std::max(m, ptr[i + 1] - ptr[i]);
    return m;
  };
  c->max_node_val = maxval(c->node_ptr);
  c->max_edge_val = maxval(c->edge_ptr);
  c->max_face_val = maxval(c->face_ptr);

  // Upload every table in one allocation.
  std::vector<const std::vector<int> *> parts = {
      &c->block_conn, &c->block_edge, &c->block_face, &c->face_ids,
      &c->node_ptr,   &c->node_ent,   &c->edge_ptr,   &c->edge_ent,
      &c->face_ptr,   &c->face_ent};
  size_t total = 0;
  for (auto *p : parts) total += p->size();
  std::vector<int> flat;
  flat.reserve(total);
  std::vector<size_t> offs;
  for (auto *p : parts) {
    offs.push_back(flat.size());
    flat.insert(flat.end(), p->begin(), p->end());
  }
  c->d_all.alloc(total, s);
  TMRG_CUDA(cudaMemcpyAsync(c->d_all.p, flat.data(), total * sizeof(int),
                            cudaMemcpyHostToDevice, s));
  TMRG_CUDA(cudaStreamSynchronize(s));
  const int *d = c->d_all.p;
  c->dev.nb = nb;
  c->dev.block_conn = d + offs[0];
  c->dev.block_edge = d + offs[1];
  c->dev.block_face = d + offs[2];
  c->dev.face_ids = d + offs[3];
  c->dev.node_ptr = d + offs[4];
  c->dev.node_ent = d + offs[5];
  c->dev.edge_ptr = d + offs[6];
  c->dev.edge_ent = d + offs[7];
  c->dev.face_ptr = d + offs[8];
  c->dev.face_ent = d + offs[9];
  return c;
}

}  // namespace tmrg
