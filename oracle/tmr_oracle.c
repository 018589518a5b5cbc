/*
  tmr_oracle.c — sequential CPU restatement of the TMR octree-forest
  adaptation path.  TEST INFRASTRUCTURE (see tmr_oracle.h): the checker,
  never the product.

  Each function names the reference lines it follows.  Where the reference
  uses a chained hash (TMROctantHash, TMROctant.cpp:599-798) only its
  set semantics matter for the results ("an element is added once; the
  first insertion wins"); this file gets the same semantics from an
  open-addressing table or from a stable sort that keeps the first of
  each run of equal keys.

  Compile with -ffp-contract=off so that every floating-point expression
  is evaluated in source order, as the reference's x86-64 build does.
*/
#include "tmr_oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define OO_MAX_LEVEL 30
#define OO_HMAX (1 << OO_MAX_LEVEL)
#define OO_MAX_ORDER 16

/* ------------------------------------------------------------------ */
/* Geometry of one hexahedral block (TMROctForest.cpp:29-72).  Corner c
   of a block sits at (c&1, (c>>1)&1, c>>2).  Edges 0-3 run along x,
   4-7 along y, 8-11 along z; faces 0/1 are x=0/1, 2/3 y=0/1, 4/5 z=0/1. */
static void edge_corners(int e, int *n1, int *n2) {
  if (e < 4) {
    *n1 = 2 * (e & 1) + 4 * (e >> 1);
    *n2 = *n1 + 1;
  } else if (e < 8) {
    *n1 = (e & 1) + 4 * ((e - 4) >> 1);
    *n2 = *n1 + 2;
  } else {
    *n1 = e - 8;
    *n2 = *n1 + 4;
  }
}
/* The four corners of face f in the reference's order
   (block_to_face_nodes, TMROctForest.cpp:37-38): the first free
   coordinate varies fastest. */
static int face_corner(int f, int k) {
  int d = f >> 1, s = f & 1;
  int a = k & 1, b = k >> 1;
  if (d == 0) return s + 2 * a + 4 * b;
  if (d == 1) return a + 2 * s + 4 * b;
  return a + 2 * b + 4 * s;
}
/* Relative orientations of two matched faces (face_orientations,
   TMROctForest.cpp:69-72): the 8 symmetries of a square. */
static const int face_orient[8][4] = {{0, 1, 2, 3}, {2, 0, 3, 1},
                                      {3, 2, 1, 0}, {1, 3, 0, 2},
                                      {0, 2, 1, 3}, {2, 3, 0, 1},
                                      {3, 1, 2, 0}, {1, 0, 3, 2}};
/* Faces / edges of the parent that child `id` touches
   (child_id_to_face_index, child_id_to_edge_index). */
static int child_face(int id, int k) {
  return 2 * k + ((id >> k) & 1);
}
static int child_edge(int id, int k) {
  int x = id & 1, y = (id >> 1) & 1, z = id >> 2;
  if (k == 0) return y + 2 * z;
  if (k == 1) return 4 + x + 2 * z;
  return 8 + x + 2 * y;
}
/* The two parent edges lying in parent face child_face(id,k)
   (child_id_to_face_to_edge_index). */
static int child_face_edge(int id, int k, int j) {
  int other[2];
  int n = 0;
  for (int d = 2; d >= 0; d--)
    if (d != k) other[n++] = d;
  return child_edge(id, other[j]);
}
/* The 4 edges bounding face f (face_to_edge_index); entries 0,1 run
   along the second free face coordinate, 2,3 along the first. */
static int face_edge(int f, int e) {
  int d = f >> 1, s = f & 1;
  int dir, a, b;
  if (d == 0) {
    dir = (e < 2) ? 2 : 1;
  } else if (d == 1) {
    dir = (e < 2) ? 2 : 0;
  } else {
    dir = (e < 2) ? 1 : 0;
  }
  int side = e & 1;
  /* edge index = 4*dir + (first other coord side) + 2*(second) */
  if (dir == 0) { /* x-edge: sides in y, z */
    a = (d == 1) ? s : side;
    b = (d == 2) ? s : side;
  } else if (dir == 1) { /* y-edge: sides in x, z */
    a = (d == 0) ? s : side;
    b = (d == 2) ? s : side;
  } else { /* z-edge: sides in x, y */
    a = (d == 0) ? s : side;
    b = (d == 1) ? s : side;
  }
  return 4 * dir + a + 2 * b;
}

/* Face coordinate transforms (TMROctForest.cpp:78-198).  `h` is the
   octant side for octant transforms, 0 for node transforms with the
   extent `hmax` passed instead. */
static void face_get(int id, int32_t ext, int32_t x, int32_t y, int32_t *u,
                     int32_t *v) {
  switch (id) {
    case 0: *u = x; *v = y; break;
    case 1: *u = ext - y; *v = x; break;
    case 2: *u = ext - x; *v = ext - y; break;
    case 3: *u = y; *v = ext - x; break;
    case 4: *u = y; *v = x; break;
    case 5: *u = x; *v = ext - y; break;
    case 6: *u = ext - y; *v = ext - x; break;
    default: *u = ext - x; *v = y; break;
  }
}
static void face_set(int id, int32_t ext, int32_t u, int32_t v, int32_t *x,
                     int32_t *y) {
  switch (id) {
    case 0: *x = u; *y = v; break;
    case 1: *x = v; *y = ext - u; break;
    case 2: *x = ext - u; *y = ext - v; break;
    case 3: *x = ext - v; *y = u; break;
    case 4: *x = v; *y = u; break;
    case 5: *x = u; *y = ext - v; break;
    case 6: *x = ext - v; *y = ext - u; break;
    default: *x = ext - u; *y = v; break;
  }
}

/* ------------------------------------------------------------------ */
/* Octant algebra (TMROctant.cpp:28-291). */
static int32_t side(int level) { return (int32_t)1 << (OO_MAX_LEVEL - level); }

static int child_id(const oo_oct *o) {
  int32_t h = side(o->level);
  return ((o->x & h) ? 1 : 0) | ((o->y & h) ? 2 : 0) | ((o->z & h) ? 4 : 0);
}
static oo_oct sibling(const oo_oct *o, int id) {
  int32_t h = side(o->level);
  oo_oct s = *o;
  int32_t xr = (o->x & h) ? o->x - h : o->x;
  int32_t yr = (o->y & h) ? o->y - h : o->y;
  int32_t zr = (o->z & h) ? o->z - h : o->z;
  s.info = 0;
  s.x = (id & 1) ? xr + h : xr;
  s.y = (id & 2) ? yr + h : yr;
  s.z = (id & 4) ? zr + h : zr;
  return s;
}
static oo_oct parent_of(const oo_oct *o) {
  oo_oct p = *o;
  p.info = 0;
  if (o->level > 0) {
    int32_t h = side(o->level);
    p.level = o->level - 1;
    p.x = o->x & ~h;
    p.y = o->y & ~h;
    p.z = o->z & ~h;
  }
  return p;
}
static oo_oct face_nbr(const oo_oct *o, int f) {
  int32_t h = side(o->level);
  oo_oct n = *o;
  n.info = 0;
  n.x += (f == 0) ? -h : (f == 1) ? h : 0;
  n.y += (f == 2) ? -h : (f == 3) ? h : 0;
  n.z += (f == 4) ? -h : (f == 5) ? h : 0;
  return n;
}
static oo_oct edge_nbr(const oo_oct *o, int e) {
  int32_t h = side(o->level);
  oo_oct n = *o;
  n.info = 0;
  int a = (e & 1) ? h : -h, b = (e & 2) ? h : -h;
  if (e < 4) {
    n.y += a;
    n.z += b;
  } else if (e < 8) {
    n.x += a;
    n.z += b;
  } else {
    n.x += a;
    n.y += b;
  }
  return n;
}
static oo_oct corner_nbr(const oo_oct *o, int c) {
  int32_t h = side(o->level);
  oo_oct n = *o;
  n.info = 0;
  n.x += (c & 1) ? h : -h;
  n.y += (c & 2) ? h : -h;
  n.z += (c & 4) ? h : -h;
  return n;
}
static int contains(const oo_oct *a, const oo_oct *b) {
  int32_t h = side(a->level);
  return b->block == a->block && b->x >= a->x && b->x < a->x + h &&
         b->y >= a->y && b->y < a->y + h && b->z >= a->z && b->z < a->z + h;
}
/* Morton position compare: the most significant differing coordinate
   bit decides, ties between coordinates go to x, then y
   (TMROctant.cpp:171-204). */
static int cmp_position(const oo_oct *a, const oo_oct *b) {
  if (a->block != b->block) return a->block < b->block ? -1 : 1;
  uint32_t dx = (uint32_t)(a->x ^ b->x), dy = (uint32_t)(a->y ^ b->y),
           dz = (uint32_t)(a->z ^ b->z);
  uint32_t any = dx | dy | dz;
  int32_t d;
  if (any == 0) return 0;
  if (dx > (any ^ dx)) {
    d = a->x - b->x;
  } else if (dy > (any ^ dy)) {
    d = a->y - b->y;
  } else {
    d = a->z - b->z;
  }
  return d > 0 ? 1 : (d < 0 ? -1 : 0);
}
static int cmp_octant(const oo_oct *a, const oo_oct *b) {
  int c = cmp_position(a, b);
  if (c) return c;
  return a->level - b->level;
}
static int cmp_node(const oo_oct *a, const oo_oct *b) {
  int c = cmp_position(a, b);
  if (c) return c;
  return a->info - b->info;
}
static int cmp_tag(const oo_oct *a, const oo_oct *b) { return a->tag - b->tag; }

typedef int (*oo_cmp)(const oo_oct *, const oo_oct *);

/* Stable merge sort. */
static void msort_rec(oo_oct *a, oo_oct *t, long n, oo_cmp cmp) {
  if (n < 2) return;
  long m = n / 2;
  msort_rec(a, t, m, cmp);
  msort_rec(a + m, t, n - m, cmp);
  long i = 0, j = m, k = 0;
  while (i < m && j < n) {
    if (cmp(&a[j], &a[i]) < 0)
      t[k++] = a[j++];
    else
      t[k++] = a[i++];
  }
  while (i < m) t[k++] = a[i++];
  while (j < n) t[k++] = a[j++];
  memcpy(a, t, sizeof(oo_oct) * (size_t)n);
}
static void stable_sort(oo_oct *a, long n, oo_cmp cmp) {
  if (n < 2) return;
  oo_oct *t = (oo_oct *)malloc(sizeof(oo_oct) * (size_t)n);
  msort_rec(a, t, n, cmp);
  free(t);
}
/* Keep the first element of each run of elements equal under `eq`. */
static long unique_first(oo_oct *a, long n, oo_cmp eq) {
  long j = 0;
  for (long i = 0; i < n; i++) {
    if (j > 0 && eq(&a[j - 1], &a[i]) == 0) continue;
    a[j++] = a[i];
  }
  return j;
}
/* TMROctantArray::sort for elements (TMROctant.cpp:357-399): order by
   (position, level), then for each position keep the last entry, i.e.
   the finest. */
static long sort_elements(oo_oct *a, long n) {
  stable_sort(a, n, cmp_octant);
  long j = 0;
  for (long i = 0; i < n; i++) {
    while (i < n - 1 && cmp_position(&a[i], &a[i + 1]) == 0) i++;
    a[j++] = a[i];
  }
  return j;
}
static long bsearch_oct(const oo_oct *a, long n, const oo_oct *q, oo_cmp cmp) {
  long lo = 0, hi = n - 1;
  while (lo <= hi) {
    long mid = lo + (hi - lo) / 2;
    int c = cmp(&a[mid], q);
    if (c == 0) return mid;
    if (c < 0)
      lo = mid + 1;
    else
      hi = mid - 1;
  }
  return -1;
}

/* ------------------------------------------------------------------ */
/* Insertion-ordered set of octants keyed by (block, x, y, z, level):
   the TMROctantHash semantics for elements.  Open addressing. */
typedef struct {
  oo_oct *items;
  long n, cap;
  long *slots;
  long nslots;
} oset;

static uint64_t oct_hash(const oo_oct *o) {
  uint64_t h = (uint64_t)(uint32_t)o->block * 0x9E3779B97F4A7C15ULL;
  h ^= (uint64_t)(uint32_t)o->x + 0x632BE59BD9B4E019ULL + (h << 6) + (h >> 2);
  h ^= (uint64_t)(uint32_t)o->y + 0x85EBCA77C2B2AE63ULL + (h << 6) + (h >> 2);
  h ^= (uint64_t)(uint32_t)o->z + 0xC2B2AE3D27D4EB4FULL + (h << 6) + (h >> 2);
  h ^= (uint64_t)(uint16_t)o->level * 0x165667B19E3779F9ULL;
  return oo_splitmix64(h);
}
static void oset_init(oset *s) {
  s->n = 0;
  s->cap = 1024;
  s->items = (oo_oct *)malloc(sizeof(oo_oct) * (size_t)s->cap);
  s->nslots = 4096;
  s->slots = (long *)malloc(sizeof(long) * (size_t)s->nslots);
  for (long i = 0; i < s->nslots; i++) s->slots[i] = -1;
}
static void oset_free(oset *s) {
  free(s->items);
  free(s->slots);
}
static int same_elem(const oo_oct *a, const oo_oct *b) {
  return a->block == b->block && a->x == b->x && a->y == b->y &&
         a->z == b->z && a->level == b->level;
}
static void oset_rehash(oset *s) {
  long ns = s->nslots * 2;
  long *sl = (long *)malloc(sizeof(long) * (size_t)ns);
  for (long i = 0; i < ns; i++) sl[i] = -1;
  for (long i = 0; i < s->n; i++) {
    uint64_t h = oct_hash(&s->items[i]) & (uint64_t)(ns - 1);
    while (sl[h] >= 0) h = (h + 1) & (uint64_t)(ns - 1);
    sl[h] = i;
  }
  free(s->slots);
  s->slots = sl;
  s->nslots = ns;
}
/* Returns 1 if added, 0 if an equal element was already present. */
static int oset_add(oset *s, const oo_oct *o) {
  if (2 * (s->n + 1) > s->nslots) oset_rehash(s);
  uint64_t mask = (uint64_t)(s->nslots - 1);
  uint64_t h = oct_hash(o) & mask;
  while (s->slots[h] >= 0) {
    if (same_elem(&s->items[s->slots[h]], o)) return 0;
    h = (h + 1) & mask;
  }
  if (s->n == s->cap) {
    s->cap *= 2;
    s->items = (oo_oct *)realloc(s->items, sizeof(oo_oct) * (size_t)s->cap);
  }
  s->items[s->n] = *o;
  s->slots[h] = s->n;
  s->n++;
  return 1;
}

/* Growable octant list (a FIFO when used as the balance queue). */
typedef struct {
  oo_oct *a;
  long n, cap, head;
} olist;
static void ol_init(olist *l) {
  l->n = 0;
  l->head = 0;
  l->cap = 1024;
  l->a = (oo_oct *)malloc(sizeof(oo_oct) * (size_t)l->cap);
}
static void ol_push(olist *l, const oo_oct *o) {
  if (l->n == l->cap) {
    l->cap *= 2;
    l->a = (oo_oct *)realloc(l->a, sizeof(oo_oct) * (size_t)l->cap);
  }
  l->a[l->n++] = *o;
}

/* ------------------------------------------------------------------ */
/* Block connectivity (TMROctForest.cpp:558-1143). */
typedef struct {
  int refcount;
  int num_nodes, num_edges, num_faces, num_blocks;
  int *block_conn;      /* 8 per block */
  int *block_edge_conn; /* 12 per block */
  int *block_face_conn; /* 6 per block */
  int *block_face_ids;  /* 6 per block: orientation relative to owner */
  int *node_block_ptr, *node_block_conn; /* entries 8*block + corner */
  int *edge_block_ptr, *edge_block_conn; /* entries 12*block + edge */
  int *face_block_ptr, *face_block_conn; /* entries 6*block + face */
  int *node_owner, *edge_owner, *face_owner;
} oo_conn;

static void csr_from(int nent, int nitems, const int *item_of, int per,
                     int **ptr_out, int **conn_out) {
  int *ptr = (int *)calloc((size_t)nitems + 1, sizeof(int));
  for (int i = 0; i < nent; i++) ptr[item_of[i] + 1]++;
  for (int i = 0; i < nitems; i++) ptr[i + 1] += ptr[i];
  int *conn = (int *)malloc(sizeof(int) * (size_t)(nent > 0 ? nent : 1));
  int *fill = (int *)malloc(sizeof(int) * (size_t)(nitems + 1));
  memcpy(fill, ptr, sizeof(int) * (size_t)(nitems + 1));
  /* entries in block order, so the first entry is the lowest block */
  for (int i = 0; i < nent; i++) conn[fill[item_of[i]]++] = i;
  (void)per;
  free(fill);
  *ptr_out = ptr;
  *conn_out = conn;
}

static void conn_free(oo_conn *c) {
  if (!c) return;
  if (--c->refcount > 0) return;
  free(c->block_conn);
  free(c->block_edge_conn);
  free(c->block_face_conn);
  free(c->block_face_ids);
  free(c->node_block_ptr);
  free(c->node_block_conn);
  free(c->edge_block_ptr);
  free(c->edge_block_conn);
  free(c->face_block_ptr);
  free(c->face_block_conn);
  free(c->node_owner);
  free(c->edge_owner);
  free(c->face_owner);
  free(c);
}

static oo_conn *conn_build(int num_nodes, const int *bc, int nb) {
  if (nb < 0 || num_nodes < 0) return NULL;
  oo_conn *c = (oo_conn *)calloc(1, sizeof(oo_conn));
  c->refcount = 1;
  c->num_nodes = num_nodes;
  c->num_blocks = nb;
  c->block_conn = (int *)malloc(sizeof(int) * 8 * (size_t)(nb > 0 ? nb : 1));
  memcpy(c->block_conn, bc, sizeof(int) * 8 * (size_t)nb);
  /* corners -> blocks */
  csr_from(8 * nb, num_nodes, c->block_conn, 8, &c->node_block_ptr,
           &c->node_block_conn);
  /* Edges: identified by their unordered corner-node pair, numbered in
     order of first appearance (block-major, local edge order). */
  c->block_edge_conn = (int *)malloc(sizeof(int) * 12 * (size_t)(nb ? nb : 1));
  int ne = 0;
  for (int b = 0; b < nb; b++) {
    for (int e = 0; e < 12; e++) {
      int a1, a2;
      edge_corners(e, &a1, &a2);
      int n1 = bc[8 * b + a1], n2 = bc[8 * b + a2];
      int found = -1;
      for (int p = c->node_block_ptr[n1];
           p < c->node_block_ptr[n1 + 1] && found < 0; p++) {
        int b2 = c->node_block_conn[p] / 8;
        if (b2 > b) continue;
        int lim = (b2 == b) ? e : 12;
        for (int e2 = 0; e2 < lim; e2++) {
          int c1, c2;
          edge_corners(e2, &c1, &c2);
          int m1 = bc[8 * b2 + c1], m2 = bc[8 * b2 + c2];
          if ((m1 == n1 && m2 == n2) || (m1 == n2 && m2 == n1)) {
            found = c->block_edge_conn[12 * b2 + e2];
            break;
          }
        }
      }
      c->block_edge_conn[12 * b + e] = (found >= 0) ? found : ne++;
    }
  }
  c->num_edges = ne;
  csr_from(12 * nb, ne, c->block_edge_conn, 12, &c->edge_block_ptr,
           &c->edge_block_conn);
  /* Faces: identified by their corner-node 4-tuple up to the 8
     orientations. */
  c->block_face_conn = (int *)malloc(sizeof(int) * 6 * (size_t)(nb ? nb : 1));
  int nf = 0;
  for (int b = 0; b < nb; b++) {
    for (int f = 0; f < 6; f++) {
      int fn[4];
      for (int k = 0; k < 4; k++) fn[k] = bc[8 * b + face_corner(f, k)];
      int found = -1;
      for (int p = c->node_block_ptr[fn[0]];
           p < c->node_block_ptr[fn[0] + 1] && found < 0; p++) {
        int b2 = c->node_block_conn[p] / 8;
        if (b2 >= b) continue;
        for (int f2 = 0; f2 < 6 && found < 0; f2++) {
          int an[4];
          for (int k = 0; k < 4; k++) an[k] = bc[8 * b2 + face_corner(f2, k)];
          for (int o = 0; o < 8; o++) {
            if (fn[0] == an[face_orient[o][0]] &&
                fn[1] == an[face_orient[o][1]] &&
                fn[2] == an[face_orient[o][2]] &&
                fn[3] == an[face_orient[o][3]]) {
              found = c->block_face_conn[6 * b2 + f2];
              break;
            }
          }
        }
      }
      c->block_face_conn[6 * b + f] = (found >= 0) ? found : nf++;
    }
  }
  c->num_faces = nf;
  csr_from(6 * nb, nf, c->block_face_conn, 6, &c->face_block_ptr,
           &c->face_block_conn);
  /* Face orientation of every block face relative to the face's owner,
     the lowest-numbered block (TMROctForest.cpp:1029-1080). */
  c->block_face_ids = (int *)calloc(6 * (size_t)(nb ? nb : 1), sizeof(int));
  for (int face = 0; face < nf; face++) {
    int own = c->face_block_conn[c->face_block_ptr[face]];
    int ob = own / 6, of = own % 6;
    int on[4];
    for (int k = 0; k < 4; k++) on[k] = bc[8 * ob + face_corner(of, k)];
    for (int p = c->face_block_ptr[face]; p < c->face_block_ptr[face + 1];
         p++) {
      int b = c->face_block_conn[p] / 6, f = c->face_block_conn[p] % 6;
      int an[4];
      for (int k = 0; k < 4; k++) an[k] = bc[8 * b + face_corner(f, k)];
      for (int o = 0; o < 8; o++) {
        if (on[0] == an[face_orient[o][0]] && on[1] == an[face_orient[o][1]] &&
            on[2] == an[face_orient[o][2]] && on[3] == an[face_orient[o][3]]) {
          c->block_face_ids[6 * b + f] = o;
          break;
        }
      }
    }
  }
  c->node_owner = (int *)malloc(sizeof(int) * (size_t)(num_nodes + 1));
  for (int n = 0; n < num_nodes; n++)
    c->node_owner[n] = (c->node_block_ptr[n + 1] > c->node_block_ptr[n])
                           ? c->node_block_conn[c->node_block_ptr[n]] / 8
                           : nb;
  c->edge_owner = (int *)malloc(sizeof(int) * (size_t)(ne + 1));
  for (int e = 0; e < ne; e++)
    c->edge_owner[e] = c->edge_block_conn[c->edge_block_ptr[e]] / 12;
  c->face_owner = (int *)malloc(sizeof(int) * (size_t)(nf + 1));
  for (int f = 0; f < nf; f++)
    c->face_owner[f] = c->face_block_conn[c->face_block_ptr[f]] / 6;
  return c;
}

/* ------------------------------------------------------------------ */
struct oo_forest {
  int order, interp;
  double knots[OO_MAX_ORDER];
  oo_conn *conn;
  oo_oct *octs;
  long noct;
  /* createNodes products */
  int have_nodes;
  int *econn;
  int *node_numbers;
  int num_local, num_owned, num_dep, ext_pre;
  int *dep_ptr, *dep_conn;
  double *dep_w;
};

static void free_mesh(oo_forest *f) {
  free(f->econn);
  free(f->node_numbers);
  free(f->dep_ptr);
  free(f->dep_conn);
  free(f->dep_w);
  f->econn = NULL;
  f->node_numbers = NULL;
  f->dep_ptr = f->dep_conn = NULL;
  f->dep_w = NULL;
  f->have_nodes = 0;
  f->num_local = f->num_owned = f->num_dep = f->ext_pre = 0;
}

/* TMROctForest::setMeshOrder (TMROctForest.cpp:1389-1427). */
void oo_set_mesh_order(oo_forest *f, int order, int interp) {
  free_mesh(f);
  if (order < 2) order = 2;
  if (order > OO_MAX_ORDER) order = OO_MAX_ORDER;
  f->order = order;
  f->interp = interp;
  memset(f->knots, 0, sizeof(f->knots));
  f->knots[0] = -1.0;
  f->knots[order - 1] = 1.0;
  for (int i = 1; i < order - 1; i++) {
    if (interp == 1 || interp == 2)
      f->knots[i] = -cos(M_PI * i / (order - 1));
    else
      f->knots[i] = -1.0 + 2.0 * i / (order - 1);
  }
}

oo_forest *oo_forest_create(int order, int interp) {
  oo_forest *f = (oo_forest *)calloc(1, sizeof(oo_forest));
  oo_set_mesh_order(f, order, interp);
  return f;
}
void oo_forest_destroy(oo_forest *f) {
  if (!f) return;
  free_mesh(f);
  free(f->octs);
  conn_free(f->conn);
  free(f);
}
int oo_set_connectivity(oo_forest *f, int nn, const int *bc, int nb) {
  free_mesh(f);
  free(f->octs);
  f->octs = NULL;
  f->noct = 0;
  conn_free(f->conn);
  f->conn = conn_build(nn, bc, nb);
  return f->conn ? 0 : -1;
}

static void set_tags(oo_forest *f) {
  for (long i = 0; i < f->noct; i++) f->octs[i].tag = (int32_t)i;
}

/* TMROctForest::createTrees (TMROctForest.cpp:1744-1833), one rank. */
void oo_create_trees(oo_forest *f, int level) {
  free_mesh(f);
  free(f->octs);
  if (level < 0) level = 0;
  if (level >= OO_MAX_LEVEL) level = OO_MAX_LEVEL - 1;
  long ne = 1L << level;
  long n = ne * ne * ne * f->conn->num_blocks;
  f->octs = (oo_oct *)malloc(sizeof(oo_oct) * (size_t)(n > 0 ? n : 1));
  int32_t h = side(level);
  long k = 0;
  for (int b = 0; b < f->conn->num_blocks; b++)
    for (int32_t x = 0; x < OO_HMAX; x += h)
      for (int32_t y = 0; y < OO_HMAX; y += h)
        for (int32_t z = 0; z < OO_HMAX; z += h) {
          oo_oct o = {b, x, y, z, 0, (int16_t)level, 0};
          f->octs[k++] = o;
        }
  f->noct = sort_elements(f->octs, n);
  set_tags(f);
}

/* TMROctForest::refine (TMROctForest.cpp:2169-2329), one rank. */
void oo_refine(oo_forest *f, const int *ref, int min_level, int max_level) {
  free_mesh(f);
  if (min_level < 0) min_level = 0;
  if (max_level > OO_MAX_LEVEL) max_level = OO_MAX_LEVEL;
  if (min_level > max_level) min_level = max_level;
  oset s;
  oset_init(&s);
  for (long i = 0; i < f->noct; i++) {
    oo_oct o = f->octs[i];
    if (ref) {
      if (ref[i] == 0) {
        oset_add(&s, &o);
      } else if (ref[i] < 0) {
        if (o.level > min_level) {
          int nl = o.level + ref[i];
          if (nl < min_level) nl = min_level;
          oo_oct q = o;
          q.level = (int16_t)nl;
          q.info = 0;
          int32_t h = side(nl);
          q.x -= q.x % h;
          q.y -= q.y % h;
          q.z -= q.z % h;
          oset_add(&s, &q);
        } else {
          oset_add(&s, &o);
        }
      } else {
        if (o.level < max_level) {
          int nl = o.level + ref[i];
          if (nl > max_level) nl = max_level;
          int r = nl - o.level;
          r = (r <= 0) ? 1 : (1 << (r - 1));
          oo_oct q = o;
          q.level = (int16_t)nl;
          q.info = 0;
          int32_t h = side(nl);
          int32_t x0 = q.x - q.x % h, y0 = q.y - q.y % h, z0 = q.z - q.z % h;
          for (int ii = 0; ii < r; ii++)
            for (int jj = 0; jj < r; jj++)
              for (int kk = 0; kk < r; kk++) {
                q.x = x0 + 2 * ii * h;
                q.y = y0 + 2 * jj * h;
                q.z = z0 + 2 * kk * h;
                oset_add(&s, &q);
              }
        } else {
          oset_add(&s, &o);
        }
      }
    } else {
      if (o.level < max_level) {
        oo_oct q = o;
        q.level += 1;
        q.info = 0;
        q = sibling(&q, 0);
        oset_add(&s, &q);
      } else {
        oset_add(&s, &o);
      }
    }
  }
  free(f->octs);
  f->octs = s.items;
  f->noct = sort_elements(s.items, s.n);
  s.items = NULL;
  free(s.slots);
  set_tags(f);
}

static oo_forest *new_like(oo_forest *f) {
  oo_forest *c = oo_forest_create(f->order, f->interp);
  c->conn = f->conn;
  if (c->conn) c->conn->refcount++;
  return c;
}

/* TMROctForest::duplicate (TMROctForest.cpp:2097-2109). */
oo_forest *oo_duplicate(oo_forest *f) {
  oo_forest *c = new_like(f);
  c->noct = f->noct;
  c->octs = (oo_oct *)malloc(sizeof(oo_oct) * (size_t)(f->noct ? f->noct : 1));
  memcpy(c->octs, f->octs, sizeof(oo_oct) * (size_t)f->noct);
  return c;
}

/* TMROctForest::coarsen (TMROctForest.cpp:2119-2164): the parent of
   every child-0, level-0 octants kept, in array order. */
oo_forest *oo_coarsen(oo_forest *f) {
  oo_forest *c = new_like(f);
  c->octs = (oo_oct *)malloc(sizeof(oo_oct) * (size_t)(f->noct ? f->noct : 1));
  long k = 0;
  for (long i = 0; i < f->noct; i++) {
    if (f->octs[i].level > 0) {
      if (child_id(&f->octs[i]) == 0) c->octs[k++] = parent_of(&f->octs[i]);
    } else {
      c->octs[k++] = f->octs[i];
    }
  }
  c->noct = k;
  set_tags(c);
  return c;
}

/* ------------------------------------------------------------------ */
/* Balance (TMROctForest.cpp:2525-3089). */
static int in_tree(const oo_oct *q) {
  return q->x >= 0 && q->x < OO_HMAX && q->y >= 0 && q->y < OO_HMAX &&
         q->z >= 0 && q->z < OO_HMAX;
}
static void bal_add(oset *s, olist *queue, const oo_oct *q) {
  if (oset_add(s, q)) ol_push(queue, q);
}
/* addFaceNeighbors (TMROctForest.cpp:2525-2584): q's parent-sized box
   (side 2h) mapped across block face `fi`. */
static void bal_face(oo_forest *f, int fi, const oo_oct *q, oset *s,
                     olist *queue) {
  oo_conn *c = f->conn;
  int b = q->block;
  int face = c->block_face_conn[6 * b + fi];
  int id = c->block_face_ids[6 * b + fi];
  int32_t h = side(q->level), ext = OO_HMAX - 2 * h;
  int32_t u, v;
  if (fi < 2)
    face_get(id, ext, q->y, q->z, &u, &v);
  else if (fi < 4)
    face_get(id, ext, q->x, q->z, &u, &v);
  else
    face_get(id, ext, q->x, q->y, &u, &v);
  for (int p = c->face_block_ptr[face]; p < c->face_block_ptr[face + 1]; p++) {
    int ab = c->face_block_conn[p] / 6, af = c->face_block_conn[p] % 6;
    if (ab == b) continue;
    int aid = c->block_face_ids[6 * ab + af];
    oo_oct n = {ab, 0, 0, 0, 0, q->level, 0};
    if (af < 2) {
      n.x = ext * (af % 2);
      face_set(aid, ext, u, v, &n.y, &n.z);
    } else if (af < 4) {
      n.y = ext * (af % 2);
      face_set(aid, ext, u, v, &n.x, &n.z);
    } else {
      n.z = ext * (af % 2);
      face_set(aid, ext, u, v, &n.x, &n.y);
    }
    bal_add(s, queue, &n);
  }
}
/* addEdgeNeighbors (TMROctForest.cpp:2601-2671). */
static void bal_edge(oo_forest *f, int ei, const oo_oct *q, oset *s,
                     olist *queue) {
  oo_conn *c = f->conn;
  int b = q->block;
  int edge = c->block_edge_conn[12 * b + ei];
  int32_t h = side(q->level), ext = OO_HMAX - 2 * h;
  int32_t uc = (ei < 4) ? q->x : (ei < 8) ? q->y : q->z;
  int a1, a2;
  edge_corners(ei, &a1, &a2);
  int n1 = c->block_conn[8 * b + a1], n2 = c->block_conn[8 * b + a2];
  for (int p = c->edge_block_ptr[edge]; p < c->edge_block_ptr[edge + 1]; p++) {
    int ab = c->edge_block_conn[p] / 12, ae = c->edge_block_conn[p] % 12;
    if (ab == b) continue;
    int c1, c2;
    edge_corners(ae, &c1, &c2);
    int m1 = c->block_conn[8 * ab + c1], m2 = c->block_conn[8 * ab + c2];
    int32_t u = (n1 == m2 && n2 == m1) ? ext - uc : uc;
    oo_oct n = {ab, 0, 0, 0, 0, q->level, 0};
    if (ae < 4) {
      n.x = u;
      n.y = ext * (ae % 2);
      n.z = ext * (ae / 2);
    } else if (ae < 8) {
      n.x = ext * (ae % 2);
      n.y = u;
      n.z = ext * ((ae - 4) / 2);
    } else {
      n.x = ext * (ae % 2);
      n.y = ext * ((ae - 8) / 2);
      n.z = u;
    }
    bal_add(s, queue, &n);
  }
}
/* addCornerNeighbors (TMROctForest.cpp:2688-2745). */
static void bal_corner(oo_forest *f, int ci, const oo_oct *q, oset *s,
                       olist *queue) {
  oo_conn *c = f->conn;
  int b = q->block;
  int node = c->block_conn[8 * b + ci];
  int32_t h = side(q->level), ext = OO_HMAX - 2 * h;
  for (int p = c->node_block_ptr[node]; p < c->node_block_ptr[node + 1];
       p++) {
    int ab = c->node_block_conn[p] / 8, ac = c->node_block_conn[p] % 8;
    if (ab == b) continue;
    oo_oct n = {ab, ext * (ac % 2), ext * ((ac % 4) / 2), ext * (ac / 4),
                0, q->level, 0};
    bal_add(s, queue, &n);
  }
}
static void bal_outside(oo_forest *f, const oo_oct *q, oset *s, olist *queue,
                        int allow_corner) {
  int ex = (q->x < 0 || q->x >= OO_HMAX);
  int ey = (q->y < 0 || q->y >= OO_HMAX);
  int ez = (q->z < 0 || q->z >= OO_HMAX);
  if (allow_corner && ex && ey && ez) {
    int ci = (q->x < 0 ? 0 : 1) + (q->y < 0 ? 0 : 2) + (q->z < 0 ? 0 : 4);
    bal_corner(f, ci, q, s, queue);
  } else if ((ex && ey) || (ex && ez) || (ey && ez)) {
    int e;
    if (ey && ez)
      e = (q->y < 0 ? 0 : 1) + (q->z < 0 ? 0 : 2);
    else if (ex && ez)
      e = (q->x < 0 ? 4 : 5) + (q->z < 0 ? 0 : 2);
    else
      e = (q->x < 0 ? 8 : 9) + (q->y < 0 ? 0 : 2);
    bal_edge(f, e, q, s, queue);
  } else {
    int fi;
    if (ex)
      fi = q->x < 0 ? 0 : 1;
    else if (ey)
      fi = q->y < 0 ? 2 : 3;
    else
      fi = q->z < 0 ? 4 : 5;
    bal_face(f, fi, q, s, queue);
  }
}
/* balanceOctant (TMROctForest.cpp:2763-2895). */
static void balance_octant(oo_forest *f, const oo_oct *o, oset *s,
                           olist *queue, int corner) {
  if (o->level <= 1) return;
  oo_oct p = parent_of(o);
  for (int fi = 0; fi < 6; fi++) {
    oo_oct n = face_nbr(&p, fi);
    oo_oct q = sibling(&n, 0);
    if (in_tree(&q))
      bal_add(s, queue, &q);
    else
      bal_outside(f, &q, s, queue, 0);
  }
  for (int e = 0; e < 12; e++) {
    oo_oct n = edge_nbr(&p, e);
    oo_oct q = sibling(&n, 0);
    if (in_tree(&q))
      bal_add(s, queue, &q);
    else
      bal_outside(f, &q, s, queue, 0);
  }
  if (corner) {
    for (int ci = 0; ci < 8; ci++) {
      oo_oct n = corner_nbr(&p, ci);
      oo_oct q = sibling(&n, 0);
      if (in_tree(&q))
        bal_add(s, queue, &q);
      else
        bal_outside(f, &q, s, queue, 1);
    }
  }
}

void oo_balance(oo_forest *f, int corner) {
  free_mesh(f);
  oset s;
  oset_init(&s);
  olist queue;
  ol_init(&queue);
  for (long i = 0; i < f->noct; i++) {
    oo_oct q = sibling(&f->octs[i], 0);
    oset_add(&s, &q);
    balance_octant(f, &q, &s, &queue, corner);
  }
  while (queue.head < queue.n) {
    oo_oct q = queue.a[queue.head++];
    balance_octant(f, &q, &s, &queue, corner);
  }
  free(queue.a);
  /* Sibling expansion (TMROctForest.cpp:3039-3053), then sort and keep
     the finest octant at each position. */
  long n0 = s.n;
  for (long i = 0; i < n0; i++) {
    oo_oct q = s.items[i];
    if (q.level > 0) {
      for (int j = 0; j < 8; j++) {
        oo_oct t = sibling(&q, j);
        oset_add(&s, &t);
      }
    }
  }
  free(f->octs);
  f->octs = s.items;
  f->noct = sort_elements(s.items, s.n);
  s.items = NULL;
  free(s.slots);
  set_tags(f);
}

/* ------------------------------------------------------------------ */
/* createNodes and its helpers (TMROctForest.cpp:3455-5519). */
static long find_elem(oo_forest *f, const oo_oct *q) {
  return bsearch_oct(f->octs, f->noct, q, cmp_octant);
}
/* checkAdjacentFaces (TMROctForest.cpp:3464-3513). */
static int adj_face_exists(oo_forest *f, int fi, const oo_oct *nb) {
  oo_conn *c = f->conn;
  int32_t h = side(nb->level), ext = OO_HMAX - h;
  int b = nb->block;
  int face = c->block_face_conn[6 * b + fi];
  int id = c->block_face_ids[6 * b + fi];
  int32_t u, v;
  if (fi < 2)
    face_get(id, ext, nb->y, nb->z, &u, &v);
  else if (fi < 4)
    face_get(id, ext, nb->x, nb->z, &u, &v);
  else
    face_get(id, ext, nb->x, nb->y, &u, &v);
  for (int p = c->face_block_ptr[face]; p < c->face_block_ptr[face + 1]; p++) {
    int ab = c->face_block_conn[p] / 6, af = c->face_block_conn[p] % 6;
    if (ab == b) continue;
    int aid = c->block_face_ids[6 * ab + af];
    oo_oct o = {ab, 0, 0, 0, 0, nb->level, 0};
    if (af < 2) {
      o.x = ext * (af % 2);
      face_set(aid, ext, u, v, &o.y, &o.z);
    } else if (af < 4) {
      o.y = ext * (af % 2);
      face_set(aid, ext, u, v, &o.x, &o.z);
    } else {
      o.z = ext * (af % 2);
      face_set(aid, ext, u, v, &o.x, &o.y);
    }
    if (find_elem(f, &o) >= 0) return 1;
  }
  return 0;
}
/* checkAdjacentEdges (TMROctForest.cpp:3524-3605). */
static int adj_edge_exists(oo_forest *f, int ei, const oo_oct *nb) {
  oo_conn *c = f->conn;
  int32_t h = side(nb->level), ext = OO_HMAX - h;
  int b = nb->block;
  int32_t uc = (ei < 4) ? nb->x : (ei < 8) ? nb->y : nb->z;
  int edge = c->block_edge_conn[12 * b + ei];
  int a1, a2;
  edge_corners(ei, &a1, &a2);
  int n1 = c->block_conn[8 * b + a1], n2 = c->block_conn[8 * b + a2];
  for (int p = c->edge_block_ptr[edge]; p < c->edge_block_ptr[edge + 1]; p++) {
    int ab = c->edge_block_conn[p] / 12, ae = c->edge_block_conn[p] % 12;
    if (ab == b) continue;
    int c1, c2;
    edge_corners(ae, &c1, &c2);
    int m1 = c->block_conn[8 * ab + c1], m2 = c->block_conn[8 * ab + c2];
    int32_t u = (n1 == m2 && n2 == m1) ? ext - uc : uc;
    oo_oct o = {ab, 0, 0, 0, 0, nb->level, 0};
    if (ae < 4) {
      o.x = u;
      o.y = ext * (ae % 2);
      o.z = ext * (ae / 2);
    } else if (ae < 8) {
      o.x = ext * (ae % 2);
      o.y = u;
      o.z = ext * ((ae - 4) / 2);
    } else {
      o.x = ext * (ae % 2);
      o.y = ext * ((ae - 8) / 2);
      o.z = u;
    }
    if (find_elem(f, &o) >= 0) return 1;
  }
  return 0;
}
static int encode_info(const oo_oct *o, int face_info, int edge_info) {
  int id = child_id(o), info = 0;
  for (int k = 0; k < 3; k++) {
    if (face_info & (1 << child_face(id, k))) info |= 1 << k;
    if (edge_info & (1 << child_edge(id, k))) info |= 1 << (k + 3);
  }
  return info;
}
static void decode_info(const oo_oct *o, int info, int *face_info,
                        int *edge_info) {
  int id = child_id(o), fi = 0, ei = 0;
  for (int k = 0; k < 3; k++) {
    if (info & (1 << k)) {
      fi |= 1 << child_face(id, k);
      for (int j = 0; j < 2; j++) ei |= 1 << child_face_edge(id, k, j);
    }
    if (info & (1 << (k + 3))) ei |= 1 << child_edge(id, k);
  }
  if (face_info) *face_info = fi;
  if (edge_info) *edge_info = ei;
}
/* computeDepFacesAndEdges (TMROctForest.cpp:3619-3702). */
static void dep_faces_edges(oo_forest *f) {
  for (long i = 0; i < f->noct; i++) {
    oo_oct *o = &f->octs[i];
    int fi_bits = 0, ei_bits = 0;
    if (o->level > 0) {
      int id = child_id(o);
      oo_oct p = parent_of(o);
      for (int k = 0; k < 3; k++) {
        int fi = child_face(id, k);
        oo_oct n = face_nbr(&p, fi);
        if (in_tree(&n)) {
          if (find_elem(f, &n) >= 0) fi_bits |= 1 << fi;
        } else if (adj_face_exists(f, fi, &n)) {
          fi_bits |= 1 << fi;
        }
      }
      for (int k = 0; k < 3; k++) {
        int e = child_edge(id, k);
        oo_oct n = edge_nbr(&p, e);
        int fx0 = n.x < 0, fy0 = n.y < 0, fz0 = n.z < 0;
        int fx = fx0 || n.x >= OO_HMAX, fy = fy0 || n.y >= OO_HMAX,
            fz = fz0 || n.z >= OO_HMAX;
        if ((fx && fy) || (fy && fz) || (fx && fz)) {
          if (adj_edge_exists(f, e, &n)) ei_bits |= 1 << e;
        } else if (fx || fy || fz) {
          int fi = fx * (fx0 ? 0 : 1) + fy * (fy0 ? 2 : 3) + fz * (fz0 ? 4 : 5);
          if (adj_face_exists(f, fi, &n)) ei_bits |= 1 << e;
        } else if (find_elem(f, &n) >= 0) {
          ei_bits |= 1 << e;
        }
      }
      o->info = (int16_t)encode_info(o, fi_bits, ei_bits);
    } else {
      o->info = 0;
    }
  }
}

/* transformNode (TMROctForest.cpp:3847-4039). */
static void transform_node(oo_forest *f, oo_oct *o, int edge_dir,
                           int *edge_rev, int *src_face_id) {
  oo_conn *c = f->conn;
  const int32_t hmax = OO_HMAX;
  int fx0 = o->x == 0, fy0 = o->y == 0, fz0 = o->z == 0;
  int fx = fx0 || o->x == hmax, fy = fy0 || o->y == hmax,
      fz = fz0 || o->z == hmax;
  if (edge_rev) *edge_rev = 0;
  if (src_face_id) *src_face_id = 0;
  if (!(fx || fy || fz)) return;
  int b = o->block;
  if (fx && fy && fz) {
    int corner = (fx0 ? 0 : 1) + (fy0 ? 0 : 2) + (fz0 ? 0 : 4);
    int node = c->block_conn[8 * b + corner];
    if (b != c->node_owner[node]) {
      int e = c->node_block_conn[c->node_block_ptr[node]];
      int ab = e / 8, ac = e % 8;
      o->block = ab;
      o->x = hmax * (ac % 2);
      o->y = hmax * ((ac % 4) / 2);
      o->z = hmax * (ac / 4);
    }
  } else if ((fy && fz) || (fx && fz) || (fx && fy)) {
    int ei;
    int32_t u;
    if (fy && fz) {
      ei = (fy0 ? 0 : 1) + (fz0 ? 0 : 2);
      u = o->x;
    } else if (fx && fz) {
      ei = (fx0 ? 4 : 5) + (fz0 ? 0 : 2);
      u = o->y;
    } else {
      ei = (fx0 ? 8 : 9) + (fy0 ? 0 : 2);
      u = o->z;
    }
    int edge = c->block_edge_conn[12 * b + ei];
    if (b != c->edge_owner[edge]) {
      int e = c->edge_block_conn[c->edge_block_ptr[edge]];
      int ab = e / 12, ae = e % 12;
      int a1, a2, c1, c2;
      edge_corners(ei, &a1, &a2);
      edge_corners(ae, &c1, &c2);
      int n1 = c->block_conn[8 * b + a1], n2 = c->block_conn[8 * b + a2];
      int m1 = c->block_conn[8 * ab + c1], m2 = c->block_conn[8 * ab + c2];
      int rev = (n1 == m2 && n2 == m1);
      if (edge_rev) *edge_rev = rev;
      int32_t uo = rev ? hmax - u : u;
      o->block = ab;
      if (ae < 4) {
        o->x = uo;
        o->y = hmax * (ae % 2);
        o->z = hmax * (ae / 2);
      } else if (ae < 8) {
        o->x = hmax * (ae % 2);
        o->y = uo;
        o->z = hmax * ((ae - 4) / 2);
      } else {
        o->x = hmax * (ae % 2);
        o->y = hmax * ((ae - 8) / 2);
        o->z = uo;
      }
    }
  } else {
    int fi = fx * (fx0 ? 0 : 1) + fy * (fy0 ? 2 : 3) + fz * (fz0 ? 4 : 5);
    int face = c->block_face_conn[6 * b + fi];
    if (b != c->face_owner[face]) {
      int id = c->block_face_ids[6 * b + fi];
      if (src_face_id) *src_face_id = id;
      int32_t u, v;
      if (fi < 2)
        face_get(id, hmax, o->y, o->z, &u, &v);
      else if (fi < 4)
        face_get(id, hmax, o->x, o->z, &u, &v);
      else
        face_get(id, hmax, o->x, o->y, &u, &v);
      if (edge_rev) {
        int32_t x = 0, y = 0, z = 0;
        if (edge_dir == 0)
          x = 1;
        else if (edge_dir == 1)
          y = 1;
        else if (edge_dir == 2)
          z = 1;
        if (fi < 2)
          face_get(id, 0, y, z, &y, &z);
        else if (fi < 4)
          face_get(id, 0, x, z, &x, &z);
        else
          face_get(id, 0, x, y, &x, &y);
        *edge_rev = (x < 0 || y < 0 || z < 0);
      }
      int e = c->face_block_conn[c->face_block_ptr[face]];
      int ab = e / 6, af = e % 6;
      o->block = ab;
      if (af < 2) {
        o->x = hmax * (af % 2);
        o->y = u;
        o->z = v;
      } else if (af < 4) {
        o->x = u;
        o->y = hmax * (af % 2);
        o->z = v;
      } else {
        o->x = u;
        o->y = v;
        o->z = hmax * (af % 2);
      }
    }
  }
  if (o->x == hmax) o->x = hmax - 1;
  if (o->y == hmax) o->y = hmax - 1;
  if (o->z == hmax) o->z = hmax - 1;
}

/* Node labels (initLabel, TMROctForest.cpp:6798-6811). */
static void node_labels(int order, int interp, int lab[4]) {
  if (order > 3 || (order >= 3 && interp == 2)) {
    for (int i = 0; i < 4; i++) lab[i] = i;
  } else {
    for (int i = 0; i < 4; i++) lab[i] = 0;
  }
}

typedef struct {
  oo_oct *a;
  long n;
  int *offset; /* node_offset */
} onodes;

static long node_find(const onodes *N, const oo_oct *q) {
  return bsearch_oct(N->a, N->n, q, cmp_node);
}

/* createLocalNodes (TMROctForest.cpp:4290-4640), one rank. */
static void create_local_nodes(oo_forest *f, onodes *N) {
  int order = f->order;
  int lab[4];
  node_labels(order, f->interp, lab);
  olist L;
  ol_init(&L);
  for (long i = 0; i < f->noct; i++) {
    const oo_oct *e = &f->octs[i];
    if (order == 2) {
      int32_t h = side(e->level);
      for (int kk = 0; kk < 2; kk++)
        for (int jj = 0; jj < 2; jj++)
          for (int ii = 0; ii < 2; ii++) {
            oo_oct n = {e->block, e->x + h * ii, e->y + h * jj, e->z + h * kk,
                        0, 1, (int16_t)lab[0]};
            transform_node(f, &n, -1, NULL, NULL);
            ol_push(&L, &n);
          }
    } else {
      int32_t h = (int32_t)1 << (OO_MAX_LEVEL - e->level - 1);
      for (int kk = 0; kk < 3; kk++)
        for (int jj = 0; jj < 3; jj++)
          for (int ii = 0; ii < 3; ii++) {
            oo_oct n = {e->block, e->x + h * ii, e->y + h * jj, e->z + h * kk,
                        0, 0, 0};
            int fx = (ii != 1), fy = (jj != 1), fz = (kk != 1);
            if (fx && fy && fz) {
              n.level = 1;
              n.info = (int16_t)lab[0];
            } else if ((fy && fz) || (fx && fz) || (fx && fy)) {
              n.level = (int16_t)(order - 2);
              n.info = (int16_t)lab[1];
            } else if (fx || fy || fz) {
              n.level = (int16_t)((order - 2) * (order - 2));
              n.info = (int16_t)lab[2];
            } else {
              n.level = (int16_t)((order - 2) * (order - 2) * (order - 2));
              n.info = (int16_t)lab[3];
            }
            transform_node(f, &n, -1, NULL, NULL);
            ol_push(&L, &n);
          }
    }
  }
  /* Nodes the dependent relations refer to (TMROctForest.cpp:4375-4532);
     these carry tag -1 and lose to any element node at the same key. */
  for (long i = 0; i < f->noct; i++) {
    const oo_oct *e = &f->octs[i];
    if (!e->info) continue;
    int fi_bits, ei_bits;
    decode_info(e, e->info, &fi_bits, &ei_bits);
    oo_oct p = parent_of(e);
    int32_t h = side(e->level), hp = side(p.level);
    for (int ei = 0; ei < 12; ei++) {
      if (!(ei_bits & (1 << ei))) continue;
      int np = (order == 2) ? 2 : 3;
      int32_t step = (order == 2) ? hp : h;
      for (int ii = 0; ii < np; ii++) {
        oo_oct n = {p.block, 0, 0, 0, -1, 1, (int16_t)lab[0]};
        if (ei < 4) {
          n.x = p.x + ii * step;
          n.y = p.y + hp * (ei % 2);
          n.z = p.z + hp * (ei / 2);
        } else if (ei < 8) {
          n.x = p.x + hp * (ei % 2);
          n.y = p.y + ii * step;
          n.z = p.z + hp * ((ei - 4) / 2);
        } else {
          n.x = p.x + hp * (ei % 2);
          n.y = p.y + hp * ((ei - 8) / 2);
          n.z = p.z + ii * step;
        }
        if (order > 2 && ii == 1) {
          n.info = (int16_t)lab[1];
          n.level = (int16_t)(order - 2);
        }
        transform_node(f, &n, -1, NULL, NULL);
        ol_push(&L, &n);
      }
    }
    for (int fi = 0; fi < 6; fi++) {
      if (!(fi_bits & (1 << fi))) continue;
      int np = (order == 2) ? 2 : 3;
      int32_t step = (order == 2) ? hp : h;
      for (int jj = 0; jj < np; jj++)
        for (int ii = 0; ii < np; ii++) {
          oo_oct n = {p.block, 0, 0, 0, -1, 1, (int16_t)lab[0]};
          if (fi < 2) {
            n.x = p.x + hp * (fi % 2);
            n.y = p.y + ii * step;
            n.z = p.z + jj * step;
          } else if (fi < 4) {
            n.x = p.x + ii * step;
            n.y = p.y + hp * (fi % 2);
            n.z = p.z + jj * step;
          } else {
            n.x = p.x + ii * step;
            n.y = p.y + jj * step;
            n.z = p.z + hp * (fi % 2);
          }
          if (order > 2) {
            int ei2 = (ii == 0 || ii == 2), ej2 = (jj == 0 || jj == 2);
            if (ei2 && ej2) {
              n.info = (int16_t)lab[0];
              n.level = 1;
            } else if (ei2 || ej2) {
              n.info = (int16_t)lab[1];
              n.level = (int16_t)(order - 2);
            } else {
              n.info = (int16_t)lab[2];
              n.level = (int16_t)((order - 2) * (order - 2));
            }
          }
          transform_node(f, &n, -1, NULL, NULL);
          ol_push(&L, &n);
        }
    }
  }
  /* Hash semantics: first insertion of each node key wins. */
  stable_sort(L.a, L.n, cmp_node);
  N->n = unique_first(L.a, L.n, cmp_node);
  N->a = L.a;
}

static int node_index(oo_forest *f, const onodes *N, oo_oct *q, int edge_dir,
                      int *rev, int *fid) {
  transform_node(f, q, edge_dir, rev, fid);
  long t = node_find(N, q);
  if (t < 0) {
    fprintf(stderr, "tmr_oracle: node not found\n");
    abort();
  }
  return (int)t;
}

/* createLocalConn (TMROctForest.cpp:4660-4867). */
static void create_local_conn(oo_forest *f, const onodes *N) {
  int o = f->order, npe = o * o * o;
  int lab[4];
  node_labels(o, f->interp, lab);
  f->econn = (int *)calloc((size_t)npe * (size_t)(f->noct ? f->noct : 1),
                           sizeof(int));
  for (long i = 0; i < f->noct; i++) {
    int *c = &f->econn[npe * i];
    const oo_oct *e = &f->octs[i];
    int32_t h = (int32_t)1 << (OO_MAX_LEVEL - e->level - 1);
    for (int kk = 0; kk < 2; kk++)
      for (int jj = 0; jj < 2; jj++)
        for (int ii = 0; ii < 2; ii++) {
          oo_oct n = {e->block, e->x + 2 * h * ii, e->y + 2 * h * jj,
                      e->z + 2 * h * kk, 0, 0, (int16_t)lab[0]};
          int t = node_index(f, N, &n, -1, NULL, NULL);
          c[(o - 1) * ii + (o - 1) * o * jj + (o - 1) * o * o * kk] =
              N->offset[t];
        }
    if (o < 3) continue;
    for (int ei = 0; ei < 12; ei++) {
      oo_oct n = {e->block, 0, 0, 0, 0, 0, (int16_t)lab[1]};
      if (ei < 4) {
        n.x = e->x + h;
        n.y = e->y + 2 * h * (ei % 2);
        n.z = e->z + 2 * h * (ei / 2);
      } else if (ei < 8) {
        n.x = e->x + 2 * h * (ei % 2);
        n.y = e->y + h;
        n.z = e->z + 2 * h * ((ei - 4) / 2);
      } else {
        n.x = e->x + 2 * h * (ei % 2);
        n.y = e->y + 2 * h * ((ei - 8) / 2);
        n.z = e->z + h;
      }
      int rev = 0;
      int t = node_index(f, N, &n, ei / 4, &rev, NULL);
      for (int a = 1; a < o - 1; a++) {
        int off;
        if (ei < 4)
          off = a + (o - 1) * (ei % 2) * o + (o - 1) * (ei / 2) * o * o;
        else if (ei < 8)
          off = (o - 1) * (ei % 2) + a * o + (o - 1) * ((ei - 4) / 2) * o * o;
        else
          off = (o - 1) * (ei % 2) + (o - 1) * ((ei - 8) / 2) * o + a * o * o;
        c[off] = N->offset[t] + (rev ? o - 2 - a : a - 1);
      }
    }
    for (int fi = 0; fi < 6; fi++) {
      oo_oct n = {e->block, 0, 0, 0, 0, 0, (int16_t)lab[2]};
      if (fi < 2) {
        n.x = e->x + 2 * h * (fi % 2);
        n.y = e->y + h;
        n.z = e->z + h;
      } else if (fi < 4) {
        n.x = e->x + h;
        n.y = e->y + 2 * h * (fi % 2);
        n.z = e->z + h;
      } else {
        n.x = e->x + h;
        n.y = e->y + h;
        n.z = e->z + 2 * h * (fi % 2);
      }
      int fid = 0;
      int t = node_index(f, N, &n, -1, NULL, &fid);
      for (int b2 = 1; b2 < o - 1; b2++)
        for (int a = 1; a < o - 1; a++) {
          int32_t u, v;
          face_get(fid, o - 1, a, b2, &u, &v);
          int off;
          if (fi < 2)
            off = (o - 1) * (fi % 2) + a * o + b2 * o * o;
          else if (fi < 4)
            off = a + (o - 1) * (fi % 2) * o + b2 * o * o;
          else
            off = a + b2 * o + (o - 1) * (fi % 2) * o * o;
          c[off] = N->offset[t] + (u - 1) + (v - 1) * (o - 2);
        }
    }
    oo_oct n = {e->block, e->x + h, e->y + h, e->z + h, 0, 0, (int16_t)lab[3]};
    int t = node_index(f, N, &n, -1, NULL, NULL);
    for (int kk = 1; kk < o - 1; kk++)
      for (int jj = 1; jj < o - 1; jj++)
        for (int ii = 1; ii < o - 1; ii++)
          c[ii + jj * o + kk * o * o] = N->offset[t] + (ii - 1) +
                                        (jj - 1) * (o - 2) +
                                        (kk - 1) * (o - 2) * (o - 2);
  }
}

/* Start/end of the dependent run along an element edge
   (labelDependentNodes, TMROctForest.cpp:3741-3760). */
static void dep_edge_range(oo_forest *f, int id, int ei, int *start,
                           int *end) {
  int o = f->order;
  int s = (ei < 4) ? (id & 1) : (ei < 8) ? ((id >> 1) & 1) : (id >> 2);
  int m3 = (o == 3 && f->interp != 2);
  if (s == 0) {
    *start = 1;
    *end = m3 ? o - 1 : o;
  } else {
    *start = m3 ? 1 : 0;
    *end = o - 1;
  }
}
static int edge_offset(int o, int ei, int a) {
  if (ei < 4) return a + (o - 1) * (ei % 2) * o + (o - 1) * (ei / 2) * o * o;
  if (ei < 8) return (o - 1) * (ei % 2) + a * o + (o - 1) * ((ei - 4) / 2) * o * o;
  return (o - 1) * (ei % 2) + (o - 1) * ((ei - 8) / 2) * o + a * o * o;
}
static int face_offset(int o, int fi, int a, int b) {
  if (fi < 2) return (o - 1) * (fi % 2) + a * o + b * o * o;
  if (fi < 4) return a + (o - 1) * (fi % 2) * o + b * o * o;
  return a + b * o + (o - 1) * (fi % 2) * o * o;
}

/* labelDependentNodes (TMROctForest.cpp:3711-3832). */
static void label_dependent(oo_forest *f, int *nodes) {
  int o = f->order, npe = o * o * o;
  for (long i = 0; i < f->noct; i++) {
    const oo_oct *e = &f->octs[i];
    if (!e->info) continue;
    int fi_bits, ei_bits;
    decode_info(e, e->info, &fi_bits, &ei_bits);
    const int *c = &f->econn[npe * i];
    for (int fi = 0; fi < 6; fi++)
      if (fi_bits & (1 << fi))
        for (int k = 0; k < 4; k++) ei_bits |= 1 << face_edge(fi, k);
    int id = child_id(e);
    for (int ei = 0; ei < 12; ei++) {
      if (!(ei_bits & (1 << ei))) continue;
      int s, en;
      dep_edge_range(f, id, ei, &s, &en);
      for (int a = s; a < en; a++) nodes[c[edge_offset(o, ei, a)]] = -1;
    }
    for (int fi = 0; fi < 6; fi++) {
      if (!(fi_bits & (1 << fi))) continue;
      for (int b2 = 1; b2 < o - 1; b2++)
        for (int a = 1; a < o - 1; a++) nodes[c[face_offset(o, fi, a, b2)]] = -1;
    }
  }
}

/* eval_bernstein_weights (TMRInterpolation.h:309-439): the weights of the
   coarse edge's Bernstein control points for the control point u of the two
   refined half-edges, u in [-(order-1), order-1].  The reference lists the
   de Casteljau subdivision at t = 1/2 for orders 2-5: control point r of the
   left half (u = r - (order-1)) takes C(r, i) / 2^r of coarse point i <= r,
   control point r of the right half (u = r) takes
   C(order-1-r, i-r) / 2^(order-1-r) of coarse point i >= r.  Every value is
   a short dyadic fraction, exact in double.  Returns 1 (and writes nothing,
   as the reference writes nothing) for orders outside 2-5. */
static int bernstein_dep_weights(int order, int u, double *N) {
  if (order < 2 || order > 5) return 1;
  int p = order - 1;
  for (int i = 0; i < order; i++) N[i] = 0.0;
  if (u <= 0) {
    int r = u + p;
    double c = 1.0;
    for (int i = 0; i <= r; i++) {
      N[i] = c / (double)(1 << r);
      c = c * (r - i) / (i + 1);
    }
  } else {
    int r = u, m = p - r;
    double c = 1.0;
    for (int i = 0; i <= m; i++) {
      N[r + i] = c / (double)(1 << m);
      c = c * (m - i) / (i + 1);
    }
  }
  return 0;
}

/* eval_bernstein_interp_weights (TMRInterpolation.h:441-560): degree
   elevation weights of fine control point u on a coarse element one order
   lower, exactly as the reference tabulates them.  Note that for coarse
   order 4 the reference's rows u = 2 and u = 3 are the natural elevation
   rows of u = 3 and u = 2 (the table is reproduced as written).  Returns 1
   when the orders differ by more than one or the coarse order is outside
   2-5 (the reference leaves N unset then). */
static int bernstein_interp_weights(int mo, int co, int u, double *N) {
  if (mo - co != 1 || co < 2 || co > 5 || u < 0 || u > mo - 1) return 1;
  for (int i = 0; i < co; i++) N[i] = 0.0;
  if (u == 0) {
    N[0] = 1.0;
  } else if (u == mo - 1) {
    N[co - 1] = 1.0;
  } else if (co == 2) {
    N[0] = 0.5; N[1] = 0.5;
  } else if (co == 3) {
    if (u == 1) { N[0] = 1. / 3; N[1] = 2. / 3; }
    else { N[1] = 2. / 3; N[2] = 1. / 3; }
  } else if (co == 4) {
    if (u == 1) { N[0] = 0.25; N[1] = 0.75; }
    else if (u == 2) { N[2] = 0.75; N[3] = 0.25; }
    else { N[1] = 0.5; N[2] = 0.5; }
  } else {
    if (u == 1) { N[0] = 0.2; N[1] = 0.8; }
    else if (u == 2) { N[1] = 0.4; N[2] = 0.6; }
    else if (u == 3) { N[2] = 0.6; N[3] = 0.4; }
    else { N[3] = 0.8; N[4] = 0.2; }
  }
  return 0;
}

/* bernstein_shape_functions (TMRInterpolation.h:164-177): the Bernstein
   basis at u in [-1, 1] by the reference's triangular recurrence. */
static void bernstein(int order, double u, double *N) {
  double u1 = 0.5 * (1.0 - u), u2 = 0.5 * (u + 1.0);
  N[0] = 1.0;
  for (int j = 1; j < order; j++) {
    double s = 0.0;
    for (int k = 0; k < j; k++) {
      double t = N[k];
      N[k] = s + u1 * t;
      s = u2 * t;
    }
    N[j] = s;
  }
}

static void lagrange(int order, double u, const double *knots, double *N) {
  for (int i = 0; i < order; i++) {
    N[i] = 1.0;
    for (int j = 0; j < order; j++) {
      if (i != j) {
        double d = 1.0 / (knots[i] - knots[j]);
        N[i] *= (u - knots[j]) * d;
      }
    }
  }
}

/* getEdgeNodes (TMROctForest.cpp:4886-4963). */
static void parent_edge_nodes(oo_forest *f, const onodes *N, const oo_oct *p,
                              int ei, int *out) {
  int o = f->order;
  int32_t h = (int32_t)1 << (OO_MAX_LEVEL - p->level - 1);
  int32_t hp = side(p->level);
  int lab[4];
  node_labels(o, f->interp, lab);
  int np = (o == 2) ? 2 : 3;
  int32_t step = (o == 2) ? hp : h;
  for (int ii = 0; ii < np; ii++) {
    oo_oct n = {p->block, 0, 0, 0, 0, 1, 0};
    if (ei < 4) {
      n.x = p->x + ii * step;
      n.y = p->y + hp * (ei % 2);
      n.z = p->z + hp * (ei / 2);
    } else if (ei < 8) {
      n.x = p->x + hp * (ei % 2);
      n.y = p->y + ii * step;
      n.z = p->z + hp * ((ei - 4) / 2);
    } else {
      n.x = p->x + hp * (ei % 2);
      n.y = p->y + hp * ((ei - 8) / 2);
      n.z = p->z + ii * step;
    }
    if (o == 2 || ii != 1) {
      n.info = (int16_t)lab[0];
      int t = node_index(f, N, &n, -1, NULL, NULL);
      out[(o == 2) ? ii : (ii / 2) * (o - 1)] = N->offset[t];
    } else {
      n.info = (int16_t)lab[1];
      int rev = 0;
      int t = node_index(f, N, &n, ei / 4, &rev, NULL);
      for (int k = 1; k < o - 1; k++)
        out[k] = N->offset[t] + (rev ? o - 2 - k : k - 1);
    }
  }
}

/* getFaceNodes (TMROctForest.cpp:4984-5146). */
static void parent_face_nodes(oo_forest *f, const onodes *N, const oo_oct *p,
                              int fi, int *out) {
  int o = f->order;
  int32_t h = (int32_t)1 << (OO_MAX_LEVEL - p->level - 1);
  int lab[4];
  node_labels(o, f->interp, lab);
  int np = (o == 2) ? 2 : 3;
  int32_t step = (o == 2) ? 2 * h : h;
  for (int jj = 0; jj < np; jj++)
    for (int ii = 0; ii < np; ii++) {
      oo_oct n = {p->block, 0, 0, 0, 0, 1, 0};
      if (fi < 2) {
        n.x = p->x + 2 * h * (fi % 2);
        n.y = p->y + ii * step;
        n.z = p->z + jj * step;
      } else if (fi < 4) {
        n.x = p->x + ii * step;
        n.y = p->y + 2 * h * (fi % 2);
        n.z = p->z + jj * step;
      } else {
        n.x = p->x + ii * step;
        n.y = p->y + jj * step;
        n.z = p->z + 2 * h * (fi % 2);
      }
      if (o == 2) {
        n.info = (int16_t)lab[0];
        int t = node_index(f, N, &n, -1, NULL, NULL);
        out[ii + 2 * jj] = N->offset[t];
        continue;
      }
      int ci = (ii == 0 || ii == 2), cj = (jj == 0 || jj == 2);
      if (ci && cj) {
        n.info = (int16_t)lab[0];
        int t = node_index(f, N, &n, -1, NULL, NULL);
        out[(ii / 2) * (o - 1) + (jj / 2) * (o - 1) * o] = N->offset[t];
      } else if (ci || cj) {
        n.info = (int16_t)lab[1];
        int e = (ii == 0) ? 0 : (ii == 2) ? 1 : (jj == 0) ? 2 : 3;
        int rev = 0;
        int t = node_index(f, N, &n, face_edge(fi, e) / 4, &rev, NULL);
        int incr = 1, start = (jj / 2) * (o - 1) * o;
        if (ii == 0 || ii == 2) {
          incr = o;
          start = (ii / 2) * (o - 1);
        }
        for (int k = 1; k < o - 1; k++)
          out[start + k * incr] = N->offset[t] + (rev ? o - 2 - k : k - 1);
      } else {
        n.info = (int16_t)lab[2];
        int fid = 0;
        int t = node_index(f, N, &n, -1, NULL, &fid);
        for (int k = 1; k < o - 1; k++)
          for (int j = 1; j < o - 1; j++) {
            int32_t u, v;
            face_get(fid, o - 1, j, k, &u, &v);
            out[j + k * o] = N->offset[t] + (u - 1) + (v - 1) * (o - 2);
          }
      }
    }
}

/* Element nodes on edge ei / face fi, in the edge/face's own order
   (TMROctForest.cpp:5190-5206, 5236-5262). */
static void elem_edge_nodes(int o, const int *c, int ei, int *out) {
  for (int a = 0; a < o; a++) out[a] = c[edge_offset(o, ei, a)];
}
static void elem_face_nodes(int o, const int *c, int fi, int *out) {
  for (int b = 0; b < o; b++)
    for (int a = 0; a < o; a++) out[a + b * o] = c[face_offset(o, fi, a, b)];
}

/* createDependentConn (TMROctForest.cpp:5157-5519), Lagrange knots. */
static void create_dep_conn(oo_forest *f, const int *nn, const onodes *N) {
  int o = f->order, npe = o * o * o;
  int nd = f->num_dep;
  f->dep_ptr = (int *)calloc((size_t)nd + 1, sizeof(int));
  int en[OO_MAX_ORDER], fn[OO_MAX_ORDER * OO_MAX_ORDER];
  int pen[OO_MAX_ORDER], pfn[OO_MAX_ORDER * OO_MAX_ORDER];
  double Nu[OO_MAX_ORDER], Nv[OO_MAX_ORDER];
  for (long i = 0; i < f->noct; i++) {
    const oo_oct *e = &f->octs[i];
    if (!e->info) continue;
    int ei_bits;
    decode_info(e, e->info, NULL, &ei_bits);
    const int *c = &f->econn[npe * i];
    for (int ei = 0; ei < 12; ei++) {
      if (!(ei_bits & (1 << ei))) continue;
      elem_edge_nodes(o, c, ei, en);
      for (int k = 0; k < o; k++) {
        int d = nn[en[k]];
        if (d < 0 && f->dep_ptr[-d] == 0) f->dep_ptr[-d] = o;
      }
    }
  }
  for (long i = 0; i < f->noct; i++) {
    const oo_oct *e = &f->octs[i];
    if (!e->info) continue;
    int fi_bits;
    decode_info(e, e->info, &fi_bits, NULL);
    const int *c = &f->econn[npe * i];
    for (int fi = 0; fi < 6; fi++) {
      if (!(fi_bits & (1 << fi))) continue;
      elem_face_nodes(o, c, fi, fn);
      for (int k = 0; k < o * o; k++) {
        int d = nn[fn[k]];
        if (d < 0 && f->dep_ptr[-d] == 0) f->dep_ptr[-d] = o * o;
      }
    }
  }
  for (int i = 0; i < nd; i++) f->dep_ptr[i + 1] += f->dep_ptr[i];
  int nnz = f->dep_ptr[nd];
  f->dep_conn = (int *)calloc((size_t)(nnz ? nnz : 1), sizeof(int));
  f->dep_w = (double *)calloc((size_t)(nnz ? nnz : 1), sizeof(double));
  for (long i = 0; i < f->noct; i++) {
    const oo_oct *e = &f->octs[i];
    if (!e->info) continue;
    int fi_bits, ei_bits;
    decode_info(e, e->info, &fi_bits, &ei_bits);
    oo_oct p = parent_of(e);
    int id = child_id(e);
    int x = id % 2, y = (id % 4) / 2, z = id / 4;
    const int *c = &f->econn[npe * i];
    for (int ei = 0; ei < 12; ei++) {
      if (!(ei_bits & (1 << ei))) continue;
      elem_edge_nodes(o, c, ei, en);
      parent_edge_nodes(f, N, &p, ei, pen);
      for (int k = 0; k < o; k++) {
        int d = nn[en[k]];
        if (d >= 0) continue;
        d = -d - 1;
        if (f->dep_ptr[d + 1] - f->dep_ptr[d] != o) continue;
        int ptr = f->dep_ptr[d];
        for (int j = 0; j < o; j++) f->dep_conn[ptr + j] = pen[j];
        int s = (ei < 4) ? x : (ei < 8) ? y : z;
        if (f->interp == 2) { /* TMROctForest.cpp:5364-5373 */
          bernstein_dep_weights(o, (o - 1) * (s - 1) + k, &f->dep_w[ptr]);
          continue;
        }
        double u = 1.0 * (s - 1) + 0.5 * (1.0 + f->knots[k]);
        lagrange(o, u, f->knots, &f->dep_w[ptr]);
      }
    }
    for (int fi = 0; fi < 6; fi++) {
      if (!(fi_bits & (1 << fi))) continue;
      elem_face_nodes(o, c, fi, fn);
      parent_face_nodes(f, N, &p, fi, pfn);
      for (int jj = 0; jj < o; jj++)
        for (int ii = 0; ii < o; ii++) {
          int d = nn[fn[ii + jj * o]];
          if (d >= 0) continue;
          d = -d - 1;
          if (f->dep_ptr[d + 1] - f->dep_ptr[d] != o * o) continue;
          if (f->interp == 2) { /* TMROctForest.cpp:5453-5473 */
            int ub = -(o - 1) + ii, vb = -(o - 1) + jj;
            if (fi < 2) {
              ub += (o - 1) * y;
              vb += (o - 1) * z;
            } else if (fi < 4) {
              ub += (o - 1) * x;
              vb += (o - 1) * z;
            } else {
              ub += (o - 1) * x;
              vb += (o - 1) * y;
            }
            bernstein_dep_weights(o, ub, Nu);
            bernstein_dep_weights(o, vb, Nv);
            int ptr = f->dep_ptr[d];
            for (int j = 0; j < o * o; j++) {
              f->dep_conn[ptr + j] = pfn[j];
              f->dep_w[ptr + j] = Nu[j % o] * Nv[j / o];
            }
            continue;
          }
          double u = -1.0 + 0.5 * (1.0 + f->knots[ii]);
          double v = -1.0 + 0.5 * (1.0 + f->knots[jj]);
          if (fi < 2) {
            u += 1.0 * y;
            v += 1.0 * z;
          } else if (fi < 4) {
            u += 1.0 * x;
            v += 1.0 * z;
          } else {
            u += 1.0 * x;
            v += 1.0 * y;
          }
          lagrange(o, u, f->knots, Nu);
          lagrange(o, v, f->knots, Nv);
          int ptr = f->dep_ptr[d];
          for (int j = 0; j < o * o; j++) {
            f->dep_conn[ptr + j] = pfn[j];
            f->dep_w[ptr + j] = Nu[j % o] * Nv[j / o];
          }
        }
    }
  }
}

static int cmp_int(const void *a, const void *b) {
  int x = *(const int *)a, y = *(const int *)b;
  return (x > y) - (x < y);
}

/* createNodes (TMROctForest.cpp:4064-4268), one rank. */
void oo_create_nodes(oo_forest *f) {
  if (f->have_nodes) return;
  if (f->interp == 2 && f->order > 5) {
    /* the reference's eval_bernstein_weights covers orders 2-5 only */
    fprintf(stderr, "tmr_oracle: Bernstein dependent weights exist for orders 2-5\n");
    abort();
  }
  dep_faces_edges(f);
  onodes N;
  create_local_nodes(f, &N);
  N.offset = (int *)malloc(sizeof(int) * (size_t)(N.n ? N.n : 1));
  int nl = 0;
  for (long i = 0; i < N.n; i++) {
    N.offset[i] = nl;
    nl += N.a[i].level;
  }
  f->num_local = nl;
  create_local_conn(f, &N);
  int *nn = (int *)calloc((size_t)(nl ? nl : 1), sizeof(int));
  label_dependent(f, nn);
  int nd = 0;
  for (int i = 0; i < nl; i++)
    if (nn[i] == -1) nn[i] = -(++nd);
  f->num_dep = nd;
  create_dep_conn(f, nn, &N);
  /* A node that only a dependent relation created keeps tag -1 and is
     treated as owned elsewhere (TMROctForest.cpp:4122-4145): on one rank
     it is numbered -num_dep-1 (+k).  Element nodes always win the key. */
  {
    int idx = 0;
    for (long i = 0; i < N.n; i++) {
      if (nn[idx] >= 0 && N.a[i].tag != 0)
        for (int k = 0; k < N.a[i].level; k++) nn[idx + k] = -nd - 1;
      idx += N.a[i].level;
    }
  }
  int no = 0;
  for (int i = 0; i < nl; i++)
    if (nn[i] >= 0) nn[i] = no++;
  f->num_owned = no;
  {
    int idx = 0;
    for (long i = 0; i < N.n; i++) {
      if (N.a[i].tag != 0 && nn[idx] == -nd - 1)
        for (int k = 0; k < N.a[i].level; k++) nn[idx + k] = -nd - 1 + k;
      idx += N.a[i].level;
    }
  }
  int npe = f->order * f->order * f->order;
  for (long i = 0; i < (long)npe * f->noct; i++) f->econn[i] = nn[f->econn[i]];
  for (int i = 0; i < f->dep_ptr[nd]; i++) f->dep_conn[i] = nn[f->dep_conn[i]];
  qsort(nn, (size_t)nl, sizeof(int), cmp_int);
  f->ext_pre = 0;
  while (f->ext_pre < nl && nn[f->ext_pre] < 0) f->ext_pre++;
  f->node_numbers = nn;
  f->have_nodes = 1;
  free(N.a);
  free(N.offset);
}

int oo_num_octants(oo_forest *f) { return (int)f->noct; }
void oo_get_octants(oo_forest *f, int *out) {
  for (long i = 0; i < f->noct; i++) {
    const oo_oct *o = &f->octs[i];
    out[7 * i + 0] = o->block;
    out[7 * i + 1] = o->x;
    out[7 * i + 2] = o->y;
    out[7 * i + 3] = o->z;
    out[7 * i + 4] = o->tag;
    out[7 * i + 5] = o->level;
    out[7 * i + 6] = o->info;
  }
}
void oo_node_sizes(oo_forest *f, int *out) {
  out[0] = f->num_local;
  out[1] = f->num_owned;
  out[2] = f->num_dep;
  out[3] = f->ext_pre;
  out[4] = (int)f->noct;
  out[5] = f->dep_ptr ? f->dep_ptr[f->num_dep] : 0;
}
void oo_get_conn(oo_forest *f, int *out) {
  int npe = f->order * f->order * f->order;
  memcpy(out, f->econn, sizeof(int) * (size_t)npe * (size_t)f->noct);
}
void oo_get_node_numbers(oo_forest *f, int *out) {
  memcpy(out, f->node_numbers, sizeof(int) * (size_t)f->num_local);
}
void oo_get_dep(oo_forest *f, int *ptr, int *conn, double *w) {
  int nd = f->num_dep;
  memcpy(ptr, f->dep_ptr, sizeof(int) * (size_t)(nd + 1));
  memcpy(conn, f->dep_conn, sizeof(int) * (size_t)f->dep_ptr[nd]);
  memcpy(w, f->dep_w, sizeof(double) * (size_t)f->dep_ptr[nd]);
}
void oo_get_knots(oo_forest *f, double *k) {
  memcpy(k, f->knots, sizeof(double) * (size_t)f->order);
}

/* ------------------------------------------------------------------ */
/* createInterpolation (TMROctForest.cpp:6228-6793), one rank. */
struct oo_interp {
  int nrows, nnz, cap_rows, cap_nnz;
  int *rows, *end_ptr, *cols;
  double *w;
};

/* findEnclosing (TMROctForest.cpp:6228-6377). */
static long find_enclosing(oo_forest *coarse, int order, const double *knots,
                           const oo_oct *node) {
  const oo_oct *a = coarse->octs;
  long size = coarse->noct;
  int32_t h = side(node->level);
  int ii = node->info % order, jj = (node->info % (order * order)) / order,
      kk = node->info / (order * order);
  int32_t xi = -1, yi = -1, zi = -1;
  if (ii == 0 || ii == order - 1)
    xi = node->x + (ii / (order - 1)) * h;
  else if (order % 2 == 1 && ii == order / 2)
    xi = node->x + h / 2;
  if (jj == 0 || jj == order - 1)
    yi = node->y + (jj / (order - 1)) * h;
  else if (order % 2 == 1 && jj == order / 2)
    yi = node->y + h / 2;
  if (kk == 0 || kk == order - 1)
    zi = node->z + (kk / (order - 1)) * h;
  else if (order % 2 == 1 && kk == order / 2)
    zi = node->z + h / 2;
  double xd = node->x + 0.5 * h * (1.0 + knots[ii]);
  double yd = node->y + 0.5 * h * (1.0 + knots[jj]);
  double zd = node->z + 0.5 * h * (1.0 + knots[kk]);
  long low = 0, high = size - 1, mid = low + (high - low) / 2;
  while (mid != low) {
    if (contains(&a[mid], node)) break;
    int st = cmp_position(&a[mid], node);
    if (st == 0) break;
    if (st < 0)
      low = mid + 1;
    else
      high = mid - 1;
    mid = low + (high - low) / 2;
  }
  oo_oct bound = {node->block, node->x + h, node->y + h, node->z + h, 0, 0, 0};
  while (mid < size && cmp_position(&a[mid], &bound) <= 0) {
    if (a[mid].block == node->block) {
      int32_t hm = side(a[mid].level);
      int xin, yin, zin;
      if (xi >= 0)
        xin = (a[mid].x <= xi && xi <= a[mid].x + hm);
      else
        xin = (a[mid].x <= xd && xd <= a[mid].x + hm);
      if (yi >= 0)
        yin = (a[mid].y <= yi && yi <= a[mid].y + hm);
      else
        yin = (a[mid].y <= yd && yd <= a[mid].y + hm);
      if (zi >= 0)
        zin = (a[mid].z <= zi && zi <= a[mid].z + hm);
      else
        zin = (a[mid].z <= zd && zd <= a[mid].z + hm);
      if (xin && yin && zin) return mid;
    }
    mid++;
  }
  return -1;
}

typedef struct {
  int index;
  double weight;
} oo_iw;

/* TMRIndexWeight::uniqueSort (TMRBase.h:103-130): sort by index (stable),
   summing the weights of equal indices in order. */
static int unique_sort_iw(oo_iw *a, int n) {
  for (int i = 1; i < n; i++) { /* stable insertion sort */
    oo_iw t = a[i];
    int j = i - 1;
    while (j >= 0 && a[j].index > t.index) {
      a[j + 1] = a[j];
      j--;
    }
    a[j + 1] = t;
  }
  int j = 0;
  for (int i = 0; i < n; i++, j++) {
    if (i != j) a[j] = a[i];
    while (i < n - 1 && a[i].index == a[i + 1].index) {
      a[j].weight += a[i + 1].weight;
      i++;
    }
  }
  return j;
}

/* The 1-D weights of one direction of computeElemInterp: the coarse
   basis (Lagrange at the coarse knots, or Bernstein: the basis at u when
   the orders agree, the degree-elevation table when they differ) at the
   fine node's coordinate. */
static void dir_basis(oo_forest *fine, oo_forest *coarse, int i, int32_t nx, int32_t h,
                      int32_t ox, int32_t hc, double *N) {
  int mo = fine->order, co = coarse->order;
  const double *kn = fine->knots;
  if (fine->interp == 2 && mo != co) {
    bernstein_interp_weights(mo, co, i, N);
    return;
  }
  double u = -1.0 + 2.0 * (nx + 0.5 * h * (1.0 + kn[i]) - ox) / hc;
  if (fine->interp == 2)
    bernstein(mo, u, N);
  else
    lagrange(co, u, coarse->knots, N);
}

/* computeElemInterp (TMROctForest.cpp:6396-6594), Lagrange and Bernstein
   branches. */
static int elem_interp(oo_forest *fine, const oo_oct *node, oo_forest *coarse,
                       const oo_oct *oct, oo_iw *w) {
  int mo = fine->order, co = coarse->order;
  int i = node->info % mo, j = (node->info % (mo * mo)) / mo,
      k = node->info / (mo * mo);
  int32_t h = side(node->level), hc = side(oct->level);
  double Nu[OO_MAX_ORDER], Nv[OO_MAX_ORDER], Nw[OO_MAX_ORDER];
  int is = 0, ie = co, js = 0, je = co, ks = 0, ke = co;
  if ((i == 0 && oct->x == node->x) || (i == mo - 1 && oct->x == node->x + h)) {
    is = 0; ie = 1; Nu[0] = 1.0;
  } else if ((i == 0 && oct->x + hc == node->x) ||
             (i == mo - 1 && oct->x + hc == node->x + h)) {
    is = co - 1; ie = co; Nu[is] = 1.0;
  } else {
    dir_basis(fine, coarse, i, node->x, h, oct->x, hc, Nu);
  }
  if ((j == 0 && oct->y == node->y) || (j == mo - 1 && oct->y == node->y + h)) {
    js = 0; je = 1; Nv[0] = 1.0;
  } else if ((j == 0 && oct->y + hc == node->y) ||
             (j == mo - 1 && oct->y + hc == node->y + h)) {
    js = co - 1; je = co; Nv[js] = 1.0;
  } else {
    dir_basis(fine, coarse, j, node->y, h, oct->y, hc, Nv);
  }
  if ((k == 0 && oct->z == node->z) || (k == mo - 1 && oct->z == node->z + h)) {
    ks = 0; ke = 1; Nw[0] = 1.0;
  } else if ((k == 0 && oct->z + hc == node->z) ||
             (k == mo - 1 && oct->z + hc == node->z + h)) {
    ks = co - 1; ke = co; Nw[ks] = 1.0;
  } else {
    dir_basis(fine, coarse, k, node->z, h, oct->z, hc, Nw);
  }
  const int *c = &coarse->econn[(long)co * co * co * oct->tag];
  int n = 0;
  for (int kk = ks; kk < ke; kk++)
    for (int jj = js; jj < je; jj++)
      for (int ii = is; ii < ie; ii++) {
        int off = ii + jj * co + kk * co * co;
        double wt = Nu[ii] * Nv[jj] * Nw[kk];
        if (c[off] >= 0) {
          w[n].index = c[off];
          w[n].weight = wt;
          n++;
        } else {
          int d = -c[off] - 1;
          for (int p = coarse->dep_ptr[d]; p < coarse->dep_ptr[d + 1]; p++) {
            w[n].index = coarse->dep_conn[p];
            w[n].weight = wt * coarse->dep_w[p];
            n++;
          }
        }
      }
  return unique_sort_iw(w, n);
}

static void interp_add(oo_interp *I, int row, const oo_iw *w, int n) {
  if (I->nrows == I->cap_rows) {
    I->cap_rows = I->cap_rows ? 2 * I->cap_rows : 1024;
    I->rows = (int *)realloc(I->rows, sizeof(int) * (size_t)I->cap_rows);
    I->end_ptr = (int *)realloc(I->end_ptr, sizeof(int) * (size_t)I->cap_rows);
  }
  while (I->nnz + n > I->cap_nnz) {
    I->cap_nnz = I->cap_nnz ? 2 * I->cap_nnz : 4096;
    I->cols = (int *)realloc(I->cols, sizeof(int) * (size_t)I->cap_nnz);
    I->w = (double *)realloc(I->w, sizeof(double) * (size_t)I->cap_nnz);
  }
  for (int k = 0; k < n; k++) {
    I->cols[I->nnz + k] = w[k].index;
    I->w[I->nnz + k] = w[k].weight;
  }
  I->nnz += n;
  I->rows[I->nrows] = row;
  I->end_ptr[I->nrows] = I->nnz;
  I->nrows++;
}

oo_interp *oo_create_interp(oo_forest *fine, oo_forest *coarse) {
  oo_create_nodes(fine);
  oo_create_nodes(coarse);
  oo_interp *I = (oo_interp *)calloc(1, sizeof(oo_interp));
  int mo = fine->order, co = coarse->order, npe = mo * mo * mo;
  char *done = (char *)calloc((size_t)(fine->num_owned ? fine->num_owned : 1), 1);
  long maxw = (long)co * co * co * co * co;
  oo_iw *w = (oo_iw *)malloc(sizeof(oo_iw) * (size_t)maxw);
  for (long i = 0; i < fine->noct; i++) {
    const int *c = &fine->econn[npe * i];
    for (int j = 0; j < npe; j++) {
      if (c[j] < 0 || c[j] >= fine->num_owned || done[c[j]]) continue;
      done[c[j]] = 1;
      oo_oct node = fine->octs[i];
      node.info = (int16_t)j;
      long t = find_enclosing(coarse, mo, fine->knots, &node);
      if (t < 0) {
        fprintf(stderr, "tmr_oracle: no enclosing coarse octant\n");
        abort();
      }
      int n = elem_interp(fine, &node, coarse, &coarse->octs[t], w);
      interp_add(I, c[j], w, n);
    }
  }
  free(done);
  free(w);
  return I;
}
void oo_interp_sizes(oo_interp *I, int *out) {
  out[0] = I->nrows;
  out[1] = I->nnz;
}
void oo_interp_get(oo_interp *I, int *rows, int *end_ptr, int *cols,
                   double *w) {
  memcpy(rows, I->rows, sizeof(int) * (size_t)I->nrows);
  memcpy(end_ptr, I->end_ptr, sizeof(int) * (size_t)I->nrows);
  memcpy(cols, I->cols, sizeof(int) * (size_t)I->nnz);
  memcpy(w, I->w, sizeof(double) * (size_t)I->nnz);
}
void oo_interp_destroy(oo_interp *I) {
  if (!I) return;
  free(I->rows);
  free(I->end_ptr);
  free(I->cols);
  free(I->w);
  free(I);
}

/* ------------------------------------------------------------------ */
/* P applies.  TACS's TACSBVecInterp is not in the reference tree
   (called at TMRConformFilter.cpp:163, TMRMatrixFilter.cpp:315); these
   follow the natural definitions and are "parity unpinned":
     mult:            y = P x
     multTranspose:   y = P^T x
     multWeightTranspose: y_j = (P^T x)_j / (P^T 1)_j  */
void oo_csr_mult(int n, const int *rp, const int *cols, const double *vals,
                 int k, const double *x, double *y) {
  for (int i = 0; i < n; i++)
    for (int v = 0; v < k; v++) {
      double s = 0.0;
      for (int p = rp[i]; p < rp[i + 1]; p++)
        s += vals[p] * x[(long)cols[p] * k + v];
      y[(long)i * k + v] = s;
    }
}
void oo_csr_mult_t(int n, int nc, const int *rp, const int *cols,
                   const double *vals, int k, const double *x, double *y) {
  memset(y, 0, sizeof(double) * (size_t)nc * (size_t)k);
  for (int i = 0; i < n; i++)
    for (int p = rp[i]; p < rp[i + 1]; p++)
      for (int v = 0; v < k; v++)
        y[(long)cols[p] * k + v] += vals[p] * x[(long)i * k + v];
}
void oo_csr_mult_wt(int n, int nc, const int *rp, const int *cols,
                    const double *vals, int k, const double *x, double *y) {
  double *wsum = (double *)calloc((size_t)(nc ? nc : 1), sizeof(double));
  oo_csr_mult_t(n, nc, rp, cols, vals, k, x, y);
  for (int i = 0; i < n; i++)
    for (int p = rp[i]; p < rp[i + 1]; p++) wsum[cols[p]] += vals[p];
  for (int j = 0; j < nc; j++)
    for (int v = 0; v < k; v++)
      y[(long)j * k + v] = (wsum[j] != 0.0) ? y[(long)j * k + v] / wsum[j] : 0.0;
  free(wsum);
}

/* ------------------------------------------------------------------ */
/* Seeded inputs: splitmix64 of (seed, stream, index). */
uint64_t oo_splitmix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ULL;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ULL;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBULL;
  return x ^ (x >> 31);
}
double oo_uniform(uint64_t seed, uint64_t stream, uint64_t index) {
  uint64_t r = oo_splitmix64(oo_splitmix64(seed * 0x100000001B3ULL + stream) ^
                             (index * 0xD6E8FEB86659FD93ULL));
  return (double)(r >> 11) * (1.0 / 9007199254740992.0);
}

/* ------------------------------------------------------------------ */
/* Matrix density filter (TMRMatrixFilter.cpp:30-235).  Parity unpinned:
   the mass matrix is assembled by TACS in the reference (absent here).
   Restatement: trilinear elements for order 2, quadratic and cubic
   Bernstein hexahedra for orders 3 and 4 (TMRMatrixCreator.h:76-92), on
   blocks that are cubes of side block_len (elem_mass).  Dependent nodes
   are condensed: each element merges its expanded block over its distinct
   independent nodes (first-appearance order; products summed in
   (a, b, p, q) loop order), and the element blocks are summed in element
   order. */
struct oo_filter {
  int n, nnz, N;
  double r;
  int *rowptr, *cols;
  double *vals, *Ainv, *B, *Tinv;
};

typedef struct {
  long key;
  long seq;
  double v;
} oo_fent;

static int cmp_fent(const void *a, const void *b) {
  const oo_fent *x = (const oo_fent *)a, *y = (const oo_fent *)b;
  if (x->key != y->key) return x->key < y->key ? -1 : 1;
  return (x->seq > y->seq) - (x->seq < y->seq);
}

static void filter_horner(oo_filter *F, int tr, int vpn, const double *in,
                          double *out) {
  long n = F->n, len = n * (long)vpn;
  double *t1 = (double *)malloc(sizeof(double) * (size_t)(len ? len : 1));
  double *cur = (double *)malloc(sizeof(double) * (size_t)(len ? len : 1));
  double *nxt = (double *)malloc(sizeof(double) * (size_t)(len ? len : 1));
  const double *pre = tr ? F->Tinv : F->Ainv, *post = tr ? F->Ainv : F->Tinv;
  for (long i = 0; i < len; i++) t1[i] = pre[i / vpn] * in[i];
  memcpy(cur, t1, sizeof(double) * (size_t)len);
  for (int it = 0; it < F->N; it++) {
    for (long i = 0; i < n; i++)
      for (int v = 0; v < vpn; v++) {
        double acc = 0.0;
        for (int p = F->rowptr[i]; p < F->rowptr[i + 1]; p++) {
          int j = F->cols[p];
          double xv = cur[(long)j * vpn + v];
          if (tr) xv = F->B[j] * xv;
          acc = acc + F->vals[p] * xv;
        }
        double r = tr ? acc + t1[i * vpn + v] : F->B[i] * acc + t1[i * vpn + v];
        nxt[i * vpn + v] = r;
      }
    double *t = cur;
    cur = nxt;
    nxt = t;
  }
  for (long i = 0; i < len; i++) out[i] = cur[i] * post[i / vpn];
  free(t1);
  free(cur);
  free(nxt);
}

/* 1-D Bernstein mass of degree p on [0, 1]:
   int B_i B_j = C(p, i) C(p, j) / ((2p + 1) C(2p, i + j)), one division. */
static double bern_mass_1d(int p, int i, int j) {
  double ci = 1.0, cj = 1.0, c2 = 1.0;
  for (int k = 1; k <= i; k++) ci = ci * (p - k + 1) / k;
  for (int k = 1; k <= j; k++) cj = cj * (p - k + 1) / k;
  for (int k = 1; k <= i + j; k++) c2 = c2 * (2 * p - k + 1) / k;
  return (ci * cj) / ((2 * p + 1) * c2);
}

/* Element mass of an order-o element on a cube of side `side`
   (TMRMatrixCreator.h:76-92): the trilinear element for order 2, the
   quadratic and cubic Bernstein hexahedra for orders 3 and 4, whose
   consistent mass matrices are tensor products of the 1-D Bernstein
   masses (TACS integrates them exactly on axis-aligned cubes).  Order 2
   keeps the exact form s^3 / (27 * 2^k) (k = coordinates in which the two
   corners differ); orders 3-4 form ((s^3 m_x) m_y) m_z. */
static double elem_mass(int o, double s3, int a, int b) {
  if (o == 2) {
    int x = a ^ b;
    int k = (x & 1) + ((x >> 1) & 1) + (x >> 2);
    return s3 / (27.0 * (double)(1 << k));
  }
  int p = o - 1;
  int ia = a % o, ja = (a / o) % o, ka = a / (o * o);
  int ib = b % o, jb = (b / o) % o, kb = b / (o * o);
  return ((s3 * bern_mass_1d(p, ia, ib)) * bern_mass_1d(p, ja, jb)) * bern_mass_1d(p, ka, kb);
}

oo_filter *oo_filter_create(oo_forest *f, double block_len, double r, int N) {
  if (f->order < 2 || f->order > 4) return NULL;
  oo_create_nodes(f);
  oo_filter *F = (oo_filter *)calloc(1, sizeof(oo_filter));
  F->n = f->num_owned;
  F->N = N;
  F->r = r;
  const int o = f->order, npe = o * o * o, mx = o * o; /* dependent rows <= o^2 */
  long cap = 1 << 16, ne = 0;
  oo_fent *E = (oo_fent *)malloc(sizeof(oo_fent) * (size_t)cap);
  int *ni = (int *)malloc(sizeof(int) * (size_t)npe * mx);
  double *nw = (double *)malloc(sizeof(double) * (size_t)npe * mx);
  int *nc = (int *)malloc(sizeof(int) * (size_t)npe);
  int *U = (int *)malloc(sizeof(int) * (size_t)npe * mx);
  double *L = NULL;
  long Lcap = 0;
  for (long e = 0; e < f->noct; e++) {
    const int *ec = &f->econn[(long)npe * e];
    int K = 0;
    for (int a = 0; a < npe; a++) {
      int g = ec[a];
      if (g >= 0) {
        nc[a] = 1;
        ni[a * mx] = g;
        nw[a * mx] = 1.0;
      } else {
        int d = -g - 1;
        nc[a] = f->dep_ptr[d + 1] - f->dep_ptr[d];
        for (int p = 0; p < nc[a]; p++) {
          ni[a * mx + p] = f->dep_conn[f->dep_ptr[d] + p];
          nw[a * mx + p] = f->dep_w[f->dep_ptr[d] + p];
        }
      }
      for (int p = 0; p < nc[a]; p++) {
        int u = 0;
        while (u < K && U[u] != ni[a * mx + p]) u++;
        if (u == K) U[K++] = ni[a * mx + p];
      }
    }
    if ((long)K * K > Lcap) {
      Lcap = (long)K * K;
      L = (double *)realloc(L, sizeof(double) * (size_t)Lcap);
    }
    for (long u = 0; u < (long)K * K; u++) L[u] = 0.0;
    double side = block_len / (double)(1 << f->octs[e].level);
    double s3 = side * side * side;
    for (int a = 0; a < npe; a++)
      for (int b = 0; b < npe; b++) {
        double mab = elem_mass(o, s3, a, b);
        for (int p = 0; p < nc[a]; p++) {
          int u = 0;
          while (U[u] != ni[a * mx + p]) u++;
          double t = mab * nw[a * mx + p];
          for (int q = 0; q < nc[b]; q++) {
            int v = 0;
            while (U[v] != ni[b * mx + q]) v++;
            L[(long)u * K + v] = L[(long)u * K + v] + t * nw[b * mx + q];
          }
        }
      }
    while (ne + (long)K * K > cap) {
      cap *= 2;
      E = (oo_fent *)realloc(E, sizeof(oo_fent) * (size_t)cap);
    }
    for (int u = 0; u < K; u++)
      for (int v = 0; v < K; v++) {
        E[ne].key = (long)U[u] * (long)F->n + U[v];
        E[ne].seq = ne;
        E[ne].v = L[(long)u * K + v];
        ne++;
      }
  }
  free(ni);
  free(nw);
  free(nc);
  free(U);
  free(L);
  qsort(E, (size_t)ne, sizeof(oo_fent), cmp_fent);
  F->rowptr = (int *)calloc((size_t)F->n + 1, sizeof(int));
  F->cols = (int *)malloc(sizeof(int) * (size_t)(ne ? ne : 1));
  F->vals = (double *)malloc(sizeof(double) * (size_t)(ne ? ne : 1));
  int nnz = 0;
  for (long i = 0; i < ne;) {
    long j = i;
    double s = E[i].v;
    while (j + 1 < ne && E[j + 1].key == E[i].key) {
      j++;
      s = s + E[j].v;
    }
    F->cols[nnz] = (int)(E[i].key % F->n);
    F->vals[nnz] = s;
    F->rowptr[E[i].key / F->n + 1]++;
    nnz++;
    i = j + 1;
  }
  for (int i = 0; i < F->n; i++) F->rowptr[i + 1] += F->rowptr[i];
  F->nnz = nnz;
  free(E);
  F->Ainv = (double *)malloc(sizeof(double) * (size_t)(F->n ? F->n : 1));
  F->B = (double *)malloc(sizeof(double) * (size_t)(F->n ? F->n : 1));
  F->Tinv = (double *)malloc(sizeof(double) * (size_t)(F->n ? F->n : 1));
  for (int i = 0; i < F->n; i++) {
    double D = 0.0;
    for (int p = F->rowptr[i]; p < F->rowptr[i + 1]; p++) D = D + F->vals[p];
    if (D == 0.0) {
      F->Ainv[i] = 1.0;
      F->B[i] = 0.0;
    } else {
      double t = pow(D, 2.0 / 3.0);
      F->Ainv[i] = 1.0 / (1.0 + r * r / t);
      F->B[i] = F->Ainv[i] * r * r / (t * D);
    }
    F->Tinv[i] = 1.0;
  }
  double *ones = (double *)malloc(sizeof(double) * (size_t)(F->n ? F->n : 1));
  double *y = (double *)malloc(sizeof(double) * (size_t)(F->n ? F->n : 1));
  for (int i = 0; i < F->n; i++) ones[i] = 1.0;
  filter_horner(F, 0, 1, ones, y);
  for (int i = 0; i < F->n; i++) F->Tinv[i] = (y[i] != 0.0) ? 1.0 / y[i] : 0.0;
  free(ones);
  free(y);
  return F;
}
void oo_filter_sizes(oo_filter *F, int *out) {
  out[0] = F->n;
  out[1] = F->nnz;
}
void oo_filter_get_matrix(oo_filter *F, int *rowptr, int *cols, double *vals,
                          double *Ainv, double *B, double *Tinv) {
  memcpy(rowptr, F->rowptr, sizeof(int) * (size_t)(F->n + 1));
  memcpy(cols, F->cols, sizeof(int) * (size_t)F->nnz);
  memcpy(vals, F->vals, sizeof(double) * (size_t)F->nnz);
  memcpy(Ainv, F->Ainv, sizeof(double) * (size_t)F->n);
  memcpy(B, F->B, sizeof(double) * (size_t)F->n);
  memcpy(Tinv, F->Tinv, sizeof(double) * (size_t)F->n);
}
void oo_filter_apply(oo_filter *F, int vpn, const double *in, double *out) {
  filter_horner(F, 0, vpn, in, out);
}
void oo_filter_apply_t(oo_filter *F, int vpn, const double *in, double *out) {
  filter_horner(F, 1, vpn, in, out);
}
void oo_filter_destroy(oo_filter *F) {
  if (!F) return;
  free(F->rowptr);
  free(F->cols);
  free(F->vals);
  free(F->Ainv);
  free(F->B);
  free(F->Tinv);
  free(F);
}
