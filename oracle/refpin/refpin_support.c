/*
 * Stand-ins for the runtime the reference's pbvh.c links against
 * (guarded allocator, bitmap, GHash/GSet, task range, custom data, mesh
 * normals) — TEST INFRASTRUCTURE ONLY, part of the reference-pinning harness.
 * Single threaded; nothing here does arithmetic that a pinned result depends
 * on, except the vertex-iterator step, which only selects which stored
 * coordinates the reference's own loops read.
 */
#include "refpin_prelude.h"

#include <stdarg.h>
#include <time.h>

static void refpin_unreachable(const char *what)
{
  fprintf(stderr, "refpin: %s is not part of the pinned paths\n", what);
  abort();
}

/* ---- allocator: a 16-byte header keeps the size for realloc / recalloc ---- */
typedef struct MemHead {
  size_t len;
  size_t pad;
} MemHead;

void *MEM_mallocN(size_t len, const char *str)
{
  (void)str;
  MemHead *h = malloc(sizeof(MemHead) + (len ? len : 1));
  if (!h) {
    refpin_unreachable("out of memory");
  }
  h->len = len;
  return h + 1;
}
void *MEM_callocN(size_t len, const char *str)
{
  void *p = MEM_mallocN(len, str);
  memset(p, 0, len);
  return p;
}
void *MEM_malloc_arrayN(size_t n, size_t size, const char *str)
{
  return MEM_mallocN(n * size, str);
}
void *MEM_calloc_arrayN(size_t n, size_t size, const char *str)
{
  return MEM_callocN(n * size, str);
}
static size_t mem_len(const void *p)
{
  return p ? ((const MemHead *)p - 1)->len : 0;
}
void *MEM_reallocN_id(void *p, size_t len, const char *str)
{
  void *q = MEM_mallocN(len, str);
  if (p) {
    size_t old = mem_len(p);
    memcpy(q, p, old < len ? old : len);
    MEM_freeN(p);
  }
  return q;
}
void *MEM_recallocN_id(void *p, size_t len, const char *str)
{
  size_t old = mem_len(p);
  void *q = MEM_reallocN_id(p, len, str);
  if (len > old) {
    memset((char *)q + old, 0, len - old);
  }
  return q;
}
void *MEM_dupallocN(const void *p)
{
  if (!p) {
    return NULL;
  }
  void *q = MEM_mallocN(mem_len(p), "dup");
  memcpy(q, p, mem_len(p));
  return q;
}
void MEM_freeN(void *p)
{
  if (p) {
    free((MemHead *)p - 1);
  }
}

void BLI_bitmap_set_all(BLI_bitmap *b, bool set, size_t bits)
{
  memset(b, set ? 0xff : 0, (bits + 31) / 32 * 4);
}

/* ---- GHash / GSet: open addressing on pointer-sized keys ---- */
struct GHash {
  void **keys;
  void **vals;
  unsigned char *used;
  size_t cap, len;
};

static size_t gh_slot(const GHash *gh, const void *key)
{
  uint64_t x = (uint64_t)(uintptr_t)key;
  x ^= x >> 33;
  x *= 0xff51afd7ed558ccdULL;
  x ^= x >> 33;
  return (size_t)x & (gh->cap - 1);
}

static GHash *gh_new(size_t reserve)
{
  GHash *gh = calloc(1, sizeof(GHash));
  gh->cap = 16;
  while (gh->cap < reserve * 2 + 2) {
    gh->cap *= 2;
  }
  gh->keys = calloc(gh->cap, sizeof(void *));
  gh->vals = calloc(gh->cap, sizeof(void *));
  gh->used = calloc(gh->cap, 1);
  return gh;
}

static void gh_grow(GHash *gh)
{
  GHash old = *gh;
  gh->cap *= 2;
  gh->len = 0;
  gh->keys = calloc(gh->cap, sizeof(void *));
  gh->vals = calloc(gh->cap, sizeof(void *));
  gh->used = calloc(gh->cap, 1);
  for (size_t i = 0; i < old.cap; i++) {
    if (old.used[i]) {
      size_t s = gh_slot(gh, old.keys[i]);
      while (gh->used[s]) {
        s = (s + 1) & (gh->cap - 1);
      }
      gh->used[s] = 1;
      gh->keys[s] = old.keys[i];
      gh->vals[s] = old.vals[i];
      gh->len++;
    }
  }
  free(old.keys);
  free(old.vals);
  free(old.used);
}

/* Returns true if the key was present; *r_slot is its slot either way. */
static bool gh_ensure(GHash *gh, void *key, size_t *r_slot)
{
  if ((gh->len + 1) * 2 > gh->cap) {
    gh_grow(gh);
  }
  size_t s = gh_slot(gh, key);
  while (gh->used[s]) {
    if (gh->keys[s] == key) {
      *r_slot = s;
      return true;
    }
    s = (s + 1) & (gh->cap - 1);
  }
  gh->used[s] = 1;
  gh->keys[s] = key;
  gh->vals[s] = NULL;
  gh->len++;
  *r_slot = s;
  return false;
}

GHash *BLI_ghash_int_new_ex(const char *info, unsigned int reserve)
{
  (void)info;
  return gh_new(reserve);
}
bool BLI_ghash_ensure_p(GHash *gh, void *key, void ***r_val)
{
  size_t s;
  bool found = gh_ensure(gh, key, &s);
  *r_val = &gh->vals[s];
  return found;
}
void BLI_ghash_free(GHash *gh, void *keyfree, void *valfree)
{
  (void)keyfree;
  (void)valfree;
  if (gh) {
    free(gh->keys);
    free(gh->vals);
    free(gh->used);
    free(gh);
  }
}
void BLI_ghashIterator_init(GHashIterator *it, GHash *gh)
{
  it->gh = gh;
  it->slot = -1;
  BLI_ghashIterator_step(it);
}
void BLI_ghashIterator_step(GHashIterator *it)
{
  do {
    it->slot++;
  } while ((size_t)it->slot < it->gh->cap && !it->gh->used[it->slot]);
}
bool BLI_ghashIterator_done(const GHashIterator *it)
{
  return (size_t)it->slot >= it->gh->cap;
}
void *BLI_ghashIterator_getKey(GHashIterator *it)
{
  return it->gh->keys[it->slot];
}
void *BLI_ghashIterator_getValue(GHashIterator *it)
{
  return it->gh->vals[it->slot];
}
GSet *BLI_gset_ptr_new(const char *info)
{
  (void)info;
  return gh_new(16);
}
bool BLI_gset_add(GSet *gs, void *key)
{
  size_t s;
  return !gh_ensure(gs, key, &s);
}
unsigned int BLI_gset_len(const GSet *gs)
{
  return gs ? (unsigned int)gs->len : 0u;
}
void BLI_gset_free(GSet *gs, void *keyfree)
{
  BLI_ghash_free(gs, keyfree, NULL);
}
void BLI_gsetIterator_init(GSetIterator *it, GSet *gs)
{
  BLI_ghashIterator_init(it, gs);
}
void *BLI_gsetIterator_getKey(GSetIterator *it)
{
  return BLI_ghashIterator_getKey(it);
}

/* ---- task range: the callback over [start, stop) in order, one thread; the
 * per-thread chunk is a copy of settings->userdata_chunk, freed at the end ---- */
void BLI_task_parallel_range(const int start,
                             const int stop,
                             void *userdata,
                             TaskParallelRangeFunc func,
                             const TaskParallelSettings *settings)
{
  TaskParallelTLS tls = {NULL};
  void *chunk = NULL;
  if (settings && settings->userdata_chunk && settings->userdata_chunk_size) {
    chunk = malloc(settings->userdata_chunk_size);
    memcpy(chunk, settings->userdata_chunk, settings->userdata_chunk_size);
    tls.userdata_chunk = chunk;
  }
  for (int i = start; i < stop; i++) {
    func(userdata, i, &tls);
  }
  if (chunk) {
    if (settings->func_reduce) {
      settings->func_reduce(userdata, settings->userdata_chunk, chunk);
    }
    if (settings->func_free) {
      settings->func_free(userdata, chunk);
    }
    free(chunk);
  }
}

double PIL_check_seconds_timer(void)
{
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

/* ---- custom data: the first layer of a type ---- */
void *CustomData_get_layer(const CustomData *data, int type)
{
  if (!data) {
    return NULL;
  }
  for (int i = 0; i < data->totlayer; i++) {
    if (data->layers[i].type == type) {
      return data->layers[i].data;
    }
  }
  return NULL;
}
int CustomData_get_offset(const CustomData *data, int type)
{
  (void)data;
  (void)type;
  return -1;
}

/* ---- mesh normals: the driver keeps them in the Mesh it passes ---- */
typedef struct RefpinMeshNormals {
  const Mesh *mesh;
  float (*normals)[3];
} RefpinMeshNormals;
static RefpinMeshNormals g_normals;
void refpin_set_mesh_normals(const Mesh *mesh, float (*normals)[3])
{
  g_normals.mesh = mesh;
  g_normals.normals = normals;
}
void BKE_mesh_vertex_normals_ensure(const Mesh *mesh)
{
  (void)mesh;
}
float (*BKE_mesh_vertex_normals_for_write(Mesh *mesh))[3]
{
  return mesh == g_normals.mesh ? g_normals.normals : NULL;
}

/* ---- vertex iterator step (FACES and GRIDS) ---- */
bool refpin_vertex_iter_next(PBVHVertexIter *vi)
{
  for (;;) {
    vi->pos++;
    if (vi->pos >= vi->end) {
      return false;
    }
    if (vi->grids) {
      const int area = vi->key.grid_area;
      const int g = vi->pos / area, e = vi->pos % area;
      const int grid = vi->grid_indices[g];
      CCGElem *elem = CCG_elem_offset(&vi->key, vi->grids[grid], e);
      /* pbvh_vertex_iter_init sets grid_hidden in unique mode only. */
      vi->gh = (vi->mode == PBVH_ITER_UNIQUE && vi->grid_hidden) ? vi->grid_hidden[grid] : NULL;
      vi->co = CCG_elem_co(&vi->key, elem);
      vi->fno = vi->key.has_normals ? CCG_elem_no(&vi->key, elem) : NULL;
      vi->mask = vi->key.has_mask ? CCG_elem_mask(&vi->key, elem) : NULL;
      vi->index = grid * area + e;
      vi->visible = true;
      if (vi->mode == PBVH_ITER_UNIQUE && vi->gh && BLI_BITMAP_TEST(vi->gh, e)) {
        continue;
      }
      return true;
    }
    const int v = vi->vert_indices[vi->pos];
    vi->mvert = &vi->mverts[v];
    vi->visible = !(vi->mvert->flag & ME_HIDE);
    if (vi->respect_hide && vi->mode == PBVH_ITER_UNIQUE && !vi->visible) {
      continue;
    }
    vi->co = vi->mvert->co;
    vi->no = vi->vert_normals ? vi->vert_normals[v] : NULL;
    vi->index = v;
    vi->mask = vi->vmask ? &vi->vmask[v] : NULL;
    return true;
  }
}

/* ---- not on the pinned paths ---- */
void BKE_mesh_calc_normals_looptri(MVert *mverts, int numVerts, const MLoop *mloop,
                                   const MLoopTri *looptri, int looptri_num,
                                   float (*r_tri_nors)[3])
{
  refpin_unreachable("BKE_mesh_calc_normals_looptri");
}
GSet *BKE_pbvh_bmesh_node_unique_verts(PBVHNode *node)
{
  refpin_unreachable("dyntopo");
  return NULL;
}
GSet *BKE_pbvh_bmesh_node_other_verts(PBVHNode *node)
{
  refpin_unreachable("dyntopo");
  return NULL;
}
bool pbvh_bmesh_node_raycast(PBVHNode *node, const float ray_start[3], const float ray_normal[3],
                             struct IsectRayPrecalc *isect_precalc, float *dist,
                             bool use_original, int *r_active_vertex_index,
                             float *r_face_normal)
{
  refpin_unreachable("dyntopo");
  return false;
}
bool pbvh_bmesh_node_nearest_to_ray(PBVHNode *node, const float ray_start[3],
                                    const float ray_normal[3], float *depth, float *dist_sq,
                                    bool use_original)
{
  refpin_unreachable("dyntopo");
  return false;
}
void pbvh_bmesh_normals_update(PBVHNode **nodes, int totnode)
{
  refpin_unreachable("dyntopo");
}
int BM_elem_flag_test(const void *ele, int hflag)
{
  refpin_unreachable("dyntopo");
  return 0;
}
void BM_mesh_elem_index_ensure(BMesh *bm, int htype)
{
  refpin_unreachable("dyntopo");
}
/* Draw buffers: refpin_draw.c compiles the reference's; BMesh stays out. */
GPU_PBVH_Buffers *GPU_pbvh_bmesh_buffers_build(bool smooth_shading)
{
  refpin_unreachable("dyntopo draw buffers");
  return NULL;
}
void GPU_pbvh_bmesh_buffers_update(GPU_PBVH_Buffers *buffers, ...)
{
  refpin_unreachable("dyntopo draw buffers");
}
void GPU_pbvh_bmesh_buffers_update_free(GPU_PBVH_Buffers *buffers)
{
  refpin_unreachable("dyntopo draw buffers");
}

void mid_v3_v3v3(float r[3], const float a[3], const float b[3])
{
  refpin_unreachable("raycast root projection");
}

