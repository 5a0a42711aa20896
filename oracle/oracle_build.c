/*
 * CPU oracle, part 1: PBVH build, topology tables and falloff-curve tables.
 * TEST INFRASTRUCTURE ONLY (see oracle.h).  Each function cites the reference
 * code it restates (paths relative to the reference project root).
 */
#include <float.h>
#include <limits.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "oracle_internal.h"

/* ------------------------------------------------------------------------- */
/* Float helpers: lib/intern/math_base_inline.c:402-409, math_vector_inline.c */

static inline float o_min_ff(float a, float b) { return (a < b) ? a : b; }
static inline float o_max_ff(float a, float b) { return (a > b) ? a : b; }

/* BB_reset / BB_expand / BB_expand_with_bb / BB_widest_axis /
 * BBC_update_centroid: kernel/intern/pbvh.c:1973-2023 */
static void bb_reset(float bb[6])
{
  bb[0] = bb[1] = bb[2] = FLT_MAX;
  bb[3] = bb[4] = bb[5] = -FLT_MAX;
}
static void bb_expand(float bb[6], const float co[3])
{
  for (int i = 0; i < 3; i++) {
    bb[i] = o_min_ff(bb[i], co[i]);
    bb[3 + i] = o_max_ff(bb[3 + i], co[i]);
  }
}
static void bb_expand_bb(float bb[6], const float bb2[6])
{
  for (int i = 0; i < 3; i++) {
    bb[i] = o_min_ff(bb[i], bb2[i]);
    bb[3 + i] = o_max_ff(bb[3 + i], bb2[3 + i]);
  }
}
static int bb_widest_axis(const float bb[6])
{
  float dim[3];
  for (int i = 0; i < 3; i++) {
    dim[i] = bb[3 + i] - bb[i];
  }
  if (dim[0] > dim[1]) {
    if (dim[0] > dim[2]) {
      return 0;
    }
    return 2;
  }
  if (dim[1] > dim[2]) {
    return 1;
  }
  return 2;
}

typedef struct BBC {
  float bb[6];
  float c[3];
} BBC;

static void bbc_update_centroid(BBC *b)
{
  for (int i = 0; i < 3; i++) {
    b->c[i] = (b->bb[i] + b->bb[3 + i]) * 0.5f;
  }
}

/* ------------------------------------------------------------------------- */
/* Build (pbvh.c:2070-2514) */

typedef struct BuildCtx {
  OrMesh *m;
  BBC *prim_bbc;
  float *vb; /* node BBs being written (grows with nodes) */
  int vb_cap;
  unsigned char *vert_bitmap;
  int *map_val, *map_stamp;
  int *vi_pool;
  int vi_cap;
} BuildCtx;

/* pbvh.c:2070-2088 */
static int partition_indices(int *prim_indices, int lo, int hi, int axis, float mid,
                             const BBC *prim_bbc)
{
  int i = lo, j = hi;
  for (;;) {
    for (; prim_bbc[prim_indices[i]].c[axis] < mid; i++) {
    }
    for (; mid < prim_bbc[prim_indices[j]].c[axis]; j--) {
    }
    if (!(i < j)) {
      return i;
    }
    int t = prim_indices[i];
    prim_indices[i] = prim_indices[j];
    prim_indices[j] = t;
    i++;
  }
}

/* face_materials_match / grid_materials_match: pbvh.c:2058-2066 (ME_SMOOTH = 1). */
static int prim_materials_match(const OrMesh *m, int pa, int pb)
{
  if (m->type == OR_FACES) {
    int a = m->lt_poly[pa], b = m->lt_poly[pb];
    return ((m->poly_flag[a] & 1) == (m->poly_flag[b] & 1)) && (m->poly_mat[a] == m->poly_mat[b]);
  }
  return 1; /* one material for every grid */
}

/* pbvh.c:2091-2131 */
static int partition_indices_material(OrMesh *m, int lo, int hi)
{
  int *indices = m->prim_indices;
  int first = indices[lo];
  int i = lo, j = hi;
  for (;;) {
    for (; prim_materials_match(m, first, indices[i]); i++) {
    }
    for (; !prim_materials_match(m, first, indices[j]); j--) {
    }
    if (!(i < j)) {
      return i;
    }
    int t = indices[i];
    indices[i] = indices[j];
    indices[j] = t;
    i++;
  }
}

/* pbvh_grow_nodes: pbvh.c:2133-2144 */
static void grow_nodes(BuildCtx *ctx, int totnode)
{
  OrMesh *m = ctx->m;
  if (totnode > m->node_cap) {
    int cap = m->node_cap + m->node_cap / 3;
    if (cap < totnode) {
      cap = totnode;
    }
    m->nodes = (OrNode *)realloc(m->nodes, sizeof(OrNode) * cap);
    memset(m->nodes + m->node_cap, 0, sizeof(OrNode) * (cap - m->node_cap));
    ctx->vb = (float *)realloc(ctx->vb, sizeof(float) * 6 * cap);
    m->node_cap = cap;
  }
  m->totnode = totnode;
}

/* update_vb: pbvh.c:2240-2247 (reverse prim order) */
static void update_vb(BuildCtx *ctx, int node, int offset, int count)
{
  float *vb = ctx->vb + 6 * node;
  bb_reset(vb);
  for (int i = offset + count - 1; i >= offset; i--) {
    bb_expand_bb(vb, ctx->prim_bbc[ctx->m->prim_indices[i]].bb);
  }
}

/* map_insert_vert: pbvh.c:2149-2171.  The value stored for a vertex is its
 * insertion rank among unique (positive) or shared (negative, ~rank) vertices,
 * so the resulting order does not depend on the hash map's iteration order. */
static int map_insert_vert(BuildCtx *ctx, int stamp, int *face_verts, int *uniq_verts, int v)
{
  if (ctx->map_stamp[v] != stamp) {
    int value;
    ctx->map_stamp[v] = stamp;
    if (!ctx->vert_bitmap[v]) {
      ctx->vert_bitmap[v] = 1;
      value = *uniq_verts;
      (*uniq_verts)++;
    }
    else {
      value = ~(*face_verts);
      (*face_verts)++;
    }
    ctx->map_val[v] = value;
    return value;
  }
  return ctx->map_val[v];
}

/* build_mesh_leaf_node: pbvh.c:2174-2238 */
static void build_mesh_leaf_node(BuildCtx *ctx, int node_index)
{
  OrMesh *m = ctx->m;
  OrNode *node = &m->nodes[node_index];
  int uniq = 0, face = 0;
  const int stamp = node_index + 1;
  for (int i = 0; i < node->totprim; i++) {
    const int lt = m->prim_indices[node->prim_off + i];
    for (int j = 0; j < 3; j++) {
      map_insert_vert(ctx, stamp, &face, &uniq, m->lt_v[3 * lt + j]);
    }
  }
  const int tot = uniq + face;
  if (m->vert_entries + tot > ctx->vi_cap) {
    int cap = ctx->vi_cap * 2 + tot + 1024;
    ctx->vi_pool = (int *)realloc(ctx->vi_pool, sizeof(int) * cap);
    ctx->vi_cap = cap;
  }
  int *vert_indices = ctx->vi_pool + m->vert_entries;
  /* Every vertex inserted for this leaf carries the stamp; place each at its rank. */
  for (int i = 0; i < node->totprim; i++) {
    const int lt = m->prim_indices[node->prim_off + i];
    for (int j = 0; j < 3; j++) {
      const int v = m->lt_v[3 * lt + j];
      int ndx = ctx->map_val[v];
      if (ndx < 0) {
        ndx = -ndx + uniq - 1;
      }
      vert_indices[ndx] = v;
    }
  }
  node->uniq = uniq;
  node->face_verts = face;
  node->vert_off = m->vert_entries;
  m->vert_entries += tot;
}

/* build_leaf: pbvh.c:2309-2325 */
static void build_leaf(BuildCtx *ctx, int node_index, int offset, int count)
{
  OrMesh *m = ctx->m;
  m->nodes[node_index].flag |= OR_Leaf;
  m->nodes[node_index].prim_off = offset;
  m->nodes[node_index].totprim = count;
  update_vb(ctx, node_index, offset, count);
  if (m->type == OR_FACES) {
    build_mesh_leaf_node(ctx, node_index);
  }
}

/* leaf_needs_material_split: pbvh.c:2329-2362 */
static int leaf_needs_material_split(OrMesh *m, int offset, int count)
{
  if (count <= 1) {
    return 0;
  }
  const int first = m->prim_indices[offset];
  for (int i = offset + count - 1; i > offset; i--) {
    if (!prim_materials_match(m, first, m->prim_indices[i])) {
      return 1;
    }
  }
  return 0;
}

/* build_sub: pbvh.c:2372-2425 */
static void build_sub(BuildCtx *ctx, int node_index, const float *cb_in, int offset, int count)
{
  OrMesh *m = ctx->m;
  float cb_backing[6];
  const float *cb = cb_in;
  int end;
  const int below_leaf_limit = count <= m->leaf_limit;
  if (below_leaf_limit) {
    if (!leaf_needs_material_split(m, offset, count)) {
      build_leaf(ctx, node_index, offset, count);
      return;
    }
  }
  m->nodes[node_index].children_offset = m->totnode;
  grow_nodes(ctx, m->totnode + 2);
  update_vb(ctx, node_index, offset, count);
  if (!below_leaf_limit) {
    if (!cb) {
      bb_reset(cb_backing);
      for (int i = offset + count - 1; i >= offset; i--) {
        bb_expand(cb_backing, ctx->prim_bbc[m->prim_indices[i]].c);
      }
      cb = cb_backing;
    }
    const int axis = bb_widest_axis(cb);
    end = partition_indices(m->prim_indices, offset, offset + count - 1, axis,
                            (cb[3 + axis] + cb[axis]) * 0.5f, ctx->prim_bbc);
  }
  else {
    end = partition_indices_material(m, offset, offset + count - 1);
  }
  const int child = m->nodes[node_index].children_offset;
  build_sub(ctx, child, NULL, offset, end - offset);
  build_sub(ctx, child + 1, NULL, end, offset + count - end);
}

/* pbvh_build: pbvh.c:2427-2450 */
static void pbvh_build(BuildCtx *ctx, const float cb[6], int totprim)
{
  OrMesh *m = ctx->m;
  m->totprim = totprim;
  m->prim_indices = (int *)malloc(sizeof(int) * (totprim > 0 ? totprim : 1));
  for (int i = 0; i < totprim; i++) {
    m->prim_indices[i] = i;
  }
  m->node_cap = 0;
  m->nodes = NULL;
  m->totnode = 0;
  grow_nodes(ctx, 100);
  m->totnode = 1;
  build_sub(ctx, 0, cb, 0, totprim);
}

static void finish_build(BuildCtx *ctx)
{
  OrMesh *m = ctx->m;
  const int n = m->totnode;
  m->sf.vb = (float *)malloc(sizeof(float) * 6 * n);
  m->sf.orig_vb = (float *)malloc(sizeof(float) * 6 * n);
  m->sd.vb = (double *)malloc(sizeof(double) * 6 * n);
  m->sd.orig_vb = (double *)malloc(sizeof(double) * 6 * n);
  memcpy(m->sf.vb, ctx->vb, sizeof(float) * 6 * n);
  memcpy(m->sf.orig_vb, ctx->vb, sizeof(float) * 6 * n);
  for (int i = 0; i < 6 * n; i++) {
    m->sd.vb[i] = m->sd.orig_vb[i] = (double)ctx->vb[i];
  }
  /* Leaves in left-first DFS order (pbvh.c:2700-2701 push right then left). */
  m->leaf_nodes = (int *)malloc(sizeof(int) * n);
  m->nleaf = 0;
  int *stack = (int *)malloc(sizeof(int) * (n + 1));
  int sp = 0;
  stack[sp++] = 0;
  while (sp) {
    int node = stack[--sp];
    if (m->nodes[node].flag & OR_Leaf) {
      m->leaf_nodes[m->nleaf++] = node;
    }
    else {
      stack[sp++] = m->nodes[node].children_offset + 1;
      stack[sp++] = m->nodes[node].children_offset;
    }
  }
  free(stack);
  m->vert_indices = ctx->vi_pool;
  free(ctx->vb);
}

/* ------------------------------------------------------------------------- */
/* Topology tables used by the gather-form kernels */

static void build_vertex_looptri_csr(OrMesh *m)
{
  const int V = m->totvert, T = m->totlt;
  m->vt_off = (int *)calloc(V + 1, sizeof(int));
  for (int t = 0; t < T; t++) {
    for (int j = 0; j < 3; j++) {
      m->vt_off[m->lt_v[3 * t + j] + 1]++;
    }
  }
  for (int v = 0; v < V; v++) {
    m->vt_off[v + 1] += m->vt_off[v];
  }
  m->vt_idx = (int *)malloc(sizeof(int) * (size_t)(3 * T + 1));
  int *fill = (int *)malloc(sizeof(int) * (V + 1));
  memcpy(fill, m->vt_off, sizeof(int) * (V + 1));
  for (int t = 0; t < T; t++) {
    for (int j = 0; j < 3; j++) {
      m->vt_idx[fill[m->lt_v[3 * t + j]]++] = t;
    }
  }
  free(fill);
}

/* One-ring: for each polygon around v (ascending polygon index), the previous
 * and next corner vertex of v in that polygon, keeping first occurrences. */
static void build_one_ring_csr(OrMesh *m)
{
  const int V = m->totvert, P = m->totpoly;
  int *pc = (int *)calloc(V + 1, sizeof(int));
  for (int p = 0; p < P; p++) {
    for (int k = 0; k < m->poly_totloop[p]; k++) {
      pc[m->loop_v[m->poly_loopstart[p] + k] + 1]++;
    }
  }
  for (int v = 0; v < V; v++) {
    pc[v + 1] += pc[v];
  }
  int *pidx = (int *)malloc(sizeof(int) * (size_t)(pc[V] + 1));
  int *pcorner = (int *)malloc(sizeof(int) * (size_t)(pc[V] + 1));
  int *fill = (int *)malloc(sizeof(int) * (V + 1));
  memcpy(fill, pc, sizeof(int) * (V + 1));
  for (int p = 0; p < P; p++) {
    for (int k = 0; k < m->poly_totloop[p]; k++) {
      int v = m->loop_v[m->poly_loopstart[p] + k];
      pidx[fill[v]] = p;
      pcorner[fill[v]] = k;
      fill[v]++;
    }
  }
  m->nb_off = (int *)calloc(V + 1, sizeof(int));
  int cap = pc[V] * 2 + 16;
  m->nb_idx = (int *)malloc(sizeof(int) * cap);
  int n = 0;
  for (int v = 0; v < V; v++) {
    m->nb_off[v] = n;
    for (int e = pc[v]; e < pc[v + 1]; e++) {
      const int p = pidx[e], k = pcorner[e];
      const int ls = m->poly_loopstart[p], tl = m->poly_totloop[p];
      const int cand[2] = {m->loop_v[ls + (k + tl - 1) % tl], m->loop_v[ls + (k + 1) % tl]};
      for (int c = 0; c < 2; c++) {
        int dup = 0;
        for (int q = m->nb_off[v]; q < n; q++) {
          if (m->nb_idx[q] == cand[c]) {
            dup = 1;
            break;
          }
        }
        if (!dup && cand[c] != v) {
          m->nb_idx[n++] = cand[c];
        }
      }
    }
  }
  m->nb_off[V] = n;
  free(pc);
  free(pidx);
  free(pcorner);
  free(fill);
}

static void build_lt_leaf(OrMesh *m)
{
  m->lt_leaf = (int *)malloc(sizeof(int) * (m->totlt > 0 ? m->totlt : 1));
  for (int k = 0; k < m->nleaf; k++) {
    const OrNode *nd = &m->nodes[m->leaf_nodes[k]];
    for (int i = 0; i < nd->totprim; i++) {
      m->lt_leaf[m->prim_indices[nd->prim_off + i]] = m->leaf_nodes[k];
    }
  }
}

/* ------------------------------------------------------------------------- */
/* Mesh creation */

typedef struct OMVert {
  float co[3];
  char flag, bweight, pad[2];
} OMVert;
typedef struct OMPoly {
  int loopstart, totloop;
  short mat_nr;
  char flag, pad;
} OMPoly;
typedef struct OMLoop {
  unsigned int v, e;
} OMLoop;
typedef struct OMLoopTri {
  unsigned int tri[3];
  unsigned int poly;
} OMLoopTri;

/* BKE_pbvh_build_mesh: pbvh.c:2452-2514 */
OrMesh *or_mesh_create_faces(const void *mverts, int totvert, const void *mpolys, int totpoly,
                             const void *mloops, int totloop, const void *looptris, int totlt,
                             const float *mask, const float *automask, int leaf_limit)
{
  const OMVert *mv = (const OMVert *)mverts;
  const OMPoly *mp = (const OMPoly *)mpolys;
  const OMLoop *ml = (const OMLoop *)mloops;
  const OMLoopTri *mlt = (const OMLoopTri *)looptris;
  OrMesh *m = (OrMesh *)calloc(1, sizeof(OrMesh));
  m->type = OR_FACES;
  m->totvert = totvert;
  m->totpoly = totpoly;
  m->totloop = totloop;
  m->totlt = totlt;
  m->leaf_limit = leaf_limit > 0 ? leaf_limit : 10000;
  m->poly_loopstart = (int *)malloc(sizeof(int) * (totpoly + 1));
  m->poly_totloop = (int *)malloc(sizeof(int) * (totpoly + 1));
  m->poly_mat = (short *)malloc(sizeof(short) * (totpoly + 1));
  m->poly_flag = (char *)malloc(totpoly + 1);
  for (int p = 0; p < totpoly; p++) {
    m->poly_loopstart[p] = mp[p].loopstart;
    m->poly_totloop[p] = mp[p].totloop;
    m->poly_mat[p] = mp[p].mat_nr;
    m->poly_flag[p] = mp[p].flag;
  }
  m->loop_v = (int *)malloc(sizeof(int) * (totloop + 1));
  for (int l = 0; l < totloop; l++) {
    m->loop_v[l] = (int)ml[l].v;
  }
  m->lt_v = (int *)malloc(sizeof(int) * 3 * (size_t)(totlt + 1));
  m->lt_poly = (int *)malloc(sizeof(int) * (totlt + 1));
  for (int t = 0; t < totlt; t++) {
    for (int j = 0; j < 3; j++) {
      m->lt_v[3 * t + j] = m->loop_v[mlt[t].tri[j]];
    }
    m->lt_poly[t] = (int)mlt[t].poly;
  }
  const size_t V = (size_t)totvert;
  m->sf.co = (float *)malloc(sizeof(float) * 3 * V);
  m->sf.no = (float *)calloc(3 * V, sizeof(float));
  m->sd.co = (double *)malloc(sizeof(double) * 3 * V);
  m->sd.no = (double *)calloc(3 * V, sizeof(double));
  for (size_t v = 0; v < V; v++) {
    for (int j = 0; j < 3; j++) {
      m->sf.co[3 * v + j] = mv[v].co[j];
      m->sd.co[3 * v + j] = (double)mv[v].co[j];
    }
  }
  if (mask) {
    m->sf.mask = (float *)malloc(sizeof(float) * V);
    m->sd.mask = (double *)malloc(sizeof(double) * V);
    for (size_t v = 0; v < V; v++) {
      m->sf.mask[v] = mask[v];
      m->sd.mask[v] = (double)mask[v];
    }
  }
  if (automask) {
    m->automask = (float *)malloc(sizeof(float) * V);
    memcpy(m->automask, automask, sizeof(float) * V);
  }
  m->vtag = (unsigned char *)calloc(V + 1, 1);

  BuildCtx ctx;
  memset(&ctx, 0, sizeof(ctx));
  ctx.m = m;
  ctx.prim_bbc = (BBC *)malloc(sizeof(BBC) * (totlt > 0 ? totlt : 1));
  ctx.vert_bitmap = (unsigned char *)calloc(V + 1, 1);
  ctx.map_val = (int *)malloc(sizeof(int) * (V + 1));
  ctx.map_stamp = (int *)calloc(V + 1, sizeof(int));
  float cb[6];
  bb_reset(cb);
  for (int i = 0; i < totlt; i++) {
    BBC *bbc = &ctx.prim_bbc[i];
    bb_reset(bbc->bb);
    for (int j = 0; j < 3; j++) {
      bb_expand(bbc->bb, m->sf.co + 3 * m->lt_v[3 * i + j]);
    }
    bbc_update_centroid(bbc);
    bb_expand(cb, bbc->c);
  }
  pbvh_build(&ctx, cb, totlt);
  finish_build(&ctx);
  free(ctx.prim_bbc);
  free(ctx.vert_bitmap);
  free(ctx.map_val);
  free(ctx.map_stamp);

  build_vertex_looptri_csr(m);
  build_one_ring_csr(m);
  build_lt_leaf(m);
  return m;
}

/* ------------------------------------------------------------------------- */
/* GRIDS: BKE_pbvh_build_grids (pbvh.c:2516-2561) and the CCG adjacency of
 * subdiv_ccg.c:397-549 (built from the base topology given by the caller,
 * since OpenSubdiv's topology refiner is not part of the reference). */

OrMesh *or_mesh_create_grids(int num_grids, int grid_size, const float *grids_co,
                             const float *grids_no, const float *grids_mask, int num_faces,
                             const int *face_start, const int *face_ngrids, const int *face_verts,
                             const int *face_edges, int num_base_verts, int num_base_edges,
                             const int *edge_verts, int leaf_limit)
{
  OrMesh *m = (OrMesh *)calloc(1, sizeof(OrMesh));
  m->type = OR_GRIDS;
  m->num_grids = num_grids;
  m->grid_size = grid_size;
  m->grid_area = grid_size * grid_size;
  m->totvert = num_grids * m->grid_area;
  m->num_faces = num_faces;
  const int gs = grid_size, area = m->grid_area;
  int totcorner = 0;
  m->face_start = (int *)malloc(sizeof(int) * (num_faces + 1));
  m->face_ngrids = (int *)malloc(sizeof(int) * (num_faces + 1));
  for (int f = 0; f < num_faces; f++) {
    m->face_start[f] = face_start[f];
    m->face_ngrids[f] = face_ngrids[f];
    totcorner += face_ngrids[f];
  }
  m->face_verts = (int *)malloc(sizeof(int) * (totcorner + 1));
  m->face_edges = (int *)malloc(sizeof(int) * (totcorner + 1));
  memcpy(m->face_verts, face_verts, sizeof(int) * totcorner);
  memcpy(m->face_edges, face_edges, sizeof(int) * totcorner);
  m->num_base_verts = num_base_verts;
  m->num_base_edges = num_base_edges;
  m->grid_face = (int *)malloc(sizeof(int) * (num_grids + 1));
  for (int f = 0; f < num_faces; f++) {
    for (int c = 0; c < face_ngrids[f]; c++) {
      m->grid_face[face_start[f] + c] = f;
    }
  }
  /* subdiv_ccg_init_faces_edge_neighborhood: subdiv_ccg.c:397-466.  Corner c of
   * a face uses face_verts/face_edges at (face_start + c) (grids and corners
   * share the order, subdiv_ccg.c:425-427). */
  m->edge_off = (int *)calloc(num_base_edges + 1, sizeof(int));
  for (int f = 0; f < num_faces; f++) {
    for (int c = 0; c < face_ngrids[f]; c++) {
      m->edge_off[face_edges[face_start[f] + c] + 1]++;
    }
  }
  for (int e = 0; e < num_base_edges; e++) {
    m->edge_off[e + 1] += m->edge_off[e];
  }
  m->edge_elems = (int *)malloc(sizeof(int) * (size_t)(m->edge_off[num_base_edges] * 2 * gs + 1));
  int *efill = (int *)malloc(sizeof(int) * (num_base_edges + 1));
  memcpy(efill, m->edge_off, sizeof(int) * (num_base_edges + 1));
#define ELEM_AT(g, x, y) ((g)*area + (y)*gs + (x))
  for (int f = 0; f < num_faces; f++) {
    const int n = face_ngrids[f];
    for (int corner = 0; corner < n; corner++) {
      const int vertex_index = face_verts[face_start[f] + corner];
      const int edge_index = face_edges[face_start[f] + corner];
      const int flipped = (edge_verts[2 * edge_index] != vertex_index);
      const int cur = face_start[f] + corner;
      const int next = face_start[f] + (corner + 1) % n;
      int *bc = m->edge_elems + (size_t)efill[edge_index]++ * 2 * gs;
      int k = 0;
      if (flipped) {
        for (int i = 0; i < gs; i++) {
          bc[k++] = ELEM_AT(next, gs - i - 1, gs - 1);
        }
        for (int i = 0; i < gs; i++) {
          bc[k++] = ELEM_AT(cur, gs - 1, i);
        }
      }
      else {
        for (int i = 0; i < gs; i++) {
          bc[k++] = ELEM_AT(cur, gs - 1, gs - i - 1);
        }
        for (int i = 0; i < gs; i++) {
          bc[k++] = ELEM_AT(next, i, gs - 1);
        }
      }
    }
  }
  free(efill);
  /* subdiv_ccg_init_faces_vertex_neighborhood: subdiv_ccg.c:500-531 */
  m->bvert_off = (int *)calloc(num_base_verts + 1, sizeof(int));
  for (int f = 0; f < num_faces; f++) {
    for (int c = 0; c < face_ngrids[f]; c++) {
      m->bvert_off[face_verts[face_start[f] + c] + 1]++;
    }
  }
  for (int v = 0; v < num_base_verts; v++) {
    m->bvert_off[v + 1] += m->bvert_off[v];
  }
  m->bvert_elems = (int *)malloc(sizeof(int) * (m->bvert_off[num_base_verts] + 1));
  int *vfill = (int *)malloc(sizeof(int) * (num_base_verts + 1));
  memcpy(vfill, m->bvert_off, sizeof(int) * (num_base_verts + 1));
  for (int f = 0; f < num_faces; f++) {
    for (int c = 0; c < face_ngrids[f]; c++) {
      const int g = face_start[f] + c;
      m->bvert_elems[vfill[face_verts[g]]++] = ELEM_AT(g, gs - 1, gs - 1);
    }
  }
  free(vfill);
#undef ELEM_AT

  const size_t E = (size_t)m->totvert;
  m->sf.co = (float *)malloc(sizeof(float) * 3 * E);
  m->sf.no = (float *)malloc(sizeof(float) * 3 * E);
  m->sd.co = (double *)malloc(sizeof(double) * 3 * E);
  m->sd.no = (double *)malloc(sizeof(double) * 3 * E);
  memcpy(m->sf.co, grids_co, sizeof(float) * 3 * E);
  if (grids_no) {
    memcpy(m->sf.no, grids_no, sizeof(float) * 3 * E);
  }
  else {
    memset(m->sf.no, 0, sizeof(float) * 3 * E);
  }
  for (size_t i = 0; i < 3 * E; i++) {
    m->sd.co[i] = (double)m->sf.co[i];
    m->sd.no[i] = (double)m->sf.no[i];
  }
  if (grids_mask) {
    m->sf.mask = (float *)malloc(sizeof(float) * E);
    m->sd.mask = (double *)malloc(sizeof(double) * E);
    for (size_t i = 0; i < E; i++) {
      m->sf.mask[i] = grids_mask[i];
      m->sd.mask[i] = (double)grids_mask[i];
    }
  }
  m->leaf_limit = leaf_limit > 0 ? leaf_limit : (10000 / area > 1 ? 10000 / area : 1);

  BuildCtx ctx;
  memset(&ctx, 0, sizeof(ctx));
  ctx.m = m;
  ctx.prim_bbc = (BBC *)malloc(sizeof(BBC) * (num_grids > 0 ? num_grids : 1));
  float cb[6];
  bb_reset(cb);
  for (int i = 0; i < num_grids; i++) {
    BBC *bbc = &ctx.prim_bbc[i];
    bb_reset(bbc->bb);
    for (int j = 0; j < area; j++) {
      bb_expand(bbc->bb, m->sf.co + 3 * ((size_t)i * area + j));
    }
    bbc_update_centroid(bbc);
    bb_expand(cb, bbc->c);
  }
  pbvh_build(&ctx, cb, num_grids);
  finish_build(&ctx);
  free(ctx.prim_bbc);
  return m;
}

void or_mesh_free(OrMesh *m)
{
  if (!m) {
    return;
  }
  void *ptrs[] = {m->poly_loopstart, m->poly_totloop, m->poly_mat,   m->poly_flag, m->loop_v,
                  m->lt_v,           m->lt_poly,      m->vt_off,     m->vt_idx,    m->nb_off,
                  m->nb_idx,         m->lt_leaf,      m->vtag,       m->automask,  m->face_start,
                  m->face_ngrids,    m->face_verts,   m->face_edges, m->grid_face, m->edge_off,
                  m->edge_elems,     m->bvert_off,    m->bvert_elems, m->nodes,    m->prim_indices,
                  m->vert_indices,   m->leaf_nodes,   m->sf.co,      m->sf.no,     m->sf.mask,
                  m->sf.vb,          m->sf.orig_vb,   m->sd.co,      m->sd.no,     m->sd.mask,
                  m->sd.vb,          m->sd.orig_vb,   m->sf.orig_co, m->sf.orig_no, m->sd.orig_co,
                  m->sd.orig_no,     m->sf.layer_disp, m->sd.layer_disp};
  for (size_t i = 0; i < sizeof(ptrs) / sizeof(ptrs[0]); i++) {
    free(ptrs[i]);
  }
  free(m);
}

/* ------------------------------------------------------------------------- */
/* Falloff curve (kernel/intern/colortools.c) */

typedef struct OBez {
  float vec[3][3];
  int h1, h2;
} OBez;

#define O_HD_AUTO 1

static inline float o_len_v2(const float v[2]) { return sqrtf(v[0] * v[0] + v[1] * v[1]); }
static inline float o_len_v3(const float v[3])
{
  return sqrtf(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
}

/* calchandle_curvemap: colortools.c:440-~560 (auto handles only; the brush
 * presets set no handle flags, so every point is HD_AUTO). */
static void calchandle_curvemap(OBez *bezt, const OBez *prev, const OBez *next)
{
  const float *p1, *p3;
  float *p2 = bezt->vec[1];
  float pt[3];
  float dvec_a[2], dvec_b[2], len, len_a, len_b;
  if (prev == NULL) {
    p3 = next->vec[1];
    pt[0] = 2.0f * p2[0] - p3[0];
    pt[1] = 2.0f * p2[1] - p3[1];
    p1 = pt;
  }
  else {
    p1 = prev->vec[1];
  }
  if (next == NULL) {
    p1 = prev->vec[1];
    pt[0] = 2.0f * p2[0] - p1[0];
    pt[1] = 2.0f * p2[1] - p1[1];
    p3 = pt;
  }
  else {
    p3 = next->vec[1];
  }
  dvec_a[0] = p2[0] - p1[0];
  dvec_a[1] = p2[1] - p1[1];
  dvec_b[0] = p3[0] - p2[0];
  dvec_b[1] = p3[1] - p2[1];
  len_a = o_len_v2(dvec_a);
  len_b = o_len_v2(dvec_b);
  if (len_a == 0.0f) {
    len_a = 1.0f;
  }
  if (len_b == 0.0f) {
    len_b = 1.0f;
  }
  if (bezt->h1 == O_HD_AUTO || bezt->h2 == O_HD_AUTO) {
    float tvec[2];
    tvec[0] = dvec_b[0] / len_b + dvec_a[0] / len_a;
    tvec[1] = dvec_b[1] / len_b + dvec_a[1] / len_a;
    len = o_len_v2(tvec) * 2.5614f;
    if (len != 0.0f) {
      if (bezt->h1 == O_HD_AUTO) {
        len_a /= len;
        bezt->vec[0][0] = p2[0] + tvec[0] * -len_a;
        bezt->vec[0][1] = p2[1] + tvec[1] * -len_a;
      }
      if (bezt->h2 == O_HD_AUTO) {
        len_b /= len;
        bezt->vec[2][0] = p2[0] + tvec[0] * len_b;
        bezt->vec[2][1] = p2[1] + tvec[1] * len_b;
      }
    }
  }
}

/* KERNEL_curve_forward_diff_bezier: curve.cc:1710-1736 */
static void forward_diff_bezier(float q0, float q1, float q2, float q3, float *p, int it,
                                int stride_floats)
{
  float rt0, rt1, rt2, rt3, f;
  f = (float)it;
  rt0 = q0;
  rt1 = 3.0f * (q1 - q0) / f;
  f *= f;
  rt2 = 3.0f * (q0 - 2.0f * q1 + q2) / f;
  f *= it;
  rt3 = (q3 - q0 + 3.0f * (q1 - q2)) / f;
  q0 = rt0;
  q1 = rt1 + rt2 + rt3;
  q2 = 2 * rt2 + 6 * rt3;
  q3 = 6 * rt3;
  for (int a = 0; a <= it; a++) {
    *p = q0;
    p += stride_floats;
    q0 += q1;
    q1 += q2;
    q2 += q3;
  }
}

/* BKE_fcurve_correct_bezpart: fcurve.c:1407-1444 */
static void correct_bezpart(const float v1[2], float v2[2], float v3[2], const float v4[2])
{
  float h1[2], h2[2], len1, len2, len, fac;
  h1[0] = v1[0] - v2[0];
  h1[1] = v1[1] - v2[1];
  h2[0] = v4[0] - v3[0];
  h2[1] = v4[1] - v3[1];
  len = v4[0] - v1[0];
  len1 = fabsf(h1[0]);
  len2 = fabsf(h2[0]);
  if ((len1 + len2) == 0.0f) {
    return;
  }
  if (len1 > len) {
    fac = len / len1;
    v2[0] = (v1[0] - fac * h1[0]);
    v2[1] = (v1[1] - fac * h1[1]);
  }
  if (len2 > len) {
    fac = len / len2;
    v3[0] = (v4[0] - fac * h2[0]);
    v3[1] = (v4[1] - fac * h2[1]);
  }
}

/* curvemap_calc_extend with CUMA_EXTEND_EXTRAPOLATE off: colortools.c:563-595 */
static float calc_extend_horizontal(float x, const float first[2], const float last[2])
{
  if (x <= first[0]) {
    return first[1];
  }
  if (x >= last[0]) {
    return last[1];
  }
  return 0.0f;
}

/* KERNEL_curvemap_reset presets (colortools.c:249-~330) on clip rect [0,1]^2,
 * negative slope. Returns the point count. */
static int curve_preset_points(int preset, float *xs, float *ys)
{
  switch (preset) {
    case 0: /* LINE */
      xs[0] = 0.0f, ys[0] = 1.0f, xs[1] = 1.0f, ys[1] = 0.0f;
      return 2;
    case 1: /* SHARP */
      xs[0] = 0, ys[0] = 1, xs[1] = 0.25f, ys[1] = 0.50f, xs[2] = 0.75f, ys[2] = 0.04f;
      xs[3] = 1, ys[3] = 0;
      return 4;
    case 2: /* SMOOTH */
      xs[0] = 0, ys[0] = 1, xs[1] = 0.25f, ys[1] = 0.94f, xs[2] = 0.75f, ys[2] = 0.06f;
      xs[3] = 1, ys[3] = 0;
      return 4;
    case 3: /* MAX */
      xs[0] = 0, ys[0] = 1, xs[1] = 1, ys[1] = 1;
      return 2;
    case 5: /* ROUND */
      xs[0] = 0, ys[0] = 1, xs[1] = 0.5f, ys[1] = 0.90f, xs[2] = 0.86f, ys[2] = 0.5f;
      xs[3] = 1, ys[3] = 0;
      return 4;
    case 6: /* ROOT */
      xs[0] = 0, ys[0] = 1, xs[1] = 0.25f, ys[1] = 0.95f, xs[2] = 0.75f, ys[2] = 0.44f;
      xs[3] = 1, ys[3] = 0;
      return 4;
    default:
      return 0;
  }
}

/* curvemap_make_table: colortools.c:597-771 */
static void curve_make(int preset, OrCurve *cu)
{
  float xs[9], ys[9];
  const int totpoint = curve_preset_points(preset, xs, ys);
  memset(cu, 0, sizeof(*cu));
  cu->flag = 1; /* CUMA_DO_CLIP */
  if (totpoint == 0) {
    return;
  }
  cu->mintable = 0.0f;
  cu->maxtable = 1.0f;
  OBez bezt[9];
  memset(bezt, 0, sizeof(bezt));
  for (int a = 0; a < totpoint; a++) {
    cu->mintable = o_min_ff(cu->mintable, xs[a]);
    cu->maxtable = o_max_ff(cu->maxtable, xs[a]);
    bezt[a].vec[1][0] = xs[a];
    bezt[a].vec[1][1] = ys[a];
    bezt[a].h1 = bezt[a].h2 = O_HD_AUTO;
  }
  const OBez *prev = NULL;
  for (int a = 0; a < totpoint; a++) {
    const OBez *next = (a != totpoint - 1) ? &bezt[a + 1] : NULL;
    calchandle_curvemap(&bezt[a], prev, next);
    prev = &bezt[a];
  }
  if (totpoint > 2) {
    float hlen, nlen, vec[3];
    if (bezt[0].h2 == O_HD_AUTO) {
      float d[3] = {bezt[0].vec[1][0] - bezt[0].vec[2][0], bezt[0].vec[1][1] - bezt[0].vec[2][1],
                    bezt[0].vec[1][2] - bezt[0].vec[2][2]};
      hlen = o_len_v3(d);
      vec[0] = bezt[1].vec[0][0];
      vec[1] = bezt[1].vec[0][1];
      vec[2] = bezt[1].vec[0][2];
      if (vec[0] < bezt[0].vec[1][0]) {
        vec[0] = bezt[0].vec[1][0];
      }
      for (int i = 0; i < 3; i++) {
        vec[i] -= bezt[0].vec[1][i];
      }
      nlen = o_len_v3(vec);
      if (nlen > FLT_EPSILON) {
        for (int i = 0; i < 3; i++) {
          vec[i] *= hlen / nlen;
        }
        for (int i = 0; i < 3; i++) {
          bezt[0].vec[2][i] = vec[i] + bezt[0].vec[1][i];
        }
        for (int i = 0; i < 3; i++) {
          bezt[0].vec[0][i] = bezt[0].vec[1][i] - vec[i];
        }
      }
    }
    const int a = totpoint - 1;
    if (bezt[a].h2 == O_HD_AUTO) {
      float d[3] = {bezt[a].vec[1][0] - bezt[a].vec[0][0], bezt[a].vec[1][1] - bezt[a].vec[0][1],
                    bezt[a].vec[1][2] - bezt[a].vec[0][2]};
      hlen = o_len_v3(d);
      vec[0] = bezt[a - 1].vec[2][0];
      vec[1] = bezt[a - 1].vec[2][1];
      vec[2] = bezt[a - 1].vec[2][2];
      if (vec[0] > bezt[a].vec[1][0]) {
        vec[0] = bezt[a].vec[1][0];
      }
      for (int i = 0; i < 3; i++) {
        vec[i] -= bezt[a].vec[1][i];
      }
      nlen = o_len_v3(vec);
      if (nlen > FLT_EPSILON) {
        for (int i = 0; i < 3; i++) {
          vec[i] *= hlen / nlen;
        }
        for (int i = 0; i < 3; i++) {
          bezt[a].vec[0][i] = vec[i] + bezt[a].vec[1][i];
        }
        for (int i = 0; i < 3; i++) {
          bezt[a].vec[2][i] = bezt[a].vec[1][i] - vec[i];
        }
      }
    }
  }
  const int totpt = (totpoint - 1) * OR_CM_RESOL;
  float *allpoints = (float *)calloc((size_t)totpt * 2, sizeof(float));
  float *point = allpoints;
  for (int a = 0; a < totpoint - 1; a++, point += 2 * OR_CM_RESOL) {
    correct_bezpart(bezt[a].vec[1], bezt[a].vec[2], bezt[a + 1].vec[0], bezt[a + 1].vec[1]);
    forward_diff_bezier(bezt[a].vec[1][0], bezt[a].vec[2][0], bezt[a + 1].vec[0][0],
                        bezt[a + 1].vec[1][0], point, OR_CM_RESOL - 1, 2);
    forward_diff_bezier(bezt[a].vec[1][1], bezt[a].vec[2][1], bezt[a + 1].vec[0][1],
                        bezt[a + 1].vec[1][1], point + 1, OR_CM_RESOL - 1, 2);
  }
  cu->ext_in[0] = bezt[0].vec[0][0] - bezt[0].vec[1][0];
  cu->ext_in[1] = bezt[0].vec[0][1] - bezt[0].vec[1][1];
  float ext_in_range = sqrtf(cu->ext_in[0] * cu->ext_in[0] + cu->ext_in[1] * cu->ext_in[1]);
  cu->ext_in[0] /= ext_in_range;
  cu->ext_in[1] /= ext_in_range;
  const int out_a = totpoint - 1;
  cu->ext_out[0] = bezt[out_a].vec[1][0] - bezt[out_a].vec[2][0];
  cu->ext_out[1] = bezt[out_a].vec[1][1] - bezt[out_a].vec[2][1];
  float ext_out_range = sqrtf(cu->ext_out[0] * cu->ext_out[0] + cu->ext_out[1] * cu->ext_out[1]);
  cu->ext_out[0] /= ext_out_range;
  cu->ext_out[1] /= ext_out_range;

  float range = (1.0f / 256.0f) * (cu->maxtable - cu->mintable);
  cu->range = 1.0f / range;
  float *firstpoint = allpoints;
  float *lastpoint = allpoints + 2 * (totpt - 1);
  point = allpoints;
  for (int a = 0; a <= OR_CM_TABLE; a++) {
    float cur_x = cu->mintable + range * (float)a;
    cu->table[2 * a] = cur_x;
    while (cur_x >= point[0] && point != lastpoint) {
      point += 2;
    }
    if (point == firstpoint || (point == lastpoint && cur_x >= point[0])) {
      if (fabsf(cur_x - point[0]) <= 1e-6f) {
        cu->table[2 * a + 1] = point[1];
      }
      else {
        cu->table[2 * a + 1] = calc_extend_horizontal(cur_x, firstpoint, lastpoint);
      }
    }
    else {
      float fac1 = point[0] - point[-2];
      float fac2 = point[0] - cur_x;
      if (fac1 > FLT_EPSILON) {
        fac1 = fac2 / fac1;
      }
      else {
        fac1 = 0.0f;
      }
      cu->table[2 * a + 1] = fac1 * point[-1] + (1.0f - fac1) * point[1];
    }
  }
  free(allpoints);
}

void or_curve_build(int preset, OrCurve *cu) { curve_make(preset, cu); }

void or_curve_table(int preset, float *table_xy, float *params)
{
  OrCurve cu;
  curve_make(preset, &cu);
  memcpy(table_xy, cu.table, sizeof(cu.table));
  params[0] = cu.mintable;
  params[1] = cu.maxtable;
  params[2] = cu.range;
  params[3] = cu.ext_in[0];
  params[4] = cu.ext_in[1];
  params[5] = cu.ext_out[0];
  params[6] = cu.ext_out[1];
}

/* ------------------------------------------------------------------------- */
/* Accessors */

int or_num_nodes(const OrMesh *m) { return m->totnode; }
int or_num_leaves(const OrMesh *m) { return m->nleaf; }
int or_num_verts(const OrMesh *m) { return m->totvert; }
int or_num_leaf_vert_entries(const OrMesh *m) { return m->vert_entries; }

void or_get_nodes(const OrMesh *m, int *children_offset, int *flag, int *prim_off, int *totprim,
                  int *uniq, int *face_verts, int *vert_off)
{
  for (int i = 0; i < m->totnode; i++) {
    const OrNode *n = &m->nodes[i];
    const int leaf = n->flag & OR_Leaf;
    children_offset[i] = leaf ? -1 : n->children_offset;
    flag[i] = n->flag;
    prim_off[i] = leaf ? n->prim_off : -1;
    totprim[i] = leaf ? n->totprim : 0;
    uniq[i] = leaf ? n->uniq : 0;
    face_verts[i] = leaf ? n->face_verts : 0;
    vert_off[i] = leaf ? n->vert_off : -1;
  }
}
void or_get_prim_indices(const OrMesh *m, int *out)
{
  memcpy(out, m->prim_indices, sizeof(int) * m->totprim);
}
void or_get_vert_indices(const OrMesh *m, int *out)
{
  memcpy(out, m->vert_indices, sizeof(int) * m->vert_entries);
}
void or_get_bbs(const OrMesh *m, float *vb, float *orig_vb)
{
  memcpy(vb, m->sf.vb, sizeof(float) * 6 * m->totnode);
  memcpy(orig_vb, m->sf.orig_vb, sizeof(float) * 6 * m->totnode);
}
void or_get_bbs64(const OrMesh *m, double *vb, double *orig_vb)
{
  memcpy(vb, m->sd.vb, sizeof(double) * 6 * m->totnode);
  memcpy(orig_vb, m->sd.orig_vb, sizeof(double) * 6 * m->totnode);
}
void or_get_co(const OrMesh *m, float *out)
{
  memcpy(out, m->sf.co, sizeof(float) * 3 * (size_t)m->totvert);
}
void or_get_no(const OrMesh *m, float *out)
{
  memcpy(out, m->sf.no, sizeof(float) * 3 * (size_t)m->totvert);
}
void or_get_mask(const OrMesh *m, float *out)
{
  if (m->sf.mask) {
    memcpy(out, m->sf.mask, sizeof(float) * (size_t)m->totvert);
  }
}
void or_get_co64(const OrMesh *m, double *out)
{
  memcpy(out, m->sd.co, sizeof(double) * 3 * (size_t)m->totvert);
}
void or_get_no64(const OrMesh *m, double *out)
{
  memcpy(out, m->sd.no, sizeof(double) * 3 * (size_t)m->totvert);
}
void or_set_co(OrMesh *m, const float *co)
{
  memcpy(m->sf.co, co, sizeof(float) * 3 * (size_t)m->totvert);
  for (size_t i = 0; i < 3 * (size_t)m->totvert; i++) {
    m->sd.co[i] = (double)co[i];
  }
}
