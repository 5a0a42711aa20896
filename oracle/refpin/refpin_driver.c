/*
 * Driver of the reference-pinning harness — TEST INFRASTRUCTURE ONLY.
 *
 * A flat C API (loaded by tests/ through ctypes) over the reference's own
 * compiled PBVH code: BKE_pbvh_new + BKE_pbvh_build_mesh / _build_grids
 * (pbvh.c:2563, :2452-2514, :2516-2561 of the complete copy),
 * BKE_pbvh_search_gather (:2736-2767), BKE_pbvh_node_mark_update (:3641),
 * BKE_pbvh_vert_mark_update (:3729), BKE_pbvh_update_normals (:4559) and
 * BKE_pbvh_update_bounds (:3319).  The one piece of logic written here is the
 * sculpt sphere search callback, which the reference does not ship (its
 * sculpt.c is missing); it is the brush specification's test: per axis the
 * closest point of the box, hit iff the squared distance is < radius_sq.
 */
#include "refpin_prelude.h"

#include "pbvh_intern.h"

void refpin_set_mesh_normals(const Mesh *mesh, float (*normals)[3]);

/* pbvh.c's LEAF_LIMIT (Makefile substitution); the reference's value by default. */
int refpin_leaf_limit = 10000;
void rp_set_leaf_limit(int leaf_limit)
{
  refpin_leaf_limit = leaf_limit;
}

typedef struct RefPin {
  PBVH *pbvh;
  Mesh mesh;
  /* FACES */
  MVert *verts;
  MPoly *polys;
  MLoop *loops;
  MLoopTri *looptris;
  float (*normals)[3];
  float *mask;
  CustomData vdata;
  CustomDataLayer mask_layer;
  int totvert;
  /* GRIDS */
  CCGKey key;
  float *grid_mem;
  CCGElem **grids;
  DMFlagMat *flagmats;
  BLI_bitmap **grid_hidden;
  int totgrid;
} RefPin;

RefPin *rp_build_faces(const void *mverts, int totvert, const void *mpolys, int totpoly,
                       const void *mloops, int totloop, const void *looptris, int totlt,
                       const float *vert_normals, const float *mask)
{
  RefPin *r = calloc(1, sizeof(RefPin));
  r->totvert = totvert;
  r->verts = malloc(sizeof(MVert) * (size_t)(totvert ? totvert : 1));
  memcpy(r->verts, mverts, sizeof(MVert) * (size_t)totvert);
  r->polys = malloc(sizeof(MPoly) * (size_t)(totpoly ? totpoly : 1));
  memcpy(r->polys, mpolys, sizeof(MPoly) * (size_t)totpoly);
  r->loops = malloc(sizeof(MLoop) * (size_t)(totloop ? totloop : 1));
  memcpy(r->loops, mloops, sizeof(MLoop) * (size_t)totloop);
  /* BKE_pbvh_free releases the looptri array (pbvh.c:2606). */
  r->looptris = MEM_mallocN(sizeof(MLoopTri) * (size_t)(totlt ? totlt : 1), "looptris");
  memcpy(r->looptris, looptris, sizeof(MLoopTri) * (size_t)totlt);
  r->normals = malloc(sizeof(float[3]) * (size_t)(totvert ? totvert : 1));
  memcpy(r->normals, vert_normals, sizeof(float[3]) * (size_t)totvert);
  if (mask) {
    r->mask = malloc(sizeof(float) * (size_t)(totvert ? totvert : 1));
    memcpy(r->mask, mask, sizeof(float) * (size_t)totvert);
    r->mask_layer.type = CD_PAINT_MASK;
    r->mask_layer.data = r->mask;
    r->vdata.layers = &r->mask_layer;
    r->vdata.totlayer = 1;
  }
  refpin_set_mesh_normals(&r->mesh, r->normals);
  r->pbvh = BKE_pbvh_new();
  BKE_pbvh_build_mesh(r->pbvh, &r->mesh, r->polys, r->loops, r->verts, totvert, &r->vdata,
                      NULL, NULL, r->looptris, totlt);
  return r;
}

/* co, no: num_grids * grid_size^2 * 3 floats; mask nullable. */
RefPin *rp_build_grids(int num_grids, int grid_size, const float *co, const float *no,
                       const float *mask)
{
  RefPin *r = calloc(1, sizeof(RefPin));
  const int area = grid_size * grid_size;
  r->key.grid_size = grid_size;
  r->key.grid_area = area;
  r->key.has_normals = 1;
  r->key.has_mask = mask != NULL;
  r->key.mask_offset = mask ? (int)sizeof(float[3]) : -1;
  r->key.normal_offset = (int)sizeof(float[3]) + (mask ? (int)sizeof(float) : 0);
  r->key.elem_size = r->key.normal_offset + (int)sizeof(float[3]);
  r->key.grid_bytes = r->key.elem_size * area;
  const int nf = r->key.elem_size / (int)sizeof(float);
  r->totgrid = num_grids;
  r->grid_mem = malloc(sizeof(float) * (size_t)nf * (size_t)area * (size_t)(num_grids ? num_grids : 1));
  r->grids = malloc(sizeof(CCGElem *) * (size_t)(num_grids ? num_grids : 1));
  for (int g = 0; g < num_grids; g++) {
    r->grids[g] = (CCGElem *)(r->grid_mem + (size_t)g * (size_t)area * (size_t)nf);
    for (int e = 0; e < area; e++) {
      const size_t i = (size_t)g * (size_t)area + (size_t)e;
      CCGElem *el = CCG_elem_offset(&r->key, r->grids[g], e);
      memcpy(CCG_elem_co(&r->key, el), co + 3 * i, sizeof(float[3]));
      memcpy(CCG_elem_no(&r->key, el), no + 3 * i, sizeof(float[3]));
      if (mask) {
        *CCG_elem_mask(&r->key, el) = mask[i];
      }
    }
  }
  /* One material for every grid: leaf_needs_material_split reads the flag mats
   * of every grid (pbvh.c:2329-2362). */
  r->flagmats = calloc((size_t)(num_grids ? num_grids : 1), sizeof(DMFlagMat));
  /* No hidden elements: one NULL bitmap per grid, as subdiv_ccg allocates it
   * (BKE_pbvh_count_grid_quads reads it per leaf grid). */
  r->grid_hidden = calloc((size_t)(num_grids ? num_grids : 1), sizeof(BLI_bitmap *));
  r->pbvh = BKE_pbvh_new();
  BKE_pbvh_build_grids(r->pbvh, r->grids, num_grids, &r->key, NULL, r->flagmats,
                       r->grid_hidden);
  return r;
}

void rp_free(RefPin *r)
{
  if (!r) {
    return;
  }
  BKE_pbvh_free(r->pbvh);
  free(r->verts);
  free(r->polys);
  free(r->loops);
  free(r->normals);
  free(r->mask);
  free(r->grid_mem);
  free(r->grids);
  free(r->flagmats);
  free(r->grid_hidden);
  free(r);
}

int rp_num_nodes(const RefPin *r)
{
  return r->pbvh->totnode;
}
int rp_leaf_limit(const RefPin *r)
{
  return r->pbvh->leaf_limit;
}

/* Per node: children_offset (-1 for leaves), flag, offset of its prims in the
 * prim_indices array (-1 for internal nodes), totprim, uniq_verts, face_verts. */
void rp_get_nodes(const RefPin *r, int *children_offset, int *flag, int *prim_off, int *totprim,
                  int *uniq, int *face_verts)
{
  const PBVH *p = r->pbvh;
  for (int i = 0; i < p->totnode; i++) {
    const PBVHNode *n = &p->nodes[i];
    const int leaf = (n->flag & PBVH_Leaf) != 0;
    children_offset[i] = leaf ? -1 : n->children_offset;
    flag[i] = n->flag;
    prim_off[i] = leaf ? (int)(n->prim_indices - p->prim_indices) : -1;
    totprim[i] = leaf ? (int)n->totprim : 0;
    uniq[i] = leaf ? (int)n->uniq_verts : 0;
    face_verts[i] = leaf ? (int)n->face_verts : 0;
  }
}
void rp_get_prim_indices(const RefPin *r, int *out)
{
  memcpy(out, r->pbvh->prim_indices, sizeof(int) * (size_t)r->pbvh->totprim);
}
/* vert_indices of one leaf (uniq_verts + face_verts entries; FACES only). */
void rp_get_node_vert_indices(const RefPin *r, int node, int *out)
{
  const PBVHNode *n = &r->pbvh->nodes[node];
  if (n->vert_indices) {
    memcpy(out, n->vert_indices, sizeof(int) * (size_t)(n->uniq_verts + n->face_verts));
  }
}
/* face_vert_indices of one leaf (3 per prim; FACES only). */
void rp_get_node_face_vert_indices(const RefPin *r, int node, int *out)
{
  const PBVHNode *n = &r->pbvh->nodes[node];
  if (n->face_vert_indices) {
    memcpy(out, n->face_vert_indices, sizeof(int[3]) * (size_t)n->totprim);
  }
}
void rp_get_bbs(const RefPin *r, float *vb, float *orig_vb)
{
  const PBVH *p = r->pbvh;
  for (int i = 0; i < p->totnode; i++) {
    memcpy(vb + 6 * i, &p->nodes[i].vb, sizeof(float[6]));
    memcpy(orig_vb + 6 * i, &p->nodes[i].orig_vb, sizeof(float[6]));
  }
}

typedef struct SphereSearch {
  float center[3];
  float radius_sq;
  int original;
} SphereSearch;

static bool sphere_cb(PBVHNode *node, void *data_v)
{
  const SphereSearch *s = data_v;
  float bmin[3], bmax[3];
  if (s->original) {
    BKE_pbvh_node_get_original_BB(node, bmin, bmax);
  }
  else {
    BKE_pbvh_node_get_BB(node, bmin, bmax);
  }
  float t[3];
  for (int i = 0; i < 3; i++) {
    const float c = s->center[i];
    const float nearest = bmin[i] > c ? bmin[i] : (bmax[i] < c ? bmax[i] : c);
    t[i] = c - nearest;
  }
  return t[0] * t[0] + t[1] * t[1] + t[2] * t[2] < s->radius_sq;
}

/* BKE_pbvh_search_gather with the sphere callback; node indices out. */
int rp_search_sphere(RefPin *r, const float center[3], float radius_sq, int original,
                     int *out_nodes)
{
  SphereSearch s = {{center[0], center[1], center[2]}, radius_sq, original};
  PBVHNode **nodes = NULL;
  int tot = 0;
  BKE_pbvh_search_gather(r->pbvh, sphere_cb, &s, &nodes, &tot);
  for (int i = 0; i < tot; i++) {
    out_nodes[i] = (int)(nodes[i] - r->pbvh->nodes);
  }
  MEM_SAFE_FREE(nodes);
  return tot;
}

/* FACES: new positions (3 floats per vertex) written into the MVert array. */
void rp_set_co(RefPin *r, const float *co)
{
  for (int v = 0; v < r->totvert; v++) {
    memcpy(r->verts[v].co, co + 3 * v, sizeof(float[3]));
  }
}
/* GRIDS: new element positions (3 floats per element). */
void rp_set_grid_co(RefPin *r, const float *co)
{
  const int area = r->key.grid_area;
  for (int g = 0; g < r->totgrid; g++) {
    for (int e = 0; e < area; e++) {
      memcpy(CCG_elem_offset_co(&r->key, r->grids[g], e), co + 3 * ((size_t)g * area + e),
             sizeof(float[3]));
    }
  }
}
void rp_get_no(const RefPin *r, float *out)
{
  memcpy(out, r->normals, sizeof(float[3]) * (size_t)r->totvert);
}
void rp_node_mark_update(RefPin *r, int node)
{
  BKE_pbvh_node_mark_update(&r->pbvh->nodes[node]);
}
void rp_vert_mark_update(RefPin *r, int vertex)
{
  BKE_pbvh_vert_mark_update(r->pbvh, vertex);
}
void rp_update_normals(RefPin *r)
{
  BKE_pbvh_update_normals(r->pbvh, NULL);
}
void rp_update_bounds(RefPin *r, int flag)
{
  BKE_pbvh_update_bounds(r->pbvh, flag);
}
int rp_node_flag(const RefPin *r, int node)
{
  return r->pbvh->nodes[node].flag;
}

/* ---- falloff curve (colortools.c) ---- */
void KERNEL_curvemapping_set_defaults(CurveMapping *cumap, int tot, float minx, float miny,
                                      float maxx, float maxy);
void KERNEL_curvemap_reset(CurveMap *cuma, const rctf *clipr, int preset, int slope);
void KERNEL_curvemapping_changed(CurveMapping *cumap, const bool rem_doubles);
float KERNEL_curvemapping_evaluateF(const CurveMapping *cumap, int cur, float value);
void KERNEL_curvemapping_free_data(CurveMapping *cumap);

/* A brush falloff curve as the brush specification sets it up: one curve on
 * the clip rectangle [0,1]^2, reset to `preset` with negative slope, clipping
 * on, horizontal extension (CUMA_EXTEND_EXTRAPOLATE off), then
 * KERNEL_curvemapping_changed builds the 257-entry table. */
static void brush_curve(CurveMapping *cumap, int preset)
{
  memset(cumap, 0, sizeof(*cumap));
  KERNEL_curvemapping_set_defaults(cumap, 1, 0.0f, 0.0f, 1.0f, 1.0f);
  cumap->flag &= ~CUMA_EXTEND_EXTRAPOLATE;
  cumap->preset = preset;
  KERNEL_curvemap_reset(&cumap->cm[0], &cumap->clipr, preset, CURVEMAP_SLOPE_NEGATIVE);
  KERNEL_curvemapping_changed(cumap, false);
}

/* table_xy: (CM_TABLE + 1) x (x, y); params: mintable, maxtable, range,
 * ext_in[2], ext_out[2]. */
void rp_curve_table(int preset, float *table_xy, float *params)
{
  CurveMapping cumap;
  brush_curve(&cumap, preset);
  const CurveMap *cuma = &cumap.cm[0];
  for (int i = 0; i <= CM_TABLE; i++) {
    table_xy[2 * i] = cuma->table[i].x;
    table_xy[2 * i + 1] = cuma->table[i].y;
  }
  params[0] = cuma->mintable;
  params[1] = cuma->maxtable;
  params[2] = cuma->range;
  params[3] = cuma->ext_in[0];
  params[4] = cuma->ext_in[1];
  params[5] = cuma->ext_out[0];
  params[6] = cuma->ext_out[1];
  KERNEL_curvemapping_free_data(&cumap);
}

/* KERNEL_curvemapping_evaluateF of the brush curve at n values. */
void rp_curve_evaluate(int preset, const float *values, int n, float *out)
{
  CurveMapping cumap;
  brush_curve(&cumap, preset);
  for (int i = 0; i < n; i++) {
    out[i] = KERNEL_curvemapping_evaluateF(&cumap, 0, values[i]);
  }
  KERNEL_curvemapping_free_data(&cumap);
}

/* ---- ray cast (pbvh.c:3897-3929, 4042-4108, 4204-4262) ---- */
typedef struct RaycastCb {
  PBVH *pbvh;
  const float *start, *normal;
  IsectRayPrecalc isect;
  float depth;
  int active_vertex, active_face;
  float face_normal[3];
  bool hit;
} RaycastCb;

/* The sculpt ray-cast callback of the brush specification (the reference's
 * sculpt.c, which would hold it, is absent): a node is ray cast when its entry
 * distance is below the running minimum; a hit lowers the minimum to the hit
 * depth. */
static void raycast_cb(PBVHNode *node, void *data_v, float *tmin)
{
  RaycastCb *d = data_v;
  if (BKE_pbvh_node_get_tmin(node) < *tmin) {
    if (BKE_pbvh_node_raycast(d->pbvh, node, NULL, false, d->start, d->normal, &d->isect,
                              &d->depth, &d->active_vertex, &d->active_face, d->face_normal)) {
      d->hit = true;
      *tmin = d->depth;
    }
  }
}

/* BKE_pbvh_raycast with that callback; depth in = ray length, out = hit depth. */
int rp_raycast(RefPin *r, const float start[3], const float normal[3], int original, float *depth,
               int *active_vertex, int *active_face, float face_normal[3])
{
  RaycastCb d;
  memset(&d, 0, sizeof(d));
  d.pbvh = r->pbvh;
  d.start = start;
  d.normal = normal;
  d.depth = *depth;
  d.active_vertex = d.active_face = -1;
  isect_ray_tri_watertight_v3_precalc(&d.isect, normal);
  BKE_pbvh_raycast(r->pbvh, raycast_cb, &d, start, normal, original != 0);
  *depth = d.depth;
  *active_vertex = d.active_vertex;
  *active_face = d.active_face;
  memcpy(face_normal, d.face_normal, sizeof(float[3]));
  return d.hit ? 1 : 0;
}

/* ---- nearest to ray (pbvh.c:4315-4494) ---- */
typedef struct NearestCb {
  PBVH *pbvh;
  const float *start, *normal;
  float depth, dist_sq;
  bool hit;
} NearestCb;

/* The sculpt nearest-to-ray callback of the brush specification (the
 * reference's sculpt.c, which would hold it, is absent), the same rule as the
 * ray cast's: a node is searched when its squared distance to the ray is
 * below the running minimum; a found triangle lowers the minimum to its
 * squared distance. */
static void nearest_cb(PBVHNode *node, void *data_v, float *tmin)
{
  NearestCb *d = data_v;
  if (BKE_pbvh_node_get_tmin(node) < *tmin) {
    if (BKE_pbvh_node_find_nearest_to_ray(d->pbvh, node, NULL, false, d->start, d->normal,
                                          &d->depth, &d->dist_sq)) {
      d->hit = true;
      *tmin = d->dist_sq;
    }
  }
}

/* BKE_pbvh_find_nearest_to_ray with that callback; depth and dist_sq in =
 * the starting values (FLT_MAX), out = the nearest triangle's. */
int rp_nearest_to_ray(RefPin *r, const float start[3], const float normal[3], int original,
                      float *depth, float *dist_sq)
{
  NearestCb d;
  memset(&d, 0, sizeof(d));
  d.pbvh = r->pbvh;
  d.start = start;
  d.normal = normal;
  d.depth = *depth;
  d.dist_sq = *dist_sq;
  BKE_pbvh_find_nearest_to_ray(r->pbvh, nearest_cb, &d, start, normal, original != 0);
  *depth = d.depth;
  *dist_sq = d.dist_sq;
  return d.hit ? 1 : 0;
}

/* The PBVH of a harness mesh (the draw-buffer functions of refpin_draw.c take it). */
PBVH *rp_pbvh(RefPin *r)
{
  return r->pbvh;
}

/* The reference's Kelvinlet displacement of one element (kelvinlet.c):
 * BKE_kelvinlet_init_params(radius, force, 1, poisson), then type 0 grab,
 * 1 grab_biscale, 2 grab_triscale (dn = brush delta), 3 scale, 4 twist
 * (dn = surface normal). */
#include "BKE_kelvinlet.h"
void rp_kelvinlet(int type, float radius, float force, float poisson, const float co[3],
                  const float location[3], const float dn[3], float out[3])
{
  KelvinletParams p;
  BKE_kelvinlet_init_params(&p, radius, force, 1.0f, poisson);
  switch (type) {
    case 0:
      BKE_kelvinlet_grab(out, &p, co, location, dn);
      break;
    case 1:
      BKE_kelvinlet_grab_biscale(out, &p, co, location, dn);
      break;
    case 2:
      BKE_kelvinlet_grab_triscale(out, &p, co, location, dn);
      break;
    case 3:
      BKE_kelvinlet_scale(out, &p, co, location, dn);
      break;
    default:
      BKE_kelvinlet_twist(out, &p, co, location, dn);
      break;
  }
}
