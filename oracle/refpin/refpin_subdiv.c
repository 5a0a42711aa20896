/*
 * Multires part of the reference-pinning harness — TEST INFRASTRUCTURE ONLY.
 *
 * Compiles the reference's subdiv_ccg.c (whole file, included below so that
 * its static set-up functions can be called) and drives it without
 * OpenSubdiv:
 *   - the topology refiner is a table of query functions answered from the
 *     base mesh's arrays (face -> corner vertices / edges, edge -> vertices);
 *   - the grid elements are written from the caller's positions, normals and
 *     masks, standing in for the limit-surface evaluation (subdiv_ccg.c:200-
 *     312) that needs OpenSubdiv; grid_faces and material flags are assigned
 *     as that evaluation assigns them.
 * The reference's own code then builds the layers and element storage
 * (subdiv_ccg_init_layers, subdiv_ccg_alloc_elements, subdiv_ccg_init_faces),
 * the edge and vertex adjacency (subdiv_ccg_init_faces_neighborhood,
 * :397-540), the PBVH (BKE_pbvh_build_grids), and per update
 * BKE_pbvh_update_normals -> BKE_pbvh_get_grid_updates ->
 * KERNEL_subdiv_ccg_update_normals (inner normals, face-seam stitching,
 * boundary and corner averaging of positions, normals and masks) and
 * BKE_pbvh_update_bounds.
 */
#include "refpin_prelude.h"

#include "subdiv_ccg_ref.c"

#include "pbvh_intern.h"

void rp_set_leaf_limit(int leaf_limit);

typedef struct BaseTopology {
  int num_verts, num_edges, num_faces;
  int *face_start, *face_ncorners, *face_verts, *face_edges, *edge_verts;
} BaseTopology;

static const BaseTopology *topo_of(const OpenSubdiv_TopologyRefiner *r)
{
  return (const BaseTopology *)r->user_data;
}
static int tr_num_vertices(const OpenSubdiv_TopologyRefiner *r)
{
  return topo_of(r)->num_verts;
}
static int tr_num_edges(const OpenSubdiv_TopologyRefiner *r)
{
  return topo_of(r)->num_edges;
}
static int tr_num_faces(const OpenSubdiv_TopologyRefiner *r)
{
  return topo_of(r)->num_faces;
}
static int tr_num_face_vertices(const OpenSubdiv_TopologyRefiner *r, int face)
{
  return topo_of(r)->face_ncorners[face];
}
static void tr_face_vertices(const OpenSubdiv_TopologyRefiner *r, int face, int *out)
{
  const BaseTopology *t = topo_of(r);
  memcpy(out, t->face_verts + t->face_start[face], sizeof(int) * (size_t)t->face_ncorners[face]);
}
static void tr_face_edges(const OpenSubdiv_TopologyRefiner *r, int face, int *out)
{
  const BaseTopology *t = topo_of(r);
  memcpy(out, t->face_edges + t->face_start[face], sizeof(int) * (size_t)t->face_ncorners[face]);
}
static void tr_edge_vertices(const OpenSubdiv_TopologyRefiner *r, int edge, int out[2])
{
  out[0] = topo_of(r)->edge_verts[2 * edge];
  out[1] = topo_of(r)->edge_verts[2 * edge + 1];
}
static int tr_num_vertex_edges(const OpenSubdiv_TopologyRefiner *r, int vertex)
{
  const BaseTopology *t = topo_of(r);
  int n = 0;
  for (int e = 0; e < t->num_edges; e++) {
    n += (t->edge_verts[2 * e] == vertex) + (t->edge_verts[2 * e + 1] == vertex);
  }
  return n;
}
static void tr_vertex_edges(const OpenSubdiv_TopologyRefiner *r, int vertex, int *out)
{
  const BaseTopology *t = topo_of(r);
  int n = 0;
  for (int e = 0; e < t->num_edges; e++) {
    if (t->edge_verts[2 * e] == vertex || t->edge_verts[2 * e + 1] == vertex) {
      out[n++] = e;
    }
  }
}

typedef struct RefGrids {
  BaseTopology topo;
  OpenSubdiv_TopologyRefiner refiner;
  Subdiv subdiv;
  SubdivCCG *ccg;
  CCGKey key;
  PBVH *pbvh;
} RefGrids;

static int *dup_ints(const int *src, size_t n)
{
  int *p = malloc(sizeof(int) * (n ? n : 1));
  memcpy(p, src, sizeof(int) * n);
  return p;
}

/* Base topology as in or_mesh_create_grids: per face its first corner and
 * corner count; per corner its base vertex and the base edge to the next
 * corner; per edge its two vertices.  co / no: one xyz per grid element in
 * grid order; mask nullable.  leaf_limit replaces pbvh.c's LEAF_LIMIT. */
RefGrids *rg_create(int num_faces, const int *face_start, const int *face_ncorners,
                    const int *face_verts, const int *face_edges, int num_base_verts,
                    int num_base_edges, const int *edge_verts, int grid_size, const float *co,
                    const float *no, const float *mask, int leaf_limit)
{
  RefGrids *g = calloc(1, sizeof(RefGrids));
  int ncorners = 0;
  for (int f = 0; f < num_faces; f++) {
    ncorners += face_ncorners[f];
  }
  g->topo.num_verts = num_base_verts;
  g->topo.num_edges = num_base_edges;
  g->topo.num_faces = num_faces;
  g->topo.face_start = dup_ints(face_start, (size_t)num_faces);
  g->topo.face_ncorners = dup_ints(face_ncorners, (size_t)num_faces);
  g->topo.face_verts = dup_ints(face_verts, (size_t)ncorners);
  g->topo.face_edges = dup_ints(face_edges, (size_t)ncorners);
  g->topo.edge_verts = dup_ints(edge_verts, 2 * (size_t)num_base_edges);
  OpenSubdiv_TopologyRefiner *r = &g->refiner;
  r->getNumVertices = tr_num_vertices;
  r->getNumEdges = tr_num_edges;
  r->getNumFaces = tr_num_faces;
  r->getNumFaceVertices = tr_num_face_vertices;
  r->getFaceVertices = tr_face_vertices;
  r->getNumFaceEdges = tr_num_face_vertices;
  r->getFaceEdges = tr_face_edges;
  r->getEdgeVertices = tr_edge_vertices;
  r->getNumVertexEdges = tr_num_vertex_edges;
  r->getVertexEdges = tr_vertex_edges;
  r->user_data = &g->topo;
  g->subdiv.topology_refiner = r;

  /* KERNEL_subdiv_to_ccg (subdiv_ccg.c:543-561) up to the grid evaluation. */
  SubdivCCG *ccg = MEM_callocN(sizeof(SubdivCCG), "subdiv ccg");
  g->ccg = ccg;
  ccg->subdiv = &g->subdiv;
  ccg->level = 1;
  while (KERNEL_subdiv_grid_size_from_level(ccg->level) < grid_size) {
    ccg->level++;
  }
  ccg->grid_size = KERNEL_subdiv_grid_size_from_level(ccg->level);
  SubdivToCCGSettings settings = {grid_size, true, mask != NULL};
  subdiv_ccg_init_layers(ccg, &settings);
  subdiv_ccg_alloc_elements(ccg, &g->subdiv);
  subdiv_ccg_init_faces(ccg);
  subdiv_ccg_init_faces_neighborhood(ccg);

  /* Stand-in for subdiv_ccg_evaluate_grids: the elements, grid -> face, flags. */
  KERNEL_subdiv_ccg_key_top_level(&g->key, ccg);
  const int area = g->key.grid_area;
  for (int f = 0; f < num_faces; f++) {
    for (int c = 0; c < ccg->faces[f].num_grids; c++) {
      const int grid = ccg->faces[f].start_grid_index + c;
      ccg->grid_faces[grid] = &ccg->faces[f];
      for (int e = 0; e < area; e++) {
        const size_t i = (size_t)grid * (size_t)area + (size_t)e;
        CCGElem *el = CCG_elem_offset(&g->key, ccg->grids[grid], e);
        memcpy(CCG_elem_co(&g->key, el), co + 3 * i, sizeof(float[3]));
        memcpy(CCG_elem_no(&g->key, el), no + 3 * i, sizeof(float[3]));
        if (mask) {
          *CCG_elem_mask(&g->key, el) = mask[i];
        }
      }
    }
  }

  rp_set_leaf_limit(leaf_limit);
  g->pbvh = BKE_pbvh_new();
  BKE_pbvh_build_grids(g->pbvh, ccg->grids, ccg->num_grids, &g->key, (void **)ccg->grid_faces,
                       ccg->grid_flag_mats, ccg->grid_hidden);
  g->pbvh->subdiv_ccg = ccg;
  return g;
}

void rg_free(RefGrids *g)
{
  if (!g) {
    return;
  }
  BKE_pbvh_free(g->pbvh);
  g->ccg->subdiv = NULL; /* owned here, not by the CCG */
  KERNEL_subdiv_ccg_destroy(g->ccg);
  free(g->topo.face_start);
  free(g->topo.face_ncorners);
  free(g->topo.face_verts);
  free(g->topo.face_edges);
  free(g->topo.edge_verts);
  free(g);
}

int rg_num_grids(const RefGrids *g)
{
  return g->ccg->num_grids;
}
int rg_num_nodes(const RefGrids *g)
{
  return g->pbvh->totnode;
}
void rg_get_bbs(const RefGrids *g, float *vb, float *orig_vb)
{
  for (int i = 0; i < g->pbvh->totnode; i++) {
    memcpy(vb + 6 * i, &g->pbvh->nodes[i].vb, sizeof(float[6]));
    memcpy(orig_vb + 6 * i, &g->pbvh->nodes[i].orig_vb, sizeof(float[6]));
  }
}
/* Element data out / in (xyz per element, one mask per element). */
void rg_get(const RefGrids *g, float *co, float *no, float *mask)
{
  const int area = g->key.grid_area;
  for (int grid = 0; grid < g->ccg->num_grids; grid++) {
    for (int e = 0; e < area; e++) {
      const size_t i = (size_t)grid * (size_t)area + (size_t)e;
      CCGElem *el = CCG_elem_offset(&g->key, g->ccg->grids[grid], e);
      if (co) {
        memcpy(co + 3 * i, CCG_elem_co(&g->key, el), sizeof(float[3]));
      }
      if (no) {
        memcpy(no + 3 * i, CCG_elem_no(&g->key, el), sizeof(float[3]));
      }
      if (mask && g->key.has_mask) {
        mask[i] = *CCG_elem_mask(&g->key, el);
      }
    }
  }
}
void rg_set(RefGrids *g, const float *co, const float *mask)
{
  const int area = g->key.grid_area;
  for (int grid = 0; grid < g->ccg->num_grids; grid++) {
    for (int e = 0; e < area; e++) {
      const size_t i = (size_t)grid * (size_t)area + (size_t)e;
      CCGElem *el = CCG_elem_offset(&g->key, g->ccg->grids[grid], e);
      if (co) {
        memcpy(CCG_elem_co(&g->key, el), co + 3 * i, sizeof(float[3]));
      }
      if (mask && g->key.has_mask) {
        *CCG_elem_mask(&g->key, el) = mask[i];
      }
    }
  }
}
void rg_node_mark_update(RefGrids *g, int node)
{
  BKE_pbvh_node_mark_update(&g->pbvh->nodes[node]);
}
void rg_update_normals(RefGrids *g)
{
  BKE_pbvh_update_normals(g->pbvh, g->ccg);
}
void rg_update_bounds(RefGrids *g, int flag)
{
  BKE_pbvh_update_bounds(g->pbvh, flag);
}
/* Adjacency the reference built: per base edge its adjacent-face count and
 * boundary coordinates (2 * grid_size per face: grid, x, y), per base vertex
 * its corner coordinates. */
int rg_edge_num_faces(const RefGrids *g, int edge)
{
  return g->ccg->adjacent_edges[edge].num_adjacent_faces;
}
void rg_edge_coords(const RefGrids *g, int edge, int face, int *out)
{
  const SubdivCCGCoord *c = g->ccg->adjacent_edges[edge].boundary_coords[face];
  for (int i = 0; i < 2 * g->ccg->grid_size; i++) {
    out[3 * i] = c[i].grid_index;
    out[3 * i + 1] = c[i].x;
    out[3 * i + 2] = c[i].y;
  }
}
int rg_vertex_num_faces(const RefGrids *g, int vertex)
{
  return g->ccg->adjacent_vertices[vertex].num_adjacent_faces;
}
void rg_vertex_coords(const RefGrids *g, int vertex, int *out)
{
  const SubdivCCGAdjacentVertex *v = &g->ccg->adjacent_vertices[vertex];
  for (int i = 0; i < v->num_adjacent_faces; i++) {
    out[3 * i] = v->corner_coords[i].grid_index;
    out[3 * i + 1] = v->corner_coords[i].x;
    out[3 * i + 2] = v->corner_coords[i].y;
  }
}

/* pbvh.c calls the multires normal update under its upstream name. */
void BKE_subdiv_ccg_update_normals(SubdivCCG *subdiv_ccg, struct CCGFace **effected_faces,
                                   int num_effected_faces)
{
  KERNEL_subdiv_ccg_update_normals(subdiv_ccg, effected_faces, num_effected_faces);
}
int BKE_subdiv_ccg_grid_to_face_index(const SubdivCCG *subdiv_ccg, const int grid_index)
{
  return KERNEL_subdiv_ccg_grid_to_face_index(subdiv_ccg, grid_index);
}
void LIB_parallel_range_settings_defaults(TaskParallelSettings *settings)
{
  memset(settings, 0, sizeof(*settings));
  settings->use_threading = true;
}

/* ---- OpenSubdiv evaluation and mesh conversion: not pinned ---- */
static void subdiv_unreachable(const char *what)
{
  fprintf(stderr, "refpin: %s needs OpenSubdiv and is not pinned\n", what);
  abort();
}
int *KERNEL_subdiv_face_ptex_offset_get(Subdiv *subdiv)
{
  subdiv_unreachable("ptex offsets");
  return NULL;
}
void KERNEL_subdiv_rotate_grid_to_quad(int corner, float grid_u, float grid_v, float *r_quad_u,
                                       float *r_quad_v)
{
  subdiv_unreachable("grid rotation");
}
void KERNEL_subdiv_eval_limit_point(Subdiv *subdiv, int ptex_face_index, float u, float v,
                                    float r_P[3])
{
  subdiv_unreachable("limit evaluation");
}
void KERNEL_subdiv_eval_limit_point_and_normal(Subdiv *subdiv, int ptex_face_index, float u,
                                               float v, float r_P[3], float r_N[3])
{
  subdiv_unreachable("limit evaluation");
}
void KERNEL_subdiv_eval_final_point(Subdiv *subdiv, int ptex_face_index, float u, float v,
                                    float r_P[3])
{
  subdiv_unreachable("limit evaluation");
}
bool KERNEL_subdiv_eval_begin_from_mesh(Subdiv *subdiv, const Mesh *mesh,
                                        const float (*coarse_vertex_cos)[3], int evaluator_type,
                                        void *evaluator_cache)
{
  subdiv_unreachable("evaluator");
  return false;
}
void KERNEL_subdiv_stats_begin(SubdivStats *stats, int value)
{
  (void)stats;
  (void)value;
}
void KERNEL_subdiv_stats_end(SubdivStats *stats, int value)
{
  (void)stats;
  (void)value;
}
void KERNEL_subdiv_free(Subdiv *subdiv)
{
  (void)subdiv;
}
bool KERNEL_subdiv_ccg_mask_init_from_paint(SubdivCCGMaskEvaluator *mask_evaluator,
                                            const Mesh *mesh)
{
  subdiv_unreachable("mask evaluator");
  return false;
}
void KERNEL_subdiv_ccg_material_flags_init_from_mesh(
    SubdivCCGMaterialFlagsEvaluator *material_flags_evaluator, const Mesh *mesh)
{
  subdiv_unreachable("material evaluator");
}
Mesh *KERNEL_mesh_new_nomain_from_template(const Mesh *me_src, int verts_len, int edges_len,
                                           int tessface_len, int loops_len, int polys_len)
{
  subdiv_unreachable("mesh conversion");
  return NULL;
}
int poly_find_loop_from_vert(const MPoly *poly, const MLoop *loopstart, unsigned int vert)
{
  subdiv_unreachable("coarse mesh adjacency");
  return -1;
}

/* BKE_pbvh_raycast on the grids PBVH with the sculpt ray-cast callback of the
 * brush specification (the same rule as rp_raycast): active vertex = grid
 * element index, active face = grid index. */
typedef struct GridRaycastCb {
  PBVH *pbvh;
  const float *start, *normal;
  IsectRayPrecalc isect;
  float depth;
  int active_vertex, active_grid;
  float face_normal[3];
  bool hit;
} GridRaycastCb;

static void grid_raycast_cb(PBVHNode *node, void *data_v, float *tmin)
{
  GridRaycastCb *d = data_v;
  if (BKE_pbvh_node_get_tmin(node) < *tmin) {
    if (BKE_pbvh_node_raycast(d->pbvh, node, NULL, false, d->start, d->normal, &d->isect,
                              &d->depth, &d->active_vertex, &d->active_grid, d->face_normal)) {
      d->hit = true;
      *tmin = d->depth;
    }
  }
}

int rg_raycast(RefGrids *g, const float start[3], const float normal[3], int original,
               float *depth, int *active_vertex, int *active_grid, float face_normal[3])
{
  GridRaycastCb d;
  memset(&d, 0, sizeof(d));
  d.pbvh = g->pbvh;
  d.start = start;
  d.normal = normal;
  d.depth = *depth;
  d.active_vertex = d.active_grid = -1;
  isect_ray_tri_watertight_v3_precalc(&d.isect, normal);
  BKE_pbvh_raycast(g->pbvh, grid_raycast_cb, &d, start, normal, original != 0);
  *depth = d.depth;
  *active_vertex = d.active_vertex;
  *active_grid = d.active_grid;
  memcpy(face_normal, d.face_normal, sizeof(float[3]));
  return d.hit ? 1 : 0;
}

/* BKE_pbvh_find_nearest_to_ray on the grids PBVH with the callback of
 * rp_nearest_to_ray (pbvh_grids_node_nearest_to_ray inside a leaf). */
typedef struct GridNearestCb {
  PBVH *pbvh;
  const float *start, *normal;
  float depth, dist_sq;
  bool hit;
} GridNearestCb;

static void grid_nearest_cb(PBVHNode *node, void *data_v, float *tmin)
{
  GridNearestCb *d = data_v;
  if (BKE_pbvh_node_get_tmin(node) < *tmin) {
    if (BKE_pbvh_node_find_nearest_to_ray(d->pbvh, node, NULL, false, d->start, d->normal,
                                          &d->depth, &d->dist_sq)) {
      d->hit = true;
      *tmin = d->dist_sq;
    }
  }
}

int rg_nearest_to_ray(RefGrids *g, const float start[3], const float normal[3], int original,
                      float *depth, float *dist_sq)
{
  GridNearestCb d;
  memset(&d, 0, sizeof(d));
  d.pbvh = g->pbvh;
  d.start = start;
  d.normal = normal;
  d.depth = *depth;
  d.dist_sq = *dist_sq;
  BKE_pbvh_find_nearest_to_ray(g->pbvh, grid_nearest_cb, &d, start, normal, original != 0);
  *depth = d.depth;
  *dist_sq = d.dist_sq;
  return d.hit ? 1 : 0;
}

PBVH *rg_pbvh(RefGrids *g)
{
  return g->pbvh;
}
