/*
 * CPU oracle for the sculpt-brush dab path — TEST INFRASTRUCTURE ONLY.
 *
 * This library is the checker: a plain-C restatement of the reference's PBVH
 * build, node search, vertex-normal update, bounding-box refit and falloff-curve
 * tables (Kielan/dune_sculpt, source/dune/kernel/intern/pbvh.c, colortools.c,
 * mesh_evaluate.c, subdiv_ccg.c; lib/intern/math_*), plus the brush math the
 * reference lacks (its sculpt.c is absent), written from the project's brush
 * specification.  Every arithmetic step runs twice: once in FP32 (the parity
 * target of the GPU path, bit-for-bit) and once in FP64 (the error reference).
 *
 * Only tests, the smoke check and the benchmark's CPU-baseline leg may load it.
 * The GPU product never links or calls it.
 *
 * Parity pinning: the reference ships no tests, fixtures or golden vectors for
 * this path and does not build as shipped (its public headers are missing).
 * oracle/refpin compiles the reference's own pbvh.c, subdiv_ccg.c,
 * poly-normal, vector-math and colortools.c code from the reference tree
 * behind stand-in headers, and tests/test_refpin.py checks this restatement
 * against it: PBVH build, node search, bounding boxes, multires normals with
 * seam stitching, falloff tables and curve evaluation bit for bit; FACES vertex
 * normals within 1e-6 (the reference's float atomics add in task order).  The
 * brush math has no reference code (sculpt.c is missing): it is pinned only by
 * known-answer tests written from the reference's definitions.
 */
#ifndef ORACLE_H
#define ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct OrMesh OrMesh;

/* Field order matches SGPU_Brush in include/sculpt_gpu.h. */
typedef struct OrBrush {
  int sculpt_tool; /* 1 draw, 2 smooth, 3 pinch, 4 inflate, 16 crease, 18 clay strips
                      (eBrushSculptTool) */
  int flag;        /* eBrushFlags subset: BRUSH_FRONTFACE (1 << 27) */
  int symmetry;    /* PAINT_SYMM_X | _Y | _Z */
  int curve_preset;
  float radius;
  float strength;
  float normal_radius_factor;
  float area_radius_factor;
  float plane_offset;
  float view_normal[3];
  int use_original_bb;
  float crease_pinch_factor;
  int elastic_deform_type;                /* BRUSH_ELASTIC_DEFORM_* */
  float elastic_deform_volume_preservation; /* Kelvinlet Poisson ratio */
  float height;                            /* layer height */
} OrBrush;

/* ---- mesh (PBVH_FACES) ---- */
OrMesh *or_mesh_create_faces(const void *mverts, int totvert, const void *mpolys, int totpoly,
                             const void *mloops, int totloop, const void *looptris, int totlt,
                             const float *mask, const float *automask, int leaf_limit);
void or_mesh_free(OrMesh *m);

/* ---- mesh (PBVH_GRIDS) ----
 * grids_co/no: num_grids*grid_size^2*3 floats, mask: num_grids*grid_size^2 (nullable).
 * face_start/face_ngrids: per base face, first grid and corner count.
 * face_verts/face_edges: per face corner, base vertex / base edge (edge i joins corner i, i+1).
 * edge_verts: per base edge, its two base vertices. */
OrMesh *or_mesh_create_grids(int num_grids, int grid_size, const float *grids_co,
                             const float *grids_no, const float *grids_mask, int num_faces,
                             const int *face_start, const int *face_ngrids, const int *face_verts,
                             const int *face_edges, int num_base_verts, int num_base_edges,
                             const int *edge_verts, int leaf_limit);

/* The stroke-start positions and normals that grab and elastic deform read
 * (the undo node's original coordinates); or_stroke stores them itself at the
 * start of a stroke that uses one of those tools. */
void or_store_original(OrMesh *m);
/* One dab of grab / elastic deform over all symmetry passes (b->symmetry) of
 * the unmirrored location and grab delta; the leaves come from the library's
 * own gather.  Returns vertex-passes displaced (FP32 state). */
int or_orig_dab(OrMesh *m, const OrBrush *b, const float location[3], const float grab_delta[3]);
/* The Kelvinlet displacement (kelvinlet.c:6-190) of one element, FP32:
 * params from BKE_kelvinlet_init_params(radius, force, 1, poisson); type 0-4. */
void or_kelvinlet(int type, float radius, float force, float poisson, const float co[3],
                  const float location[3], const float delta_or_normal[3], float out[3]);

int or_num_nodes(const OrMesh *m);
int or_num_leaves(const OrMesh *m);
int or_num_verts(const OrMesh *m);
void or_get_nodes(const OrMesh *m, int *children_offset, int *flag, int *prim_off, int *totprim,
                  int *uniq, int *face_verts, int *vert_off);
void or_get_prim_indices(const OrMesh *m, int *out);
int or_num_leaf_vert_entries(const OrMesh *m);
void or_get_vert_indices(const OrMesh *m, int *out);
void or_get_bbs(const OrMesh *m, float *vb, float *orig_vb);
void or_get_bbs64(const OrMesh *m, double *vb, double *orig_vb);
void or_get_co(const OrMesh *m, float *out);
void or_get_no(const OrMesh *m, float *out);
void or_get_mask(const OrMesh *m, float *out);
void or_get_co64(const OrMesh *m, double *out);
void or_get_no64(const OrMesh *m, double *out);
void or_set_co(OrMesh *m, const float *co);

/* Left-first DFS node search with the sphere callback; returns the count. */
int or_search_sphere(OrMesh *m, const float center[3], float radius_sq, int original,
                     int *out_nodes);

/* Initial normals: every vertex tagged, every leaf flagged, one normal update. */
void or_recalc_all_normals(OrMesh *m);

/* Single steps, FP32 state (tests of the fine-grained entry points). */
int or_brush_pass(OrMesh *m, const OrBrush *b, const float location[3],
                  const float grab_delta[3], const int *nodes, int totnode, float *area_out);
void or_update_normals(OrMesh *m);
void or_update_bounds(OrMesh *m, int flag);
void or_node_mark_update(OrMesh *m, int node);
void or_vert_mark_update(OrMesh *m, int vertex);
void or_get_vert_tags(const OrMesh *m, unsigned char *out);

/* Whole stroke: per dab, symmetry passes (search + brush), normals, bounds(UpdateBB);
 * bounds(UpdateOriginalBB) at the end.  which: 1 = FP32, 2 = FP64, 3 = both.
 * Returns vertices displaced (FP32 run if it ran).  dabs: ndabs * 6 floats;
 * dab_tools (nullable) overrides the tool per dab. */
int64_t or_stroke(OrMesh *m, const OrBrush *b, const float *dabs, int ndabs,
                  const int *dab_tools, int which, int nthreads, int64_t *per_dab_counts);

/* Copies the FP32 state (positions, normals, mask, boxes, stroke-start data)
 * into the FP64 state, widening each value exactly. */
void or_sync64(OrMesh *m);

/* The area normal and centre of one pass over the given leaves (node
 * indices) at location, in FP32 (out32: normal, centre) and in FP64 from the
 * same positions and normals (out64; the FP64 state is set to the FP32 one
 * first, or_sync64). */
void or_area_normal_center(OrMesh *m, const OrBrush *b, const float location[3],
                           const int *nodes, int totnode, float out32[6], double out64[6]);

/* The FP32 stroke, with the rounding error of each measured dab (every
 * stride-th, from dab 0) against FP64, stage by stage from the same input:
 * the FP64 state is set to the FP32 one (or_sync64) before the brush, before
 * the normal update and before the bounds refit, each stage runs in both
 * precisions from the same node flags and vertex tags, and err[5*d .. 5*d+4]
 * receives max|x32 - x64| / max|x64| of the positions (brush, and the GRIDS
 * seam averages), max|x32 - x64| of the normals, the norm-wise relative
 * error of the node boxes, and max|x32 - x64| of the area normal and of the
 * area centre over the dab's passes (0 without the area reduction); -1 for
 * dabs not measured.  The FP32 state ends as or_stroke(..., which = 1) leaves
 * it.  Returns the FP32 vertices displaced. */
int64_t or_stroke_local_error(OrMesh *m, const OrBrush *b, const float *dabs, int ndabs,
                              const int *dab_tools, int stride, int nthreads, double *err);

/* BKE_pbvh_raycast (PBVH_FACES) with the sculpt ray-cast callback of the brush
 * specification.  depth: in = ray length, out = nearest hit depth.  Returns 1
 * on a hit (active vertex, its face and the hit triangle's normal set).
 * r_nleaves (nullable): leaves whose box the ray meets. */
int or_raycast(OrMesh *m, const float ray_start[3], const float ray_normal[3], int original,
               float *depth, int *active_vertex, int *active_face, float face_normal[3],
               int *r_nleaves);

/* BKE_pbvh_find_nearest_to_ray (PBVH_FACES and PBVH_GRIDS) with the sculpt
 * nearest-to-ray callback of the brush specification: leaves in order of
 * their box's squared distance to the ray, a leaf searched while that
 * distance is below the running minimum, the triangle (grid quad) of
 * smallest squared distance inside (strictly smaller wins).  depth and
 * dist_sq: in = starting values (FLT_MAX), out = the nearest triangle's
 * depth along the ray and squared distance.  Returns 1 when some triangle was
 * taken.  r_nleaves (nullable): leaves listed. */
int or_nearest_to_ray(OrMesh *m, const float ray_start[3], const float ray_normal[3],
                      int original, float *depth, float *dist_sq, int *r_nleaves);

/* Test helper: grid quads whose two triangles both meet the ray, the second
 * one closer. */
int or_grids_special_quads(OrMesh *m, const float ray_start[3], const float ray_normal[3]);

/* Falloff curve of a brush preset (colortools.c): table 257*(x,y), params
 * {mintable, maxtable, range, ext_in[2], ext_out[2]}. */
void or_curve_table(int preset, float *table_xy, float *params);
float or_curve_strength(int preset, float dist, float radius);

#ifdef __cplusplus
}
#endif

/* ---- headless draw buffers ----
 * pbvh_update_draw_buffers (pbvh.c:3240-3290) with GPU_pbvh_mesh_buffers_build
 * / _update (gpu_buffers.c:174-400) and GPU_pbvh_grid_buffers_update
 * (gpu_buffers.c:548-725), writing the 36-byte interleaved vertex format into
 * one buffer, node after node.  Bytes the reference leaves unwritten are left
 * as the caller initialised them. */
typedef struct OrDrawSetup {
  const int *face_sets;              /* per poly (FACES) / base face (GRIDS), nullable */
  int face_sets_color_seed, face_sets_color_default;
  const unsigned char *loop_colors;  /* FACES: r g b a per loop, nullable */
  const float *vert_colors;          /* FACES: rgba per vertex, nullable */
  int use_sculpt_vertex_colors;
  const unsigned char *grid_flag_mats; /* GRIDS: DMFlagMat records (4 bytes), nullable */
  const unsigned char *vert_flag;    /* FACES: MVert.flag per vertex, nullable (none hidden) */
  const int *lt_loops;               /* FACES: 3 loop indices per looptri (loop colours) */
} OrDrawSetup;
/* Layout per node: vert_off[totnode + 1], tot_tri, smooth, material (nullable
 * outputs); marks every leaf PBVH_RebuildDrawBuffers | PBVH_UpdateDrawBuffers.
 * Returns the vertex count. */
int64_t or_draw_build(OrMesh *m, const OrDrawSetup *s, int64_t *vert_off, int *tot_tri,
                      int *smooth, int *material);
/* Fills every leaf flagged PBVH_UpdateDrawBuffers at vert_off * 36 in vbo,
 * sets overlay[node] (show_overlay) for those, clears the two draw flags. */
void or_draw_update(OrMesh *m, const OrDrawSetup *s, const int64_t *vert_off, unsigned char *vbo,
                    int *overlay);
/* BKE_paint_face_set_overlay_color_get (paint.c:2219-2236), rgb bytes. */
void or_face_set_color(int face_set, int seed, unsigned char rgb[3]);

#endif
