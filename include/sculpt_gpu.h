/*
 * libsculptgpu — GB300 (sm_103a) implementation of the sculpt-brush dab path of
 * Kielan/dune_sculpt behind a plain C ABI.
 *
 * Every entry point takes plain pointers and sizes and returns an int status
 * (SGPU_OK or an SGPU_ERR_* code); nothing aborts.  Device memory belongs to a
 * mesh handle; host arrays passed in are read and copied.  A handle owns one
 * CUDA stream and is not thread-safe; distinct handles may be used from
 * distinct threads.  There is no CPU fallback: without a usable GB300 every
 * compute entry point returns SGPU_ERR_CUDA.
 *
 * Reference interfaces replaced (paths relative to the reference project):
 *   BKE_pbvh_new / BKE_pbvh_build_mesh / BKE_pbvh_build_grids / BKE_pbvh_free
 *       source/dune/kernel/intern/pbvh.c:2563, :2452, :2516, :2570
 *   BKE_pbvh_search_gather (sphere callback)     pbvh.c:2736-2767
 *   do_draw/smooth/inflate/clay_strips_brush     absent in the reference (its
 *       sculpt.c is missing); signature shape do_X_brush(sd, ob, nodes, totnode)
 *       is fixed here, with the brush math of the project's brush specification
 *   BKE_pbvh_update_normals                      pbvh.c:4559-4587
 *   BKE_pbvh_update_bounds                       pbvh.c:3319-3339
 *   BKE_pbvh_node_mark_update                    pbvh.c:3641-3645
 *   BKE_pbvh_node_get_BB / _get_original_BB      pbvh.c:3830-3840
 *   KERNEL_curvemapping_evaluateF (brush falloff) colortools.c:942-980
 */
#ifndef SCULPT_GPU_H
#define SCULPT_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---- */
#define SGPU_OK 0
#define SGPU_ERR_INVALID_ARG 1
#define SGPU_ERR_OOM 2
#define SGPU_ERR_CUDA 3
#define SGPU_ERR_TIMEOUT 4
#define SGPU_ERR_BOUNDS 5
#define SGPU_ERR_UNSUPPORTED 6

/* ---- element layouts (source/dune/types/types_meshdata.h) ---- */
typedef struct SGPU_MVert { /* MVert, types_meshdata.h:13-17 */
  float co[3];
  char flag, bweight;
  char _pad[2];
} SGPU_MVert;

typedef struct SGPU_MPoly { /* MPoly, types_meshdata.h:50-56 */
  int loopstart;
  int totloop;
  short mat_nr;
  char flag, _pad;
} SGPU_MPoly;

typedef struct SGPU_MLoop { /* MLoop, types_meshdata.h:69-74 */
  unsigned int v;
  unsigned int e;
} SGPU_MLoop;

typedef struct SGPU_MLoopTri { /* MLoopTri, types_meshdata.h:178-181 */
  unsigned int tri[3];
  unsigned int poly;
} SGPU_MLoopTri;

/* ---- PBVHNodeFlags (values the reference's pbvh.c relies on) ---- */
#define SGPU_PBVH_Leaf 1
#define SGPU_PBVH_UpdateNormals 2
#define SGPU_PBVH_UpdateBB 4
#define SGPU_PBVH_UpdateOriginalBB 8
#define SGPU_PBVH_UpdateDrawBuffers 16
#define SGPU_PBVH_UpdateRedraw 32

/* ---- brush (subset of Brush, types_brush.h:138-362) ---- */
#define SGPU_TOOL_DRAW 1         /* SCULPT_TOOL_DRW (types_brush_enums.h:411) */
#define SGPU_TOOL_SMOOTH 2       /* SCULPT_TOOL_SMOOTH */
#define SGPU_TOOL_PINCH 3        /* SCULPT_TOOL_PINCH */
#define SGPU_TOOL_INFLATE 4      /* SCULPT_TOOL_INFLATE */
#define SGPU_TOOL_GRAB 5         /* SCULPT_TOOL_GRAB */
#define SGPU_TOOL_LAYER 6        /* SCULPT_TOOL_LAYER */
#define SGPU_TOOL_CREASE 16      /* SCULPT_TOOL_CREASE */
#define SGPU_TOOL_CLAY_STRIPS 18 /* SCULPT_TOOL_CLAY_STRIPS */
#define SGPU_TOOL_ELASTIC_DEFORM 21 /* SCULPT_TOOL_ELASTIC_DEFORM (Kelvinlets, kelvinlet.c) */
/* Brush.elastic_deform_type (types_brush_enums.h:195-199) */
#define SGPU_ELASTIC_DEFORM_GRAB 0
#define SGPU_ELASTIC_DEFORM_GRAB_BISCALE 1
#define SGPU_ELASTIC_DEFORM_GRAB_TRISCALE 2
#define SGPU_ELASTIC_DEFORM_SCALE 3
#define SGPU_ELASTIC_DEFORM_TWIST 4
#define SGPU_BRUSH_FRONTFACE (1 << 27)
#define SGPU_SYMM_X 1 /* PAINT_SYMM_X, types_scene.h:2174 */
#define SGPU_SYMM_Y 2
#define SGPU_SYMM_Z 4
#define SGPU_CURVE_PRESET_LINE 0
#define SGPU_CURVE_PRESET_SHARP 1
#define SGPU_CURVE_PRESET_SMOOTH 2
#define SGPU_CURVE_PRESET_MAX 3
#define SGPU_CURVE_PRESET_ROUND 5
#define SGPU_CURVE_PRESET_ROOT 6

typedef struct SGPU_Brush {
  int sculpt_tool;            /* SGPU_TOOL_* */
  int flag;                   /* SGPU_BRUSH_FRONTFACE or 0 */
  int symmetry;               /* SGPU_SYMM_* bits */
  int curve_preset;           /* falloff curve, SGPU_CURVE_PRESET_* */
  float radius;               /* object-space radius */
  float strength;             /* bstrength */
  float normal_radius_factor; /* default 0.5 (types_brush_defaults.h:25) */
  float area_radius_factor;   /* default 0.5 (types_brush_defaults.h:27) */
  float plane_offset;         /* clay strips plane offset */
  float view_normal[3];       /* front-face reference direction */
  int use_original_bb;        /* cull against orig_vb instead of vb */
  float crease_pinch_factor;  /* crease: pinch strength (default 0.5, types_brush_defaults.h:23) */
  int elastic_deform_type;    /* SGPU_ELASTIC_DEFORM_* */
  float elastic_deform_volume_preservation; /* Kelvinlet Poisson ratio, in [0, 1) */
  float height;               /* Brush.height: the layer brush's layer height */
} SGPU_Brush;

/* One dab of a stroke: location and grab delta (stroke direction). */
typedef struct SGPU_Dab {
  float location[3];
  float grab_delta[3];
} SGPU_Dab;

typedef struct SGPU_MeshInfo {
  int type; /* 0 PBVH_FACES, 1 PBVH_GRIDS */
  int totvert; /* vertices, or grid elements */
  int totnode;
  int totleaf;
  int leaf_limit;
  int totprim;
  int leaf_vert_entries; /* FACES: total vert_indices entries over leaves */
  int grid_size;
} SGPU_MeshInfo;

typedef struct SGPU_StrokeStats {
  int64_t verts_displaced; /* sum over dabs and symmetry passes of verts moved */
  float gpu_ms;            /* CUDA-event time of the stroke on the mesh stream */
  int kernel_launches;     /* kernels launched by the library for the stroke */
  int graph_nodes;         /* nodes of the captured graph (graph mode) */
} SGPU_StrokeStats;

typedef struct sgpu_mesh sgpu_mesh;

/* ---- library ---- */
const char *sgpu_version(void);
const char *sgpu_last_error(void);
int sgpu_device_info(int *sm_count, int *cc_major, int *cc_minor);

/* ---- mesh lifetime ----
 * BKE_pbvh_new + BKE_pbvh_build_mesh (pbvh.c:2452-2514).  vert_normals (3 floats
 * per vertex) may be NULL: the normals are then computed by the normal update
 * over every vertex.  mask (CD_PAINT_MASK, one float per vertex) and automask
 * (one factor per vertex) may be NULL.  leaf_limit <= 0 selects the reference's
 * LEAF_LIMIT (10000 primitives, pbvh.c:1950). */
int sgpu_mesh_create_faces(const SGPU_MVert *verts, int totvert, const SGPU_MPoly *polys,
                           int totpoly, const SGPU_MLoop *loops, int totloop,
                           const SGPU_MLoopTri *looptris, int totlooptri,
                           const float *vert_normals, const float *mask, const float *automask,
                           int leaf_limit, sgpu_mesh **r_mesh);

/* BKE_pbvh_build_grids (pbvh.c:2516-2561) over grids in the CCG layout of
 * subdiv_ccg.c:40-89 (co, mask, no per element; given here as separate arrays
 * of num_grids*grid_size^2 elements).  The base topology gives the seam
 * adjacency (subdiv_ccg.c:397-549): per face its first grid and corner count,
 * per corner its base vertex and the base edge to the next corner, per base
 * edge its two vertices.  grids_no may be NULL (computed). */
int sgpu_mesh_create_grids(int num_grids, int grid_size, const float *grids_co,
                           const float *grids_no, const float *grids_mask, int num_faces,
                           const int *face_start, const int *face_ngrids, const int *face_verts,
                           const int *face_edges, int num_base_verts, int num_base_edges,
                           const int *edge_verts, int leaf_limit, sgpu_mesh **r_mesh);

int sgpu_mesh_destroy(sgpu_mesh *mesh); /* BKE_pbvh_free, pbvh.c:2570 */
int sgpu_mesh_info(const sgpu_mesh *mesh, SGPU_MeshInfo *r_info);
int sgpu_mesh_sync(sgpu_mesh *mesh);
void *sgpu_mesh_stream(sgpu_mesh *mesh); /* the handle's cudaStream_t */

/* ---- per-call entry points (one reference call each) ---- */

/* BKE_pbvh_search_gather with the sphere callback: leaves whose box (vb, or
 * orig_vb when original != 0) is closer than sqrt(radius_sq) to center, in the
 * reference's left-first DFS order.  The list stays on the device as the
 * mesh's current node list.  r_nodes (host, capacity >= totleaf) and r_tot may
 * be NULL; when given they receive node indices and count (synchronises). */
int sgpu_search_sphere(sgpu_mesh *mesh, const float center[3], float radius_sq, int original,
                       int *r_nodes, int *r_tot);

/* do_<tool>_brush(sd, ob, nodes, totnode) for one symmetry pass: location and
 * grab_delta are already mirrored for the pass, as the reference's stroke
 * cache does.  nodes == NULL uses the device list of the last search; otherwise
 * the host list (node indices) is uploaded.  Marks the nodes for update
 * (BKE_pbvh_node_mark_update) and tags the moved vertices (vert_bitmap). */
int sgpu_do_draw_brush(sgpu_mesh *mesh, const SGPU_Brush *brush, const float location[3],
                       const float grab_delta[3], const int *nodes, int totnode);
int sgpu_do_smooth_brush(sgpu_mesh *mesh, const SGPU_Brush *brush, const float location[3],
                         const float grab_delta[3], const int *nodes, int totnode);
int sgpu_do_inflate_brush(sgpu_mesh *mesh, const SGPU_Brush *brush, const float location[3],
                          const float grab_delta[3], const int *nodes, int totnode);
int sgpu_do_clay_strips_brush(sgpu_mesh *mesh, const SGPU_Brush *brush, const float location[3],
                              const float grab_delta[3], const int *nodes, int totnode);
int sgpu_do_pinch_brush(sgpu_mesh *mesh, const SGPU_Brush *brush, const float location[3],
                        const float grab_delta[3], const int *nodes, int totnode);
int sgpu_do_crease_brush(sgpu_mesh *mesh, const SGPU_Brush *brush, const float location[3],
                         const float grab_delta[3], const int *nodes, int totnode);
/* Layer: per pass like the above, from the stroke-start positions and
 * normals and a per-vertex layer height that sgpu_mesh_store_original resets
 * (needs it at the stroke start; sgpu_stroke does it itself). */
int sgpu_do_layer_brush(sgpu_mesh *mesh, const SGPU_Brush *brush, const float location[3],
                        const float grab_delta[3], const int *nodes, int totnode);
/* Original-data brushes (grab, elastic deform): one DAB over all symmetry
 * passes of brush->symmetry, from the unmirrored location and grab delta — the
 * reference combines these brushes' proxies once per dab onto the original
 * coordinates, so every vertex of the gathered leaves is rebuilt from its
 * stroke-start position.  The library gathers the leaves itself (grab: leaves
 * whose orig_vb meets any pass sphere; elastic deform: every leaf, as
 * SCULPT_tool_needs_all_pbvh_nodes has it): nodes must be NULL.  Needs
 * sgpu_mesh_store_original at the stroke start (the undo push that keeps
 * the original coordinates); sgpu_stroke stores them itself. */
int sgpu_do_grab_brush(sgpu_mesh *mesh, const SGPU_Brush *brush, const float location[3],
                       const float grab_delta[3], const int *nodes, int totnode);
int sgpu_do_elastic_deform_brush(sgpu_mesh *mesh, const SGPU_Brush *brush,
                                 const float location[3], const float grab_delta[3],
                                 const int *nodes, int totnode);
/* Copies the current positions and normals as the stroke-start ones and
 * resets the layer heights. */
int sgpu_mesh_store_original(sgpu_mesh *mesh);
/* Dispatch on brush->sculpt_tool. */
int sgpu_do_brush(sgpu_mesh *mesh, const SGPU_Brush *brush, const float location[3],
                  const float grab_delta[3], const int *nodes, int totnode);

/* The area normal and centre that a draw, clay-strips, pinch or crease pass
 * computes before it moves vertices (SCULPT_calc_area_normal_and_center of
 * the absent sculpt.c; the compensated tree reduction of the brush
 * specification): normals of the visited vertices within
 * radius * normal_radius_factor of location, positions within
 * radius * area_radius_factor, over the device list of the last search
 * (nodes == NULL) or the given leaves.  Moves nothing.  Synchronous. */
int sgpu_calc_area_normal_and_center(sgpu_mesh *mesh, const SGPU_Brush *brush,
                                     const float location[3], const int *nodes, int totnode,
                                     float r_area_no[3], float r_area_co[3]);

/* BKE_pbvh_update_normals (FACES: tagged vertices of flagged leaves; GRIDS:
 * inner grid normals of the affected faces plus seam stitching). */
int sgpu_pbvh_update_normals(sgpu_mesh *mesh);
/* BKE_pbvh_update_bounds(pbvh, flag) with SGPU_PBVH_Update* bits. */
int sgpu_pbvh_update_bounds(sgpu_mesh *mesh, int flag);
/* BKE_pbvh_node_mark_update on one node index. */
int sgpu_pbvh_node_mark_update(sgpu_mesh *mesh, int node);

/* ---- whole strokes ----
 * Per dab: for every enabled symmetry pass the sphere search and the brush,
 * then the normal update and update_bounds(UpdateBB); update_bounds(
 * UpdateOriginalBB) once at the end.  dab_tools (nullable) overrides the tool
 * per dab (mixed strokes).  A stroke with grab, elastic deform or layer dabs
 * first stores the stroke-start positions and normals (every mode).  mode:
 * 0 = launched call by call, 1 = the stroke captured once as a CUDA graph and
 * replayed.  stats may be NULL. */
#define SGPU_STROKE_EAGER 0
#define SGPU_STROKE_GRAPH 1
/* 2: one persistent launch of the whole stroke (cluster team); a stroke with
 * elastic deform dabs (every vertex moves in every dab) runs as mode 1 */
#define SGPU_STROKE_TEAM 2
int sgpu_stroke(sgpu_mesh *mesh, const SGPU_Brush *brush, const SGPU_Dab *dabs, int ndabs,
                const int *dab_tools, int mode, SGPU_StrokeStats *stats);

/* Cluster size (CTAs of 256 threads working on one mesh) of the persistent
 * stroke kernel for this mesh: 1, 2, 4, 8 or 16, or SGPU_TEAM_GRID: every
 * SM of the GPU works on the one stroke (one CTA per SM in a cooperative
 * launch; the CTAs meet at barriers in global memory whose waits are bounded:
 * a wait that runs out ends the launch and the call returns
 * SGPU_ERR_TIMEOUT).  A batch with SGPU_TEAM_GRID runs its strokes one after
 * another.  Default: the autotuner's cached team for the stroke (see
 * sgpu_autotune_team), else 8. */
#define SGPU_TEAM_GRID (-1)
/* Batches only (sgpu_batch_stroke, sgpu_autotune_batch): every SM works on
 * every stroke of the batch at once, dab by dab (one cooperative launch).
 * Each phase of a dab pools the work of all meshes — culled leaves in runs of
 * 32 vertices, area blocks, smooth hits, claimed GRIDS faces, touched-leaf
 * refit chunks, tagged vertices — and deals it over the whole GPU, so meshes
 * of any size mix without one team holding a large mesh alone.  Strokes with
 * grab, elastic deform or layer dabs, more than 1024 meshes, or GRIDS grids
 * above 33x33 return SGPU_ERR_UNSUPPORTED.  Results equal each mesh's own
 * stroke bit for bit. */
#define SGPU_TEAM_LOCKSTEP (-2)
int sgpu_mesh_set_team(sgpu_mesh *mesh, int cluster_size);
int sgpu_mesh_get_team(const sgpu_mesh *mesh, int *cluster_size);
/* Autotuner of the persistent stroke kernel's team shape.  Times the stroke
 * in SGPU_STROKE_TEAM mode on every candidate team — the whole GPU, then
 * clusters of 1, 2, 4, 8 and 16 CTAs (one CTA per SM, the full register
 * file) — restoring the mesh state between trials (second of two trials), and
 * keeps the fastest for the mesh.  The choice is also cached process-wide
 * under (mesh type, log2 of the vertex count, the set of tools in the stroke,
 * symmetry passes): a mesh whose team was never set (sgpu_mesh_set_team or
 * this call) strokes on the cached team of its stroke's key.  The block size
 * is fixed at 256 threads: the area reduction's 256-lane tree is part of the
 * brush specification.  r_ms (nullable) receives SGPU_AUTOTUNE_CANDIDATES
 * timings in that order (-1 where a candidate cannot run). */
#define SGPU_AUTOTUNE_CANDIDATES 6
int sgpu_autotune_team(sgpu_mesh *mesh, const SGPU_Brush *brush, const SGPU_Dab *dabs,
                       int ndabs, const int *dab_tools, int *r_cluster, float *r_ms);

/* Autotuner of a batch's team shape (the arguments of sgpu_batch_stroke):
 * times SGPU_BATCH_TEAM on the candidates (cluster, CTAs per SM) = (16, 1),
 * (8, 1), (8, 2), (4, 1), (4, 2), (2, 2), the whole GPU (strokes one after
 * another) and SGPU_TEAM_LOCKSTEP with 1 and 2 CTAs per SM (strokes
 * together; skipped where the batch does not allow it), restoring every mesh
 * between trials, and caches the fastest under
 * (mesh count, log2 of the total vertex count, the set of tools), where
 * sgpu_batch_stroke with cluster_size 0 finds it.  Two CTAs per SM run the
 * build with 128 registers per thread: twice the teams, slower each.
 * r_ms (nullable): SGPU_AUTOTUNE_BATCH_CANDIDATES timings, -1 where a
 * candidate cannot run. */
#define SGPU_AUTOTUNE_BATCH_CANDIDATES 9
int sgpu_autotune_batch(sgpu_mesh **meshes, int nmesh, const SGPU_Brush *brushes,
                        const SGPU_Dab *dabs, const int *dab_offsets, const int *dab_tools,
                        int *r_cluster, int *r_ctas_per_sm, float *r_ms);

/* Profile of one SGPU_STROKE_TEAM stroke: the persistent kernel's time split
 * by phase (time of the team's first thread from phase start to the barrier
 * that ends it) and the algorithmic bytes each phase moved.  Phases: 0 node
 * search, 1 area normal/centre, 2 brush sweep (smooth: candidate test and
 * first sweep), 3 smooth sweeps after the first, 4 normals and leaf refit,
 * 5 ancestor flush, 6 job set-up and end-of-stroke bounds, 7 GRIDS inner
 * normals with face seams and centres, 8 GRIDS base edges and corners
 * (phase 4 holds the refit of GRIDS meshes). */
#define SGPU_TEAM_PHASES 9
typedef struct SGPU_TeamProfile {
  float total_ms; /* CUDA-event time of the launch */
  double phase_ms[SGPU_TEAM_PHASES];
  double phase_bytes[SGPU_TEAM_PHASES];
} SGPU_TeamProfile;
int sgpu_stroke_team_profile(sgpu_mesh *mesh, const SGPU_Brush *brush, const SGPU_Dab *dabs,
                             int ndabs, const int *dab_tools, SGPU_TeamProfile *out,
                             SGPU_StrokeStats *stats);
/* The same profile for one SGPU_BATCH_TEAM batch (arguments of
 * sgpu_batch_stroke; cluster_size 0 takes the cached team).  The phase times
 * are those of the launch's first thread.  Cluster teams: each phase
 * includes the wait at the barrier that ends it.  SGPU_TEAM_LOCKSTEP: each
 * phase is the first CTA's own work, phase 6 holds its barrier waits, and
 * phase 5 the flushes (run by each mesh's home CTA at the next dab start).
 * stats (nullable): one per mesh. */
int sgpu_batch_team_profile(sgpu_mesh **meshes, int nmesh, const SGPU_Brush *brushes,
                            const SGPU_Dab *dabs, const int *dab_offsets, const int *dab_tools,
                            int cluster_size, SGPU_TeamProfile *out, SGPU_StrokeStats *stats);

/* ---- ray cast ----
 * Replaces BKE_pbvh_raycast (pbvh.c:3916) driven by the sculpt ray-cast
 * callback, which the reference calls but does not ship (sculpt.c is absent):
 * leaves in order of their box entry distance (BKE_pbvh_search_callback_occluded,
 * pbvh.c:2853), a leaf cast while its entry distance is below the running
 * minimum, pbvh_faces_node_raycast (pbvh.c:4042) or pbvh_grids_node_raycast
 * (pbvh.c:4110) inside it.  GRIDS: the active vertex is the grid element index
 * and the active face the grid index.  nrays independent
 * rays; ray_starts / ray_normals 3 floats each (unit directions);
 * ray_lengths (nullable: FLT_MAX) the initial depth; original selects
 * orig_vb.  Results per ray: depth (initial depth when no hit), hit 0/1,
 * active vertex (caller numbering, -1 without a hit), active face (poly, -1)
 * and the hit triangle's normal (3 floats, zero without a hit); the last three
 * outputs are nullable.  The first call with more rays than any before it
 * allocates the batch buffers (device and page-locked host); the first call
 * for a given (nrays, original) captures the call (copies in, kernels, copies
 * out) as a CUDA graph that later calls with the same shape replay. */
int sgpu_raycast(sgpu_mesh *mesh, int nrays, const float *ray_starts, const float *ray_normals,
                 const float *ray_lengths, int original, float *r_depths, int *r_hits,
                 int *r_active_vertices, int *r_active_faces, float *r_face_normals);

/* ---- nearest to ray ----
 * Replaces BKE_pbvh_find_nearest_to_ray (pbvh.c:4339-4352) driven by the
 * sculpt nearest-to-ray callback (absent with sculpt.c; fixed by the brush
 * specification like the ray cast's): the location of a dab when the cursor
 * ray misses the surface.  Leaves are visited in order of their box's squared
 * distance from the ray (nearest_to_ray_aabb_dist_sq, pbvh.c:4315-4337; a box
 * whose nearest point lies behind the ray origin is skipped), a leaf is
 * searched while that distance is below the running minimum, and inside it
 * the triangle (PBVH_FACES looptri, PBVH_GRIDS quad triangle) of smallest
 * squared distance from the ray wins (pbvh_faces_node_nearest_to_ray /
 * pbvh_grids_node_nearest_to_ray, pbvh.c:4354-4460; a quad's second triangle
 * is tested only when its first one is taken).  Per ray: r_depths the depth
 * along the ray of the nearest point, r_dist_sq its squared distance, r_hits
 * 1 when a triangle was taken (the values start at FLT_MAX).  The location
 * the stroke uses is ray_start + ray_normal * depth.  Shares the ray cast's
 * buffers and graph cache (a graph per (nrays, original, query)). */
int sgpu_find_nearest_to_ray(sgpu_mesh *mesh, int nrays, const float *ray_starts,
                             const float *ray_normals, int original, float *r_depths,
                             float *r_dist_sq, int *r_hits);

/* ---- headless draw buffers ----
 * Replaces the PBVH draw-buffer path without GL: pbvh_update_draw_buffers
 * (pbvh.c:3240-3290) reached from BKE_pbvh_draw_cb (pbvh.c:4615) with every
 * node that needs an update, and inside it GPU_pbvh_mesh_buffers_build /
 * _update (gpu_buffers.c:174-305, 307-400) and GPU_pbvh_grid_buffers_update
 * (gpu_buffers.c:548-725) with the update flags pbvh.c always passes (mask,
 * vertex colours, face sets).  The vertex buffer is one device array holding
 * every leaf's buffer in node order, in the reference's interleaved vertex
 * format ("pos" f32x3, "nor" i16x3, "msk" u8, "ac" u16x4, "fset" u8x3, packed
 * by VertexFormat_pack, gpu_vertex_format.cc:300-330): */
#define SGPU_DRAW_STRIDE 36   /* bytes per vertex */
#define SGPU_DRAW_OFS_POS 0
#define SGPU_DRAW_OFS_NOR 16
#define SGPU_DRAW_OFS_MSK 22
#define SGPU_DRAW_OFS_COL 24
#define SGPU_DRAW_OFS_FSET 32
/* Padding bytes and attributes the reference leaves unwritten (colours of a
 * mesh without colour layers, the mask of grids without a mask) are zero.
 * FACES: 3 vertices per visible looptri (visible: no corner has ME_HIDE and
 * face_sets[poly] > 0; without face sets nothing is visible, as
 * gpu_pbvh_is_looptri_visible has it).  GRIDS: grid_size^2 vertices per grid
 * when smooth, 4 per grid quad when flat. */
#define SGPU_ME_SMOOTH 1 /* MPoly.flag, DMFlagMat.flag */
#define SGPU_ME_HIDE 16  /* MVert.flag */
typedef struct SGPU_DMFlagMat { /* DMFlagMat: per grid, its face's material and flag */
  short mat_nr;
  char flag;
  char _pad;
} SGPU_DMFlagMat;
typedef struct SGPU_DrawSetup {
  const int *face_sets;     /* CD_SCULPT_FACE_SETS per poly (FACES) / base face (GRIDS); nullable */
  int face_sets_color_seed; /* BKE_pbvh_face_sets_color_set */
  int face_sets_color_default;
  const unsigned char *loop_colors; /* FACES: CD_MLOOPCOL, r g b a per loop; nullable */
  const float *vert_colors;         /* FACES: CD_PROP_COLOR, rgba per vertex; nullable */
  int use_sculpt_vertex_colors;     /* U.experimental.use_sculpt_vertex_colors */
  const SGPU_DMFlagMat *grid_flag_mats; /* GRIDS: per grid; NULL = every grid ME_SMOOTH, mat 0 */
} SGPU_DrawSetup;
/* GPU_pbvh_*_buffers_build for every leaf: the visible prims, smooth or flat
 * (from the leaf's first prim), material, and each leaf's place in the vertex
 * buffer; allocates the buffer and marks every leaf PBVH_RebuildDrawBuffers |
 * PBVH_UpdateDrawBuffers.  Face-set and colour layers are read here: call it
 * again after they change (the reference rebuilds on PBVH_RebuildDrawBuffers).
 * Synchronous. */
int sgpu_draw_buffers_build(sgpu_mesh *mesh, const SGPU_DrawSetup *setup);
/* The update: every leaf flagged PBVH_UpdateDrawBuffers gets its buffer filled
 * from the current positions, normals and mask, its show_overlay recomputed,
 * and PBVH_RebuildDrawBuffers | PBVH_UpdateDrawBuffers cleared on every leaf.
 * One kernel on the mesh stream; returns without waiting. */
int sgpu_draw_buffers_update(sgpu_mesh *mesh);
/* The update timed with CUDA events on the mesh stream (synchronous); with
 * all_leaves every leaf is flagged PBVH_UpdateDrawBuffers first (outside the
 * timed interval), a full refresh. */
int sgpu_draw_buffers_update_timed(sgpu_mesh *mesh, int all_leaves, float *gpu_ms);
/* Layout per node (reference node order, internal nodes empty):
 * vert_off[totnode + 1] first vertex of the node's buffer, and the buffer's
 * tot_tri (visible looptris; 0 for grids, as the grid buffers leave it),
 * smooth 0/1 and material_index.  Any output may be NULL.  Host data, no GPU
 * work. */
int sgpu_draw_buffers_layout(sgpu_mesh *mesh, int64_t *vert_off, int *tot_tri, int *smooth,
                             int *material_index);
/* show_overlay per node after the last update (!empty_mask || !default_face_set). */
int sgpu_draw_buffers_overlay(sgpu_mesh *mesh, int *show_overlay);
/* Copies the whole vertex buffer (vert_off[totnode] * SGPU_DRAW_STRIDE bytes). */
int sgpu_draw_buffers_get(sgpu_mesh *mesh, void *dst, size_t bytes);
/* The device address and size of the vertex buffer (owned by the handle). */
int sgpu_draw_buffers_device(sgpu_mesh *mesh, void **d_vbo, size_t *bytes);

/* ---- batches of independent meshes ----
 * Mesh i strokes with brushes[i] over dabs[dab_offsets[i] .. dab_offsets[i+1]);
 * dab_tools (nullable) is indexed like dabs.
 *   SGPU_BATCH_SEQUENTIAL: one graph-mode stroke per mesh, one after another.
 *   SGPU_BATCH_TEAM: one persistent launch; cluster teams take meshes from a
 *     work queue, longest estimated stroke first; SGPU_TEAM_GRID runs the
 *     strokes one after another on the whole GPU; SGPU_TEAM_LOCKSTEP runs
 *     them together on the whole GPU with every phase's work pooled over the
 *     meshes.  A mesh may appear once per batch.
 * cluster_size 0 uses the team sgpu_autotune_batch cached for a batch like
 * this one, else the first mesh's setting.  stats (nullable) gets one
 * entry per mesh; r_total_ms the CUDA-event time of the whole batch. */
#define SGPU_BATCH_SEQUENTIAL 0
#define SGPU_BATCH_TEAM 1
int sgpu_batch_stroke(sgpu_mesh **meshes, int nmesh, const SGPU_Brush *brushes,
                      const SGPU_Dab *dabs, const int *dab_offsets, const int *dab_tools,
                      int mode, int cluster_size, SGPU_StrokeStats *stats, float *r_total_ms);

/* The stroke with host buffers, as a host application calls it: verts_in (and
 * vert_normals_in, nullable) are copied to the device, every leaf box is
 * refit, the stroke runs (mode as in sgpu_stroke), and the positions are
 * copied back to verts_out.  stats->gpu_ms covers the copies and the kernels.
 * FACES meshes.  When verts_out is page-locked and mapped (sgpu_host_alloc),
 * host threads copy verts_in into it while the stroke runs and the device
 * then writes the blocks of 256 vertices that changed (bitwise, all 16 bytes
 * of the record); verts_out may then be verts_in itself, and must not
 * otherwise overlap it. */
int sgpu_stroke_host(sgpu_mesh *mesh, const SGPU_Brush *brush, const SGPU_Dab *dabs, int ndabs,
                     const int *dab_tools, const SGPU_MVert *verts_in,
                     const float *vert_normals_in, SGPU_MVert *verts_out, int mode,
                     SGPU_StrokeStats *stats);

/* The same for a GRIDS mesh: grids_co_in (and grids_no_in, nullable) hold 3
 * floats per grid element in the element order of sgpu_mesh_create_grids;
 * grids_co_out receives the positions after the stroke, same layout.  When
 * grids_co_out is page-locked and mapped (sgpu_host_alloc), host threads copy
 * grids_co_in into it while the stroke runs and the device then writes the
 * grids whose positions changed (bitwise), instead of copying every position
 * back; grids_co_out may then be grids_co_in itself, and must not otherwise
 * overlap it. */
int sgpu_stroke_host_grids(sgpu_mesh *mesh, const SGPU_Brush *brush, const SGPU_Dab *dabs,
                           int ndabs, const int *dab_tools, const float *grids_co_in,
                           const float *grids_no_in, float *grids_co_out, int mode,
                           SGPU_StrokeStats *stats);

/* ---- per-stroke restore (undo) ----
 * snapshot copies positions, normals, mask, node boxes and node flags into
 * device memory owned by the handle; restore copies them back. */
int sgpu_mesh_snapshot(sgpu_mesh *mesh);
int sgpu_mesh_restore(sgpu_mesh *mesh);

/* ---- measurement ---- */
#define SGPU_KERNEL_KINDS 10
typedef struct SGPU_KernelProfile {
  char name[24];   /* kernel kind */
  int launches;    /* launches of this kind in the stroke */
  float total_ms;  /* sum of per-launch CUDA-event durations */
  double alg_bytes; /* algorithmic bytes moved by those launches */
} SGPU_KernelProfile;
/* Runs the stroke call by call with CUDA events around every launch and the
 * kernels' algorithmic-byte counters on; out has SGPU_KERNEL_KINDS entries. */
int sgpu_stroke_profile(sgpu_mesh *mesh, const SGPU_Brush *brush, const SGPU_Dab *dabs,
                        int ndabs, const int *dab_tools, SGPU_KernelProfile *out,
                        SGPU_StrokeStats *stats);
/* Evicts L2 on the mesh stream: writes a 256 MiB device buffer (larger than
 * L2), then reads another 256 MiB buffer so that the dirty lines of the write
 * are written back before the next kernel. */
int sgpu_mesh_flush_l2(sgpu_mesh *mesh);
/* Page-locked host memory for the host-buffer path. */
void *sgpu_host_alloc(size_t bytes);
int sgpu_host_free(void *ptr);

/* ---- allocation-free smooth dab ----
 * No counterpart in the reference.  For callers that cannot allocate device
 * memory — an application embedding this library under a device-memory budget
 * it fixed up front, a plug-in host that forbids allocation, an interactive
 * loop that must not allocate while a stroke runs — and so cannot create a mesh handle
 * (creating one allocates).  They pass device arrays they already own: co (4
 * floats per vertex, the MVert layout, moved in place), normals (4 floats per
 * vertex, read only for SGPU_BRUSH_FRONTFACE; may be NULL otherwise), mask and
 * automask (may be NULL), the one-ring as CSR nb_off/nb_idx, and the candidate
 * vertices verts[nverts] (each vertex once, e.g. the unique vertices of the
 * leaves sgpu_search_sphere found).  One smooth-brush pass at location, with
 * the same sweeps and arithmetic as sgpu_do_smooth_brush; vertices are not
 * tagged and nodes not marked (there is no mesh handle).
 * The Jacobi scratch is a fixed device array of SGPU_NOALLOC_MAX_VERTS float4
 * (1 MiB) that every GPU loading the library holds until exit; nverts above
 * that returns SGPU_ERR_INVALID_ARG.  The first call on a device looks up the
 * array's device address (again after a device reset): a call with
 * nverts = 0 at set-up does only that, and with
 * lazy module loading (the CUDA default) it also makes the driver load the
 * module that holds the array, so that no later call loads it inside a fixed
 * memory budget (CUDA_MODULE_LOADING=EAGER loads it with the library).  All
 * calls share the array: calls that overlap on the GPU race.  No cudaMalloc,
 * no cudaFree.  Every entry of verts and nb_idx must index the caller's co
 * array (and normals, mask, automask); nothing checks this on the device.
 * The call waits for its stream (a cudaStream_t; NULL = default stream). */
#define SGPU_NOALLOC_MAX_VERTS 65536
int sgpu_smooth_dab_noalloc(float *co, const float *normals, const float *mask,
                            const float *automask, const int *nb_off, const int *nb_idx,
                            const int *verts, int nverts, const SGPU_Brush *brush,
                            const float location[3], void *stream);

/* ---- failure injection (host side; for tests) ----
 * SGPU_INJECT_ALLOC_FAIL, value n > 0: the n-th device allocation of mesh
 *   creation from now on fails as out of memory (the create call returns
 *   SGPU_ERR_OOM and frees what it had allocated); 0 disarms.
 * SGPU_INJECT_WAIT_NS, value > 0: the wait limit of the whole-GPU team's
 *   barriers in nanoseconds; 0 restores the default (2 s).
 * SGPU_INJECT_BARRIER_EXTRA, value 1: those barriers wait for one arrival
 *   more than the launch has, so every wait runs out after the limit and the
 *   stroke returns SGPU_ERR_TIMEOUT; 0 disarms.
 * No GPU fault is involved: the kernel gives up, records the status and
 * returns.  Returns SGPU_ERR_INVALID_ARG for an unknown hook. */
#define SGPU_INJECT_ALLOC_FAIL 1
#define SGPU_INJECT_WAIT_NS 2
#define SGPU_INJECT_BARRIER_EXTRA 3
/* SGPU_DEBUG_LOCKSTEP_PER_SM, value 1 or 2: every SGPU_TEAM_LOCKSTEP launch
 * runs that many CTAs per SM (the build the autotuner may also choose); 0
 * restores the team shape's choice.  A test hook, not a failure. */
#define SGPU_DEBUG_LOCKSTEP_PER_SM 4
int sgpu_debug_inject(int what, int64_t value);

/* ---- data access (synchronous) ---- */
int sgpu_get_verts(sgpu_mesh *mesh, SGPU_MVert *out);          /* FACES */
int sgpu_set_verts(sgpu_mesh *mesh, const SGPU_MVert *verts);  /* FACES */
int sgpu_get_positions(sgpu_mesh *mesh, float *out_xyz);       /* 3 floats per vertex/element */
int sgpu_set_positions(sgpu_mesh *mesh, const float *xyz);
int sgpu_get_normals(sgpu_mesh *mesh, float *out_xyz);
int sgpu_get_mask(sgpu_mesh *mesh, float *out);
/* Node bounding boxes, 6 floats each (min xyz, max xyz), reference node order. */
int sgpu_get_node_bbs(sgpu_mesh *mesh, float *vb, float *orig_vb);
/* Node table in reference order: children_offset (-1 for leaves), flag,
 * prim_off/totprim (leaves), uniq_verts, face_verts, vert_off (FACES leaves). */
int sgpu_get_nodes(sgpu_mesh *mesh, int *children_offset, int *flag, int *prim_off, int *totprim,
                   int *uniq_verts, int *face_verts, int *vert_off);
int sgpu_get_prim_indices(sgpu_mesh *mesh, int *out);
int sgpu_get_vert_indices(sgpu_mesh *mesh, int *out);

/* Brush falloff table (curvemap_make_table, colortools.c:597-771) for a preset:
 * 257 (x, y) pairs and {mintable, maxtable, range, ext_in[2], ext_out[2]}. */
int sgpu_curve_table(int preset, float *table_xy, float *params);

#ifdef __cplusplus
}
#endif

#endif /* SCULPT_GPU_H */
