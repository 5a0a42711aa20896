/*
 * Reference-pinning harness — TEST INFRASTRUCTURE ONLY.
 *
 * The reference's kernel/intern/pbvh.c, the poly-normal helpers of
 * mesh_evaluate.c, the triangle/quad normals of lib/intern/math_geom.cc and the
 * falloff-curve code of kernel/intern/colortools.c are compiled here, unmodified,
 * from the reference tree (see Makefile).  They include public headers the
 * reference does not ship (BKE_pbvh.h, BLI_math.h, BLI_ghash.h, BKE_ccg.h,
 * ...); every such header in include/ forwards to this file, which declares
 * what those sources use.
 *
 * What comes from the reference itself, compiled as it lies:
 *   - types/types_meshdata.h, types_mesh.h, types_customdata.h, types_color.h
 *     (MVert, MPoly, MLoop, MLoopTri, Mesh, CustomData, CurveMapping);
 *   - lib/intern/math_base_inline.c (up to line 605) and math_vector_inline.c
 *     (min_ff, max_ff, normalize_v3, ...: every float operation of the update
 *     path).
 * What is this harness's own (the interface the missing headers would give):
 *   - small utility macros (the reference's lib/lib_utildefines.h does not
 *     preprocess: lib_compiler_compat.h has an unbalanced #endif);
 *   - the PBVH flag and type enums, callback typedefs and the vertex-iterator
 *     struct with a step function behind the begin/end macros (fields named
 *     as pbvh_vertex_iter_init, pbvh.c:2928-2986 of the complete copy, fills
 *     them);
 *   - the CCG key and element accessors, laid out as subdiv_ccg.c:62-89 does
 *     (co | mask | normal);
 *   - MEM_*, bitmap, GHash/GSet, task-range and atomic stand-ins (single
 *     threaded: the task range runs its callback over the nodes in order, so
 *     the float atomics of the normal accumulation add in node order);
 *   - no-op or aborting stand-ins for the draw, BMesh and subdivision calls
 *     that the pinned paths never reach.
 */
#pragma once

#include <float.h>
#include <limits.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "dunelib/lib_sys_types.h"

/* ---- utility macros used by the compiled sources ---- */
#define POINTER_FROM_INT(i) ((void *)(intptr_t)(i))
#define POINTER_AS_INT(p) ((int)(intptr_t)(p))
#define POINTER_FROM_UINT(i) ((void *)(uintptr_t)(i))
#define POINTER_AS_UINT(p) ((unsigned int)(uintptr_t)(p))
#define UNLIKELY(x) __builtin_expect(!!(x), 0)
#define LIKELY(x) __builtin_expect(!!(x), 1)
#define UNUSED(x) UNUSED_##x __attribute__((__unused__))
#define UNUSED_VARS(...) ((void)0)
#define ATTR_FALLTHROUGH __attribute__((fallthrough))
#define ARRAY_SIZE(a) (sizeof(a) / sizeof(*(a)))
#define SWAP(type, a, b) \
  do { \
    type sw_ap_ = (a); \
    (a) = (b); \
    (b) = sw_ap_; \
  } while (0)
#define ELEM(v, ...) refpin_elem_((int)(v), (int[]){__VA_ARGS__}, sizeof((int[]){__VA_ARGS__}) / sizeof(int))
static inline bool refpin_elem_(int v, const int *list, size_t n)
{
  for (size_t i = 0; i < n; i++) {
    if (list[i] == v) {
      return true;
    }
  }
  return false;
}

#include "types_color.h"
#include "types_customdata.h"
#include "types_mesh.h"
#include "types_meshdata.h"

/* ---- assertions (the reference names them BLI_/LIB_) ---- */
#ifndef BLI_assert
#  define BLI_assert(a) ((void)0)
#endif
#ifndef BLI_assert_msg
#  define BLI_assert_msg(a, msg) ((void)0)
#endif

/* Spellings the partial rewrite left in pbvh.c (assert-only lines). */
#define LI_assert(a) ((void)0)
#define lib_assert(a) ((void)0)
#define CLAMP(a, b, c) \
  { \
    if ((a) < (b)) { \
      (a) = (b); \
    } \
    else if ((a) > (c)) { \
      (a) = (c); \
    } \
  } \
  (void)0

/* ---- the reference's inline math, compiled from its own sources ---- */
#ifndef MINLINE
#  define MINLINE static inline
#endif
#ifndef MALWAYS_INLINE
#  define MALWAYS_INLINE static inline
#endif
/* Forward use inside math_vector_inline.c (the missing BLI_math_vector.h
 * declares it in the reference's build). */
MINLINE bool is_zero_v3(const float v[3]);
MINLINE int float_as_int(float f);
MINLINE float int_as_float(int i);
/* math_inline_ref.h is generated by the Makefile: math_base_inline.c lines
 * 21-605 (min_ff, max_ff, max_ii, ...; the file's next function,
 * compare_threshold_relative, names an undeclared variable and does not
 * compile) followed by math_vector_inline.c lines 5-1463 (the whole file
 * inside its include guard). */
#include "math_inline_ref.h"

/* lib/intern/math_geom.cc (extracted by the Makefile into refpin_math_geom.c) */
float normal_tri_v3(float n[3], const float v1[3], const float v2[3], const float v3[3]);
float normal_quad_v3(
    float n[3], const float v1[3], const float v2[3], const float v3[3], const float v4[3]);

/* Ray helpers of lib/intern/math_geom.cc.  pbvh.c names the precalc structs
 * struct IsectRayAABB_Precalc / struct DistRayAABB_Precalc, math_geom.cc names
 * them IsectRayAABBPrecalc / DistRayAABBPrecalc; the fields are the ones
 * math_geom.cc reads and writes (isect_ray_tri_watertight_v3_precalc :1755,
 * dist_squared_ray_to_aabb_v3_precalc :643, isect_ray_aabb_v3_precalc :3017). */
typedef struct IsectRayPrecalc {
  int kx, ky, kz;
  float sx, sy, sz;
} IsectRayPrecalc;
typedef struct IsectRayAABB_Precalc {
  float ray_origin[3];
  float ray_inv_dir[3];
  int sign[3];
} IsectRayAABB_Precalc, IsectRayAABBPrecalc;
typedef struct DistRayAABB_Precalc {
  float ray_origin[3];
  float ray_direction[3];
  float ray_inv_dir[3];
} DistRayAABB_Precalc, DistRayAABBPrecalc;
void isect_ray_tri_watertight_v3_precalc(IsectRayPrecalc *isect_precalc, const float ray_direction[3]);
bool isect_ray_tri_watertight_v3(const float ray_origin[3], const IsectRayPrecalc *isect_precalc,
                                 const float v0[3], const float v1[3], const float v2[3],
                                 float *r_dist, float r_uv[2]);
void isect_ray_aabb_v3_precalc(IsectRayAABBPrecalc *data, const float ray_origin[3],
                               const float ray_direction[3]);
bool isect_ray_aabb_v3(const IsectRayAABBPrecalc *data, const float bb_min[3],
                       const float bb_max[3], float *tmin);
void dist_squared_ray_to_aabb_v3_precalc(DistRayAABBPrecalc *neasrest_precalc,
                                         const float ray_origin[3], const float ray_direction[3]);
float dist_squared_ray_to_aabb_v3(const DistRayAABBPrecalc *data, const float bb_min[3],
                                  const float bb_max[3], float r_point[3], float *r_depth);
float dist_squared_ray_to_seg_v3(const float ray_origin[3], const float ray_direction[3],
                                 const float v0[3], const float v1[3], float r_point[3],
                                 float *r_depth);
float dist_squared_to_ray_v3_normalized(const float ray_origin[3], const float ray_direction[3],
                                        const float co[3]);
void aabb_get_near_far_from_plane(const float plane_no[3], const float bbmin[3],
                                  const float bbmax[3], float bb_near[3], float bb_afar[3]);
bool isect_ray_line_v3(const float ray_origin[3], const float ray_direction[3], const float v0[3],
                       const float v1[3], float *r_lambda);
void interp_v3_v3v3(float r[3], const float a[3], const float b[3], const float t);
void closest_on_tri_to_point_v3(float r[3], const float p[3], const float v1[3],
                                const float v2[3], const float v3[3]);

/* Bezier knot used by the curve-table build of colortools.c (DNA_curve_types.h
 * is not in the reference): the fields colortools.c reads and writes. */
typedef struct BezTriple {
  float vec[3][3];
  char h1, h2;
  char f1, f2, f3;
} BezTriple;
/* Handle types (eBezTriple_Handle); colortools.c compares against these. */
enum { HD_FREE = 0, HD_AUTO = 1, HD_VECT = 2, HD_ALIGN = 3, HD_AUTO_ANIM = 4 };

/* ---- names colortools.c uses (its headers are not in the reference) ---- */
#define POINTER_OFFSET(v, ofs) ((void *)((char *)(v) + (ofs)))
/* The partial rewrite calls these under other prefixes than it defines them. */
#define KERNEL_curve_forward_diff_bezier BKE_curve_forward_diff_bezier
#define KERNEL_curve_correct_bezpart BKE_fcurve_correct_bezpart
#define BKE_curvemap_evaluateF KERNEL_curvemap_evaluateF
#define CUMA_SELECT CUMA_SEL
enum { CURVEMAP_SLOPE_NEGATIVE = 0, CURVEMAP_SLOPE_POSITIVE = 1, CURVEMAP_SLOPE_POS_NEG = 2 };
void BKE_curve_forward_diff_bezier(float q0, float q1, float q2, float q3, float *p, int it,
                                   int stride);
void BKE_fcurve_correct_bezpart(const float v1[2], float v2[2], float v3[2], const float v4[2]);
float KERNEL_curvemap_evaluateF(const CurveMapping *cumap, const CurveMap *cuma, float value);
static inline float LIB_rctf_size_x(const rctf *r)
{
  return r->xmax - r->xmin;
}
static inline float LIB_rctf_size_y(const rctf *r)
{
  return r->ymax - r->ymin;
}
#define BLI_rctf_size_x LIB_rctf_size_x
static inline void LIB_rctf_init(rctf *r, float xmin, float xmax, float ymin, float ymax)
{
  r->xmin = xmin;
  r->xmax = xmax;
  r->ymin = ymin;
  r->ymax = ymax;
}

/* ---- guarded allocator stand-ins (intern/guardedalloc) ---- */
void *MEM_mallocN(size_t len, const char *str);
void *MEM_callocN(size_t len, const char *str);
void *MEM_malloc_arrayN(size_t n, size_t size, const char *str);
void *MEM_calloc_arrayN(size_t n, size_t size, const char *str);
void *MEM_reallocN_id(void *p, size_t len, const char *str);
void *MEM_recallocN_id(void *p, size_t len, const char *str);
void *MEM_dupallocN(const void *p);
void MEM_freeN(void *p);
#define MEM_reallocN(p, len) MEM_reallocN_id(p, len, __func__)
#define MEM_recallocN(p, len) MEM_recallocN_id(p, len, __func__)
#define MEM_SAFE_FREE(v) \
  do { \
    if (v) { \
      MEM_freeN(v); \
      (v) = NULL; \
    } \
  } while (0)

/* ---- bitmap ---- */
typedef unsigned int BLI_bitmap;
typedef unsigned int LIB_bitmap;
#define BLI_BITMAP_NEW(n, name) ((BLI_bitmap *)MEM_callocN(((size_t)(n) + 31) / 32 * 4, name))
#define BLI_BITMAP_TEST(b, i) (((b)[(unsigned)(i) >> 5] >> ((unsigned)(i)&31u)) & 1u)
#define BLI_BITMAP_TEST_BOOL(b, i) (BLI_BITMAP_TEST(b, i) != 0)
#define BLI_BITMAP_ENABLE(b, i) ((b)[(unsigned)(i) >> 5] |= (1u << ((unsigned)(i)&31u)))
#define BLI_BITMAP_DISABLE(b, i) ((b)[(unsigned)(i) >> 5] &= ~(1u << ((unsigned)(i)&31u)))
#define BLI_BITMAP_SET(b, i, v) ((v) ? BLI_BITMAP_ENABLE(b, i) : BLI_BITMAP_DISABLE(b, i))
void BLI_bitmap_set_all(BLI_bitmap *b, bool set, size_t bits);

/* ---- GHash / GSet (integer / pointer keys; iteration order is irrelevant to
 * every caller pinned here: values carry the insertion rank) ---- */
typedef struct GHash GHash;
typedef struct GHash GSet;
typedef struct GHashIterator {
  GHash *gh;
  int slot;
} GHashIterator;
typedef GHashIterator GSetIterator;
GHash *BLI_ghash_int_new_ex(const char *info, unsigned int reserve);
bool BLI_ghash_ensure_p(GHash *gh, void *key, void ***r_val);
void BLI_ghash_free(GHash *gh, void *keyfree, void *valfree);
void BLI_ghashIterator_init(GHashIterator *it, GHash *gh);
void BLI_ghashIterator_step(GHashIterator *it);
bool BLI_ghashIterator_done(const GHashIterator *it);
void *BLI_ghashIterator_getKey(GHashIterator *it);
void *BLI_ghashIterator_getValue(GHashIterator *it);
#define GHASH_ITER(gh_iter_, ghash_) \
  for (BLI_ghashIterator_init(&gh_iter_, ghash_); BLI_ghashIterator_done(&gh_iter_) == false; \
       BLI_ghashIterator_step(&gh_iter_))
GSet *BLI_gset_ptr_new(const char *info);
bool BLI_gset_add(GSet *gs, void *key);
unsigned int BLI_gset_len(const GSet *gs);
void BLI_gset_free(GSet *gs, void *keyfree);
void BLI_gsetIterator_init(GSetIterator *it, GSet *gs);
void *BLI_gsetIterator_getKey(GSetIterator *it);
#define GSET_ITER(gs_iter_, gset_) GHASH_ITER(gs_iter_, gset_)
#define GSET_ITER_INDEX(gs_iter_, gset_, i_) \
  for (BLI_ghashIterator_init(&gs_iter_, gset_), i_ = 0; \
       BLI_ghashIterator_done(&gs_iter_) == false; BLI_ghashIterator_step(&gs_iter_), i_++)

/* ---- task range (serial) ---- */
typedef struct TaskParallelTLS {
  void *userdata_chunk;
} TaskParallelTLS;
typedef void (*TaskParallelReduceFunc)(const void *__restrict userdata,
                                       void *__restrict chunk_join,
                                       void *__restrict chunk);
typedef void (*TaskParallelFreeFunc)(const void *__restrict userdata, void *__restrict chunk);
typedef struct TaskParallelSettings {
  bool use_threading;
  int min_iter_per_thread;
  void *userdata_chunk;
  size_t userdata_chunk_size;
  TaskParallelReduceFunc func_reduce;
  TaskParallelFreeFunc func_free;
} TaskParallelSettings;
typedef void (*TaskParallelRangeFunc)(void *__restrict userdata,
                                      const int iter,
                                      const TaskParallelTLS *__restrict tls);
void BLI_task_parallel_range(const int start,
                             const int stop,
                             void *userdata,
                             TaskParallelRangeFunc func,
                             const TaskParallelSettings *settings);

/* ---- atomics (single threaded) ---- */
static inline float atomic_add_and_fetch_fl(float *p, const float x)
{
  *p = *p + x;
  return *p;
}

/* ---- time ---- */
double PIL_check_seconds_timer(void);

/* ---- custom data ---- */
void *CustomData_get_layer(const CustomData *data, int type);
int CustomData_get_offset(const CustomData *data, int type);

/* ---- CCG grid elements (subdiv_ccg.c:62-89: co | mask | normal) ---- */
typedef struct CCGElem CCGElem;
typedef struct CCGKey {
  int level;
  int elem_size;
  int grid_size;
  int grid_area;
  int grid_bytes;
  int normal_offset;
  int mask_offset;
  int has_normals;
  int has_mask;
} CCGKey;
typedef struct CCGFace CCGFace;
static inline float *CCG_elem_co(const CCGKey *key, CCGElem *elem)
{
  (void)key;
  return (float *)elem;
}
static inline float *CCG_elem_no(const CCGKey *key, CCGElem *elem)
{
  return (float *)((char *)elem + key->normal_offset);
}
static inline float *CCG_elem_mask(const CCGKey *key, CCGElem *elem)
{
  return (float *)((char *)elem + key->mask_offset);
}
static inline CCGElem *CCG_elem_offset(const CCGKey *key, CCGElem *elem, int offset)
{
  return (CCGElem *)((char *)elem + (size_t)offset * (size_t)key->elem_size);
}
static inline CCGElem *CCG_grid_elem(const CCGKey *key, CCGElem *elem, int x, int y)
{
  return CCG_elem_offset(key, elem, y * key->grid_size + x);
}
static inline float *CCG_elem_offset_co(const CCGKey *key, CCGElem *elem, int offset)
{
  return CCG_elem_co(key, CCG_elem_offset(key, elem, offset));
}
static inline float *CCG_elem_offset_no(const CCGKey *key, CCGElem *elem, int offset)
{
  return CCG_elem_no(key, CCG_elem_offset(key, elem, offset));
}
static inline float *CCG_elem_offset_mask(const CCGKey *key, CCGElem *elem, int offset)
{
  return CCG_elem_mask(key, CCG_elem_offset(key, elem, offset));
}
static inline float *CCG_grid_elem_co(const CCGKey *key, CCGElem *elem, int x, int y)
{
  return CCG_elem_co(key, CCG_grid_elem(key, elem, x, y));
}
static inline float *CCG_grid_elem_no(const CCGKey *key, CCGElem *elem, int x, int y)
{
  return CCG_elem_no(key, CCG_grid_elem(key, elem, x, y));
}
static inline float *CCG_grid_elem_mask(const CCGKey *key, CCGElem *elem, int x, int y)
{
  return CCG_elem_mask(key, CCG_grid_elem(key, elem, x, y));
}
static inline CCGElem *CCG_elem_next(const CCGKey *key, CCGElem *elem)
{
  return CCG_elem_offset(key, elem, 1);
}

typedef struct DMFlagMat {
  short mat_nr;
  char flag;
} DMFlagMat;

/* ---- multires grids (subdiv_ccg.c; KERNEL_subdiv_ccg.h, KERNEL_subdiv.h and
 * OpenSubdiv's topology-refiner C API are not in the reference): the types
 * with the fields subdiv_ccg.c reads and writes.  The topology refiner is a
 * table of query functions; the harness answers them from the base mesh's
 * face / edge / vertex arrays (refpin_subdiv.c). ---- */
typedef struct OpenSubdiv_TopologyRefiner OpenSubdiv_TopologyRefiner;
struct OpenSubdiv_TopologyRefiner {
  int (*getNumVertices)(const OpenSubdiv_TopologyRefiner *r);
  int (*getNumEdges)(const OpenSubdiv_TopologyRefiner *r);
  int (*getNumFaces)(const OpenSubdiv_TopologyRefiner *r);
  int (*getNumFaceVertices)(const OpenSubdiv_TopologyRefiner *r, int face);
  void (*getFaceVertices)(const OpenSubdiv_TopologyRefiner *r, int face, int *out);
  int (*getNumFaceEdges)(const OpenSubdiv_TopologyRefiner *r, int face);
  void (*getFaceEdges)(const OpenSubdiv_TopologyRefiner *r, int face, int *out);
  void (*getEdgeVertices)(const OpenSubdiv_TopologyRefiner *r, int edge, int out[2]);
  int (*getNumVertexEdges)(const OpenSubdiv_TopologyRefiner *r, int vertex);
  void (*getVertexEdges)(const OpenSubdiv_TopologyRefiner *r, int vertex, int *out);
  void *user_data;
};
typedef struct SubdivStats {
  double dummy;
} SubdivStats;
enum { SUBDIV_STATS_SUBDIV_TO_CCG = 0 };
typedef struct Subdiv {
  OpenSubdiv_TopologyRefiner *topology_refiner;
  void *displacement_evaluator;
  SubdivStats stats;
} Subdiv;
typedef struct SubdivCCGCoord {
  int grid_index;
  short x, y;
} SubdivCCGCoord;
typedef struct SubdivCCGFace {
  int num_grids;
  int start_grid_index;
} SubdivCCGFace;
typedef struct SubdivCCGAdjacentEdge {
  int num_adjacent_faces;
  SubdivCCGCoord **boundary_coords;
} SubdivCCGAdjacentEdge;
typedef struct SubdivCCGAdjacentVertex {
  int num_adjacent_faces;
  SubdivCCGCoord *corner_coords;
} SubdivCCGAdjacentVertex;
typedef struct SubdivCCGNeighbors {
  SubdivCCGCoord *coords;
  int size;
  int num_duplicates;
  SubdivCCGCoord coords_fixed[256];
} SubdivCCGNeighbors;
typedef enum SubdivCCGAdjacencyType {
  SUBDIV_CCG_ADJACENT_NONE,
  SUBDIV_CCG_ADJACENT_VERTEX,
  SUBDIV_CCG_ADJACENT_EDGE,
} SubdivCCGAdjacencyType;
typedef struct SubdivToCCGSettings {
  int resolution;
  bool need_normal;
  bool need_mask;
} SubdivToCCGSettings;
typedef struct SubdivCCGMaskEvaluator SubdivCCGMaskEvaluator;
struct SubdivCCGMaskEvaluator {
  float (*eval_mask)(SubdivCCGMaskEvaluator *ev, int ptex_face_index, float u, float v);
  void (*free)(SubdivCCGMaskEvaluator *ev);
  void *user_data;
};
typedef struct SubdivCCGMaterialFlagsEvaluator SubdivCCGMaterialFlagsEvaluator;
struct SubdivCCGMaterialFlagsEvaluator {
  DMFlagMat (*eval_material_flags)(SubdivCCGMaterialFlagsEvaluator *ev, int coarse_face_index);
  void (*free)(SubdivCCGMaterialFlagsEvaluator *ev);
  void *user_data;
};
typedef struct SubdivCCG {
  Subdiv *subdiv;
  int level;
  int grid_size;
  int grid_element_size;
  bool has_normal, has_mask;
  int normal_offset, mask_offset;
  int num_grids;
  CCGElem **grids;
  unsigned char *grids_storage;
  DMFlagMat *grid_flag_mats;
  BLI_bitmap **grid_hidden;
  int num_faces;
  SubdivCCGFace *faces;
  SubdivCCGFace **grid_faces;
  int num_adjacent_edges;
  SubdivCCGAdjacentEdge *adjacent_edges;
  int num_adjacent_vertices;
  SubdivCCGAdjacentVertex *adjacent_vertices;
  void *edges, *vertices;
  struct {
    int *start_face_grid_index;
  } cache_;
} SubdivCCG;
#define LIB_INLINE static inline
#define LIB_BITMAP_NEW BLI_BITMAP_NEW
#define LIB_task_parallel_range BLI_task_parallel_range
#define LIB_gset_ptr_new BLI_gset_ptr_new
#define LIB_gset_add BLI_gset_add
#define LIB_gset_free BLI_gset_free
void LIB_parallel_range_settings_defaults(TaskParallelSettings *settings);
static inline int KERNEL_subdiv_grid_size_from_level(const int level)
{
  return (1 << (level - 1)) + 1;
}
static inline int bitscan_forward_i(int a)
{
  return __builtin_ctz((unsigned int)a);
}
void KERNEL_subdiv_ccg_key_top_level(CCGKey *key, const SubdivCCG *subdiv_ccg);
void KERNEL_subdiv_ccg_recalc_normals(SubdivCCG *subdiv_ccg);
void KERNEL_subdiv_ccg_average_grids(SubdivCCG *subdiv_ccg);
void KERNEL_subdiv_ccg_destroy(SubdivCCG *subdiv_ccg);
#define LIB_assert(a) ((void)0)
#define UNUSED_VARS_NDEBUG(...) ((void)0)
enum { SUBDIV_EVALUATOR_TYPE_CPU = 0 };
/* Grid evaluation through OpenSubdiv (not in the reference, not pinned). */
int *KERNEL_subdiv_face_ptex_offset_get(Subdiv *subdiv);
#define BKE_subdiv_face_ptex_offset_get KERNEL_subdiv_face_ptex_offset_get
void KERNEL_subdiv_rotate_grid_to_quad(int corner, float grid_u, float grid_v, float *r_quad_u,
                                       float *r_quad_v);
void KERNEL_subdiv_eval_limit_point(Subdiv *subdiv, int ptex_face_index, float u, float v,
                                    float r_P[3]);
void KERNEL_subdiv_eval_limit_point_and_normal(Subdiv *subdiv, int ptex_face_index, float u,
                                               float v, float r_P[3], float r_N[3]);
void KERNEL_subdiv_eval_final_point(Subdiv *subdiv, int ptex_face_index, float u, float v,
                                    float r_P[3]);
bool KERNEL_subdiv_eval_begin_from_mesh(Subdiv *subdiv, const Mesh *mesh,
                                        const float (*coarse_vertex_cos)[3], int evaluator_type,
                                        void *evaluator_cache);
void KERNEL_subdiv_stats_begin(SubdivStats *stats, int value);
void KERNEL_subdiv_stats_end(SubdivStats *stats, int value);
void KERNEL_subdiv_free(Subdiv *subdiv);
bool KERNEL_subdiv_ccg_mask_init_from_paint(SubdivCCGMaskEvaluator *mask_evaluator,
                                            const Mesh *mesh);
void KERNEL_subdiv_ccg_material_flags_init_from_mesh(
    SubdivCCGMaterialFlagsEvaluator *material_flags_evaluator, const Mesh *mesh);
Mesh *KERNEL_mesh_new_nomain_from_template(const Mesh *me_src, int verts_len, int edges_len,
                                           int tessface_len, int loops_len, int polys_len);
int poly_find_loop_from_vert(const MPoly *poly, const MLoop *loopstart, unsigned int vert);
void KERNEL_subdiv_ccg_update_normals(SubdivCCG *subdiv_ccg, struct CCGFace **effected_faces,
                                      int num_effected_faces);
void BKE_subdiv_ccg_update_normals(SubdivCCG *subdiv_ccg, struct CCGFace **effected_faces,
                                   int num_effected_faces);
int BKE_subdiv_ccg_grid_to_face_index(const SubdivCCG *subdiv_ccg, const int grid_index);

/* ---- BMesh (dyntopo; never reached by the pinned FACES / GRIDS paths) ---- */
typedef struct BMesh {
  CustomData vdata;
  int totvert, totface;
} BMesh;
typedef struct BMVert BMVert;
typedef struct BMFace BMFace;
typedef struct BMLog BMLog;
#define BM_VERT 1
#define BM_FACE 8
#define BM_ELEM_HIDDEN (1 << 4)
int BM_elem_flag_test(const void *ele, int hflag);
void BM_mesh_elem_index_ensure(BMesh *bm, int htype);

/* ---- the PBVH public interface (BKE_pbvh.h is not in the reference) ---- */
typedef struct PBVH PBVH;
typedef struct PBVHNode PBVHNode;
typedef struct PBVHProxyNode {
  float (*co)[3];
} PBVHProxyNode;
typedef struct PBVHColorBufferNode {
  float (*color)[4];
} PBVHColorBufferNode;
typedef enum PBVHType { PBVH_FACES, PBVH_GRIDS, PBVH_BMESH } PBVHType;
/* Node flags: distinct bits.  The values used by the GPU library's C ABI
 * (SGPU_PBVH_*) are the same bits for the ones both share. */
typedef enum PBVHNodeFlags {
  PBVH_Leaf = 1 << 0,
  PBVH_UpdateNormals = 1 << 1,
  PBVH_UpdateBB = 1 << 2,
  PBVH_UpdateOriginalBB = 1 << 3,
  PBVH_UpdateDrawBuffers = 1 << 4,
  PBVH_UpdateRedraw = 1 << 5,
  PBVH_UpdateMask = 1 << 6,
  PBVH_UpdateVisibility = 1 << 8,
  PBVH_RebuildDrawBuffers = 1 << 9,
  PBVH_FullyHidden = 1 << 10,
  PBVH_FullyMasked = 1 << 11,
  PBVH_FullyUnmasked = 1 << 12,
  PBVH_UpdateTopology = 1 << 13,
  PBVH_UpdateColor = 1 << 14,
} PBVHNodeFlags;
typedef struct PBVHFrustumPlanes {
  float (*planes)[4];
  int num_planes;
} PBVHFrustumPlanes;
typedef bool (*BKE_pbvh_SearchCallback)(PBVHNode *node, void *data);
typedef void (*BKE_pbvh_HitCallback)(PBVHNode *node, void *data);
typedef void (*BKE_pbvh_HitOccludedCallback)(PBVHNode *node, void *data, float *tmin);
typedef void (*BKE_pbvh_SearchNearestCallback)(PBVHNode *node, void *data, float *tmin);

#define PBVH_ITER_ALL 0
#define PBVH_ITER_UNIQUE 1

/* Vertex iterator.  The fields pbvh_vertex_iter_init (pbvh.c) fills are
 * named as it names them; the cursor (pos, end) and the step function are
 * this harness's: refpin_vertex_iter_next walks FACES vertex lists
 * (vert_indices[0 .. totvert), unique vertices first) or every element of the
 * node's grids, and sets co / no / mask / visible for the loop body. */
typedef struct PBVHVertexIter {
  /* filled by pbvh_vertex_iter_init */
  bool respect_hide;
  bool visible;
  CCGKey key;
  CCGElem **grids;
  CCGElem *grid;
  int *grid_indices;
  int totgrid;
  int gridsize;
  BLI_bitmap **grid_hidden;
  BLI_bitmap *gh;
  MVert *mverts;
  MVert *mvert;
  const int *vert_indices;
  int totvert;
  float (*vert_normals)[3];
  float *vmask;
  float (*vcol)[4];
  GSetIterator bm_unique_verts;
  GSetIterator bm_other_verts;
  CustomData *bm_vdata;
  int cd_vert_mask_offset;
  /* set per visited vertex */
  float *co;
  float *no;
  float *fno;
  float *mask;
  int index;
  /* cursor */
  int pos, end, mode;
} PBVHVertexIter;

void pbvh_vertex_iter_init(PBVH *pbvh, PBVHNode *node, PBVHVertexIter *vi, int mode);
bool refpin_vertex_iter_next(PBVHVertexIter *vi);

#define BKE_pbvh_vertex_iter_begin(pbvh, node, vi, mode_) \
  memset(&vi, 0, sizeof(vi)); \
  pbvh_vertex_iter_init(pbvh, node, &vi, mode_); \
  vi.mode = (mode_); \
  vi.pos = -1; \
  vi.end = vi.grids ? vi.totgrid * vi.key.grid_area : vi.totvert; \
  while (refpin_vertex_iter_next(&vi)) {

#define BKE_pbvh_vertex_iter_end }

/* pbvh.c functions called before their definition */
void BKE_pbvh_node_mark_rebuild_draw(PBVHNode *node);
void BKE_pbvh_node_fully_hidden_set(PBVHNode *node, int fully_hidden);
void BKE_pbvh_node_get_grids(PBVH *pbvh, PBVHNode *node, int **r_grid_indices, int *r_totgrid,
                             int *r_maxgrid, int *r_gridsize, struct CCGElem ***r_griddata);
void BKE_pbvh_node_num_verts(PBVH *pbvh, PBVHNode *node, int *r_uniquevert, int *r_totvert);
void BKE_pbvh_node_get_verts(PBVH *pbvh, PBVHNode *node, const int **r_vert_indices,
                             struct MVert **r_verts);
void BKE_pbvh_search_gather(PBVH *pbvh, BKE_pbvh_SearchCallback scb, void *search_data,
                            PBVHNode ***r_array, int *r_tot);
void BKE_pbvh_get_grid_updates(PBVH *pbvh, bool clear, void ***r_gridfaces, int *r_totface);
void BKE_pbvh_parallel_range_settings(TaskParallelSettings *settings, bool use_threading,
                                      int totnode);
PBVHType BKE_pbvh_type(const PBVH *pbvh);
float BKE_pbvh_node_get_tmin(PBVHNode *node);
bool BKE_pbvh_node_raycast(PBVH *pbvh, PBVHNode *node, float (*origco)[3], bool use_origco,
                           const float ray_start[3], const float ray_normal[3],
                           struct IsectRayPrecalc *isect_precalc, float *depth,
                           int *active_vertex_index, int *active_face_grid_index,
                           float *face_normal);
void BKE_pbvh_raycast(PBVH *pbvh, BKE_pbvh_HitOccludedCallback cb, void *data,
                      const float ray_start[3], const float ray_normal[3], bool original);
void BKE_pbvh_find_nearest_to_ray(PBVH *pbvh, BKE_pbvh_SearchNearestCallback cb, void *data,
                                  const float ray_start[3], const float ray_normal[3],
                                  bool original);
bool BKE_pbvh_node_find_nearest_to_ray(PBVH *pbvh, PBVHNode *node, float (*origco)[3],
                                       bool use_origco, const float ray_start[3],
                                       const float ray_normal[3], float *depth, float *dist_sq);
GSet *BKE_pbvh_bmesh_node_unique_verts(PBVHNode *node);
GSet *BKE_pbvh_bmesh_node_other_verts(PBVHNode *node);
void BKE_pbvh_node_fully_masked_set(PBVHNode *node, int fully_masked);
void BKE_pbvh_node_fully_unmasked_set(PBVHNode *node, int fully_masked);
void mid_v3_v3v3(float r[3], const float a[3], const float b[3]);
BLI_bitmap **BKE_pbvh_grid_hidden(const PBVH *pbvh);
const CCGKey *BKE_pbvh_get_grid_key(const PBVH *pbvh);
int BKE_pbvh_count_grid_quads(BLI_bitmap **grid_hidden, const int *grid_indices, int totgrid,
                              int gridsize);

/* ---- mesh helpers (kernel/intern) ---- */
void BKE_mesh_calc_poly_normal(const MPoly *mpoly, const MLoop *loopstart, const MVert *mvarray,
                               float r_no[3]);
void BKE_mesh_vertex_normals_ensure(const Mesh *mesh);
float (*BKE_mesh_vertex_normals_for_write(Mesh *mesh))[3];
void BKE_mesh_calc_normals_looptri(MVert *mverts, int numVerts, const MLoop *mloop,
                                   const MLoopTri *looptri, int looptri_num, float (*r_tri_nors)[3]);
bool paint_is_face_hidden(const MLoopTri *lt, const MVert *mvert, const MLoop *mloop);
bool paint_is_grid_face_hidden(const unsigned int *grid_hidden, int gridsize, int x, int y);

/* ---- draw buffers (gpu_buffers.c, compiled by refpin_draw.c over host arrays) ---- */
typedef struct GPU_PBVH_Buffers GPU_PBVH_Buffers;
#define GPU_PBVH_BUFFERS_SHOW_MASK (1 << 1)
#define GPU_PBVH_BUFFERS_SHOW_VCOL (1 << 2)
#define GPU_PBVH_BUFFERS_SHOW_SCULPT_FACE_SETS (1 << 3)
void GPU_pbvh_buffers_free(GPU_PBVH_Buffers *buffers);
GPU_PBVH_Buffers *GPU_pbvh_mesh_buffers_build(const MPoly *mpoly, const MLoop *mloop,
                                              const MLoopTri *looptri, const MVert *verts,
                                              const int *face_indices, const int *sculpt_face_sets,
                                              int face_indices_len, const struct Mesh *mesh);
GPU_PBVH_Buffers *GPU_pbvh_grid_buffers_build(int totgrid, BLI_bitmap **grid_hidden);
GPU_PBVH_Buffers *GPU_pbvh_bmesh_buffers_build(bool smooth_shading);
void GPU_pbvh_mesh_buffers_update(GPU_PBVH_Buffers *buffers, const MVert *mvert,
                                  const float (*vert_normals)[3], const float *vmask,
                                  const MLoopCol *vcol, const int *sculpt_face_sets,
                                  int face_sets_color_seed, int face_sets_color_default,
                                  const MPropCol *vtcol, int update_flags);
void GPU_pbvh_grid_buffers_update(GPU_PBVH_Buffers *buffers, struct SubdivCCG *subdiv_ccg,
                                  CCGElem **grids, const DMFlagMat *grid_flag_mats,
                                  int *grid_indices, int totgrid, const int *sculpt_face_sets,
                                  int face_sets_color_seed, int face_sets_color_default,
                                  const CCGKey *key, int update_flags);
void GPU_pbvh_bmesh_buffers_update(GPU_PBVH_Buffers *buffers, ...);
void GPU_pbvh_grid_buffers_update_free(GPU_PBVH_Buffers *buffers, const DMFlagMat *grid_flag_mats,
                                       const int *grid_indices);
void GPU_pbvh_bmesh_buffers_update_free(GPU_PBVH_Buffers *buffers);
void GPU_pbvh_buffers_update_flush(GPU_PBVH_Buffers *buffers);
