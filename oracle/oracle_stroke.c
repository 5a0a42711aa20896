/*
 * CPU oracle, part 2: the numeric core instantiated in FP32 and FP64, and the
 * exported entry points.  TEST INFRASTRUCTURE ONLY (see oracle.h).
 */
#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "oracle_internal.h"

void or_curve_build(int preset, OrCurve *cu);

#define REAL float
#define SFX(n) n##_f
#define STATE OrStateF
#define RSQRT sqrtf
#define RFABS fabsf
#include "oracle_core.inc"
#undef REAL
#undef SFX
#undef STATE
#undef RSQRT
#undef RFABS

#define REAL double
#define SFX(n) n##_d
#define STATE OrStateD
#define RSQRT sqrt
#define RFABS fabs
#include "oracle_core.inc"
#undef REAL
#undef SFX
#undef STATE
#undef RSQRT
#undef RFABS

/* FP32 face normals for the draw-buffer restatement (oracle_draw.c). */
void or_poly_normal_fp32(const OrMesh *m, int p, float r[3])
{
  poly_normal_f(m, m->sf.co, p, r);
}
void or_normal_quad_fp32(float n[3], const float *v1, const float *v2, const float *v3,
                         const float *v4)
{
  normal_quad_f(n, v1, v2, v3, v4);
}

int or_search_sphere(OrMesh *m, const float center[3], float radius_sq, int original,
                     int *out_nodes)
{
  return search_f(m, &m->sf, 0, center, radius_sq, original, 0, out_nodes);
}

void or_recalc_all_normals(OrMesh *m)
{
  recalc_all_normals_f(m, &m->sf);
  recalc_all_normals_d(m, &m->sd);
}

int or_brush_pass(OrMesh *m, const OrBrush *b, const float location[3],
                  const float grab_delta[3], const int *nodes, int totnode, float *area_out)
{
  OrCurve cu;
  or_curve_build(b->curve_preset, &cu);
  if (b->sculpt_tool == OR_TOOL_LAYER && !m->sf.orig_co) {
    store_original_f(m, &m->sf); /* the layer reads the stroke-start positions */
  }
  return (int)brush_pass_f(m, &m->sf, &cu, b, location, grab_delta, b->view_normal, nodes,
                           totnode, area_out);
}

void or_update_normals(OrMesh *m) { update_normals_f(m, &m->sf); }

void or_update_bounds(OrMesh *m, int flag) { update_bounds_f(m, &m->sf, flag); }

void or_node_mark_update(OrMesh *m, int node)
{
  if (node >= 0 && node < m->totnode) {
    mark_nodes_f(m, &node, 1);
  }
}

/* BKE_pbvh_vert_mark_update (pbvh.c:3729): tag one vertex for the normal update. */
void or_vert_mark_update(OrMesh *m, int vertex)
{
  if (vertex >= 0 && vertex < m->totvert) {
    m->vtag[vertex] = 1;
  }
}

/* The vert_bitmap tags (one byte per vertex, 0 or 1). */
void or_get_vert_tags(const OrMesh *m, unsigned char *out)
{
  memcpy(out, m->vtag, (size_t)m->totvert);
}

int64_t or_stroke(OrMesh *m, const OrBrush *b, const float *dabs, int ndabs,
                  const int *dab_tools, int which, int nthreads, int64_t *per_dab_counts)
{
#ifdef _OPENMP
  if (nthreads > 0) {
    omp_set_num_threads(nthreads);
  }
#else
  (void)nthreads;
#endif
  int64_t total = 0;
  if (which & 1) {
    total = stroke_f(m, &m->sf, b, dabs, ndabs, dab_tools, per_dab_counts);
  }
  if (which & 2) {
    const int64_t t64 =
        stroke_d(m, &m->sd, b, dabs, ndabs, dab_tools, (which & 1) ? NULL : per_dab_counts);
    if (!(which & 1)) {
      total = t64;
    }
  }
  return total;
}

void or_store_original(OrMesh *m)
{
  store_original_f(m, &m->sf);
  store_original_d(m, &m->sd);
}

int or_orig_dab(OrMesh *m, const OrBrush *b, const float location[3], const float grab_delta[3])
{
  OrCurve cu;
  or_curve_build(b->curve_preset, &cu);
  if (!m->sf.orig_co) {
    store_original_f(m, &m->sf);
  }
  int *nodes = (int *)malloc(sizeof(int) * (m->totnode + 1));
  const int64_t n = orig_dab_full_f(m, &m->sf, &cu, b, location, grab_delta, nodes);
  free(nodes);
  return (int)n;
}

void or_kelvinlet(int type, float radius, float force, float poisson, const float co[3],
                  const float location[3], const float delta_or_normal[3], float out[3])
{
  Kelvinlet_f p;
  kelvinlet_init_f(&p, radius, force, 1.0f, poisson);
  kelvinlet_disp_f(type, &p, co, location, delta_or_normal, out);
}

float or_curve_strength(int preset, float dist, float radius)
{
  OrCurve cu;
  or_curve_build(preset, &cu);
  return curve_strength_f(&cu, dist, radius);
}

int or_max_threads(void)
{
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
