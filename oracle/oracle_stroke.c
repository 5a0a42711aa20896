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

/* Copies the FP32 state into the FP64 state (exact widening), so that an FP64
 * step taken from there measures the rounding error of the same FP32 step. */
static void widen(double *dst, const float *src, size_t n)
{
#pragma omp parallel for schedule(static)
  for (long long i = 0; i < (long long)n; i++) {
    dst[i] = (double)src[i];
  }
}

void or_sync64(OrMesh *m)
{
  const size_t v3 = 3 * (size_t)m->totvert, n6 = 6 * (size_t)m->totnode;
  widen(m->sd.co, m->sf.co, v3);
  widen(m->sd.no, m->sf.no, v3);
  if (m->sf.mask) {
    widen(m->sd.mask, m->sf.mask, (size_t)m->totvert);
  }
  widen(m->sd.vb, m->sf.vb, n6);
  widen(m->sd.orig_vb, m->sf.orig_vb, n6);
  if (m->sf.orig_co) {
    if (!m->sd.orig_co) {
      m->sd.orig_co = (double *)malloc(sizeof(double) * v3);
      m->sd.orig_no = (double *)malloc(sizeof(double) * v3);
      m->sd.layer_disp = (double *)malloc(sizeof(double) * (size_t)m->totvert);
    }
    widen(m->sd.orig_co, m->sf.orig_co, v3);
    widen(m->sd.orig_no, m->sf.orig_no, v3);
    widen(m->sd.layer_disp, m->sf.layer_disp, (size_t)m->totvert);
  }
}

/* max |f - d| over n values, and max |d| */
static void max_diff(const float *f, const double *d, size_t n, double *r_diff, double *r_ref)
{
  double md = 0.0, mr = 0.0;
#pragma omp parallel for schedule(static) reduction(max : md, mr)
  for (long long i = 0; i < (long long)n; i++) {
    const double e = fabs((double)f[i] - d[i]);
    const double a = fabs(d[i]);
    md = e > md ? e : md;
    mr = a > mr ? a : mr;
  }
  *r_diff = md;
  *r_ref = mr;
}

void or_area_normal_center(OrMesh *m, const OrBrush *b, const float location[3],
                           const int *nodes, int totnode, float out32[6], double out64[6])
{
  or_sync64(m);
  float nf[3], cf[3];
  double nd[3], cd[3];
  const double locd[3] = {location[0], location[1], location[2]};
  area_calc_f(m, &m->sf, b, location, nodes, totnode, nf, cf);
  area_calc_d(m, &m->sd, b, locd, nodes, totnode, nd, cd);
  for (int k = 0; k < 3; k++) {
    out32[k] = nf[k];
    out32[3 + k] = cf[k];
    out64[k] = nd[k];
    out64[3 + k] = cd[k];
  }
}

/* Node flags and vertex tags (FACES) of the oracle, saved and put back so
 * that both precisions run a stage from the same flags. */
typedef struct FlagState {
  int *flags;
  unsigned char *tags;
} FlagState;

static void flags_save(const OrMesh *m, FlagState *f)
{
  for (int n = 0; n < m->totnode; n++) {
    f->flags[n] = m->nodes[n].flag;
  }
  if (m->vtag) {
    memcpy(f->tags, m->vtag, (size_t)m->totvert);
  }
}

static void flags_load(OrMesh *m, const FlagState *f)
{
  for (int n = 0; n < m->totnode; n++) {
    m->nodes[n].flag = f->flags[n];
  }
  if (m->vtag) {
    memcpy(m->vtag, f->tags, (size_t)m->totvert);
  }
}

static void flags_alloc(const OrMesh *m, FlagState *f)
{
  f->flags = (int *)malloc(sizeof(int) * ((size_t)m->totnode + 1));
  f->tags = (unsigned char *)malloc((size_t)m->totvert + 1);
}

static void flags_free(FlagState *f)
{
  free(f->flags);
  free(f->tags);
}

static double rel_diff(const float *f, const double *d, size_t n)
{
  double diff, ref;
  max_diff(f, d, n, &diff, &ref);
  return ref > 0.0 ? diff / ref : diff;
}

int64_t or_stroke_local_error(OrMesh *m, const OrBrush *b, const float *dabs, int ndabs,
                              const int *tools, int stride, int nthreads, double *err)
{
#ifdef _OPENMP
  if (nthreads > 0) {
    omp_set_num_threads(nthreads);
  }
#else
  (void)nthreads;
#endif
  OrCurve cu;
  or_curve_build(b->curve_preset, &cu);
  const size_t V = (size_t)m->totvert, v3 = 3 * V, n6 = 6 * (size_t)m->totnode;
  int *nodes = (int *)malloc(sizeof(int) * (m->totnode + 1));
  FlagState f0, fb, fu;
  flags_alloc(m, &f0);
  flags_alloc(m, &fb);
  flags_alloc(m, &fu);
  if (stroke_needs_start_f(b, ndabs, tools)) {
    store_original_f(m, &m->sf);
  }
  int64_t total = 0;
  for (int d = 0; d < ndabs; d++) {
    double *e = err + 5 * (size_t)d;
    if (stride <= 0 || d % stride != 0) {
      total += stroke_dab_f(m, &m->sf, b, &cu, dabs, d, tools, nodes);
      for (int k = 0; k < 5; k++) {
        e[k] = -1.0;
      }
      continue;
    }
    /* brush stage from the same input */
    flags_save(m, &f0);
    or_sync64(m);
    float area_f[48];
    double area_d[48];
    total += stroke_dab_brush_f(m, &m->sf, b, &cu, dabs, d, tools, nodes, area_f);
    flags_save(m, &fb);
    flags_load(m, &f0);
    stroke_dab_brush_d(m, &m->sd, b, &cu, dabs, d, tools, nodes, area_d);
    e[0] = rel_diff(m->sf.co, m->sd.co, v3);
    double ea_no = 0.0, ea_co = 0.0;
    for (int p = 0; p < 8; p++) {
      for (int k = 0; k < 3; k++) {
        const double dn = fabs((double)area_f[6 * p + k] - area_d[6 * p + k]);
        const double dc = fabs((double)area_f[6 * p + 3 + k] - area_d[6 * p + 3 + k]);
        ea_no = dn > ea_no ? dn : ea_no;
        ea_co = dc > ea_co ? dc : ea_co;
      }
    }
    e[3] = ea_no;
    e[4] = ea_co;
    /* normal update (GRIDS: with the seam averages of positions and masks)
     * from the same positions */
    or_sync64(m);
    update_normals_f(m, &m->sf);
    flags_save(m, &fu);
    flags_load(m, &fb);
    update_normals_d(m, &m->sd);
    {
      double diff, ref;
      max_diff(m->sf.no, m->sd.no, v3, &diff, &ref);
      e[1] = diff; /* unit vectors (GRIDS: means of unit vectors) */
    }
    const double eco = rel_diff(m->sf.co, m->sd.co, v3);
    e[0] = eco > e[0] ? eco : e[0];
    /* bounds refit from the same positions */
    or_sync64(m);
    flags_load(m, &fu);
    update_bounds_f(m, &m->sf, OR_UpdateBB);
    flags_save(m, &fb);
    flags_load(m, &fu);
    update_bounds_d(m, &m->sd, OR_UpdateBB);
    flags_load(m, &fb);
    e[2] = rel_diff(m->sf.vb, m->sd.vb, n6);
    (void)V;
  }
  update_bounds_f(m, &m->sf, OR_UpdateOriginalBB);
  free(nodes);
  flags_free(&f0);
  flags_free(&fb);
  flags_free(&fu);
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
