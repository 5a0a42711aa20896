/*
 * CPU oracle, part 3: the PBVH ray cast (PBVH_FACES and PBVH_GRIDS) — TEST
 * INFRASTRUCTURE ONLY (see oracle.h).
 *
 * Restates, in FP32:
 *   isect_ray_aabb_v3_precalc / isect_ray_aabb_v3        math_geom.cc:3017-3079
 *   isect_ray_tri_watertight_v3_precalc / _v3            math_geom.cc:1755-1855
 *   axis_dominant_v3_single                               math_geom_inline.c:76-82
 *   BKE_pbvh_raycast + ray_aabb_intersect                 pbvh.c:3897-3929
 *   pbvh_iter_next_occluded                               pbvh.c:2708-2735
 *   node_tree_insert, traverse_tree                       pbvh.c:2797-2831
 *   BKE_pbvh_search_callback_occluded                     pbvh.c:2853-2890
 *   ray_face_intersection_tri / _quad                     pbvh.c:3930-3967
 *   pbvh_faces_node_raycast                               pbvh.c:4042-4108
 *   pbvh_grids_node_raycast                               pbvh.c:4110-4201
 * and for the nearest-to-ray query:
 *   dist_squared_ray_to_seg_v3                            math_geom.cc:574-608
 *   aabb_get_near_far_from_plane                          math_geom.cc:610-641
 *   dist_squared_ray_to_aabb_v3(_precalc)                 math_geom.cc:643-744
 *   isect_ray_line_v3                                     math_geom.cc:1997-2021
 *   interp_v3_v3v3                                        math_vector.c:24-31
 *   nearest_to_ray_aabb_dist_sq,
 *   BKE_pbvh_find_nearest_to_ray                          pbvh.c:4315-4352
 *   dist_squared_ray_to_tri_v3_fast,
 *   ray_face_nearest_quad / _tri                          pbvh.c:3970-4040
 *   pbvh_faces_node_nearest_to_ray,
 *   pbvh_grids_node_nearest_to_ray                        pbvh.c:4354-4460
 * and the sculpt ray-cast callback the reference calls but does not ship
 * (its sculpt.c is absent), fixed by the brush specification: a leaf is ray
 * cast when its entry distance is below the running minimum (FLT_MAX until
 * the first hit, then the hit depth), and a hit makes the hit depth the new
 * running minimum.  Positions are the current ones (no undo copy of the
 * original coordinates exists here; `original` selects orig_vb for the boxes).
 */
#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "oracle_internal.h"

typedef struct RayBox {
  float org[3], inv[3];
  int sign[3];
} RayBox;

static void raybox_init(RayBox *r, const float o[3], const float d[3])
{
  for (int i = 0; i < 3; i++) {
    r->org[i] = o[i];
    r->inv[i] = 1.0f / d[i];
    r->sign[i] = r->inv[i] < 0.0f;
  }
}

/* Entry distance into the box (tmin) when the ray line meets it. */
static int raybox_hit(const RayBox *r, const float *bmin, const float *bmax, float *tmin_out)
{
  const float *bb[2] = {bmin, bmax};
  float tmin = (bb[r->sign[0]][0] - r->org[0]) * r->inv[0];
  float tmax = (bb[1 - r->sign[0]][0] - r->org[0]) * r->inv[0];
  const float tymin = (bb[r->sign[1]][1] - r->org[1]) * r->inv[1];
  const float tymax = (bb[1 - r->sign[1]][1] - r->org[1]) * r->inv[1];
  if ((tmin > tymax) || (tymin > tmax)) {
    return 0;
  }
  if (tymin > tmin) {
    tmin = tymin;
  }
  if (tymax < tmax) {
    tmax = tymax;
  }
  const float tzmin = (bb[r->sign[2]][2] - r->org[2]) * r->inv[2];
  const float tzmax = (bb[1 - r->sign[2]][2] - r->org[2]) * r->inv[2];
  if ((tmin > tzmax) || (tzmin > tmax)) {
    return 0;
  }
  if (tzmin > tmin) {
    tmin = tzmin;
  }
  *tmin_out = tmin;
  return 1;
}

typedef struct RayTri {
  int kx, ky, kz;
  float sx, sy, sz;
} RayTri;

static void raytri_init(RayTri *p, const float d[3])
{
  const float x = fabsf(d[0]), y = fabsf(d[1]), z = fabsf(d[2]);
  const int kz = (x > y) ? ((x > z) ? 0 : 2) : ((y > z) ? 1 : 2);
  int kx = (kz != 2) ? (kz + 1) : 0;
  int ky = (kx != 2) ? (kx + 1) : 0;
  if (d[kz] < 0.0f) {
    const int t = kx;
    kx = ky;
    ky = t;
  }
  const float inv_dir_z = 1.0f / d[kz];
  p->sx = d[kx] * inv_dir_z;
  p->sy = d[ky] * inv_dir_z;
  p->sz = inv_dir_z;
  p->kx = kx;
  p->ky = ky;
  p->kz = kz;
}

static int f_bits(float f)
{
  int i;
  memcpy(&i, &f, sizeof(i));
  return i;
}
static float bits_f(int i)
{
  float f;
  memcpy(&f, &i, sizeof(f));
  return f;
}

/* Watertight ray / triangle test; *r_lambda = hit distance along the ray. */
static int raytri_hit(const float o[3], const RayTri *p, const float *v0, const float *v1,
                      const float *v2, float *r_lambda)
{
  const float a[3] = {v0[0] - o[0], v0[1] - o[1], v0[2] - o[2]};
  const float b[3] = {v1[0] - o[0], v1[1] - o[1], v1[2] - o[2]};
  const float c[3] = {v2[0] - o[0], v2[1] - o[1], v2[2] - o[2]};
  const float a_kx = a[p->kx], a_ky = a[p->ky], a_kz = a[p->kz];
  const float b_kx = b[p->kx], b_ky = b[p->ky], b_kz = b[p->kz];
  const float c_kx = c[p->kx], c_ky = c[p->ky], c_kz = c[p->kz];
  const float ax = a_kx - p->sx * a_kz;
  const float ay = a_ky - p->sy * a_kz;
  const float bx = b_kx - p->sx * b_kz;
  const float by = b_ky - p->sy * b_kz;
  const float cx = c_kx - p->sx * c_kz;
  const float cy = c_ky - p->sy * c_kz;
  const float u = cx * by - cy * bx;
  const float v = ax * cy - ay * cx;
  const float w = bx * ay - by * ax;
  if ((u < 0.0f || v < 0.0f || w < 0.0f) && (u > 0.0f || v > 0.0f || w > 0.0f)) {
    return 0;
  }
  const float det = u + v + w;
  if (det == 0.0f || !isfinite(det)) {
    return 0;
  }
  const int sign_det = f_bits(det) & (int)0x80000000u;
  const float t = (u * a_kz + v * b_kz + w * c_kz) * p->sz;
  const float sign_t = bits_f(f_bits(t) ^ sign_det);
  if (sign_t < 0.0f) {
    return 0;
  }
  const float inv_det = 1.0f / det;
  *r_lambda = t * inv_det;
  return 1;
}

static float len_sq3(const float *a, const float *b)
{
  const float d0 = a[0] - b[0], d1 = a[1] - b[1], d2 = a[2] - b[2];
  return d0 * d0 + d1 * d1 + d2 * d2;
}

/* normal_tri_v3 (math_geom.cc:31-46) followed by normalize_v3 */
static void tri_normal(float n[3], const float *v1, const float *v2, const float *v3)
{
  float n1[3], n2[3];
  n1[0] = v1[0] - v2[0];
  n2[0] = v2[0] - v3[0];
  n1[1] = v1[1] - v2[1];
  n2[1] = v2[1] - v3[1];
  n1[2] = v1[2] - v2[2];
  n2[2] = v2[2] - v3[2];
  n[0] = n1[1] * n2[2] - n1[2] * n2[1];
  n[1] = n1[2] * n2[0] - n1[0] * n2[2];
  n[2] = n1[0] * n2[1] - n1[1] * n2[0];
  float d = n[0] * n[0] + n[1] * n[1] + n[2] * n[2];
  if (d > 1.0e-35f) {
    d = sqrtf(d);
    const float s = 1.0f / d;
    n[0] = n[0] * s;
    n[1] = n[1] * s;
    n[2] = n[2] * s;
  }
  else {
    n[0] = n[1] = n[2] = 0.0f;
  }
}

/* normal_quad_v3 (math_geom.cc:48-71) followed by normalize_v3 */
static void quad_normal(float n[3], const float *v1, const float *v2, const float *v3,
                        const float *v4)
{
  float n1[3], n2[3];
  n1[0] = v1[0] - v3[0];
  n1[1] = v1[1] - v3[1];
  n1[2] = v1[2] - v3[2];
  n2[0] = v2[0] - v4[0];
  n2[1] = v2[1] - v4[1];
  n2[2] = v2[2] - v4[2];
  n[0] = n1[1] * n2[2] - n1[2] * n2[1];
  n[1] = n1[2] * n2[0] - n1[0] * n2[2];
  n[2] = n1[0] * n2[1] - n1[1] * n2[0];
  float d = n[0] * n[0] + n[1] * n[1] + n[2] * n[2];
  if (d > 1.0e-35f) {
    d = sqrtf(d);
    const float s = 1.0f / d;
    n[0] = n[0] * s;
    n[1] = n[1] * s;
    n[2] = n[2] * s;
  }
  else {
    n[0] = n[1] = n[2] = 0.0f;
  }
}

/* pbvh_grids_node_raycast: the grid quads of a leaf in prim / row / column
 * order; per quad ray_face_intersection_quad, whose second triangle is tried
 * only when the first one is not taken.  Active vertex = grid element index
 * (grid * area + y * size + x) of the corner nearest the hit; active face =
 * the grid index. */
static int grids_node_raycast(const OrMesh *m, const OrNode *nd, const float *o, const float *dir,
                              const RayTri *rt, float *depth, int *active_vertex,
                              int *active_grid, float face_normal[3])
{
  const int gs = m->grid_size, area = m->grid_area;
  static const int x_it[4] = {0, 1, 1, 0};
  static const int y_it[4] = {0, 0, 1, 1};
  int hit = 0;
  for (int i = 0; i < nd->totprim; i++) {
    const int g = m->prim_indices[nd->prim_off + i];
    const float *base = m->sf.co + 3 * (size_t)g * area;
    for (int y = 0; y < gs - 1; y++) {
      for (int x = 0; x < gs - 1; x++) {
        const float *co[4] = {base + 3 * (y * gs + x), base + 3 * (y * gs + x + 1),
                              base + 3 * ((y + 1) * gs + x + 1), base + 3 * ((y + 1) * gs + x)};
        float dt;
        int take = 0;
        if (raytri_hit(o, rt, co[0], co[1], co[2], &dt) && dt < *depth) {
          take = 1;
        }
        else if (raytri_hit(o, rt, co[0], co[2], co[3], &dt) && dt < *depth) {
          take = 1;
        }
        if (!take) {
          continue;
        }
        *depth = dt;
        hit = 1;
        quad_normal(face_normal, co[0], co[1], co[2], co[3]);
        const float loc[3] = {o[0] + dir[0] * dt, o[1] + dir[1] * dt, o[2] + dir[2] * dt};
        float nearest[3];
        for (int j = 0; j < 4; j++) {
          if (j == 0 || len_sq3(loc, co[j]) < len_sq3(loc, nearest)) {
            nearest[0] = co[j][0];
            nearest[1] = co[j][1];
            nearest[2] = co[j][2];
            *active_vertex = area * g + (y + y_it[j]) * gs + (x + x_it[j]);
          }
        }
        *active_grid = g;
      }
    }
  }
  return hit;
}

int or_raycast(OrMesh *m, const float ray_start[3], const float ray_normal[3], int original,
               float *depth, int *active_vertex, int *active_face, float face_normal[3],
               int *r_nleaves)
{
  if (m->totnode == 0) {
    if (r_nleaves) {
      *r_nleaves = 0;
    }
    return 0;
  }
  const float *boxes = original ? m->sf.orig_vb : m->sf.vb;
  RayBox rb;
  raybox_init(&rb, ray_start, ray_normal);
  RayTri rt;
  raytri_init(&rt, ray_normal);

  /* pbvh_iter_next_occluded: left-first DFS, a failing node prunes its subtree */
  int *stack = malloc(sizeof(int) * (size_t)(m->totnode + 1));
  int *leaf = malloc(sizeof(int) * (size_t)(m->nleaf + 1));
  float *tmin = malloc(sizeof(float) * (size_t)(m->nleaf + 1));
  int *left = malloc(sizeof(int) * (size_t)(m->nleaf + 1));
  int *right = malloc(sizeof(int) * (size_t)(m->nleaf + 1));
  int ns = 0, nl = 0;
  stack[ns++] = 0;
  while (ns) {
    const int n = stack[--ns];
    float t;
    if (!raybox_hit(&rb, boxes + 6 * n, boxes + 6 * n + 3, &t)) {
      continue;
    }
    const OrNode *nd = &m->nodes[n];
    if (nd->flag & OR_Leaf) {
      leaf[nl] = n;
      tmin[nl] = t;
      left[nl] = right[nl] = -1;
      /* node_tree_insert: smaller tmin to the left, ties to the right */
      if (nl > 0) {
        int at = 0;
        for (;;) {
          int *next = (t < tmin[at]) ? &left[at] : &right[at];
          if (*next < 0) {
            *next = nl;
            break;
          }
          at = *next;
        }
      }
      nl++;
      continue;
    }
    stack[ns++] = nd->children_offset + 1;
    stack[ns++] = nd->children_offset;
  }
  if (r_nleaves) {
    *r_nleaves = nl;
  }

  /* traverse_tree: in-order, with the spec'd hit callback */
  int hit = 0;
  float run_tmin = FLT_MAX;
  float d = *depth;
  int *st = stack;
  int sp = 0, cur = nl > 0 ? 0 : -1;
  while (cur >= 0 || sp > 0) {
    while (cur >= 0) {
      st[sp++] = cur;
      cur = left[cur];
    }
    cur = st[--sp];
    if (tmin[cur] < run_tmin && m->type == OR_GRIDS) {
      if (grids_node_raycast(m, &m->nodes[leaf[cur]], ray_start, ray_normal, &rt, &d,
                             active_vertex, active_face, face_normal)) {
        hit = 1;
        run_tmin = d;
      }
    }
    else if (tmin[cur] < run_tmin) {
      /* pbvh_faces_node_raycast over the leaf's looptris in prim order */
      const OrNode *nd = &m->nodes[leaf[cur]];
      int node_hit = 0;
      for (int i = 0; i < nd->totprim; i++) {
        const int t = m->prim_indices[nd->prim_off + i];
        const int *tv = m->lt_v + 3 * (size_t)t;
        const float *co[3] = {m->sf.co + 3 * (size_t)tv[0], m->sf.co + 3 * (size_t)tv[1],
                              m->sf.co + 3 * (size_t)tv[2]};
        float dt;
        if (raytri_hit(ray_start, &rt, co[0], co[1], co[2], &dt) && dt < d) {
          d = dt;
          node_hit = 1;
          tri_normal(face_normal, co[0], co[1], co[2]);
          /* location = ray_start + ray_normal * depth (madd_v3_v3v3fl) */
          const float loc[3] = {ray_start[0] + ray_normal[0] * d, ray_start[1] + ray_normal[1] * d,
                                ray_start[2] + ray_normal[2] * d};
          float nearest[3];
          for (int j = 0; j < 3; j++) {
            if (j == 0 || len_sq3(loc, co[j]) < len_sq3(loc, nearest)) {
              nearest[0] = co[j][0];
              nearest[1] = co[j][1];
              nearest[2] = co[j][2];
              *active_vertex = tv[j];
              *active_face = m->lt_poly[t];
            }
          }
        }
      }
      if (node_hit) {
        hit = 1;
        run_tmin = d;
      }
    }
    cur = right[cur];
  }
  *depth = d;
  free(stack);
  free(leaf);
  free(tmin);
  free(left);
  free(right);
  return hit;
}

/* Test helper: quads of the whole grid mesh where both triangles meet the ray
 * and the second one is closer (dB < dA) — the case in which
 * ray_face_intersection_quad's order matters. */
int or_grids_special_quads(OrMesh *m, const float ray_start[3], const float ray_normal[3])
{
  if (m->type != OR_GRIDS) {
    return 0;
  }
  RayTri rt;
  raytri_init(&rt, ray_normal);
  const int gs = m->grid_size, area = m->grid_area;
  int n = 0;
  for (int g = 0; g < m->num_grids; g++) {
    const float *base = m->sf.co + 3 * (size_t)g * area;
    for (int y = 0; y < gs - 1; y++) {
      for (int x = 0; x < gs - 1; x++) {
        const float *co[4] = {base + 3 * (y * gs + x), base + 3 * (y * gs + x + 1),
                              base + 3 * ((y + 1) * gs + x + 1), base + 3 * ((y + 1) * gs + x)};
        float da, db;
        if (raytri_hit(ray_start, &rt, co[0], co[1], co[2], &da) &&
            raytri_hit(ray_start, &rt, co[0], co[2], co[3], &db) && db < da) {
          n++;
        }
      }
    }
  }
  return n;
}

/* ---- nearest to ray ---- */

static float dot3(const float *a, const float *b)
{
  return a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
}

static void cross3(float r[3], const float *a, const float *b)
{
  r[0] = a[1] * b[2] - a[2] * b[1];
  r[1] = a[2] * b[0] - a[0] * b[2];
  r[2] = a[0] * b[1] - a[1] * b[0];
}

/* isect_ray_line_v3: parameter of the point of the line v0 -> v1 nearest the
 * ray (0 when the two are parallel, returned as no intersection). */
static int ray_line(const float *o, const float *dir, const float *v0, const float *v1,
                    float *r_lambda)
{
  const float a[3] = {v1[0] - v0[0], v1[1] - v0[1], v1[2] - v0[2]};
  const float t[3] = {v0[0] - o[0], v0[1] - o[1], v0[2] - o[2]};
  float n[3];
  cross3(n, a, dir);
  const float nlen = dot3(n, n);
  if (nlen == 0.0f) {
    return 0;
  }
  const float c[3] = {n[0] - t[0], n[1] - t[1], n[2] - t[2]};
  float cray[3];
  cross3(cray, c, dir);
  *r_lambda = dot3(cray, n) / nlen;
  return 1;
}

/* dist_squared_ray_to_seg_v3: squared distance of the segment point the line
 * parameter selects (clamped to the ends; v0 for a parallel segment) from the
 * ray, and its depth along the ray. */
static float ray_seg_dist_sq(const float *o, const float *dir, const float *v0, const float *v1,
                             float *r_depth)
{
  float lambda, p[3];
  if (ray_line(o, dir, v0, v1, &lambda)) {
    if (lambda <= 0.0f) {
      p[0] = v0[0], p[1] = v0[1], p[2] = v0[2];
    }
    else if (lambda >= 1.0f) {
      p[0] = v1[0], p[1] = v1[1], p[2] = v1[2];
    }
    else {
      const float s = 1.0f - lambda;
      p[0] = s * v0[0] + lambda * v1[0];
      p[1] = s * v0[1] + lambda * v1[1];
      p[2] = s * v0[2] + lambda * v1[2];
    }
  }
  else {
    p[0] = v0[0], p[1] = v0[1], p[2] = v0[2];
  }
  const float dvec[3] = {p[0] - o[0], p[1] - o[1], p[2] - o[2]};
  const float depth = dot3(dvec, dir);
  *r_depth = depth;
  return dot3(dvec, dvec) - depth * depth;
}

/* dist_squared_ray_to_tri_v3_fast: the nearest of the three edges (in the
 * order (v0, v2), (v1, v0), (v2, v1); the first edge, then any strictly
 * nearer one). */
static float ray_tri_dist_sq(const float *o, const float *dir, const float *v0, const float *v1,
                             const float *v2, float *r_depth)
{
  const float *tri[3] = {v0, v1, v2};
  float best = FLT_MAX;
  for (int i = 0, j = 2; i < 3; j = i++) {
    float dt = FLT_MAX;
    const float d = ray_seg_dist_sq(o, dir, tri[i], tri[j], &dt);
    if (d < best || i == 0) {
      *r_depth = dt;
      best = d;
    }
  }
  return best;
}

typedef struct RayAabb {
  float org[3], dir[3], inv[3];
} RayAabb;

static void rayaabb_init(RayAabb *r, const float o[3], const float d[3])
{
  for (int i = 0; i < 3; i++) {
    r->org[i] = o[i];
    r->dir[i] = d[i];
    r->inv[i] = (d[i] != 0.0f) ? (1.0f / d[i]) : FLT_MAX;
  }
}

/* dist_squared_ray_to_aabb_v3: 0 and the depth of the far corner when the
 * ray line meets the box, else the squared distance to the box edge nearest
 * the ray and its depth. */
static float rayaabb_dist_sq(const RayAabb *r, const float *bmin, const float *bmax,
                             float *r_depth)
{
  float lo[3], hi[3];
  for (int k = 0; k < 3; k++) {
    /* aabb_get_near_far_from_plane */
    if (r->dir[k] < 0.0f) {
      lo[k] = bmax[k];
      hi[k] = bmin[k];
    }
    else {
      lo[k] = bmin[k];
      hi[k] = bmax[k];
    }
  }
  const float tmin[3] = {(lo[0] - r->org[0]) * r->inv[0], (lo[1] - r->org[1]) * r->inv[1],
                         (lo[2] - r->org[2]) * r->inv[2]};
  const float tmax[3] = {(hi[0] - r->org[0]) * r->inv[0], (hi[1] - r->org[1]) * r->inv[1],
                         (hi[2] - r->org[2]) * r->inv[2]};
  float va[3] = {0.0f, 0.0f, 0.0f}, vb[3] = {0.0f, 0.0f, 0.0f};
  float rtmin, rtmax;
  int axis;
  if ((tmax[0] <= tmax[1]) && (tmax[0] <= tmax[2])) {
    rtmax = tmax[0];
    va[0] = vb[0] = hi[0];
    axis = 3;
  }
  else if ((tmax[1] <= tmax[0]) && (tmax[1] <= tmax[2])) {
    rtmax = tmax[1];
    va[1] = vb[1] = hi[1];
    axis = 2;
  }
  else {
    rtmax = tmax[2];
    va[2] = vb[2] = hi[2];
    axis = 1;
  }
  if ((tmin[0] >= tmin[1]) && (tmin[0] >= tmin[2])) {
    rtmin = tmin[0];
    va[0] = vb[0] = lo[0];
    axis -= 3;
  }
  else if ((tmin[1] >= tmin[0]) && (tmin[1] >= tmin[2])) {
    rtmin = tmin[1];
    va[1] = vb[1] = lo[1];
    axis -= 1;
  }
  else {
    rtmin = tmin[2];
    va[2] = vb[2] = lo[2];
    axis -= 2;
  }
  if (axis < 0) {
    axis += 3;
  }
  if (rtmin <= rtmax) {
    const float dvec[3] = {hi[0] - r->org[0], hi[1] - r->org[1], hi[2] - r->org[2]};
    *r_depth = dot3(dvec, r->dir);
    return 0.0f;
  }
  if (r->dir[axis] >= 0.0f) {
    va[axis] = lo[axis];
    vb[axis] = hi[axis];
  }
  else {
    va[axis] = hi[axis];
    vb[axis] = lo[axis];
  }
  return ray_seg_dist_sq(r->org, r->dir, va, vb, r_depth);
}

int or_nearest_to_ray(OrMesh *m, const float ray_start[3], const float ray_normal[3],
                      int original, float *depth, float *dist_sq, int *r_nleaves)
{
  if (m->totnode == 0) {
    if (r_nleaves) {
      *r_nleaves = 0;
    }
    return 0;
  }
  const float *boxes = original ? m->sf.orig_vb : m->sf.vb;
  RayAabb ra;
  rayaabb_init(&ra, ray_start, ray_normal);
  /* pbvh_iter_next_occluded with nearest_to_ray_aabb_dist_sq: a node passes
   * when the depth of its nearest point is positive; its tmin is the squared
   * distance */
  int *stack = malloc(sizeof(int) * (size_t)(m->totnode + 1));
  int *leaf = malloc(sizeof(int) * (size_t)(m->nleaf + 1));
  float *tmin = malloc(sizeof(float) * (size_t)(m->nleaf + 1));
  int *left = malloc(sizeof(int) * (size_t)(m->nleaf + 1));
  int *right = malloc(sizeof(int) * (size_t)(m->nleaf + 1));
  int ns = 0, nl = 0;
  stack[ns++] = 0;
  while (ns) {
    const int n = stack[--ns];
    float dep;
    const float t = rayaabb_dist_sq(&ra, boxes + 6 * n, boxes + 6 * n + 3, &dep);
    if (!(dep > 0.0f)) {
      continue;
    }
    const OrNode *nd = &m->nodes[n];
    if (nd->flag & OR_Leaf) {
      leaf[nl] = n;
      tmin[nl] = t;
      left[nl] = right[nl] = -1;
      if (nl > 0) { /* node_tree_insert */
        int at = 0;
        for (;;) {
          int *next = (t < tmin[at]) ? &left[at] : &right[at];
          if (*next < 0) {
            *next = nl;
            break;
          }
          at = *next;
        }
      }
      nl++;
      continue;
    }
    stack[ns++] = nd->children_offset + 1;
    stack[ns++] = nd->children_offset;
  }
  if (r_nleaves) {
    *r_nleaves = nl;
  }
  /* traverse_tree with the callback: a leaf is searched when its tmin is below
   * the running minimum; a found triangle makes its squared distance the
   * running minimum */
  int hit = 0;
  float run_tmin = FLT_MAX;
  float dep = *depth, dsq = *dist_sq;
  int *st = stack;
  int sp = 0, cur = nl > 0 ? 0 : -1;
  const int gs = m->grid_size, area = m->grid_area;
  while (cur >= 0 || sp > 0) {
    while (cur >= 0) {
      st[sp++] = cur;
      cur = left[cur];
    }
    cur = st[--sp];
    if (tmin[cur] < run_tmin) {
      const OrNode *nd = &m->nodes[leaf[cur]];
      int node_hit = 0;
      if (m->type == OR_GRIDS) {
        /* pbvh_grids_node_nearest_to_ray: quads in (grid, row, column) order;
         * ray_face_nearest_quad tests the second triangle only when the first
         * was taken */
        for (int i = 0; i < nd->totprim; i++) {
          const int g = m->prim_indices[nd->prim_off + i];
          const float *base = m->sf.co + 3 * (size_t)g * area;
          for (int y = 0; y < gs - 1; y++) {
            for (int x = 0; x < gs - 1; x++) {
              const float *c0 = base + 3 * (y * gs + x), *c1 = base + 3 * (y * gs + x + 1);
              const float *c2 = base + 3 * ((y + 1) * gs + x + 1);
              const float *c3 = base + 3 * ((y + 1) * gs + x);
              float dt, d = ray_tri_dist_sq(ray_start, ray_normal, c0, c1, c2, &dt);
              if (d < dsq) {
                dsq = d;
                dep = dt;
                node_hit = 1;
                d = ray_tri_dist_sq(ray_start, ray_normal, c0, c2, c3, &dt);
                if (d < dsq) {
                  dsq = d;
                  dep = dt;
                }
              }
            }
          }
        }
      }
      else {
        /* pbvh_faces_node_nearest_to_ray over the leaf's looptris in prim order */
        for (int i = 0; i < nd->totprim; i++) {
          const int t = m->prim_indices[nd->prim_off + i];
          const int *tv = m->lt_v + 3 * (size_t)t;
          float dt;
          const float d = ray_tri_dist_sq(ray_start, ray_normal, m->sf.co + 3 * (size_t)tv[0],
                                          m->sf.co + 3 * (size_t)tv[1],
                                          m->sf.co + 3 * (size_t)tv[2], &dt);
          if (d < dsq) {
            dsq = d;
            dep = dt;
            node_hit = 1;
          }
        }
      }
      if (node_hit) {
        hit = 1;
        run_tmin = dsq;
      }
    }
    cur = right[cur];
  }
  *depth = dep;
  *dist_sq = dsq;
  free(stack);
  free(leaf);
  free(tmin);
  free(left);
  free(right);
  return hit;
}
