/*
 * CPU oracle, headless draw buffers.  TEST INFRASTRUCTURE ONLY (see oracle.h):
 * the checker of the GPU draw-buffer fill, never part of the product.
 *
 * Restates, per leaf flagged for a draw update and in node order,
 *   pbvh_update_draw_buffers / pbvh_update_draw_buffer_cb   pbvh.c:3169-3290
 *   GPU_pbvh_mesh_buffers_build (visible looptris)          gpu_buffers.c:307-400
 *   GPU_pbvh_mesh_buffers_update (the vertex fill)          gpu_buffers.c:174-305
 *   GPU_pbvh_grid_buffers_update (the vertex fill)          gpu_buffers.c:548-725
 *   gpu_pbvh_is_looptri_visible, paint_is_face_hidden       gpu_buffers.c:166-172, paint.c:1227-1232
 *   BKE_paint_face_set_overlay_color_get, hsv_to_rgb        paint.c:2219-2236, math_color.c:6-21
 *   BLI_color_from_srgb_table, srgb_to_linearrgb           math_color.c:393-400, 577-581
 *   unit_float_to_uchar/ushort_clamp, normal_float_to_short_v3
 *                                                          math_base_inline.c:678-690,
 *                                                          math_vector_inline.c:1260-1265
 * with the update flags pbvh_get_buffers_update_flags always passes (mask,
 * vertex colours, face sets; pbvh.c:3162-3167), into the vertex format
 * "pos" f32x3 @0, "nor" i16x3 @16, "msk" u8 @22, "ac" u16x4 @24, "fset" u8x3
 * @32, stride 36 (VertexFormat_pack, gpu_vertex_format.cc:300-330).
 * BLI_hash_int_01 comes from BLI_hash.h, which the reference does not ship:
 * its published function is Bob Jenkins' lookup3 final() mix of (k, 0) with
 * the initial value 0xdeadbeef + (2 << 2) + 13 (noise.cc:70-80 holds the same
 * two-argument hash), scaled by 1 / 0xFFFFFFFF.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "oracle_internal.h"

#define OR_RebuildDrawBuffers (1 << 9)
#define ME_SMOOTH 1
#define ME_HIDE 16
#define STRIDE 36

static unsigned int rot32(unsigned int x, int k)
{
  return (x << k) | (x >> (32 - k));
}

static unsigned int hash_int(unsigned int k)
{
  unsigned int a, b, c;
  a = b = c = 0xdeadbeefu + (2u << 2) + 13u;
  a += k;
  c ^= b;
  c -= rot32(b, 14);
  a ^= c;
  a -= rot32(c, 11);
  b ^= a;
  b -= rot32(a, 25);
  c ^= b;
  c -= rot32(b, 16);
  a ^= c;
  a -= rot32(c, 4);
  b ^= a;
  b -= rot32(a, 14);
  c ^= b;
  c -= rot32(b, 24);
  return c;
}

static float hash_int_01(unsigned int k)
{
  return (float)hash_int(k) * (1.0f / (float)0xFFFFFFFFu);
}

static float clampf01(float x)
{
  if (x < 0.0f) {
    return 0.0f;
  }
  if (x > 1.0f) {
    return 1.0f;
  }
  return x;
}

static unsigned char to_uchar_clamp(float v)
{
  return (unsigned char)((v <= 0.0f) ? 0 : ((v > (1.0f - 0.5f / 255.0f)) ? 255 : ((255.0f * v) + 0.5f)));
}

static unsigned short to_ushort_clamp(float v)
{
  return (unsigned short)((v >= 1.0f - 0.5f / 65535) ? 65535 :
                          (v <= 0.0f)               ? 0 :
                                                      (v * 65535.0f + 0.5f));
}

void or_face_set_color(int face_set, int seed, unsigned char rgb[3])
{
  float hue = 0.618033988749895f * (abs(face_set) + (seed % 10));
  hue = hue - floorf(hue);
  const float sat = hash_int_01((unsigned int)(abs(face_set) + seed + 1));
  const float val = hash_int_01((unsigned int)(abs(face_set) + seed + 2));
  const float s = 0.6f + (sat * 0.25f), v = 1.0f - (val * 0.35f);
  const float nr = clampf01(fabsf(hue * 6.0f - 3.0f) - 1.0f);
  const float ng = clampf01(2.0f - fabsf(hue * 6.0f - 2.0f));
  const float nb = clampf01(2.0f - fabsf(hue * 6.0f - 4.0f));
  rgb[0] = to_uchar_clamp(((nr - 1.0f) * s + 1.0f) * v);
  rgb[1] = to_uchar_clamp(((ng - 1.0f) * s + 1.0f) * v);
  rgb[2] = to_uchar_clamp(((nb - 1.0f) * s + 1.0f) * v);
}

static float srgb_to_linear(float c)
{
  if (c < 0.04045f) {
    return (c < 0.0f) ? 0.0f : c * (1.0f / 12.92f);
  }
  return powf((c + 0.055f) * (1.0f / 1.055f), 2.4f);
}

static void put_short3(unsigned char *p, const float n[3])
{
  for (int k = 0; k < 3; k++) {
    const short s = (short)(n[k] * 32767.0f);
    memcpy(p + 2 * k, &s, 2);
  }
}

static int looptri_visible(const OrMesh *m, const OrDrawSetup *s, int lt)
{
  int hidden = 0;
  if (s->vert_flag) {
    for (int j = 0; j < 3; j++) {
      hidden = hidden || (s->vert_flag[m->lt_v[3 * lt + j]] & ME_HIDE);
    }
  }
  return !hidden && s->face_sets && s->face_sets[m->lt_poly[lt]] > 0;
}

static int leaf_smooth(const OrMesh *m, const OrDrawSetup *s, const OrNode *nd)
{
  if (nd->totprim <= 0) {
    return 0;
  }
  const int first = m->prim_indices[nd->prim_off];
  if (m->type == OR_FACES) {
    return (m->poly_flag[m->lt_poly[first]] & ME_SMOOTH) != 0;
  }
  return s->grid_flag_mats ? (s->grid_flag_mats[4 * (size_t)first + 2] & ME_SMOOTH) != 0 : 1;
}

int64_t or_draw_build(OrMesh *m, const OrDrawSetup *s, int64_t *vert_off, int *tot_tri,
                      int *smooth, int *material)
{
  int64_t off = 0;
  const int gs = m->grid_size;
  for (int n = 0; n < m->totnode; n++) {
    OrNode *nd = &m->nodes[n];
    if (vert_off) {
      vert_off[n] = off;
    }
    int tt = 0, sm = 0, mat = 0;
    if (nd->flag & OR_Leaf) {
      sm = leaf_smooth(m, s, nd);
      if (m->type == OR_FACES) {
        for (int i = 0; i < nd->totprim; i++) {
          tt += looptri_visible(m, s, m->prim_indices[nd->prim_off + i]);
        }
        if (nd->totprim > 0) {
          mat = m->poly_mat[m->lt_poly[m->prim_indices[nd->prim_off]]];
        }
        off += 3 * (int64_t)tt;
      }
      else {
        /* tot_tri stays 0: the grid buffers never set it */
        if (nd->totprim > 0 && s->grid_flag_mats) {
          short mn;
          memcpy(&mn, s->grid_flag_mats + 4 * (size_t)m->prim_indices[nd->prim_off], 2);
          mat = mn;
        }
        off += (int64_t)nd->totprim * (sm ? gs * gs : (gs - 1) * (gs - 1) * 4);
      }
      nd->flag |= OR_RebuildDrawBuffers | OR_UpdateDrawBuffers;
    }
    if (tot_tri) {
      tot_tri[n] = tt;
    }
    if (smooth) {
      smooth[n] = sm;
    }
    if (material) {
      material[n] = mat;
    }
  }
  if (vert_off) {
    vert_off[m->totnode] = off;
  }
  return off;
}

/* GPU_pbvh_mesh_buffers_update for one leaf; returns show_overlay. */
static int fill_faces(const OrMesh *m, const OrDrawSetup *s, const OrNode *nd, unsigned char *p)
{
  const float *co = m->sf.co, *vno = m->sf.no, *vmask = m->sf.mask;
  const int show_mask = vmask != NULL;
  const int show_face_sets = s->face_sets != NULL;
  const int use_vtcol = s->vert_colors && s->use_sculpt_vertex_colors;
  const int show_vcol = s->loop_colors || use_vtcol;
  const int smooth = leaf_smooth(m, s, nd);
  int empty_mask = 1, default_face_set = 1;
  int poly_prev = -1;
  float fno[3] = {0.0f, 0.0f, 0.0f};
  for (int i = 0; i < nd->totprim; i++) {
    const int lt = m->prim_indices[nd->prim_off + i];
    if (!looptri_visible(m, s, lt)) {
      continue;
    }
    const int poly = m->lt_poly[lt];
    const int *vtri = m->lt_v + 3 * lt;
    if (poly != poly_prev && !smooth) {
      or_poly_normal_fp32(m, poly, fno);
      poly_prev = poly;
    }
    unsigned char fset[3] = {255, 255, 255};
    if (show_face_sets) {
      const int fs = abs(s->face_sets[poly]);
      if (fs != s->face_sets_color_default) {
        or_face_set_color(fs, s->face_sets_color_seed, fset);
        default_face_set = 0;
      }
    }
    unsigned char cmask = 0;
    if (show_mask && !smooth) {
      const float fmask = (vmask[vtri[0]] + vmask[vtri[1]] + vmask[vtri[2]]) / 3.0f;
      cmask = (unsigned char)(fmask * 255);
    }
    for (int j = 0; j < 3; j++, p += STRIDE) {
      const int v = vtri[j];
      memcpy(p, co + 3 * (size_t)v, 12);
      put_short3(p + 16, smooth ? vno + 3 * (size_t)v : fno);
      if (show_mask && smooth) {
        cmask = (unsigned char)(vmask[v] * 255);
      }
      p[22] = cmask;
      empty_mask = empty_mask && (cmask == 0);
      if (show_vcol) {
        unsigned short sc[4];
        if (use_vtcol) {
          for (int k = 0; k < 4; k++) {
            sc[k] = to_ushort_clamp(s->vert_colors[4 * (size_t)v + k]);
          }
        }
        else {
          const unsigned char *mc = s->loop_colors + 4 * (size_t)s->lt_loops[3 * lt + j];
          for (int k = 0; k < 3; k++) {
            sc[k] = to_ushort_clamp(srgb_to_linear((float)mc[k] * (1.0f / 255.0f)));
          }
          sc[3] = to_ushort_clamp(mc[3] * (1.0f / 255.0f));
        }
        memcpy(p + 24, sc, 8);
      }
      memcpy(p + 32, fset, 3);
    }
  }
  return !empty_mask || !default_face_set;
}

/* GPU_pbvh_grid_buffers_update for one leaf; returns show_overlay. */
static int fill_grids(const OrMesh *m, const OrDrawSetup *s, const OrNode *nd, unsigned char *p)
{
  const int gs = m->grid_size, area = m->grid_area;
  const float *co = m->sf.co, *no = m->sf.no, *mask = m->sf.mask;
  const int has_mask = mask != NULL;
  const int smooth = leaf_smooth(m, s, nd);
  int empty_mask = 1, default_face_set = 1;
  const unsigned short white[4] = {65535, 65535, 65535, 65535};
  for (int i = 0; i < nd->totprim; i++) {
    const int grid = m->prim_indices[nd->prim_off + i];
    const size_t g0 = (size_t)grid * area;
    unsigned char fset[3] = {255, 255, 255};
    if (s->face_sets) {
      const int fs = abs(s->face_sets[m->grid_face[grid]]);
      if (fs != s->face_sets_color_default) {
        or_face_set_color(fs, s->face_sets_color_seed, fset);
        default_face_set = 0;
      }
    }
    if (smooth) {
      for (int y = 0; y < gs; y++) {
        for (int x = 0; x < gs; x++, p += STRIDE) {
          const size_t e = g0 + (size_t)(y * gs + x);
          memcpy(p, co + 3 * e, 12);
          put_short3(p + 16, no + 3 * e);
          if (has_mask) {
            const unsigned char cmask = (unsigned char)(mask[e] * 255);
            p[22] = cmask;
            empty_mask = empty_mask && (cmask == 0);
          }
          memcpy(p + 24, white, 8);
          memcpy(p + 32, fset, 3);
        }
      }
    }
    else {
      for (int y = 0; y < gs - 1; y++) {
        for (int x = 0; x < gs - 1; x++) {
          const size_t e[4] = {g0 + (size_t)(y * gs + x), g0 + (size_t)(y * gs + x + 1),
                               g0 + (size_t)((y + 1) * gs + x + 1), g0 + (size_t)((y + 1) * gs + x)};
          float fno[3];
          or_normal_quad_fp32(fno, co + 3 * e[3], co + 3 * e[2], co + 3 * e[1], co + 3 * e[0]);
          unsigned char cmask = 0;
          if (has_mask) {
            const float fmask = (mask[e[0]] + mask[e[1]] + mask[e[2]] + mask[e[3]]) * 0.25f;
            cmask = (unsigned char)(fmask * 255);
            empty_mask = empty_mask && (cmask == 0);
          }
          for (int k = 0; k < 4; k++, p += STRIDE) {
            memcpy(p, co + 3 * e[k], 12);
            put_short3(p + 16, fno);
            if (has_mask) {
              p[22] = cmask;
            }
            memcpy(p + 24, white, 8);
            memcpy(p + 32, fset, 3);
          }
        }
      }
    }
  }
  return !empty_mask || !default_face_set;
}

void or_draw_update(OrMesh *m, const OrDrawSetup *s, const int64_t *vert_off, unsigned char *vbo,
                    int *overlay)
{
  for (int n = 0; n < m->totnode; n++) {
    OrNode *nd = &m->nodes[n];
    if (!(nd->flag & OR_Leaf) || !(nd->flag & (OR_RebuildDrawBuffers | OR_UpdateDrawBuffers))) {
      continue;
    }
    if (nd->flag & OR_UpdateDrawBuffers) {
      unsigned char *p = vbo + (size_t)vert_off[n] * STRIDE;
      const int ov = m->type == OR_FACES ? fill_faces(m, s, nd, p) : fill_grids(m, s, nd, p);
      if (overlay) {
        overlay[n] = ov;
      }
    }
    nd->flag &= ~(OR_RebuildDrawBuffers | OR_UpdateDrawBuffers);
  }
}
