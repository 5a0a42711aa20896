/*
 * Stand-ins for the GPU-module interfaces the reference's draw-buffer code
 * (gpu_buffers.c:36-739) calls, so that it compiles and runs without a
 * graphics stack (TEST INFRASTRUCTURE ONLY).  A vertex buffer is a plain
 * host array in the packed format the reference's VertexFormat_pack computes;
 * index buffers and batches are counted and dropped (they are not compared).
 *
 * The reference's sources call several functions under names that differ
 * from their definitions (GPU_ / gpu_ / dune_ / gou_ / gpy_ prefixes of one
 * renaming pass); the macros below map each call to the one function.
 */
#ifndef REFPIN_GPU_H
#define REFPIN_GPU_H

#include <limits.h>

#include "refpin_prelude.h"

/* ---- gpu_vertex_format.h: the vertex format types (same fields) ---- */
#define GPU_VERT_ATTR_MAX_LEN 16
#define GPU_VERT_ATTR_MAX_NAMES 6
#define GPU_VERT_ATTR_NAMES_BUF_LEN 256
#define GPU_VERT_FORMAT_MAX_NAMES 63
#define TRUST_NO_ONE 0

typedef enum {
  GPU_COMP_I8 = 0,
  GPU_COMP_U8,
  GPU_COMP_I16,
  GPU_COMP_U16,
  GPU_COMP_I32,
  GPU_COMP_U32,
  GPU_COMP_F32,
  GPU_COMP_I10,
} GPUVertCompType;

typedef enum {
  GPU_FETCH_FLOAT = 0,
  GPU_FETCH_INT,
  GPU_FETCH_INT_TO_FLOAT_UNIT,
  GPU_FETCH_INT_TO_FLOAT,
} GPUVertFetchMode;

typedef struct GPUVertAttr {
  uint fetch_mode : 2;
  uint comp_type : 3;
  uint comp_len : 5;
  uint sz : 7;
  uint offset : 11;
  uint name_len : 3;
  uchar names[GPU_VERT_ATTR_MAX_NAMES];
} GPUVertAttr;

typedef struct GPUVertFormat {
  uint attr_len : 5;
  uint name_len : 6;
  uint stride : 11;
  uint packed : 1;
  uint name_offset : 8;
  uint deinterleaved : 1;
  GPUVertAttr attrs[GPU_VERT_ATTR_MAX_LEN];
  char names[GPU_VERT_ATTR_NAMES_BUF_LEN];
} GPUVertFormat;

uint gpu_vertformat_attr_add(GPUVertFormat *, const char *name, GPUVertCompType, uint comp_len,
                             GPUVertFetchMode);
void VertexFormat_pack(GPUVertFormat *format);
uint padding(uint offset, uint alignment);
#define GPU_vertformat_attr_add gpu_vertformat_attr_add

/* ---- vertex buffers: a host array ---- */
typedef enum { GPU_USAGE_STREAM, GPU_USAGE_STATIC, GPU_USAGE_DYNAMIC } GPUUsageType;
typedef struct GPUVertBuf {
  GPUVertFormat format;
  uchar *data;
  uint vertex_len;
} GPUVertBuf;
typedef struct GPUVertBufRaw {
  uint size;
  uint stride;
  unsigned char *data;
  unsigned char *data_init;
} GPUVertBufRaw;

GPUVertBuf *gpu_vertbuf_create_with_format_ex(const GPUVertFormat *format, GPUUsageType usage);
void gpu_vertbuf_data_alloc(GPUVertBuf *verts, uint v_len);
void *gpu_vertbuf_get_data(const GPUVertBuf *verts);
uint gpu_vertbuf_get_vertex_len(const GPUVertBuf *verts);
void gpu_vertbuf_attr_set(GPUVertBuf *verts, uint a_idx, uint v_idx, const void *data);
void gpu_vertbuf_attr_get_raw_data(GPUVertBuf *verts, uint a_idx, GPUVertBufRaw *access);
static inline void *gpu_vertbuf_raw_step(GPUVertBufRaw *a)
{
  unsigned char *data = a->data;
  a->data += a->stride;
  return (void *)data;
}
void gpu_vertbuf_discard(GPUVertBuf *verts);
#define GPU_vertbuf_raw_step gpu_vertbuf_raw_step
#define gou_vertbuf_attr_set gpu_vertbuf_attr_set
#define GPU_VERTBUF_DISCARD_SAFE(v) \
  do { \
    if (v) { \
      gpu_vertbuf_discard(v); \
      (v) = NULL; \
    } \
  } while (0)

/* ---- index buffers and batches: counted, not kept ---- */
typedef enum { GPU_PRIM_POINTS, GPU_PRIM_LINES, GPU_PRIM_TRIS } GPUPrimType;
typedef struct GPUIndexBuf {
  uint len;
} GPUIndexBuf;
typedef struct GPUIndexBufBuilder {
  uint len;
} GPUIndexBufBuilder;
typedef struct GPUBatch {
  int prim;
} GPUBatch;
void gpu_indexbuf_init(GPUIndexBufBuilder *b, GPUPrimType prim, uint prim_len, uint vertex_len);
void gpu_indexbuf_add_tri_verts(GPUIndexBufBuilder *b, uint v1, uint v2, uint v3);
void gpu_indexbuf_add_line_verts(GPUIndexBufBuilder *b, uint v1, uint v2);
GPUIndexBuf *gpu_indexbuf_build(GPUIndexBufBuilder *b);
void gpu_indexbuf_discard(GPUIndexBuf *e);
GPUBatch *gpu_batch_create(GPUPrimType prim, GPUVertBuf *vbo, GPUIndexBuf *elem);
void gpu_batch_discard(GPUBatch *b);
#define dune_indexbuf_init gpu_indexbuf_init
#define GPU_BATCH_DISCARD_SAFE(b) \
  do { \
    if (b) { \
      gpu_batch_discard(b); \
      (b) = NULL; \
    } \
  } while (0)
#define GPU_INDEXBUF_DISCARD_SAFE(e) \
  do { \
    if (e) { \
      gpu_indexbuf_discard(e); \
      (e) = NULL; \
    } \
  } while (0)

/* ---- the rest of the interface gpu_buffers.c reaches ---- */
typedef struct UserDefExperimental {
  char use_sculpt_vertex_colors;
} UserDefExperimental;
typedef struct UserDef {
  UserDefExperimental experimental;
} UserDef;
extern UserDef U;

#define SCULPT_FACE_SET_NONE 0 /* the sculpt header that defines it is absent */
#define lib_bitmap BLI_bitmap
#define mem_callocn MEM_callocN
#define mem_freen MEM_freeN
#define dune_mesh_calc_poly_normal BKE_mesh_calc_poly_normal
#define dune_pbvh_count_grid_quads BKE_pbvh_count_grid_quads
#define dune_subdiv_ccg_grid_to_face_index KERNEL_subdiv_ccg_grid_to_face_index
#define dune_paint_face_set_overlay_color_get BKE_paint_face_set_overlay_color_get
#define dune_mesh_looptri_get_real_edges DUNE_mesh_looptri_get_real_edges
#define BLI_color_from_srgb_table lib_color_from_srgb_table

extern float lib_color_from_srgb_table[256];
void lib_init_srgb_conversion(void);
void hsv_to_rgb(float h, float s, float v, float *r_r, float *r_g, float *r_b);
void rgba_float_to_uchar(uchar r_col[4], const float col_f[4]);
float BLI_hash_int_01(unsigned int k);
void BKE_paint_face_set_overlay_color_get(const int face_set, const int seed, uchar r_color[4]);
int BKE_pbvh_count_grid_quads(BLI_bitmap **grid_hidden, const int *grid_indices, int totgrid,
                              int gridsize);
int KERNEL_subdiv_ccg_grid_to_face_index(const SubdivCCG *subdiv_ccg, const int grid_index);
void DUNE_mesh_looptri_get_real_edges(const Mesh *mesh, const MLoopTri *looptri, int r_edges[3]);

#endif
