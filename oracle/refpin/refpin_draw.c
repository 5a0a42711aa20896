/*
 * Draw-buffer part of the reference-pinning harness — TEST INFRASTRUCTURE ONLY.
 *
 * Compiles the reference's own draw-buffer code, gpu_buffers.c (GPU_PBVH_Buffers,
 * the mesh and grid buffer build / update) and the vertex-format packing of
 * gpu_vertex_format.cc, over the host-array stand-ins of refpin_gpu.h, and
 * drives it through the reference's BKE_pbvh_draw_cb (pbvh.c:4615-4659) with
 * every node that needs an update (update_only_visible = false), which runs
 * pbvh_update_draw_buffers (pbvh.c:3240-3290).  Written here: the stand-ins
 * (a vertex buffer is a zero-initialised host array; index buffers and batches
 * are dropped), the forwarding of pbvh.c's GPU_pbvh_* calls to the compiled
 * functions, the layers the draw code reads (face sets, colours, the edges for
 * its line index buffer) and the accessors of the result.
 */
#include "refpin_gpu.h"

#include "pbvh_intern.h"

UserDef U;

#include "gpu_vertex_format_ref.c"

#include "gpu_buffers_ref.c"

/* BLI_hash_int_01 (BLI_hash.h, not shipped): BLI_hash_int(k) is
 * BLI_hash_int_2d(k, 0), the lookup3 hash that noise.cc:70-80 defines as
 * hash(kx, ky), scaled by 1 / 0xFFFFFFFF. */
unsigned int refpin_noise_hash2(unsigned int kx, unsigned int ky);
float BLI_hash_int_01(unsigned int k)
{
  return (float)refpin_noise_hash2(k, 0) * (1.0f / (float)0xFFFFFFFF);
}
float rp_hash_int_01(unsigned int k)
{
  return BLI_hash_int_01(k);
}

/* ---- vertex buffers over host memory (the semantics of gpu_vertex_buffer.cc) ---- */
GPUVertBuf *gpu_vertbuf_create_with_format_ex(const GPUVertFormat *format, GPUUsageType usage)
{
  (void)usage;
  GPUVertBuf *v = calloc(1, sizeof(GPUVertBuf));
  v->format = *format;
  if (!v->format.packed) {
    VertexFormat_pack(&v->format);
  }
  return v;
}
void gpu_vertbuf_data_alloc(GPUVertBuf *verts, uint v_len)
{
  free(verts->data);
  verts->data = calloc((size_t)v_len * verts->format.stride + 1, 1);
  verts->vertex_len = v_len;
}
void *gpu_vertbuf_get_data(const GPUVertBuf *verts)
{
  return verts->data;
}
uint gpu_vertbuf_get_vertex_len(const GPUVertBuf *verts)
{
  return verts->vertex_len;
}
void gpu_vertbuf_attr_set(GPUVertBuf *verts, uint a_idx, uint v_idx, const void *data)
{
  const GPUVertAttr *a = &verts->format.attrs[a_idx];
  memcpy(verts->data + a->offset + (size_t)v_idx * verts->format.stride, data, a->sz);
}
void gpu_vertbuf_attr_get_raw_data(GPUVertBuf *verts, uint a_idx, GPUVertBufRaw *access)
{
  const GPUVertAttr *a = &verts->format.attrs[a_idx];
  access->size = a->sz;
  access->stride = verts->format.stride;
  access->data = verts->data + a->offset;
  access->data_init = access->data;
}
void gpu_vertbuf_discard(GPUVertBuf *verts)
{
  free(verts->data);
  free(verts);
}

/* ---- index buffers and batches: dropped ---- */
void gpu_indexbuf_init(GPUIndexBufBuilder *b, GPUPrimType prim, uint prim_len, uint vertex_len)
{
  (void)prim;
  (void)prim_len;
  (void)vertex_len;
  b->len = 0;
}
void gpu_indexbuf_add_tri_verts(GPUIndexBufBuilder *b, uint v1, uint v2, uint v3)
{
  (void)v1;
  (void)v2;
  (void)v3;
  b->len += 3;
}
void gpu_indexbuf_add_line_verts(GPUIndexBufBuilder *b, uint v1, uint v2)
{
  (void)v1;
  (void)v2;
  b->len += 2;
}
GPUIndexBuf *gpu_indexbuf_build(GPUIndexBufBuilder *b)
{
  GPUIndexBuf *e = malloc(sizeof(GPUIndexBuf));
  e->len = b->len;
  return e;
}
void gpu_indexbuf_discard(GPUIndexBuf *e)
{
  free(e);
}
GPUBatch *gpu_batch_create(GPUPrimType prim, GPUVertBuf *vbo, GPUIndexBuf *elem)
{
  (void)vbo;
  (void)elem;
  GPUBatch *b = malloc(sizeof(GPUBatch));
  b->prim = prim;
  return b;
}
void gpu_batch_discard(GPUBatch *b)
{
  free(b);
}

/* ---- pbvh.c's calls (GPU_pbvh_*) to the compiled functions (gpu_pbvh_*) ---- */
void GPU_pbvh_buffers_free(GPU_PBVH_Buffers *buffers)
{
  gpu_pbvh_buffers_free(buffers);
}
GPU_PBVH_Buffers *GPU_pbvh_mesh_buffers_build(const MPoly *mpoly, const MLoop *mloop,
                                              const MLoopTri *looptri, const MVert *verts,
                                              const int *face_indices,
                                              const int *sculpt_face_sets, int face_indices_len,
                                              const struct Mesh *mesh)
{
  return gpu_pbvh_mesh_buffers_build(mpoly, mloop, looptri, verts, face_indices, sculpt_face_sets,
                                     face_indices_len, mesh);
}
GPU_PBVH_Buffers *GPU_pbvh_grid_buffers_build(int totgrid, BLI_bitmap **grid_hidden)
{
  return gpu_pbvh_grid_buffers_build(totgrid, grid_hidden);
}
void GPU_pbvh_mesh_buffers_update(GPU_PBVH_Buffers *buffers, const MVert *mvert,
                                  const float (*vert_normals)[3], const float *vmask,
                                  const MLoopCol *vcol, const int *sculpt_face_sets,
                                  int face_sets_color_seed, int face_sets_color_default,
                                  const MPropCol *vtcol, int update_flags)
{
  gpu_pbvh_mesh_buffers_update(buffers, mvert, vert_normals, vmask, vcol, sculpt_face_sets,
                               face_sets_color_seed, face_sets_color_default, vtcol, update_flags);
}
void GPU_pbvh_grid_buffers_update(GPU_PBVH_Buffers *buffers, struct SubdivCCG *subdiv_ccg,
                                  CCGElem **grids, const DMFlagMat *grid_flag_mats,
                                  int *grid_indices, int totgrid, const int *sculpt_face_sets,
                                  int face_sets_color_seed, int face_sets_color_default,
                                  const CCGKey *key, int update_flags)
{
  gpu_pbvh_grid_buffers_update(buffers, subdiv_ccg, grids, grid_flag_mats, grid_indices, totgrid,
                               sculpt_face_sets, face_sets_color_seed, face_sets_color_default, key,
                               update_flags);
}
void GPU_pbvh_grid_buffers_update_free(GPU_PBVH_Buffers *buffers, const DMFlagMat *grid_flag_mats,
                                       const int *grid_indices)
{
  gpu_pbvh_grid_buffers_update_free(buffers, grid_flag_mats, grid_indices);
}
void GPU_pbvh_buffers_update_flush(GPU_PBVH_Buffers *buffers)
{
  (void)buffers; /* the upload to the GL buffer object: nothing here */
}

/* ---- the layers the draw code reads ---- */
typedef struct RefDraw {
  CustomData vdata, ldata, pdata;
  CustomDataLayer vlayers[2], llayer, player;
  MLoop *loops;  /* the mesh's loops with loop i using edge i */
  MEdge *edges;  /* edge i: loop i's vertex to the next loop's vertex of its poly */
  int *face_sets;
} RefDraw;

static RefDraw g_draw_faces[64];
static int g_draw_faces_n;

static void draw_init_once(void)
{
  static int done = 0;
  if (!done) {
    gpu_pbvh_init();
    lib_init_srgb_conversion();
    done = 1;
  }
}

/* FACES: sculpt face sets (per poly, CD_SCULPT_FACE_SETS), loop colours
 * (CD_MLOOPCOL, 4 bytes per loop), vertex colours (CD_PROP_COLOR, 4 floats per
 * vertex) and the user preference for the latter; all nullable.  The arrays
 * are referenced, not copied. */
void rp_draw_setup_faces(PBVH *pbvh, int totpoly, const int *poly_loopstart,
                         const int *poly_totloop, int totloop, int *face_sets,
                         const unsigned char *loop_colors, const float *vert_colors,
                         int use_vert_colors, int seed, int color_default)
{
  draw_init_once();
  RefDraw *d = &g_draw_faces[g_draw_faces_n++ % 64];
  memset(d, 0, sizeof(*d));
  d->loops = malloc(sizeof(MLoop) * (size_t)totloop);
  d->edges = calloc((size_t)totloop, sizeof(MEdge));
  for (int p = 0; p < totpoly; p++) {
    const int ls = poly_loopstart[p], tl = poly_totloop[p];
    for (int i = 0; i < tl; i++) {
      const int l = ls + i, ln = ls + (i + 1) % tl;
      d->loops[l].v = pbvh->mloop[l].v;
      d->loops[l].e = (unsigned int)l;
      d->edges[l].v1 = pbvh->mloop[l].v;
      d->edges[l].v2 = pbvh->mloop[ln].v;
    }
  }
  Mesh *me = (Mesh *)pbvh->mesh;
  me->mloop = d->loops;
  me->medge = d->edges;
  int nv = 0;
  const CustomData *old = pbvh->vdata;
  for (int i = 0; old && i < old->totlayer && nv < 1; i++) {
    d->vlayers[nv++] = old->layers[i];
  }
  if (vert_colors) {
    d->vlayers[nv].type = CD_PROP_COLOR;
    d->vlayers[nv++].data = (void *)vert_colors;
  }
  d->vdata.layers = d->vlayers;
  d->vdata.totlayer = nv;
  pbvh->vdata = &d->vdata;
  if (loop_colors) {
    d->llayer.type = CD_MLOOPCOL;
    d->llayer.data = (void *)loop_colors;
    d->ldata.layers = &d->llayer;
    d->ldata.totlayer = 1;
  }
  pbvh->ldata = &d->ldata;
  if (face_sets) {
    d->player.type = CD_SCULPT_FACE_SETS;
    d->player.data = face_sets;
    d->pdata.layers = &d->player;
    d->pdata.totlayer = 1;
  }
  pbvh->pdata = &d->pdata;
  pbvh->face_sets_color_seed = seed;
  pbvh->face_sets_color_default = color_default;
  U.experimental.use_sculpt_vertex_colors = (char)(use_vert_colors != 0);
}

/* GRIDS: face sets per base face (pbvh->face_sets) and the DMFlagMat records
 * of the grids (copied into the CCG's grid_flag_mats, which the PBVH reads). */
void rp_draw_setup_grids(PBVH *pbvh, int *face_sets, const unsigned char *flag_mats, int seed,
                         int color_default)
{
  draw_init_once();
  pbvh->face_sets = face_sets;
  if (flag_mats) {
    for (int g = 0; g < pbvh->totgrid; g++) {
      memcpy(&((DMFlagMat *)pbvh->grid_flag_mats)[g].mat_nr, flag_mats + 4 * (size_t)g, 2);
      ((DMFlagMat *)pbvh->grid_flag_mats)[g].flag = (char)flag_mats[4 * (size_t)g + 2];
    }
  }
  pbvh->face_sets_color_seed = seed;
  pbvh->face_sets_color_default = color_default;
}

static void draw_nothing(void *user_data, GPU_PBVH_Buffers *buffers)
{
  (void)user_data;
  (void)buffers;
}

/* BKE_pbvh_draw_cb with every node that needs an update. */
void rp_draw(PBVH *pbvh)
{
  draw_init_once();
  BKE_pbvh_draw_cb(pbvh, false, NULL, NULL, draw_nothing, NULL);
}

/* Per node: vertex count of its buffer (-1 without buffers), tot_tri, smooth,
 * material_index, show_overlay. */
void rp_draw_node_info(const PBVH *pbvh, int node, int *out5)
{
  const GPU_PBVH_Buffers *b = pbvh->nodes[node].draw_buffers;
  if (!b) {
    out5[0] = -1;
    out5[1] = out5[2] = out5[3] = out5[4] = 0;
    return;
  }
  out5[0] = b->vert_buf ? (int)b->vert_buf->vertex_len : 0;
  out5[1] = (int)b->tot_tri;
  out5[2] = b->smooth;
  out5[3] = b->material_index;
  out5[4] = b->show_overlay;
}
/* The format as a vertex buffer packs it (its copy of g_vbo_id.format). */
static GPUVertFormat packed_format(void)
{
  draw_init_once();
  GPUVertFormat f = g_vbo_id.format;
  if (!f.packed) {
    VertexFormat_pack(&f);
  }
  return f;
}
int rp_draw_stride(void)
{
  return (int)packed_format().stride;
}
/* The node's vertex-buffer bytes (vertex count * stride). */
void rp_draw_node_bytes(const PBVH *pbvh, int node, unsigned char *dst)
{
  const GPU_PBVH_Buffers *b = pbvh->nodes[node].draw_buffers;
  if (b && b->vert_buf && b->vert_buf->data) {
    memcpy(dst, b->vert_buf->data, (size_t)b->vert_buf->vertex_len * b->vert_buf->format.stride);
  }
}
/* The packed format: per attribute (pos, nor, msk, ac, fset) offset and size. */
void rp_draw_format(int *offsets, int *sizes)
{
  const GPUVertFormat f = packed_format();
  for (uint i = 0; i < f.attr_len; i++) {
    offsets[i] = (int)f.attrs[i].offset;
    sizes[i] = (int)f.attrs[i].sz;
  }
}
void rp_face_set_color(int face_set, int seed, unsigned char rgb[3])
{
  uchar c[4];
  BKE_paint_face_set_overlay_color_get(face_set, seed, c);
  memcpy(rgb, c, 3);
}
