/*
 * Internal layout of the CPU oracle (test infrastructure; see oracle.h).
 * One topology + PBVH (built once, in FP32, exactly as the reference builds it)
 * and two numeric states: FP32 (bit-exact parity target) and FP64 (error
 * reference).
 */
#ifndef ORACLE_INTERNAL_H
#define ORACLE_INTERNAL_H

#include <stdint.h>
#include "oracle.h"

/* PBVHNodeFlags values (the enum lives in the reference's absent BKE_pbvh.h;
 * these are the values its pbvh.c call sites rely on). */
#define OR_Leaf 1
#define OR_UpdateNormals 2
#define OR_UpdateBB 4
#define OR_UpdateOriginalBB 8
#define OR_UpdateDrawBuffers 16
#define OR_UpdateRedraw 32

#define OR_FACES 0
#define OR_GRIDS 1

#define OR_TOOL_DRAW 1
#define OR_TOOL_SMOOTH 2
#define OR_TOOL_INFLATE 4
#define OR_TOOL_CLAY_STRIPS 18
#define OR_TOOL_PINCH 3
#define OR_TOOL_CREASE 16
#define OR_TOOL_GRAB 5
#define OR_TOOL_LAYER 6
#define OR_TOOL_ELASTIC_DEFORM 21
/* eBrushElasticDeformType (types_brush_enums.h:195-199) */
#define OR_ELASTIC_GRAB 0
#define OR_ELASTIC_GRAB_BISCALE 1
#define OR_ELASTIC_GRAB_TRISCALE 2
#define OR_ELASTIC_SCALE 3
#define OR_ELASTIC_TWIST 4
#define OR_BRUSH_FRONTFACE (1 << 27)

#define OR_CM_TABLE 256
#define OR_CM_RESOL 32

typedef struct OrNode {
  int children_offset; /* internal: index of the left child; the right one follows */
  int flag;
  int prim_off, totprim; /* range in prim_indices (leaves) */
  int uniq, face_verts;  /* FACES leaves: unique / shared vertex counts */
  int vert_off;          /* FACES leaves: offset in vert_indices */
} OrNode;

typedef struct OrCurve {
  float table[(OR_CM_TABLE + 1) * 2];
  float mintable, maxtable, range;
  float ext_in[2], ext_out[2];
  int flag; /* CUMA_DO_CLIP only: horizontal extension */
} OrCurve;

typedef struct OrStateF {
  float *co, *no, *mask;     /* 3V, 3V, V (mask may be NULL) */
  float *vb, *orig_vb;       /* 6N */
  float *orig_co, *orig_no;  /* 3V each: positions / normals at the stroke start */
  float *layer_disp;         /* V: the layer brush's per-vertex layer height */
} OrStateF;

typedef struct OrStateD {
  double *co, *no, *mask;
  double *vb, *orig_vb;
  double *orig_co, *orig_no;
  double *layer_disp;
} OrStateD;

struct OrMesh {
  int type;
  int totvert; /* FACES: vertices; GRIDS: grid elements */
  /* FACES topology */
  int totpoly, totloop, totlt;
  int *poly_loopstart, *poly_totloop;
  short *poly_mat;
  char *poly_flag;
  int *loop_v;
  int *lt_v;    /* 3 per looptri, vertex indices */
  int *lt_poly; /* per looptri */
  int *vt_off, *vt_idx; /* vertex -> looptri, ascending looptri index */
  int *nb_off, *nb_idx; /* vertex -> one-ring neighbours */
  int *lt_leaf;         /* looptri -> node index of its leaf */
  unsigned char *vtag;  /* vert_bitmap */
  float *automask;      /* V or NULL */
  /* GRIDS topology */
  int num_grids, grid_size, grid_area;
  int num_faces;
  int *face_start, *face_ngrids, *face_verts, *face_edges;
  int num_base_verts, num_base_edges;
  int *grid_face;                /* grid -> base face */
  int *edge_off, *edge_elems;    /* per base edge: nfaces * 2*grid_size element indices */
  int *bvert_off, *bvert_elems;  /* per base vertex: one corner element per adjacent face */
  /* PBVH */
  int leaf_limit;
  int totnode, node_cap;
  OrNode *nodes;
  int *prim_indices;
  int totprim;
  int *vert_indices;
  int vert_entries;
  int nleaf;
  int *leaf_nodes; /* DFS order */
  /* states */
  OrStateF sf;
  OrStateD sd;
};

void or_poly_normal_fp32(const OrMesh *m, int p, float r[3]);
void or_normal_quad_fp32(float n[3], const float *v1, const float *v2, const float *v3,
                         const float *v4);

#endif
