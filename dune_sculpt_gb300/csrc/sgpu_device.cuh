// Device data model and per-element math of libsculptgpu.
//
// All kernels are compiled with -fmad=false, -prec-div=true, -prec-sqrt=true
// and -ftz=false: every multiply and add rounds separately, division and
// square root are correctly rounded, so each per-vertex formula below gives
// the same FP32 bits as the reference's scalar C code evaluated in the same
// order.  The order of every reduction is fixed by the brush specification
// (no atomics on floating-point data).
#pragma once

#include <cuda_runtime.h>

#include <cfloat>
#include <cstdint>

#include "../../include/sculpt_gpu.h"
#include "sgpu_host.h"

namespace sgpu {

// Per-mesh device work area (one per handle).
struct Work {
  int cull_count;
  int err;                 // first error code raised by a kernel, 0 if none
  unsigned int ticket_area;
  unsigned int ticket_update;
  unsigned long long displaced;
  float area_no[3];
  float area_co[3];
  int area_n_co;
  unsigned int grid_epoch;  // last finished GRIDS update (work-list stamps)
};

// Compensated partial of the area reduction: (s, e) pairs for normal xyz and
// centre xyz, and the two counts.
struct AreaPart {
  float s[6];
  float e[6];
  int n_no, n_co;
};

// Device view of one mesh; passed to kernels by value.
struct DevMesh {
  int type;
  int totvert;
  int totnode;
  int nleaf;
  int totlt;
  int grid_size, grid_area;
  int nlevels;
  float4* co;  // FACES: the MVert bytes (xyz + flag/bweight/pad in w); GRIDS: xyz, 0
  float4* no;
  float* mask;      // nullable
  const float* automask;  // nullable
  // FACES topology
  const int4* lt;    // looptri: v0, v1, v2, poly
  const int2* poly;  // loopstart, totloop
  const int* loop_v;
  const int* vt_off;
  const int* vt_idx;
  const int* nb_off;
  const int* nb_idx;
  const int* lt_leaf;  // looptri -> leaf id
  unsigned char* vtag;
  // PBVH
  float4* vb;  // 2 per node: (min xyz, 0), (max xyz, 0)
  float4* orig_vb;
  const int* node_child;   // children_offset or -1
  const int* node_parent;  // -1 for the root
  const int* node_leaf;    // leaf id or -1
  const int* leaf_node;    // leaf id (left-first DFS rank) -> node
  const int* leaf_vert_off;  // FACES: nleaf+1 offsets into leaf_verts
  const int* leaf_uniq;      // FACES: unique vertex count per leaf
  const int* leaf_verts;     // FACES: vert_indices per leaf, leaf-id order
  const int* leaf_prim_off;  // nleaf+1
  const int* leaf_prims;     // prim indices, leaf-id order
  int* leaf_flag;            // PBVHNodeFlags per leaf
  const int* level_off;      // internal nodes by depth, deepest first
  const int* level_nodes;
  // GRIDS topology
  int num_faces, num_base_verts, num_base_edges;
  const int* grid_face;
  const int* face_start;
  const int* face_ngrids;
  const int* face_verts;
  const int* face_edges;
  const int* edge_off;
  const int* edge_elems;
  const int* bvert_off;
  const int* bvert_elems;
  int* face_list;
  int* edge_list;
  int* bvert_list;
  unsigned int* face_mark;
  unsigned int* edge_mark;
  unsigned int* bvert_mark;
  int* grid_counts;  // [0] faces, [1] edges, [2] base verts
  // work
  Work* work;
  int* cull_list;  // nleaf
  int* cull_off;   // nleaf+1: prefix of brush-visible vertex counts over cull_list
  AreaPart* parts;  // nleaf
  float4* scratch;  // smooth Jacobi values, totvert
  unsigned char* node_upd;  // totnode
  // Profiling: algorithmic bytes per kernel kind (nullptr outside profiling).
  unsigned long long* prof;
};

// Kernel kinds for profiling (index into DevMesh::prof and the profile table).
enum KernelKind {
  kKCull = 0,
  kKSetList,
  kKArea,
  kKBrush,
  kKSmoothCompute,
  kKSmoothApply,
  kKUpdate,
  kKGridGather,
  kKGridFaces,
  kKGridSeams,
  kKindCount
};

// Adds per-thread algorithmic bytes to the kernel's counter (warp-aggregated).
// Called by every thread of the block from converged code.
__device__ __forceinline__ void prof_add(const DevMesh& m, int kind, unsigned long long bytes) {
  if (!m.prof) return;
#pragma unroll
  for (int o = 16; o >= 1; o >>= 1) bytes += __shfl_xor_sync(0xffffffffu, bytes, o);
  if ((threadIdx.x & 31) == 0 && bytes) atomicAdd(&m.prof[kind], bytes);
}

// Brush constants of one stroke (kernel parameter).
struct DevBrush {
  int tool;
  int flag;
  float radius;
  float strength;
  float normal_radius_factor;
  float area_radius_factor;
  float plane_offset;
  float x_first, x_last;
  float mintable, range;
  float y[kCurveTable + 1];
};

// One symmetry pass (kernel parameter): mirrored location, grab delta and view
// normal; cull radius; smooth iteration strength.
struct PassParams {
  float loc[3];
  float delta[3];
  float view[3];
  float cull_radius_sq;
  int original;
  float iter_strength;
  int iteration;
};

constexpr int kBrushFrontFace = 1 << 27;
constexpr int kToolDraw = 1, kToolSmooth = 2, kToolInflate = 4, kToolClayStrips = 18;

// ---------------------------------------------------------------------------
// Math (lib/intern/math_vector_inline.c, math_geom.cc, mesh_evaluate.c)

// normalize_v3: zero below 1e-35 (math_vector_inline.c:1165-1185).
__device__ __forceinline__ float normalize3(float& x, float& y, float& z) {
  float d = x * x + y * y + z * z;
  if (d > 1.0e-35f) {
    d = sqrtf(d);
    const float mul = 1.0f / d;
    x = x * mul;
    y = y * mul;
    z = z * mul;
  } else {
    x = y = z = 0.0f;
    d = 0.0f;
  }
  return d;
}

__device__ __forceinline__ float3 normal_tri(float3 a, float3 b, float3 c) {  // math_geom.cc:31-46
  const float n1x = a.x - b.x, n2x = b.x - c.x;
  const float n1y = a.y - b.y, n2y = b.y - c.y;
  const float n1z = a.z - b.z, n2z = b.z - c.z;
  float x = n1y * n2z - n1z * n2y;
  float y = n1z * n2x - n1x * n2z;
  float z = n1x * n2y - n1y * n2x;
  normalize3(x, y, z);
  return make_float3(x, y, z);
}

__device__ __forceinline__ float3 normal_quad(float3 a, float3 b, float3 c,
                                              float3 d) {  // math_geom.cc:48-71
  const float n1x = a.x - c.x, n1y = a.y - c.y, n1z = a.z - c.z;
  const float n2x = b.x - d.x, n2y = b.y - d.y, n2z = b.z - d.z;
  float x = n1y * n2z - n1z * n2y;
  float y = n1z * n2x - n1x * n2z;
  float z = n1x * n2y - n1y * n2x;
  normalize3(x, y, z);
  return make_float3(x, y, z);
}

__device__ __forceinline__ float3 xyz(float4 v) { return make_float3(v.x, v.y, v.z); }

// BKE_mesh_calc_poly_normal, mesh_evaluate.c:62-89 (Newell for n-gons).
__device__ __forceinline__ float3 poly_normal(const DevMesh& m, int p) {
  const int2 pl = m.poly[p];
  const int* lv = m.loop_v + pl.x;
  const int tl = pl.y;
  if (tl == 4) {
    return normal_quad(xyz(m.co[lv[0]]), xyz(m.co[lv[1]]), xyz(m.co[lv[2]]), xyz(m.co[lv[3]]));
  }
  if (tl == 3) {
    return normal_tri(xyz(m.co[lv[0]]), xyz(m.co[lv[1]]), xyz(m.co[lv[2]]));
  }
  if (tl > 4) {
    float3 prev = xyz(m.co[lv[tl - 1]]);
    float x = 0.0f, y = 0.0f, z = 0.0f;
    for (int i = 0; i < tl; i++) {
      const float3 cur = xyz(m.co[lv[i]]);
      x += (prev.y - cur.y) * (prev.z + cur.z);
      y += (prev.z - cur.z) * (prev.x + cur.x);
      z += (prev.x - cur.x) * (prev.y + cur.y);
      prev = cur;
    }
    if (normalize3(x, y, z) == 0.0f) z = 1.0f;
    return make_float3(x, y, z);
  }
  return make_float3(0.0f, 0.0f, 1.0f);
}

// Compensated sum element: value = s + e.  add: TwoSum of (s, x), error into e.
struct CSum {
  float s, e;
};
__device__ __forceinline__ void cs_add(CSum& a, float x) {
  const float s = a.s + x;
  const float bp = s - a.s;
  const float err = (a.s - (s - bp)) + (x - bp);
  a.s = s;
  a.e = a.e + err;
}
__device__ __forceinline__ CSum cs_merge(CSum a, CSum b) {
  const float s = a.s + b.s;
  const float bp = s - a.s;
  const float err = (a.s - (s - bp)) + (b.s - bp);
  CSum r;
  r.s = s;
  r.e = (a.e + b.e) + err;
  return r;
}

// KERNEL_curvemapping_evaluateF with clipping to [0,1] (colortools.c:942-980)
// behind BKE_brush_curve_strength's "dist >= len -> 0" rule.  y is the table's
// y column (shared memory copy).
__device__ __forceinline__ float curve_eval(const DevBrush& b, const float* y, float value) {
  float fi = (value - b.mintable) * b.range;
  const int i = (int)fi;
  float val;
  if (fi < 0.0f || fi > (float)kCurveTable) {
    if (value <= b.x_first) {
      val = y[0];
    } else if (value >= b.x_last) {
      val = y[kCurveTable];
    } else {
      val = 0.0f;
    }
  } else if (i < 0) {
    val = y[0];
  } else if (i >= kCurveTable) {
    val = y[kCurveTable];
  } else {
    fi = fi - (float)i;
    val = (1.0f - fi) * y[i] + (fi)*y[i + 1];
  }
  if (val < 0.0f) {
    val = 0.0f;
  } else if (val > 1.0f) {
    val = 1.0f;
  }
  return val;
}

__device__ __forceinline__ float curve_strength(const DevBrush& b, const float* y, float dist,
                                                float len) {
  if (dist >= len) return 0.0f;
  return curve_eval(b, y, dist / len);
}

// Strength factor of the spec: falloff, front-face, (1 - mask), automask.
__device__ __forceinline__ float strength_factor(const DevMesh& m, const DevBrush& b,
                                                 const float* y, const PassParams& pp, int v,
                                                 float dist, float len) {
  float f = curve_strength(b, y, dist, len);
  if (b.flag & kBrushFrontFace) {
    const float4 n = m.no[v];
    const float dot = pp.view[0] * n.x + pp.view[1] * n.y + pp.view[2] * n.z;
    f = f * (dot > 0.0f ? dot : 0.0f);
  }
  if (m.mask) f = f * (1.0f - m.mask[v]);
  if (m.automask) f = f * m.automask[v];
  return f;
}

// Brush-visible vertices of a leaf: unique vertices (FACES) or all grid
// elements of its grids (GRIDS).
__device__ __forceinline__ int leaf_nverts(const DevMesh& m, int leaf) {
  if (m.type == kFaces) return m.leaf_uniq[leaf];
  return (m.leaf_prim_off[leaf + 1] - m.leaf_prim_off[leaf]) * m.grid_area;
}
__device__ __forceinline__ int leaf_vert(const DevMesh& m, int leaf, int i) {
  if (m.type == kFaces) return m.leaf_verts[m.leaf_vert_off[leaf] + i];
  const int g = m.leaf_prims[m.leaf_prim_off[leaf] + i / m.grid_area];
  return g * m.grid_area + i % m.grid_area;
}
// All vertices of a leaf (PBVH_ITER_ALL) for the bounding-box refit.
__device__ __forceinline__ int leaf_nverts_all(const DevMesh& m, int leaf) {
  if (m.type == kFaces) return m.leaf_vert_off[leaf + 1] - m.leaf_vert_off[leaf];
  return (m.leaf_prim_off[leaf + 1] - m.leaf_prim_off[leaf]) * m.grid_area;
}

__device__ __forceinline__ float dist_sq(float4 co, const float* c) {
  const float d0 = co.x - c[0], d1 = co.y - c[1], d2 = co.z - c[2];
  return d0 * d0 + d1 * d1 + d2 * d2;
}

__device__ __forceinline__ void set_err(const DevMesh& m, int code) {
  atomicCAS(&m.work->err, 0, code);
}

}  // namespace sgpu
