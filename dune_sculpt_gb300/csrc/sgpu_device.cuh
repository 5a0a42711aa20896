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
  // persistent stroke kernel: smooth hit-list counts (3-way rotation), tagged
  // vertices and touched leaves per dab (2-way by dab parity)
  int hit_count[3];
  int tag_count[2];
  int touch_count[2];
};

// Compensated partial of the area reduction: (s, e) pairs for normal xyz and
// centre xyz, and the two counts.
struct AreaPart {
  float s[6];
  float e[6];
  int n_no, n_co;
};

// Division by a divisor fixed per mesh (Granlund and Montgomery, "Division
// by invariant integers using multiplication", PLDI 1994): with
// s = 31 + ceil(log2 d) and mul = ceil(2^s / d) (below 2^32), n * mul >> s
// equals n / d for every 0 <= n < 2^31, since mul * d - 2^s < d <= 2^(s - 31)
// keeps the error term below 1 / d.
__host__ __device__ __forceinline__ unsigned int div_invariant(unsigned int n, unsigned int mul, int shift) {
  return static_cast<unsigned int>((static_cast<unsigned long long>(n) * mul) >> shift);
}
inline void div_invariant_params(unsigned int d, unsigned int* mul, int* shift) {
  int l = 0;
  while ((1ull << l) < d) l++;
  *shift = 31 + l;
  *mul = static_cast<unsigned int>(((1ull << *shift) + d - 1) / d);
}

// First-level entries of the two-level node search: every node down to depth 6.
constexpr int kCullTopMax = 127;

// Device view of one mesh; passed to kernels by value.
struct DevMesh {
  int type;
  int totvert;
  int totnode;
  int nleaf;
  int totlt;
  int grid_size, grid_area;
  // n / grid_area and n / grid_size as multiply and shift (div_invariant)
  unsigned int area_mul, size_mul;
  int area_shift, size_shift;
  int nlevels;
  float4* co;  // FACES: the MVert bytes (xyz + flag/bweight/pad in w); GRIDS: xyz, 0
  float4* no;
  float4* orig_co;  // stroke-start positions and normals (grab, elastic deform, layer); may be null
  float4* orig_no;
  float* layer_disp;  // layer brush: per-vertex layer height of the stroke
  float* mask;      // nullable
  const float* automask;  // nullable
  // FACES topology
  const int2* poly;     // loopstart, totloop
  const int4* poly_v4;  // corner vertices of a triangle (w = -1) or quad; x = -1 otherwise
  const int* loop_v;
  const int4* lt_v4;    // per looptri: its three corner vertices and its poly
  const int* vt_off;
  const int2* vt_meta;  // per vertex, its looptris in ascending order: (poly, leaf id)
  const int* nb_off;
  const int* nb_idx;
  unsigned int* vtag;  // vert_bitmap, one word per vertex
  // PBVH
  float4* vb;  // 2 per node: (min xyz, 0), (max xyz, 0)
  float4* orig_vb;
  const int* node_child;   // children_offset or -1
  const int* node_parent;  // -1 for the root
  const int* node_leaf;    // leaf id or -1
  const int* leaf_node;    // leaf id (left-first DFS rank) -> node
  const int* leaf_vert_off;  // FACES: nleaf+1 offsets into leaf_verts
  const int* leaf_uniq;      // FACES: unique vertex count per leaf
  const int* leaf_ubase;     // FACES: device index of the leaf's first unique vertex
  // FACES: the leaves joined to each leaf by a mesh edge (CSR; GRIDS: none)
  const int* leaf_adj_off;
  const int* leaf_adj;
  const int* leaf_verts;     // FACES: vert_indices per leaf, leaf-id order
  const int* leaf_prim_off;  // nleaf+1
  const int* leaf_prims;     // prim indices, leaf-id order
  int* leaf_flag;            // PBVHNodeFlags per leaf
  const int* level_off;      // internal nodes by depth, deepest first
  const int* level_nodes;
  const int* node_leaf_lo;   // first leaf id under the node
  const int* node_leaf_hi;   // one past the last leaf id under the node
  const int* node_depth;     // root = 0
  // Two-level node search of the persistent kernels: every node of depth <=
  // the mesh's split depth, as (node, first descendant, one past the last
  // descendant) — the range set only for internal nodes at the split depth,
  // whose descendants occupy one contiguous index range (children are
  // allocated in pairs before their subtrees), else (-1, -1)
  const int4* cull_top;
  int cull_ntop;  // 0: one level, every node tested directly
  int max_depth;
  // Refit chunks: each leaf's full vertex list (PBVH_ITER_ALL order) in runs
  // of kChunk entries; chunk_box holds each run's box (2 float4), refreshed by
  // every refit, so a leaf box is the union of its chunk boxes.
  const int* leaf_chunk_off;  // nleaf+1
  float4* chunk_box;
  // persistent stroke kernel work lists
  int* hit_list[2];  // smooth: vertices inside the sphere, ping-pong per iteration
  int* tag_list;     // vertices tagged in the current dab
  int* touch_list;   // leaves marked in the current dab
  // GRIDS topology
  int num_faces, num_base_verts, num_base_edges;
  const int* grid_face;
  const int4* grid_info;  // per grid: (face, face's first grid, face's grid count, 0)
  const int* face_start;
  const int* face_ngrids;
  const int* face_verts;
  const int* face_edges;
  const int* edge_off;
  const int* edge_elems;
  const int* bvert_off;
  const int* bvert_elems;
  const int* edge_face;   // face of each edge_elems slot
  const int* bvert_face;  // face of each bvert_elems slot
  int max_face_corners;
  int* face_list;
  int2* face_info;  // per claimed face (face_list order): its first grid and grid count
  int* cgrid_list;  // grids of the claimed faces
  int* edge_list;
  int* bvert_list;
  unsigned int* face_mark;
  unsigned int* edge_mark;
  unsigned int* bvert_mark;
  int* grid_counts;  // [0] faces, [1] edges, [2] base verts, [3] grids
  // per grid (corner of its face), written with the face's update in a dab:
  // [2g] = (first edge_elems slot, faces) of the base edge the corner's face
  // averages, [2g+1] = (first bvert_elems slot, faces) of its base vertex;
  // faces = 0 when another claimed face owns it or it has one face
  int2* corner_own;
  // per base edge / base vertex: the smallest key ((~epoch) << 32 | face)
  // over the faces claimed for the persistent kernel's GRIDS update; the
  // owner in an epoch is the claimed face of least index, which is the first
  // claimed one in slot order (slots are filled face by face)
  unsigned long long* edge_own;
  unsigned long long* bvert_own;
  // work
  Work* work;
  int* cull_list;  // nleaf
  int* cull_off;   // nleaf+1: prefix of brush-visible vertex counts over cull_list
  AreaPart* parts;  // nleaf * area_blocks
  int area_blocks;  // blocks of kAreaBlock visited vertices per leaf in the area reduction
  int max_leaf_verts;   // largest brush-visible vertex count of a leaf
  int max_leaf_chunks;  // largest refit chunk count of a leaf
  float4* scratch;   // smooth Jacobi values, totvert
  float4* scratch2;  // second value buffer of the slot sweeps, totvert
  int* slot_map[2];  // vertex -> smooth slot of a pass, or -1; passes alternate
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
  float crease_pinch_factor;
  int elastic_type;                   // BRUSH_ELASTIC_DEFORM_*
  float height;                       // layer height
  float kl_a, kl_b, kl_c, kl_f;       // BKE_kelvinlet_init_params of the dab
  float kl_rs[3];
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
constexpr int kToolDraw = 1, kToolSmooth = 2, kToolPinch = 3, kToolInflate = 4, kToolGrab = 5,
              kToolLayer = 6, kToolCrease = 16, kToolClayStrips = 18, kToolElasticDeform = 21;
// Tools that read the stroke-start positions (stored when a stroke starts).
__host__ __device__ __forceinline__ bool needs_stroke_start(int tool) {
  return tool == kToolGrab || tool == kToolElasticDeform || tool == kToolLayer;
}
// Tools that rebuild positions from the stroke-start ones (one dab, all passes).
__host__ __device__ __forceinline__ bool uses_original(int tool) {
  return tool == kToolGrab || tool == kToolElasticDeform;
}
// The symmetry passes of one dab (mirrored location, grab delta, view normal).
struct DabPasses {
  int npass;
  float loc[8][3];
  float delta[8][3];
  float view[8][3];
};
// Tools that reduce the area normal (and centre) before their sweep.
__host__ __device__ __forceinline__ bool uses_area(int tool) {
  return tool == kToolDraw || tool == kToolClayStrips || tool == kToolPinch || tool == kToolCrease;
}

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
  // FACES: the unique vertices of a leaf are one range in device order
  if (m.type == kFaces) return m.leaf_ubase[leaf] + i;
  const int q = static_cast<int>(div_invariant(static_cast<unsigned int>(i), m.area_mul, m.area_shift));
  const int g = m.leaf_prims[m.leaf_prim_off[leaf] + q];
  return g * m.grid_area + (i - q * m.grid_area);
}
// All vertices of a leaf (PBVH_ITER_ALL) for the bounding-box refit.
__device__ __forceinline__ int leaf_nverts_all(const DevMesh& m, int leaf) {
  if (m.type == kFaces) return m.leaf_vert_off[leaf + 1] - m.leaf_vert_off[leaf];
  return (m.leaf_prim_off[leaf + 1] - m.leaf_prim_off[leaf]) * m.grid_area;
}
__device__ __forceinline__ int leaf_vert_all(const DevMesh& m, int leaf, int i) {
  if (m.type == kFaces) return i < m.leaf_uniq[leaf] ? m.leaf_ubase[leaf] + i : m.leaf_verts[m.leaf_vert_off[leaf] + i];
  return leaf_vert(m, leaf, i);
}

constexpr int kChunk = 64;

// Box of refit chunk c of a leaf by one warp (two entries per lane, loads
// issued together), stored in chunk_box; every lane returns the box.
__device__ __forceinline__ void chunk_refit_warp(const DevMesh& m, int leaf, int c, float* mn,
                                                 float* mx) {
  const int lane = threadIdx.x & 31;
  const int nv = leaf_nverts_all(m, leaf);
  const int i0 = c * kChunk + lane, i1 = i0 + 32;
  const int e = min(nv, (c + 1) * kChunk);
  const int v0 = i0 < e ? leaf_vert_all(m, leaf, i0) : -1;
  const int v1 = i1 < e ? leaf_vert_all(m, leaf, i1) : -1;
  const float4 p0 = v0 >= 0 ? __ldcg(&m.co[v0]) : make_float4(FLT_MAX, FLT_MAX, FLT_MAX, 0.0f);
  const float4 p1 = v1 >= 0 ? __ldcg(&m.co[v1]) : p0;
  float a[3] = {p0.x, p0.y, p0.z}, b[3] = {p1.x, p1.y, p1.z};
  for (int k = 0; k < 3; k++) {
    mn[k] = v0 >= 0 ? ((a[k] < b[k]) ? a[k] : b[k]) : FLT_MAX;
    mx[k] = v0 >= 0 ? ((a[k] > b[k]) ? a[k] : b[k]) : -FLT_MAX;
  }
#pragma unroll
  for (int o = 16; o >= 1; o >>= 1)
#pragma unroll
    for (int k = 0; k < 3; k++) {
      const float omn = __shfl_xor_sync(0xffffffffu, mn[k], o);
      const float omx = __shfl_xor_sync(0xffffffffu, mx[k], o);
      mn[k] = (mn[k] < omn) ? mn[k] : omn;
      mx[k] = (mx[k] > omx) ? mx[k] : omx;
    }
  if (lane == 0) {
    const int id = m.leaf_chunk_off[leaf] + c;
    m.chunk_box[2 * id] = make_float4(mn[0], mn[1], mn[2], 0.0f);
    m.chunk_box[2 * id + 1] = make_float4(mx[0], mx[1], mx[2], 0.0f);
  }
}

// Leaf box as the union of its chunk boxes, by one warp; lane 0 writes vb,
// every lane returns the box in omn / omx.
__device__ __forceinline__ void leaf_box_from_chunks(const DevMesh& m, int leaf, float4& omn,
                                                     float4& omx) {
  const int lane = threadIdx.x & 31;
  float mn[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, mx[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
  for (int id = m.leaf_chunk_off[leaf] + lane; id < m.leaf_chunk_off[leaf + 1]; id += 32) {
    const float4 a = __ldcg(&m.chunk_box[2 * id]), b = __ldcg(&m.chunk_box[2 * id + 1]);
    mn[0] = (mn[0] < a.x) ? mn[0] : a.x;
    mn[1] = (mn[1] < a.y) ? mn[1] : a.y;
    mn[2] = (mn[2] < a.z) ? mn[2] : a.z;
    mx[0] = (mx[0] > b.x) ? mx[0] : b.x;
    mx[1] = (mx[1] > b.y) ? mx[1] : b.y;
    mx[2] = (mx[2] > b.z) ? mx[2] : b.z;
  }
#pragma unroll
  for (int o = 16; o >= 1; o >>= 1)
#pragma unroll
    for (int k = 0; k < 3; k++) {
      const float omn = __shfl_xor_sync(0xffffffffu, mn[k], o);
      const float omx = __shfl_xor_sync(0xffffffffu, mx[k], o);
      mn[k] = (mn[k] < omn) ? mn[k] : omn;
      mx[k] = (mx[k] > omx) ? mx[k] : omx;
    }
  omn = make_float4(mn[0], mn[1], mn[2], 0.0f);
  omx = make_float4(mx[0], mx[1], mx[2], 0.0f);
  if (lane == 0) {
    const int node = m.leaf_node[leaf];
    m.vb[2 * node] = omn;
    m.vb[2 * node + 1] = omx;
  }
}

__device__ __forceinline__ void leaf_box_from_chunks(const DevMesh& m, int leaf) {
  float4 mn, mx;
  leaf_box_from_chunks(m, leaf, mn, mx);
}

__device__ __forceinline__ float dist_sq(float4 co, const float* c) {
  const float d0 = co.x - c[0], d1 = co.y - c[1], d2 = co.z - c[2];
  return d0 * d0 + d1 * d1 + d2 * d2;
}

__device__ __forceinline__ void set_err(const DevMesh& m, int code) {
  atomicCAS(&m.work->err, 0, code);
}

// ---------------------------------------------------------------------------
// Per-vertex brush math shared by the per-call kernels and the persistent
// stroke kernel (one definition, so both paths round identically).

__device__ __forceinline__ void cross3(float* r, const float* a, const float* b) {
  r[0] = a[1] * b[2] - a[2] * b[1];
  r[1] = a[2] * b[0] - a[0] * b[2];
  r[2] = a[0] * b[1] - a[1] * b[0];
}

// Pass constants derived from the area normal/centre (draw, clay strips).
struct BrushFrame {
  float area_no[3];
  float off[3];  // draw: area_no * radius * strength
  float xa[3], ya[3];  // clay strips: in-plane axes; pinch: xa = stroke side axis
  float pd, inv_r, inv_rz;  // clay strips: plane offset, inverse extents
  float pinch_k;   // crease: pinch factor^2 * |strength|
  float inv_nlen;  // crease: -1 / |area_no|^2 (0 for a zero normal)
};

// Returns false when the clay-strips frame is degenerate (the pass then does
// nothing, marks nothing).
__device__ __forceinline__ bool make_frame(const DevBrush& b, const PassParams& pp,
                                           const float* area_no, const float* area_co,
                                           BrushFrame& f) {
  const float radius = b.radius;
  for (int k = 0; k < 3; k++) f.area_no[k] = area_no[k];
  const float dd = radius * b.strength;
  for (int k = 0; k < 3; k++) f.off[k] = area_no[k] * dd;
  f.pd = f.inv_r = f.inv_rz = f.pinch_k = f.inv_nlen = 0.0f;
  if (b.tool == kToolPinch) {
    cross3(f.xa, area_no, pp.delta);
    if (normalize3(f.xa[0], f.xa[1], f.xa[2]) == 0.0f) return false;
  }
  if (b.tool == kToolCrease) {
    const float corr = b.crease_pinch_factor * b.crease_pinch_factor;
    f.pinch_k = b.strength < 0.0f ? -corr * b.strength : corr * b.strength;
    const float nl = area_no[0] * area_no[0] + area_no[1] * area_no[1] + area_no[2] * area_no[2];
    f.inv_nlen = nl > FLT_EPSILON ? -1.0f / nl : 0.0f;
  }
  if (b.tool == kToolClayStrips) {
    cross3(f.xa, area_no, pp.delta);
    if (normalize3(f.xa[0], f.xa[1], f.xa[2]) == 0.0f) return false;
    cross3(f.ya, area_no, f.xa);
    if (normalize3(f.ya[0], f.ya[1], f.ya[2]) == 0.0f) return false;
    const float rsign = b.strength < 0.0f ? -radius : radius;
    const float displace = rsign * (0.18f + b.plane_offset);
    float p[3];
    for (int k = 0; k < 3; k++) p[k] = area_co[k] + area_no[k] * displace;
    f.pd = -(area_no[0] * p[0] + area_no[1] * p[1] + area_no[2] * p[2]);
    f.inv_r = 1.0f / radius;
    f.inv_rz = 1.0f / (radius * 1.25f);
  }
  return true;
}

// Draw / inflate / clay strips on one vertex.  Returns true when the vertex is
// inside the brush test (then co holds the new position); moved reports a
// non-zero strength factor.
__device__ __forceinline__ bool brush_vertex(const DevMesh& m, const DevBrush& b, const float* ys,
                                             const PassParams& pp, const BrushFrame& f, int v,
                                             float4& co, bool& moved) {
  const float radius = b.radius;
  if (b.tool == kToolDraw) {
    const float d2 = dist_sq(co, pp.loc);
    if (!(d2 <= radius * radius)) return false;
    const float sf = strength_factor(m, b, ys, pp, v, sqrtf(d2), radius);
    co.x = co.x + f.off[0] * sf;
    co.y = co.y + f.off[1] * sf;
    co.z = co.z + f.off[2] * sf;
    moved = (b.strength * sf) != 0.0f;
    return true;
  }
  if (b.tool == kToolInflate) {
    const float d2 = dist_sq(co, pp.loc);
    if (!(d2 <= radius * radius)) return false;
    const float sf = strength_factor(m, b, ys, pp, v, sqrtf(d2), radius);
    const float fade = b.strength * sf;
    const float kk = fade * radius;
    const float4 no = m.no[v];
    co.x = co.x + no.x * kk;
    co.y = co.y + no.y * kk;
    co.z = co.z + no.z * kk;
    moved = fade != 0.0f;
    return true;
  }
  if (b.tool == kToolPinch) {
    // toward the brush centre within the plane of the side axis and the normal
    const float d2 = dist_sq(co, pp.loc);
    if (!(d2 <= radius * radius)) return false;
    const float sf = strength_factor(m, b, ys, pp, v, sqrtf(d2), radius);
    const float fade = b.strength * sf;
    const float* an = f.area_no;
    const float c0 = pp.loc[0] - co.x, c1 = pp.loc[1] - co.y, c2 = pp.loc[2] - co.z;
    const float px = c0 * f.xa[0] + c1 * f.xa[1] + c2 * f.xa[2];
    const float pz = c0 * an[0] + c1 * an[1] + c2 * an[2];
    const float v0 = f.xa[0] * px + an[0] * pz;
    const float v1 = f.xa[1] * px + an[1] * pz;
    const float v2 = f.xa[2] * px + an[2] * pz;
    co.x = co.x + v0 * fade;
    co.y = co.y + v1 * fade;
    co.z = co.z + v2 * fade;
    moved = fade != 0.0f;
    return true;
  }
  if (b.tool == kToolCrease) {
    // pinch toward the centre within the area plane, then draw along the normal
    const float d2 = dist_sq(co, pp.loc);
    if (!(d2 <= radius * radius)) return false;
    const float sf = strength_factor(m, b, ys, pp, v, sqrtf(d2), radius);
    const float* an = f.area_no;
    const float k = sf * f.pinch_k;
    float v0 = (pp.loc[0] - co.x) * k, v1 = (pp.loc[1] - co.y) * k, v2 = (pp.loc[2] - co.z) * k;
    const float t = (v0 * an[0] + v1 * an[1] + v2 * an[2]) * f.inv_nlen;
    v0 = v0 + an[0] * t;
    v1 = v1 + an[1] * t;
    v2 = v2 + an[2] * t;
    co.x = co.x + (v0 + f.off[0] * sf);
    co.y = co.y + (v1 + f.off[1] * sf);
    co.z = co.z + (v2 + f.off[2] * sf);
    moved = (b.strength * sf) != 0.0f;
    return true;
  }
  // clay strips
  const float* an = f.area_no;
  const float r0 = co.x - pp.loc[0], r1 = co.y - pp.loc[1], r2 = co.z - pp.loc[2];
  const float lx = fabsf((r0 * f.xa[0] + r1 * f.xa[1] + r2 * f.xa[2]) * f.inv_r);
  const float ly = fabsf((r0 * f.ya[0] + r1 * f.ya[1] + r2 * f.ya[2]) * f.inv_r);
  const float lz = fabsf((r0 * an[0] + r1 * an[1] + r2 * an[2]) * f.inv_rz);
  if (!(lx <= 1.0f && ly <= 1.0f && lz <= 1.0f)) return false;
  const float dloc = (lx > ly) ? lx : ly;
  const float sf = strength_factor(m, b, ys, pp, v, radius * dloc, radius);
  const float fade = b.strength * sf;
  const float side = (co.x * an[0] + co.y * an[1] + co.z * an[2]) + f.pd;
  const float ns = -side;
  const float v0 = (co.x + an[0] * ns) - co.x;
  const float v1 = (co.y + an[1] * ns) - co.y;
  const float v2 = (co.z + an[2] * ns) - co.z;
  co.x = co.x + v0 * fade;
  co.y = co.y + v1 * fade;
  co.z = co.z + v2 * fade;
  moved = fade != 0.0f;
  return true;
}

// Smooth neighbour average: FACES one-ring (CSR order) or the in-grid
// 4-neighbourhood (x-1, x+1, y-1, y+1) for GRIDS.  fetch(u) gives the
// position of neighbour u; the sum runs in ring order whatever the source.
template <int kNbBatch, class Fetch>
__device__ __forceinline__ float3 ring_average(const DevMesh& m, int v, float4 c0, Fetch fetch) {
  float sx = 0.0f, sy = 0.0f, sz = 0.0f;
  int n = 0;
  if (m.type == kFaces) {
    // ring positions loaded kNbBatch at a time, summed in ring order
    const int e = m.nb_off[v + 1];
    for (int base = m.nb_off[v]; base < e; base += kNbBatch) {
      int id[kNbBatch];
#pragma unroll
      for (int j = 0; j < kNbBatch; j++) id[j] = (base + j < e) ? m.nb_idx[base + j] : -1;
      float3 c[kNbBatch];
#pragma unroll
      for (int j = 0; j < kNbBatch; j++) c[j] = id[j] >= 0 ? fetch(id[j]) : make_float3(0.0f, 0.0f, 0.0f);
#pragma unroll
      for (int j = 0; j < kNbBatch; j++) {
        if (id[j] < 0) break;
        sx += c[j].x;
        sy += c[j].y;
        sz += c[j].z;
        n++;
      }
    }
  } else {
    const int gs = m.grid_size, area = m.grid_area;
    const int g = static_cast<int>(div_invariant(static_cast<unsigned int>(v), m.area_mul, m.area_shift));
    const int r = v - g * area;
    const int y = static_cast<int>(div_invariant(static_cast<unsigned int>(r), m.size_mul, m.size_shift));
    const int x = r - y * gs;
    const int nx[4] = {x - 1, x + 1, x, x};
    const int ny[4] = {y, y, y - 1, y + 1};
    float3 c[4];
#pragma unroll
    for (int k = 0; k < 4; k++)
      c[k] = (nx[k] >= 0 && nx[k] < gs && ny[k] >= 0 && ny[k] < gs) ? fetch(g * area + ny[k] * gs + nx[k])
                                                                   : make_float3(0.0f, 0.0f, 0.0f);
#pragma unroll
    for (int k = 0; k < 4; k++) {
      if (nx[k] >= 0 && nx[k] < gs && ny[k] >= 0 && ny[k] < gs) {
        sx += c[k].x;
        sy += c[k].y;
        sz += c[k].z;
        n++;
      }
    }
  }
  if (n == 0) return make_float3(c0.x, c0.y, c0.z);
  const float inv = 1.0f / (float)n;
  return make_float3(sx * inv, sy * inv, sz * inv);
}

__device__ __forceinline__ float3 neighbor_average(const DevMesh& m, int v, float4 c0) {
  return ring_average<8>(m, v, c0, [&](int u) { return xyz(m.co[u]); });
}

// Jacobi update of one position: co + (avg - co) * fade, w kept.
__device__ __forceinline__ float4 smooth_step(float4 co, float3 avg, float fade) {
  float4 out;
  out.x = co.x + (avg.x - co.x) * fade;
  out.y = co.y + (avg.y - co.y) * fade;
  out.z = co.z + (avg.z - co.z) * fade;
  out.w = co.w;
  return out;
}

// Smooth sweeps over slots.  The first sweep of a pass gives every vertex
// inside the sphere a slot (smap[v] = slot) and stores its new position in
// the slot; sweep k reads the slot values of sweep k-1 for neighbours with a
// slot and the unchanged positions of the others (a vertex outside the
// sphere does not move, so it never enters later).  co is the vertex's own
// value after sweep k-1; a vertex now outside keeps it.
__device__ __forceinline__ float4 smooth_slot(const DevMesh& m, const DevBrush& b,
                                              const PassParams& pp, int v, float4 co,
                                              const float4* src, const int* smap) {
  const float radius = b.radius;
  const float d2 = dist_sq(co, pp.loc);
  if (!(d2 <= radius * radius)) return co;
  const float sf = strength_factor(m, b, b.y, pp, v, sqrtf(d2), radius);
  const float fade = pp.iter_strength * sf;
  const float3 avg = ring_average<4>(m, v, co, [&](int u) {
    const int sl = __ldcg(&smap[u]);
    return xyz(sl >= 0 ? __ldcg(&src[sl]) : m.co[u]);
  });
  return smooth_step(co, avg, fade);
}

// Ring of v in smooth order (FACES one-ring, GRIDS x-1, x+1, y-1, y+1 inside
// the grid) into id[]; returns its size, or -1 above kNbCache.
constexpr int kNbCache = 8;
__device__ __forceinline__ int ring_ids(const DevMesh& m, int v, int* id) {
  int n = 0;
  if (m.type == kFaces) {
    const int q0 = m.nb_off[v], q1 = m.nb_off[v + 1];
    if (q1 - q0 > kNbCache) return -1;
    n = q1 - q0;
#pragma unroll
    for (int j = 0; j < kNbCache; j++) id[j] = j < n ? m.nb_idx[q0 + j] : -1;
  } else {
    const int gs = m.grid_size, area = m.grid_area;
    const int g = static_cast<int>(div_invariant(static_cast<unsigned int>(v), m.area_mul, m.area_shift));
    const int r = v - g * area;
    const int y = static_cast<int>(div_invariant(static_cast<unsigned int>(r), m.size_mul, m.size_shift));
    const int x = r - y * gs;
    const int nx[4] = {x - 1, x + 1, x, x};
    const int ny[4] = {y, y, y - 1, y + 1};
#pragma unroll
    for (int j = 0; j < kNbCache; j++) id[j] = -1;
#pragma unroll
    for (int k = 0; k < 4; k++)
      if (nx[k] >= 0 && nx[k] < gs && ny[k] >= 0 && ny[k] < gs) id[n++] = g * area + ny[k] * gs + nx[k];
  }
  return n;
}

// First sweep of a vertex known to be inside the sphere: the same value as
// smooth_vertex, with its ring recorded in tab (tab[j * stride]: xyz = the
// neighbour's position, w = its id as int bits) for the later sweeps.
// *nring = ring size, or -1 when the ring exceeds kNbCache (tab unused).
__device__ __forceinline__ float4 smooth_first(const DevMesh& m, const DevBrush& b,
                                               const PassParams& pp, int v, float4 co,
                                               float4* tab, int stride, int* nring,
                                               bool& moved) {
  const float radius = b.radius;
  const float d2 = dist_sq(co, pp.loc);
  const float sf = strength_factor(m, b, b.y, pp, v, sqrtf(d2), radius);
  const float fade = pp.iter_strength * sf;
  moved = fade != 0.0f;
  int id[kNbCache];
  const int n = ring_ids(m, v, id);
  *nring = n;
  if (n < 0) return smooth_step(co, neighbor_average(m, v, co), fade);
  float sx = 0.0f, sy = 0.0f, sz = 0.0f;
#pragma unroll
  for (int h = 0; h < kNbCache; h += 4) {
    float3 c[4];
#pragma unroll
    for (int j = 0; j < 4; j++)
      if (h + j < n) c[j] = xyz(m.co[id[h + j]]);
#pragma unroll
    for (int j = 0; j < 4; j++) {
      if (h + j < n) {
        sx += c[j].x;
        sy += c[j].y;
        sz += c[j].z;
        tab[(h + j) * stride] = make_float4(c[j].x, c[j].y, c[j].z, __int_as_float(id[h + j]));
      }
    }
  }
  float3 avg;
  if (n == 0) {
    avg = make_float3(co.x, co.y, co.z);
  } else {
    const float inv = 1.0f / (float)n;
    avg = make_float3(sx * inv, sy * inv, sz * inv);
  }
  return smooth_step(co, avg, fade);
}

// Replaces the neighbour ids of a ring table by their slots (or -1), once
// the first sweep has given out every slot of the pass.
__device__ __forceinline__ void smooth_resolve(float4* tab, int stride, int n, const int* smap) {
  int sl[kNbCache];
#pragma unroll
  for (int j = 0; j < kNbCache; j++) sl[j] = j < n ? __ldcg(&smap[__float_as_int(tab[j * stride].w)]) : -1;
#pragma unroll
  for (int j = 0; j < kNbCache; j++)
    if (j < n) tab[j * stride].w = __int_as_float(sl[j]);
}

// smooth_slot with a resolved ring table (n entries: w = slot or -1, xyz =
// the fixed position of a neighbour without a slot).
__device__ __forceinline__ float4 smooth_slot_cached(const DevMesh& m, const DevBrush& b,
                                                     const PassParams& pp, int v, float4 co,
                                                     int n, const float4* tab, int stride,
                                                     const float4* src) {
  const float radius = b.radius;
  const float d2 = dist_sq(co, pp.loc);
  if (!(d2 <= radius * radius)) return co;
  const float sf = strength_factor(m, b, b.y, pp, v, sqrtf(d2), radius);
  const float fade = pp.iter_strength * sf;
  float sx = 0.0f, sy = 0.0f, sz = 0.0f;
#pragma unroll
  for (int h = 0; h < kNbCache; h += 4) {
    float3 c[4];
#pragma unroll
    for (int j = 0; j < 4; j++) {
      if (h + j < n) {
        const float4 e = tab[(h + j) * stride];
        const int sl = __float_as_int(e.w);
        c[j] = sl >= 0 ? xyz(__ldcg(&src[sl])) : make_float3(e.x, e.y, e.z);
      }
    }
#pragma unroll
    for (int j = 0; j < 4; j++) {
      if (h + j < n) {
        sx += c[j].x;
        sy += c[j].y;
        sz += c[j].z;
      }
    }
  }
  float3 avg;
  if (n == 0) {
    avg = make_float3(co.x, co.y, co.z);
  } else {
    const float inv = 1.0f / (float)n;
    avg = make_float3(sx * inv, sy * inv, sz * inv);
  }
  return smooth_step(co, avg, fade);
}

// One Jacobi smooth step on one vertex from the sweep-start state.  Returns
// true when inside the sphere (out then holds the new position).
__device__ __forceinline__ bool smooth_vertex(const DevMesh& m, const DevBrush& b, const float* ys,
                                              const PassParams& pp, int v, float4 co, float4& out,
                                              bool& moved) {
  const float radius = b.radius;
  const float d2 = dist_sq(co, pp.loc);
  if (!(d2 <= radius * radius)) return false;
  const float sf = strength_factor(m, b, ys, pp, v, sqrtf(d2), radius);
  const float fade = pp.iter_strength * sf;
  out = smooth_step(co, neighbor_average(m, v, co), fade);
  moved = fade != 0.0f;
  return true;
}

// FACES vertex normal (gather form of pbvh.c:2933-3009): compensated sum of
// the poly normals of the vertex's looptris lying in UpdateNormals leaves,
// ascending looptri order, then normalize_v3.  Returns the looptris used.
__device__ __forceinline__ int vertex_normal(const DevMesh& m, int v, float4& out) {
  // Entries are taken kNrmBatch at a time: their (poly, leaf) pairs, then the
  // leaf flags and corner indices, then the corner positions are each loaded
  // together; the compensated sums then run in entry order.
  constexpr int kNrmBatch = 4;
  CSum ax = {0.0f, 0.0f}, ay = {0.0f, 0.0f}, az = {0.0f, 0.0f};
  const int e = m.vt_off[v + 1];
  int used = 0;
  for (int base = m.vt_off[v]; base < e; base += kNrmBatch) {
    int2 meta[kNrmBatch];
#pragma unroll
    for (int j = 0; j < kNrmBatch; j++) meta[j] = (base + j < e) ? m.vt_meta[base + j] : make_int2(-1, -1);
    bool on[kNrmBatch];
    int4 pv[kNrmBatch];
#pragma unroll
    for (int j = 0; j < kNrmBatch; j++) {
      on[j] = meta[j].x >= 0 && (__ldcg(&m.leaf_flag[meta[j].y]) & kUpdateNormals);
      pv[j] = meta[j].x >= 0 ? m.poly_v4[meta[j].x] : make_int4(-1, -1, -1, -1);
    }
    float3 c[kNrmBatch][4];
#pragma unroll
    for (int j = 0; j < kNrmBatch; j++) {
      const bool ld = on[j] && pv[j].x >= 0;
      const int idx[4] = {pv[j].x, pv[j].y, pv[j].z, pv[j].w};
#pragma unroll
      for (int k = 0; k < 4; k++) c[j][k] = (ld && idx[k] >= 0) ? xyz(m.co[idx[k]]) : make_float3(0.0f, 0.0f, 0.0f);
    }
#pragma unroll
    for (int j = 0; j < kNrmBatch; j++) {
      if (!on[j]) continue;
      float3 fn;
      if (pv[j].x < 0) {
        fn = poly_normal(m, meta[j].x);
      } else if (pv[j].w < 0) {
        fn = normal_tri(c[j][0], c[j][1], c[j][2]);
      } else {
        fn = normal_quad(c[j][0], c[j][1], c[j][2], c[j][3]);
      }
      cs_add(ax, fn.x);
      cs_add(ay, fn.y);
      cs_add(az, fn.z);
      used++;
    }
  }
  float nx = ax.s + ax.e, ny = ay.s + ay.e, nz = az.s + az.e;
  normalize3(nx, ny, nz);
  out = make_float4(nx, ny, nz, 0.0f);
  return used;
}

__device__ __forceinline__ float fmin_ref(float a, float b) { return (a < b) ? a : b; }
__device__ __forceinline__ float fmax_ref(float a, float b) { return (a > b) ? a : b; }

// The area reduction visits each culled leaf in blocks of kAreaBlock
// vertices (256 lanes x 16); every leaf counts DevMesh::area_blocks blocks
// (the largest ceil(visited vertices / kAreaBlock) over the leaves; blocks
// past a leaf's end are empty partials).
constexpr int kAreaBlock = 4096;

// 16-byte asynchronous copy global -> shared (no register holds the data).
__device__ __forceinline__ void cp_async16(void* smem_dst, const void* gmem_src) {
  const unsigned int d = static_cast<unsigned int>(__cvta_generic_to_shared(smem_dst));
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d), "l"(gmem_src) : "memory");
}
// 4-byte asynchronous copy global -> shared (cached in L1).
__device__ __forceinline__ void cp_async4(void* smem_dst, const void* gmem_src) {
  const unsigned int d = static_cast<unsigned int>(__cvta_generic_to_shared(smem_dst));
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(d), "l"(gmem_src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
// Wait until at most 1 / 0 committed groups of this thread are in flight.
__device__ __forceinline__ void cp_async_wait_group1() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_group0() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.commit_group;\n\tcp.async.wait_group 0;" ::: "memory");
}

// Area normal/centre lanes: compensated (s, e) sums of normal xyz and centre
// xyz plus the two counts; merged pairwise in the order the spec fixes.
struct Lane {
  CSum v[6];
  int n_no, n_co;
};

__device__ __forceinline__ void lane_merge(Lane& a, const Lane& b) {
#pragma unroll
  for (int k = 0; k < 6; k++) a.v[k] = cs_merge(a.v[k], b.v[k]);
  a.n_no += b.n_no;
  a.n_co += b.n_co;
}

__device__ __forceinline__ Lane lane_shfl_down(const Lane& a, int s) {
  Lane r;
#pragma unroll
  for (int k = 0; k < 6; k++) {
    r.v[k].s = __shfl_down_sync(0xffffffffu, a.v[k].s, s);
    r.v[k].e = __shfl_down_sync(0xffffffffu, a.v[k].e, s);
  }
  r.n_no = __shfl_down_sync(0xffffffffu, a.n_no, s);
  r.n_co = __shfl_down_sync(0xffffffffu, a.n_co, s);
  return r;
}

__device__ __forceinline__ void part_store(AreaPart* p, const Lane& l) {
#pragma unroll
  for (int k = 0; k < 6; k++) {
    __stcg(&p->s[k], l.v[k].s);
    __stcg(&p->e[k], l.v[k].e);
  }
  __stcg(&p->n_no, l.n_no);
  __stcg(&p->n_co, l.n_co);
}
__device__ __forceinline__ Lane part_load(const AreaPart* p) {
  Lane l;
#pragma unroll
  for (int k = 0; k < 6; k++) {
    l.v[k].s = __ldcg(&p->s[k]);
    l.v[k].e = __ldcg(&p->e[k]);
  }
  l.n_no = __ldcg(&p->n_no);
  l.n_co = __ldcg(&p->n_co);
  return l;
}

// ---------------------------------------------------------------------------
// Brushes that read the stroke-start data (grab, elastic deform, layer), shared
// by the per-call kernels and the persistent stroke kernel.

__device__ __forceinline__ float kp2(float x) { return x * x; }
__device__ __forceinline__ float kp3(float x) { return kp2(x) * x; }
__device__ __forceinline__ float kp5(float x) { return kp2(kp2(x)) * x; }

// init_kelvinlet_grab (kelvinlet.c:23-44) for n scales.
__device__ __forceinline__ void kelvinlet_grab_k(const DevBrush& b, float radius, int n,
                                                 float* k) {
  for (int i = 0; i < n; i++) {
    const float re = sqrtf(kp2(radius) + kp2(b.kl_rs[i]));
    k[i] = ((b.kl_a - b.kl_b) / re) + ((b.kl_b * kp2(radius)) / kp3(re)) +
           ((b.kl_a * kp2(b.kl_rs[i])) / (2.0f * kp3(re)));
  }
}

// kelvinlet_scale / kelvinlet_twist (kelvinlet.c:131-186) at one point.
__device__ __forceinline__ float3 kelvinlet_field(const DevBrush& b, float3 co, const float* loc,
                                                  const float* nrm) {
  const float r0 = co.x - loc[0], r1 = co.y - loc[1], r2 = co.z - loc[2];
  const float radius = sqrtf(r0 * r0 + r1 * r1 + r2 * r2);
  const float re = sqrtf(kp2(radius) + kp2(b.kl_rs[0]));
  const float head = b.elastic_type == 3 ? (2.0f * b.kl_b - b.kl_a) : -b.kl_a;
  const float u = head * (1.0f / kp3(re)) + ((3.0f * kp2(b.kl_rs[0])) / (2.0f * kp5(re)));
  const float s = (u * b.kl_c) * b.kl_f;
  if (b.elastic_type == 3) return make_float3(r0 * s, r1 * s, r2 * s);
  const float q0 = nrm[1] * r2 - nrm[2] * r1;
  const float q1 = nrm[2] * r0 - nrm[0] * r2;
  const float q2 = nrm[0] * r1 - nrm[1] * r0;
  return make_float3(q0 * s, q1 * s, q2 * s);
}

// The Kelvinlet displacement of one element for one pass (kelvinlet.c):
// grab types scale delta, scale / twist integrate the field in four steps.
__device__ __forceinline__ float3 kelvinlet_disp(const DevBrush& b, float3 co, const float* loc,
                                                 const float* dn) {
  if (b.elastic_type <= 2) {
    const float d0 = co.x - loc[0], d1 = co.y - loc[1], d2 = co.z - loc[2];
    const float radius = sqrtf(d0 * d0 + d1 * d1 + d2 * d2);
    float k[3];
    float fade;
    if (b.elastic_type == 0) {
      kelvinlet_grab_k(b, radius, 1, k);
      fade = k[0] * b.kl_c;
    } else if (b.elastic_type == 1) {
      kelvinlet_grab_k(b, radius, 2, k);
      const float u = k[0] - k[1];
      fade = u * b.kl_c / ((1.0f / b.kl_rs[0]) - (1.0f / b.kl_rs[1]));
    } else {
      kelvinlet_grab_k(b, radius, 3, k);
      const float s0 = kp2(b.kl_rs[0]), s1 = kp2(b.kl_rs[1]), s2 = kp2(b.kl_rs[2]);
      const float w1 = -((s2 - s0) / (s2 - s1));
      const float w2 = ((s1 - s0) / (s2 - s1));
      const float u = 1.0f * k[0] + w1 * k[1] + w2 * k[2];
      fade = u * b.kl_c / (1.0f / b.kl_rs[0] + w1 / b.kl_rs[1] + w2 / b.kl_rs[2]);
    }
    return make_float3(dn[0] * fade, dn[1] * fade, dn[2] * fade);
  }
  // sculpt_kelvinet_integrate (kelvinlet.c:104-128), third step as written there
  const float3 k0 = kelvinlet_field(b, co, loc, dn);
  const float3 k1 = kelvinlet_field(
      b, make_float3(co.x + k0.x * 0.5f, co.y + k0.y * 0.5f, co.z + k0.z * 0.5f), loc, dn);
  const float3 k2 = kelvinlet_field(
      b, make_float3(co.x + k1.x * 0.5f, co.y + k1.y * 0.5f, co.z + k1.z * 0.5f), loc, dn);
  const float3 k3 = kelvinlet_field(
      b, make_float3((co.x + k2.x) - loc[0], (co.y + k2.y) - loc[1], (co.z + k2.z) - loc[2]), loc,
      dn);
  const float sixth = 1.0f / 6.0f;
  return make_float3((((k0.x + k1.x * 2.0f) + k2.x * 2.0f) + k3.x) * sixth,
                     (((k0.y + k1.y * 2.0f) + k2.y * 2.0f) + k3.y) * sixth,
                     (((k0.z + k1.z * 2.0f) + k2.z * 2.0f) + k3.z) * sixth);
}

// One vertex of a grab / elastic deform dab: its stroke-start position plus
// each pass's displacement in pass order (the reference combines its proxies
// once per dab onto the original coordinates).  Writes co.xyz; returns the
// number of passes that moved it.
__device__ __forceinline__ unsigned int orig_vertex(const DevMesh& m, const DevBrush& b,
                                                    const float* ys, const DabPasses& dp, int v,
                                                    float4& co) {
  const bool elastic = b.tool == kToolElasticDeform;
  const float radius = b.radius, rsq = radius * radius;
  unsigned int moved = 0u;
  const float4 o4 = m.orig_co[v];
  const float3 o = make_float3(o4.x, o4.y, o4.z);
  float c0 = o.x, c1 = o.y, c2 = o.z;
  for (int p = 0; p < dp.npass; p++) {
    if (elastic) {
      float3 d = kelvinlet_disp(b, o, dp.loc[p], b.elastic_type <= 2 ? dp.delta[p] : dp.view[p]);
      if (b.elastic_type <= 2) {
        const float s = b.strength * 20.0f;
        d = make_float3(d.x * s, d.y * s, d.z * s);
      }
      if (m.mask) {
        const float mk = 1.0f - m.mask[v];
        d = make_float3(d.x * mk, d.y * mk, d.z * mk);
      }
      if (m.automask) {
        const float am = m.automask[v];
        d = make_float3(d.x * am, d.y * am, d.z * am);
      }
      c0 = c0 + d.x;
      c1 = c1 + d.y;
      c2 = c2 + d.z;
      moved += (d.x != 0.0f || d.y != 0.0f || d.z != 0.0f) ? 1u : 0u;
    } else {
      const float e0 = o.x - dp.loc[p][0], e1 = o.y - dp.loc[p][1], e2 = o.z - dp.loc[p][2];
      const float d2 = e0 * e0 + e1 * e1 + e2 * e2;
      if (!(d2 <= rsq)) continue;
      float f = curve_strength(b, ys, sqrtf(d2), radius);
      if (b.flag & kBrushFrontFace) {
        const float4 n = m.orig_no[v];
        const float dot = dp.view[p][0] * n.x + dp.view[p][1] * n.y + dp.view[p][2] * n.z;
        f = f * (dot > 0.0f ? dot : 0.0f);
      }
      if (m.mask) f = f * (1.0f - m.mask[v]);
      if (m.automask) f = f * m.automask[v];
      const float fade = b.strength * f;
      c0 = c0 + dp.delta[p][0] * fade;
      c1 = c1 + dp.delta[p][1] * fade;
      c2 = c2 + dp.delta[p][2] * fade;
      moved += fade != 0.0f ? 1u : 0u;
    }
  }
  co.x = c0;
  co.y = c1;
  co.z = c2;
  return moved;
}

// Layer brush on one vertex: the sphere test on the stroke-start position,
// the layer height raised by fade * strength * (1.05 - |height|) and clamped
// to +-(1 - mask), the target o + on * (height_brush * layer), approached by
// |fade| of the way from the current position.
__device__ __forceinline__ bool layer_vertex(const DevMesh& m, const DevBrush& b, const float* ys,
                                             const PassParams& pp, int v, float4& co,
                                             bool& moved) {
  const float4 o = m.orig_co[v];
  const float e0 = o.x - pp.loc[0], e1 = o.y - pp.loc[1], e2 = o.z - pp.loc[2];
  const float d2 = e0 * e0 + e1 * e1 + e2 * e2;
  if (!(d2 <= b.radius * b.radius)) return false;
  const float fade = strength_factor(m, b, ys, pp, v, sqrtf(d2), b.radius);
  float disp = m.layer_disp[v];
  disp = disp + fade * b.strength * (1.05f - fabsf(disp));
  const float lim = m.mask ? 1.0f - m.mask[v] : 1.0f;
  disp = disp < -lim ? -lim : (disp > lim ? lim : disp);
  m.layer_disp[v] = disp;
  const float4 on = m.orig_no[v];
  const float n0 = on.x * b.height, n1 = on.y * b.height, n2 = on.z * b.height;
  const float f0 = o.x + n0 * disp, f1 = o.y + n1 * disp, f2 = o.z + n2 * disp;
  const float af = fabsf(fade);
  const float v0 = (f0 - co.x) * af, v1 = (f1 - co.y) * af, v2 = (f2 - co.z) * af;
  co.x = co.x + v0;
  co.y = co.y + v1;
  co.z = co.z + v2;
  moved = fade != 0.0f;
  return true;
}

}  // namespace sgpu
