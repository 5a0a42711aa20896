// Ray cast of the PBVH: BKE_pbvh_raycast (pbvh.c:3916-3929) with the sculpt
// ray-cast callback, for a batch of independent rays, PBVH_FACES and
// PBVH_GRIDS.
//
// The reference walks the leaves whose box the ray line meets in order of
// their entry distance (a binary tree keyed on tmin, ties after earlier DFS
// leaves: BKE_pbvh_search_callback_occluded, pbvh.c:2853-2890), ray casts a
// leaf when its tmin is below the running minimum (FLT_MAX until the first
// hit, then the hit depth) and inside a leaf accepts a triangle when its hit
// is strictly closer than the current depth (pbvh_faces_node_raycast,
// pbvh.c:4042-4108).  The result only depends on each leaf's closest hit
// (first triangle in prim order among equals) and on that leaf order, so:
//   k_ray_leaves  one CTA per ray: every node box tested (isect_ray_aabb_v3),
//                 leaves under passing ancestors listed in DFS order, their
//                 processing order (stable by tmin; a NaN tmin is never below
//                 the running minimum, and the binary tree orders the others
//                 stably), and one work item per (leaf, 256 prims);
//   k_ray_tris    every item's triangles tested (isect_ray_tri_watertight_v3),
//                 the leaf's closest (depth, prim position) by atomicMin on a
//                 64-bit key (depth bits of a non-negative float, -0 as +0);
//   k_ray_finish  one CTA per ray: the leaves in order with the callback's
//                 rule, then the winning triangle's depth, active vertex
//                 (corner nearest the hit, first among equals), face and
//                 normal (normal_tri_v3 / normal_quad_v3).
// The leaves are tested front to back in two rounds: k_ray_tris first tests
// the first_leaves leaves of smallest entry distance; k_ray_finish (round 0)
// walks them and settles every ray whose next leaf starts at or beyond the
// running minimum (the reference never casts it, nor any later one); only the
// other rays get their remaining leaves tested (round 1) and walked.
// GRIDS (pbvh_grids_node_raycast, pbvh.c:4110-4201): the units are grid quads
// (grid, row, column order) and ray_face_intersection_quad tries the second
// triangle only when the first is not taken, so a quad whose two triangles
// both meet the ray with the second closer does not reduce to a minimum.
// k_ray_tris flags such a leaf; k_ray_finish replays a flagged leaf quad by
// quad in order (256 quads at a time, their tests in parallel, the rule
// sequentially), and every other leaf by its minimum key.
//
// The same kernels (kNear) answer BKE_pbvh_find_nearest_to_ray (pbvh.c:
// 4339-4352) with the sculpt callback of the brush specification: the node
// test is nearest_to_ray_aabb_dist_sq (pbvh.c:4315-4337: tmin = the squared
// distance of the box from the ray, dist_squared_ray_to_aabb_v3; the node
// passes when the depth of that nearest point is positive), a leaf is
// searched when its tmin is below the running minimum squared distance, and
// inside it a triangle is taken when its squared distance
// (dist_squared_ray_to_tri_v3_fast, pbvh.c:3970-3989) is strictly below the
// current one.  FACES leaves reduce to their minimum key (squared distance in
// an order-preserving encoding, prim position).  In a GRIDS leaf
// (ray_face_nearest_quad, pbvh.c:3991-4017) the second triangle of a quad is
// tested only when the first was taken, which depends on the running value,
// so every GRIDS leaf is replayed quad by quad; a chunk's quads whose first
// triangle is not below the value at the chunk's start can never be taken
// and are skipped.
#include <cuda_runtime.h>

#include "sgpu_device.cuh"
#include "sgpu_ray.h"

namespace sgpu {

namespace {

constexpr int kRayThreads = 256;
constexpr int kRayChunk = 256;  // prims per work item
constexpr unsigned long long kNoKey = ~0ull;

struct RayBox {
  float org[3], inv[3];
  int sign[3];
};

__device__ __forceinline__ void raybox_init(RayBox& r, const float* o, const float* d) {
#pragma unroll
  for (int i = 0; i < 3; i++) {
    r.org[i] = o[i];
    r.inv[i] = 1.0f / d[i];
    r.sign[i] = r.inv[i] < 0.0f;
  }
}

// isect_ray_aabb_v3 (math_geom.cc:3032-3080): entry distance in *tmin_out.
__device__ __forceinline__ bool raybox_hit(const RayBox& r, float4 mn, float4 mx, float* tmin_out) {
  const float bb[2][3] = {{mn.x, mn.y, mn.z}, {mx.x, mx.y, mx.z}};
  float tmin = (bb[r.sign[0]][0] - r.org[0]) * r.inv[0];
  float tmax = (bb[1 - r.sign[0]][0] - r.org[0]) * r.inv[0];
  const float tymin = (bb[r.sign[1]][1] - r.org[1]) * r.inv[1];
  const float tymax = (bb[1 - r.sign[1]][1] - r.org[1]) * r.inv[1];
  if ((tmin > tymax) || (tymin > tmax)) return false;
  if (tymin > tmin) tmin = tymin;
  if (tymax < tmax) tmax = tymax;
  const float tzmin = (bb[r.sign[2]][2] - r.org[2]) * r.inv[2];
  const float tzmax = (bb[1 - r.sign[2]][2] - r.org[2]) * r.inv[2];
  if ((tmin > tzmax) || (tzmin > tmax)) return false;
  if (tzmin > tmin) tmin = tzmin;
  *tmin_out = tmin;
  return true;
}

struct RayTri {
  int kx, ky, kz;
  float sx, sy, sz;
};

// isect_ray_tri_watertight_v3_precalc (math_geom.cc:1755-1780).
__device__ __forceinline__ void raytri_init(RayTri& p, const float* d) {
  const float x = fabsf(d[0]), y = fabsf(d[1]), z = fabsf(d[2]);
  const int kz = (x > y) ? ((x > z) ? 0 : 2) : ((y > z) ? 1 : 2);  // axis_dominant_v3_single
  int kx = (kz != 2) ? (kz + 1) : 0;
  int ky = (kx != 2) ? (kx + 1) : 0;
  if (d[kz] < 0.0f) {
    const int t = kx;
    kx = ky;
    ky = t;
  }
  const float inv_dir_z = 1.0f / d[kz];
  p.sx = d[kx] * inv_dir_z;
  p.sy = d[ky] * inv_dir_z;
  p.sz = inv_dir_z;
  p.kx = kx;
  p.ky = ky;
  p.kz = kz;
}

__device__ __forceinline__ float comp(const float3& v, int k) {
  return k == 0 ? v.x : (k == 1 ? v.y : v.z);
}

// isect_ray_tri_watertight_v3 (math_geom.cc:1782-1855).
__device__ __forceinline__ bool raytri_hit(const float* o, const RayTri& p, float3 v0, float3 v1,
                                           float3 v2, float* r_lambda) {
  const float3 a = make_float3(v0.x - o[0], v0.y - o[1], v0.z - o[2]);
  const float3 b = make_float3(v1.x - o[0], v1.y - o[1], v1.z - o[2]);
  const float3 c = make_float3(v2.x - o[0], v2.y - o[1], v2.z - o[2]);
  const float a_kx = comp(a, p.kx), a_ky = comp(a, p.ky), a_kz = comp(a, p.kz);
  const float b_kx = comp(b, p.kx), b_ky = comp(b, p.ky), b_kz = comp(b, p.kz);
  const float c_kx = comp(c, p.kx), c_ky = comp(c, p.ky), c_kz = comp(c, p.kz);
  const float ax = a_kx - p.sx * a_kz;
  const float ay = a_ky - p.sy * a_kz;
  const float bx = b_kx - p.sx * b_kz;
  const float by = b_ky - p.sy * b_kz;
  const float cx = c_kx - p.sx * c_kz;
  const float cy = c_ky - p.sy * c_kz;
  const float u = cx * by - cy * bx;
  const float v = ax * cy - ay * cx;
  const float w = bx * ay - by * ax;
  if ((u < 0.0f || v < 0.0f || w < 0.0f) && (u > 0.0f || v > 0.0f || w > 0.0f)) return false;
  const float det = u + v + w;
  if (det == 0.0f || !isfinite(det)) return false;
  const int sign_det = __float_as_int(det) & static_cast<int>(0x80000000u);
  const float t = (u * a_kz + v * b_kz + w * c_kz) * p.sz;
  const float sign_t = __int_as_float(__float_as_int(t) ^ sign_det);
  if (sign_t < 0.0f) return false;
  const float inv_det = 1.0f / det;
  *r_lambda = t * inv_det;
  return true;
}

__device__ __forceinline__ unsigned long long depth_key(float depth, int pos) {
  unsigned int bits = __float_as_uint(depth);
  if (bits == 0x80000000u) bits = 0u;  // -0 compares equal to +0
  return (static_cast<unsigned long long>(bits) << 32) | static_cast<unsigned int>(pos);
}

// Nearest-to-ray distances (math_geom.cc), the reference's FP32 operations.
// dist_squared_ray_to_aabb_v3_precalc (:643-655).
struct RayAabb {
  float org[3], dir[3], inv[3];
};

__device__ __forceinline__ void rayaabb_init(RayAabb& r, const float* o, const float* d) {
#pragma unroll
  for (int i = 0; i < 3; i++) {
    r.org[i] = o[i];
    r.dir[i] = d[i];
    r.inv[i] = (d[i] != 0.0f) ? (1.0f / d[i]) : FLT_MAX;
  }
}

__device__ __forceinline__ float dot3(const float* a, const float* b) {
  return a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
}

__device__ __forceinline__ void cross3(float* r, const float* a, const float* b) {
  r[0] = a[1] * b[2] - a[2] * b[1];
  r[1] = a[2] * b[0] - a[0] * b[2];
  r[2] = a[0] * b[1] - a[1] * b[0];
}

// dist_squared_ray_to_seg_v3 (:574-608) with isect_ray_line_v3 (:1997-2021)
// and interp_v3_v3v3 (math_vector.c:24-31): squared distance of the segment
// point the line parameter selects (clamped; v0 for a parallel segment) from
// the ray, and its depth.
__device__ float ray_seg_dist_sq(const float* o, const float* dir, const float* v0,
                                 const float* v1, float* r_depth) {
  const float a[3] = {v1[0] - v0[0], v1[1] - v0[1], v1[2] - v0[2]};
  const float t[3] = {v0[0] - o[0], v0[1] - o[1], v0[2] - o[2]};
  float n[3];
  cross3(n, a, dir);
  const float nlen = dot3(n, n);
  float p[3] = {v0[0], v0[1], v0[2]};
  if (nlen != 0.0f) {
    const float c[3] = {n[0] - t[0], n[1] - t[1], n[2] - t[2]};
    float cray[3];
    cross3(cray, c, dir);
    const float lambda = dot3(cray, n) / nlen;
    if (lambda <= 0.0f) {
      // v0
    } else if (lambda >= 1.0f) {
      p[0] = v1[0], p[1] = v1[1], p[2] = v1[2];
    } else {
      const float sl = 1.0f - lambda;
      p[0] = sl * v0[0] + lambda * v1[0];
      p[1] = sl * v0[1] + lambda * v1[1];
      p[2] = sl * v0[2] + lambda * v1[2];
    }
  }
  const float dvec[3] = {p[0] - o[0], p[1] - o[1], p[2] - o[2]};
  const float depth = dot3(dvec, dir);
  *r_depth = depth;
  return dot3(dvec, dvec) - depth * depth;
}

// dist_squared_ray_to_tri_v3_fast (pbvh.c:3970-3989): the edges (v0, v2),
// (v1, v0), (v2, v1); the first, then any strictly nearer one.
__device__ float ray_tri_dist_sq(const float* o, const float* dir, float3 v0, float3 v1, float3 v2,
                                 float* r_depth) {
  const float tri[3][3] = {{v0.x, v0.y, v0.z}, {v1.x, v1.y, v1.z}, {v2.x, v2.y, v2.z}};
  float best = FLT_MAX;
  for (int i = 0, j = 2; i < 3; j = i++) {
    float dt = FLT_MAX;
    const float dd = ray_seg_dist_sq(o, dir, tri[i], tri[j], &dt);
    if (dd < best || i == 0) {
      *r_depth = dt;
      best = dd;
    }
  }
  return best;
}

// dist_squared_ray_to_aabb_v3 (:657-744) with aabb_get_near_far_from_plane
// (:610-641): 0 when the ray line meets the box (depth of the far corner),
// else the squared distance of the box edge nearest the ray.
__device__ float rayaabb_dist_sq(const RayAabb& r, float4 mn, float4 mx, float* r_depth) {
  const float bmin[3] = {mn.x, mn.y, mn.z}, bmax[3] = {mx.x, mx.y, mx.z};
  float lo[3], hi[3];
#pragma unroll
  for (int k = 0; k < 3; k++) {
    const bool neg = r.dir[k] < 0.0f;
    lo[k] = neg ? bmax[k] : bmin[k];
    hi[k] = neg ? bmin[k] : bmax[k];
  }
  const float tmin[3] = {(lo[0] - r.org[0]) * r.inv[0], (lo[1] - r.org[1]) * r.inv[1],
                         (lo[2] - r.org[2]) * r.inv[2]};
  const float tmax[3] = {(hi[0] - r.org[0]) * r.inv[0], (hi[1] - r.org[1]) * r.inv[1],
                         (hi[2] - r.org[2]) * r.inv[2]};
  float va[3] = {0.0f, 0.0f, 0.0f}, vb[3] = {0.0f, 0.0f, 0.0f};
  float rtmin, rtmax;
  int axis;
  if ((tmax[0] <= tmax[1]) && (tmax[0] <= tmax[2])) {
    rtmax = tmax[0];
    va[0] = vb[0] = hi[0];
    axis = 3;
  } else if ((tmax[1] <= tmax[0]) && (tmax[1] <= tmax[2])) {
    rtmax = tmax[1];
    va[1] = vb[1] = hi[1];
    axis = 2;
  } else {
    rtmax = tmax[2];
    va[2] = vb[2] = hi[2];
    axis = 1;
  }
  if ((tmin[0] >= tmin[1]) && (tmin[0] >= tmin[2])) {
    rtmin = tmin[0];
    va[0] = vb[0] = lo[0];
    axis -= 3;
  } else if ((tmin[1] >= tmin[0]) && (tmin[1] >= tmin[2])) {
    rtmin = tmin[1];
    va[1] = vb[1] = lo[1];
    axis -= 1;
  } else {
    rtmin = tmin[2];
    va[2] = vb[2] = lo[2];
    axis -= 2;
  }
  if (axis < 0) axis += 3;
  if (rtmin <= rtmax) {
    const float dvec[3] = {hi[0] - r.org[0], hi[1] - r.org[1], hi[2] - r.org[2]};
    *r_depth = dot3(dvec, r.dir);
    return 0.0f;
  }
  if (r.dir[axis] >= 0.0f) {
    va[axis] = lo[axis];
    vb[axis] = hi[axis];
  } else {
    va[axis] = hi[axis];
    vb[axis] = lo[axis];
  }
  return ray_seg_dist_sq(r.org, r.dir, va, vb, r_depth);
}

// Key of a squared distance (any sign; NaN has none): the float order as an
// unsigned order, -0 as +0 (they compare equal), then the prim position.
__device__ __forceinline__ unsigned long long dist_key(float dist, int pos) {
  unsigned int bits = __float_as_uint(dist);
  if (bits == 0x80000000u) bits = 0u;
  bits = (bits & 0x80000000u) ? ~bits : (bits | 0x80000000u);
  return (static_cast<unsigned long long>(bits) << 32) | static_cast<unsigned int>(pos);
}
__device__ __forceinline__ float key_dist(unsigned long long key) {
  unsigned int bits = static_cast<unsigned int>(key >> 32);
  bits = (bits & 0x80000000u) ? (bits & 0x7fffffffu) : ~bits;
  return __uint_as_float(bits);
}

__device__ __forceinline__ float len_sq(float3 a, float3 b) {
  const float d0 = a.x - b.x, d1 = a.y - b.y, d2 = a.z - b.z;
  return d0 * d0 + d1 * d1 + d2 * d2;
}

// Units per leaf: looptris (FACES) or grid quads (GRIDS).
__device__ __forceinline__ int leaf_units(const DevMesh& m, int leaf) {
  const int n = m.leaf_prim_off[leaf + 1] - m.leaf_prim_off[leaf];
  return m.type == kFaces ? n : n * (m.grid_size - 1) * (m.grid_size - 1);
}

// Corners of grid quad `unit` of a leaf: (x, y), (x+1, y), (x+1, y+1),
// (x, y+1) as pbvh_grids_node_raycast orders them.
struct GridQuad {
  int grid, x, y;
  float3 c[4];
};

__device__ __forceinline__ GridQuad grid_quad(const DevMesh& m, int leaf, int unit) {
  const int g1 = m.grid_size - 1, nq = g1 * g1, gs = m.grid_size;
  GridQuad q;
  q.grid = m.leaf_prims[m.leaf_prim_off[leaf] + unit / nq];
  const int r = unit % nq;
  q.y = r / g1;
  q.x = r % g1;
  const float4* base = m.co + static_cast<size_t>(q.grid) * m.grid_area;
  q.c[0] = xyz(__ldcg(&base[q.y * gs + q.x]));
  q.c[1] = xyz(__ldcg(&base[q.y * gs + q.x + 1]));
  q.c[2] = xyz(__ldcg(&base[(q.y + 1) * gs + q.x + 1]));
  q.c[3] = xyz(__ldcg(&base[(q.y + 1) * gs + q.x]));
  return q;
}

// Block-wide exclusive scan of ints (kRayThreads threads).
__device__ int ray_block_scan(int v, int* total, int* smem32) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  constexpr int nwarps = kRayThreads / 32;
  int x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) smem32[warp] = x;
  __syncthreads();
  if (warp == 0) {
    int w = lane < nwarps ? smem32[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    smem32[lane] = w;
  }
  __syncthreads();
  const int base = warp > 0 ? smem32[warp - 1] : 0;
  *total = smem32[nwarps - 1];
  __syncthreads();
  return base + x - v;
}

// Dynamic shared memory: node pass flags (char), node tmin and parents (4 B
// each), listed leaves' tmin (float).
template <bool kNear>
__global__ void __launch_bounds__(kRayThreads) k_ray_leaves(DevMesh m, RayBatch rb) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ int scan[32];
  __shared__ int s_count;
  const int ray = blockIdx.x;
  const int N = m.totnode, L = m.nleaf;
  float* s_t = reinterpret_cast<float*>(smem);
  int* s_par = reinterpret_cast<int*>(s_t + N);
  float* s_lt = reinterpret_cast<float*>(s_par + N);
  unsigned char* s_pass = reinterpret_cast<unsigned char*>(s_lt + L);
  float o[3], d[3];
#pragma unroll
  for (int k = 0; k < 3; k++) {
    o[k] = rb.rays[6 * ray + k];
    d[k] = rb.rays[6 * ray + 3 + k];
  }
  const float4* bb = rb.original ? m.orig_vb : m.vb;
  if constexpr (kNear) {
    // nearest_to_ray_aabb_dist_sq: tmin = squared distance, pass when the
    // nearest point's depth is positive
    RayAabb ra;
    rayaabb_init(ra, o, d);
    for (int n = threadIdx.x; n < N; n += kRayThreads) {
      float dep = 0.0f;
      s_t[n] = rayaabb_dist_sq(ra, __ldcg(&bb[2 * n]), __ldcg(&bb[2 * n + 1]), &dep);
      s_pass[n] = dep > 0.0f;
      s_par[n] = m.node_parent[n];
    }
  } else {
    RayBox box;
    raybox_init(box, o, d);
    for (int n = threadIdx.x; n < N; n += kRayThreads) {
      float t = 0.0f;
      s_pass[n] = raybox_hit(box, __ldcg(&bb[2 * n]), __ldcg(&bb[2 * n + 1]), &t);
      s_t[n] = t;
      s_par[n] = m.node_parent[n];
    }
  }
  __syncthreads();
  // pbvh_iter_next_occluded: a leaf is listed when it and all its ancestors
  // pass; a NaN entry distance never passes the callback's test
  const int seg = (L + kRayThreads - 1) / kRayThreads;
  const int l0 = min(L, static_cast<int>(threadIdx.x) * seg), l1 = min(L, l0 + seg);
  int mine = 0;
  for (int id = l0; id < l1; id++) {
    const int node = m.leaf_node[id];
    bool ok = s_pass[node] && !isnan(s_t[node]);
    for (int p = s_par[node]; ok && p >= 0; p = s_par[p]) ok = s_pass[p];
    mine += ok;
  }
  int total;
  int pos = ray_block_scan(mine, &total, scan);
  int* slot_leaf = rb.slot_leaf + static_cast<size_t>(ray) * L;
  float* slot_tmin = rb.slot_tmin + static_cast<size_t>(ray) * L;
  for (int id = l0; id < l1; id++) {
    const int node = m.leaf_node[id];
    bool ok = s_pass[node] && !isnan(s_t[node]);
    for (int p = s_par[node]; ok && p >= 0; p = s_par[p]) ok = s_pass[p];
    if (!ok) continue;
    slot_leaf[pos] = id;
    slot_tmin[pos] = s_t[node];
    s_lt[pos] = s_t[node];
    pos++;
  }
  if (threadIdx.x == 0) {
    rb.count[ray] = total;
    s_count = total;
  }
  __syncthreads();
  // processing order: stable by tmin (the reference's tree, ties after the
  // earlier DFS leaf)
  int* order = rb.slot_order + static_cast<size_t>(ray) * L;
  unsigned long long* key = rb.slot_key + static_cast<size_t>(ray) * L;
  for (int i = threadIdx.x; i < total; i += kRayThreads) {
    const float ti = s_lt[i];
    int rank = 0;
    for (int j = 0; j < total; j++) {
      const float tj = s_lt[j];
      rank += (tj < ti) || (tj == ti && j < i);
    }
    order[rank] = i;
    key[i] = kNoKey;
    rb.slot_special[static_cast<size_t>(ray) * L + i] = 0;
  }
  __syncthreads();
  // round-0 work items: (ray-slot, chunk of kRayChunk units) of the first
  // leaves in entry order
  if (threadIdx.x == 0) {
    const int first = min(total, rb.first_leaves);
    int nch = 0;
    for (int r = 0; r < first; r++)
      nch += (leaf_units(m, slot_leaf[order[r]]) + kRayChunk - 1) / kRayChunk;
    const int base = atomicAdd(rb.nitems, nch);
    if (base + nch > rb.item_cap) {
      atomicCAS(&m.work->err, 0, 5 /* SGPU_ERR_BOUNDS */);
    } else {
      int at = base;
      for (int r = 0; r < first; r++) {
        const int sl = order[r];
        const int c = (leaf_units(m, slot_leaf[sl]) + kRayChunk - 1) / kRayChunk;
        for (int k = 0; k < c; k++) rb.items[at++] = make_int2(ray * L + sl, k);
      }
    }
  }
}

template <bool kNear>
__global__ void __launch_bounds__(kRayThreads) k_ray_tris(DevMesh m, RayBatch rb, int round) {
  __shared__ unsigned long long s_min[kRayThreads / 32];
  const int L = m.nleaf;
  const int2* items = round == 0 ? rb.items : rb.items2;
  const int total = __ldcg(round == 0 ? rb.nitems : rb.nitems2);
  for (int it = blockIdx.x; it < total; it += gridDim.x) {
    const int2 item = items[it];
    const int ray = item.x / L;
    float o[3], d[3];
#pragma unroll
    for (int k = 0; k < 3; k++) {
      o[k] = rb.rays[6 * ray + k];
      d[k] = rb.rays[6 * ray + 3 + k];
    }
    const int leaf = rb.slot_leaf[item.x];
    const int pos = item.y * kRayChunk + static_cast<int>(threadIdx.x);
    unsigned long long key = kNoKey;
    if (kNear && pos < leaf_units(m, leaf)) {
      if (m.type == kFaces) {
        const int4 tv = m.lt_v4[m.leaf_prims[m.leaf_prim_off[leaf] + pos]];
        float dt;
        const float dd = ray_tri_dist_sq(o, d, xyz(__ldcg(&m.co[tv.x])), xyz(__ldcg(&m.co[tv.y])),
                                         xyz(__ldcg(&m.co[tv.z])), &dt);
        if (!isnan(dd)) key = dist_key(dd, pos);
      } else if (pos == 0) {
        rb.slot_special[item.x] = 1;  // GRIDS: every leaf is replayed in order
      }
    } else if (pos < leaf_units(m, leaf)) {
      RayTri rt;
      raytri_init(rt, d);
      if (m.type == kFaces) {
        const int4 tv = m.lt_v4[m.leaf_prims[m.leaf_prim_off[leaf] + pos]];
        const float3 c0 = xyz(__ldcg(&m.co[tv.x])), c1 = xyz(__ldcg(&m.co[tv.y])),
                     c2 = xyz(__ldcg(&m.co[tv.z]));
        float depth;
        if (raytri_hit(o, rt, c0, c1, c2, &depth)) key = depth_key(depth, pos);
      } else {
        const GridQuad q = grid_quad(m, leaf, pos);
        float da = 0.0f, db = 0.0f;
        const bool ha = raytri_hit(o, rt, q.c[0], q.c[1], q.c[2], &da);
        const bool hb = raytri_hit(o, rt, q.c[0], q.c[2], q.c[3], &db);
        if (ha && hb && db < da) {
          rb.slot_special[item.x] = 1;  // the leaf is replayed in order
        } else if (ha) {
          key = depth_key(da, pos);
        } else if (hb) {
          key = depth_key(db, pos);
        }
      }
    }
#pragma unroll
    for (int s = 16; s >= 1; s >>= 1) {
      const unsigned long long other = __shfl_xor_sync(0xffffffffu, key, s);
      key = other < key ? other : key;
    }
    if ((threadIdx.x & 31) == 0) s_min[threadIdx.x >> 5] = key;
    __syncthreads();
    if (threadIdx.x == 0) {
      unsigned long long k = s_min[0];
      for (int w = 1; w < kRayThreads / 32; w++) k = s_min[w] < k ? s_min[w] : k;
      if (k != kNoKey) atomicMin(&rb.slot_key[item.x], k);
    }
    __syncthreads();
  }
}

// The winning triangle's exact depth, its normal, the active vertex (corner
// nearest the hit, first among equals) and face; one thread.
__device__ void ray_write_result(const DevMesh& m, const RayBatch& rb, int ray, const float* o,
                                 const float* d, const RayTri& rt, float depth, int win_slot,
                                 int win_pos, int win_tri) {
  const size_t base = static_cast<size_t>(ray) * m.nleaf;
  float fn[3] = {0.0f, 0.0f, 0.0f};
  int av = -1, af = -1;
  if (win_slot >= 0) {
    const int leaf = rb.slot_leaf[base + win_slot];
    if (m.type == kFaces) {
      const int4 tv = m.lt_v4[m.leaf_prims[m.leaf_prim_off[leaf] + win_pos]];
      const float3 c[3] = {xyz(__ldcg(&m.co[tv.x])), xyz(__ldcg(&m.co[tv.y])),
                           xyz(__ldcg(&m.co[tv.z]))};
      float dt = depth;
      raytri_hit(o, rt, c[0], c[1], c[2], &dt);  // the exact value (-0 kept)
      depth = dt;
      const float3 n = normal_tri(c[0], c[1], c[2]);
      fn[0] = n.x, fn[1] = n.y, fn[2] = n.z;
      const float3 loc = make_float3(o[0] + d[0] * depth, o[1] + d[1] * depth, o[2] + d[2] * depth);
      float3 nearest = c[0];
      int best = 0;
      for (int j = 1; j < 3; j++)
        if (len_sq(loc, c[j]) < len_sq(loc, nearest)) {
          nearest = c[j];
          best = j;
        }
      const int id = best == 0 ? tv.x : (best == 1 ? tv.y : tv.z);
      av = rb.n2o ? rb.n2o[id] : id;
      af = tv.w;
    } else {
      const GridQuad q = grid_quad(m, leaf, win_pos);
      float da = depth, db = depth;
      const bool ha = raytri_hit(o, rt, q.c[0], q.c[1], q.c[2], &da);
      raytri_hit(o, rt, q.c[0], q.c[2], q.c[3], &db);
      // the taken triangle: from the in-order replay, or for a minimum-key
      // leaf the first triangle when it meets the ray
      const int tri = win_tri >= 0 ? win_tri : (ha ? 0 : 1);
      depth = tri == 0 ? da : db;
      const float3 n = normal_quad(q.c[0], q.c[1], q.c[2], q.c[3]);
      fn[0] = n.x, fn[1] = n.y, fn[2] = n.z;
      const float3 loc = make_float3(o[0] + d[0] * depth, o[1] + d[1] * depth, o[2] + d[2] * depth);
      float3 nearest = q.c[0];
      int best = 0;
      for (int j = 1; j < 4; j++)
        if (len_sq(loc, q.c[j]) < len_sq(loc, nearest)) {
          nearest = q.c[j];
          best = j;
        }
      // corner j of the quad is (x + {0,1,1,0}[j], y + {0,0,1,1}[j])
      const int xi = best == 1 || best == 2, yi = best >= 2;
      av = m.grid_area * q.grid + (q.y + yi) * m.grid_size + (q.x + xi);
      af = q.grid;
    }
  }
  rb.depth_out[ray] = depth;
  rb.hit[ray] = win_slot >= 0;
  rb.active_vertex[ray] = av;
  rb.active_face[ray] = af;
  rb.face_normal[3 * ray] = fn[0];
  rb.face_normal[3 * ray + 1] = fn[1];
  rb.face_normal[3 * ray + 2] = fn[2];
}

// The nearest query's result: the winning triangle's squared distance and
// depth recomputed exactly (dist_squared_ray_to_tri_v3_fast; -0 kept); the
// squared distance goes to face_normal[3 * ray], no active vertex or face.
__device__ void ray_write_near(const DevMesh& m, const RayBatch& rb, int ray, const float* o,
                               const float* d, float dist_sq, int win_slot, int win_pos,
                               int win_tri) {
  float depth = FLT_MAX;
  if (win_slot >= 0) {
    const int leaf = rb.slot_leaf[static_cast<size_t>(ray) * m.nleaf + win_slot];
    if (m.type == kFaces) {
      const int4 tv = m.lt_v4[m.leaf_prims[m.leaf_prim_off[leaf] + win_pos]];
      dist_sq = ray_tri_dist_sq(o, d, xyz(__ldcg(&m.co[tv.x])), xyz(__ldcg(&m.co[tv.y])),
                                xyz(__ldcg(&m.co[tv.z])), &depth);
    } else {
      const GridQuad q = grid_quad(m, leaf, win_pos);
      dist_sq = win_tri == 0 ? ray_tri_dist_sq(o, d, q.c[0], q.c[1], q.c[2], &depth)
                             : ray_tri_dist_sq(o, d, q.c[0], q.c[2], q.c[3], &depth);
    }
  }
  rb.depth_out[ray] = depth;
  rb.hit[ray] = win_slot >= 0;
  rb.active_vertex[ray] = -1;
  rb.active_face[ray] = -1;
  rb.face_normal[3 * ray] = dist_sq;
  rb.face_normal[3 * ray + 1] = 0.0f;
  rb.face_normal[3 * ray + 2] = 0.0f;
}

// One CTA per ray.  Round 0 walks the first first_leaves leaves in entry
// order, then either settles the ray (its next leaf would not be cast) or
// saves the state and lists the remaining leaves' work items; round 1 walks
// those for the unsettled rays.  Dynamic shared memory: per listed leaf its
// order entry, tmin and key.
// kNear: s_depth is the running squared distance, keys decode with key_dist.
template <bool kNear>
__global__ void __launch_bounds__(kRayThreads) k_ray_finish(DevMesh m, RayBatch rb, int round) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ float s_da[kRayThreads], s_db[kRayThreads];
  __shared__ unsigned char s_ha[kRayThreads], s_hb[kRayThreads];
  __shared__ unsigned s_mask[kRayThreads / 32];
  __shared__ int scan[32];
  __shared__ float s_depth, s_run_tmin;
  __shared__ int s_slot, s_cast, s_special, s_win_slot, s_win_pos, s_win_tri, s_leaf_hit;
  const int ray = blockIdx.x;
  const int L = m.nleaf;
  int k0 = 0;
  if (round == 1) {
    k0 = __ldcg(&rb.st_win[ray].w);
    if (k0 < 0) return;  // settled in round 0 (uniform over the CTA)
  }
  const int cnt = rb.count[ray];
  const int k1 = round == 0 ? min(cnt, rb.first_leaves) : cnt;
  unsigned long long* s_key = reinterpret_cast<unsigned long long*>(smem);
  float* s_tmin = reinterpret_cast<float*>(s_key + L);
  int* s_order = reinterpret_cast<int*>(s_tmin + L);
  const size_t base = static_cast<size_t>(ray) * L;
  if (threadIdx.x == 0) {
    if (round == 0) {
      s_run_tmin = FLT_MAX;
      s_depth = rb.depth_in ? rb.depth_in[ray] : FLT_MAX;
      s_win_slot = s_win_pos = s_win_tri = -1;
    } else {
      const int4 w = __ldcg(&rb.st_win[ray]);
      s_run_tmin = __ldcg(&rb.st_run[ray]);
      s_depth = __ldcg(&rb.st_depth[ray]);
      s_win_slot = w.x;
      s_win_pos = w.y;
      s_win_tri = w.z;
    }
  }
  for (int i = threadIdx.x; i < cnt; i += kRayThreads) {
    s_key[i] = __ldcg(&rb.slot_key[base + i]);
    s_tmin[i] = rb.slot_tmin[base + i];
    s_order[i] = rb.slot_order[base + i];
  }
  __syncthreads();
  int special = 0;
  if (m.type == kGrids)
    for (int k = k0 + static_cast<int>(threadIdx.x); k < k1; k += kRayThreads)
      special |= __ldcg(&rb.slot_special[base + s_order[k]]);
  float o[3], d[3];
#pragma unroll
  for (int k = 0; k < 3; k++) {
    o[k] = rb.rays[6 * ray + k];
    d[k] = rb.rays[6 * ray + 3 + k];
  }
  RayTri rt;
  raytri_init(rt, d);
  // traverse_tree with the callback: a leaf is cast when tmin < running
  // minimum; a hit inside it is taken when strictly closer than the depth
  int kr = k1;  // leaves walked by the whole CTA
  if (!__syncthreads_or(special)) {
    // every leaf of the range reduces to its minimum key: one thread walks them
    if (threadIdx.x == 0) {
      float run_tmin = s_run_tmin, depth = s_depth;
      int win_slot = s_win_slot, win_pos = s_win_pos, win_tri = s_win_tri;
      for (int k = k0; k < k1; k++) {
        const int sl = s_order[k];
        if (!(s_tmin[sl] < run_tmin)) continue;
        const unsigned long long key = s_key[sl];
        if (key == kNoKey) continue;
        const float dmin = kNear ? key_dist(key) : __uint_as_float(static_cast<unsigned int>(key >> 32));
        if (dmin < depth) {
          depth = dmin;
          win_slot = sl;
          win_pos = static_cast<int>(key & 0xffffffffu);
          win_tri = -1;
          run_tmin = depth;
        }
      }
      s_depth = depth;
      s_run_tmin = run_tmin;
      s_win_slot = win_slot;
      s_win_pos = win_pos;
      s_win_tri = win_tri;
    }
    kr = k0;
  }
  for (int k = k0; k < kr; k++) {
    __syncthreads();
    if (threadIdx.x == 0) {
      const int sl = s_order[k];
      s_slot = sl;
      s_cast = s_tmin[sl] < s_run_tmin;
      s_special = m.type == kGrids && __ldcg(&rb.slot_special[base + sl]);
      s_leaf_hit = 0;
    }
    __syncthreads();
    if (!s_cast) continue;
    const int sl = s_slot;
    if (!s_special) {
      // the leaf's closest hit: taken when strictly below the depth
      if (threadIdx.x == 0) {
        const unsigned long long key = s_key[sl];
        if (key != kNoKey) {
          const float dmin = kNear ? key_dist(key) : __uint_as_float(static_cast<unsigned int>(key >> 32));
          if (dmin < s_depth) {
            s_depth = dmin;
            s_win_slot = sl;
            s_win_pos = static_cast<int>(key & 0xffffffffu);
            s_win_tri = -1;  // decided below
            s_run_tmin = dmin;
          }
        }
      }
      continue;
    }
    const int leaf = rb.slot_leaf[base + sl];
    const int units = leaf_units(m, leaf);
    if constexpr (kNear) {
      // GRIDS: ray_face_nearest_quad quad by quad; quads whose first triangle
      // is not below the value at the chunk's start are never taken
      for (int c0 = 0; c0 < units; c0 += kRayThreads) {
        const int u = c0 + static_cast<int>(threadIdx.x);
        float d1 = FLT_MAX, d2 = FLT_MAX, dep = 0.0f;
        if (u < units) {
          const GridQuad q = grid_quad(m, leaf, u);
          d1 = ray_tri_dist_sq(o, d, q.c[0], q.c[1], q.c[2], &dep);
          d2 = ray_tri_dist_sq(o, d, q.c[0], q.c[2], q.c[3], &dep);
        }
        s_da[threadIdx.x] = d1;
        s_db[threadIdx.x] = d2;
        const unsigned bal = __ballot_sync(0xffffffffu, u < units && d1 < s_depth);
        if ((threadIdx.x & 31) == 0) s_mask[threadIdx.x >> 5] = bal;
        __syncthreads();
        if (threadIdx.x == 0) {
          float cur = s_depth;
          for (int w = 0; w < kRayThreads / 32; w++) {
            for (unsigned b = s_mask[w]; b; b &= b - 1) {
              const int t = 32 * w + __ffs(static_cast<int>(b)) - 1;
              if (!(s_da[t] < cur)) continue;
              cur = s_da[t];
              s_win_tri = 0;
              if (s_db[t] < cur) {
                cur = s_db[t];
                s_win_tri = 1;
              }
              s_win_slot = sl;
              s_win_pos = c0 + t;
              s_leaf_hit = 1;
            }
          }
          s_depth = cur;
        }
        __syncthreads();
      }
      if (threadIdx.x == 0 && s_leaf_hit) s_run_tmin = s_depth;
      continue;
    }
    // GRIDS leaf with a folded quad: ray_face_intersection_quad quad by quad
    for (int c0 = 0; c0 < units; c0 += kRayThreads) {
      const int u = c0 + static_cast<int>(threadIdx.x);
      bool ha = false, hb = false;
      float da = 0.0f, db = 0.0f;
      if (u < units) {
        const GridQuad q = grid_quad(m, leaf, u);
        ha = raytri_hit(o, rt, q.c[0], q.c[1], q.c[2], &da);
        hb = raytri_hit(o, rt, q.c[0], q.c[2], q.c[3], &db);
      }
      s_ha[threadIdx.x] = ha;
      s_hb[threadIdx.x] = hb;
      s_da[threadIdx.x] = da;
      s_db[threadIdx.x] = db;
      // quads meeting the ray, one bit per thread; the rule visits only those
      const unsigned bal = __ballot_sync(0xffffffffu, ha || hb);
      if ((threadIdx.x & 31) == 0) s_mask[threadIdx.x >> 5] = bal;
      __syncthreads();
      if (threadIdx.x == 0) {
        float dep = s_depth;
        for (int w = 0; w < kRayThreads / 32; w++) {
          for (unsigned b = s_mask[w]; b; b &= b - 1) {
            const int t = 32 * w + __ffs(static_cast<int>(b)) - 1;
            if (s_ha[t] && s_da[t] < dep) {
              dep = s_da[t];
              s_win_tri = 0;
            } else if (s_hb[t] && s_db[t] < dep) {
              dep = s_db[t];
              s_win_tri = 1;
            } else {
              continue;
            }
            s_win_slot = sl;
            s_win_pos = c0 + t;
            s_leaf_hit = 1;
          }
        }
        s_depth = dep;
      }
      __syncthreads();
    }
    if (threadIdx.x == 0 && s_leaf_hit) s_run_tmin = s_depth;
  }
  __syncthreads();
  if (round == 0 && k1 < cnt && s_tmin[s_order[k1]] < s_run_tmin) {
    // the next leaf would be cast: keep the state, list the remaining leaves
    if (threadIdx.x == 0) {
      rb.st_depth[ray] = s_depth;
      rb.st_run[ray] = s_run_tmin;
      rb.st_win[ray] = make_int4(s_win_slot, s_win_pos, s_win_tri, k1);
    }
    int nch = 0;
    for (int k = k1 + static_cast<int>(threadIdx.x); k < cnt; k += kRayThreads)
      nch += (leaf_units(m, rb.slot_leaf[base + s_order[k]]) + kRayChunk - 1) / kRayChunk;
    int all;
    int off = ray_block_scan(nch, &all, scan);
    if (threadIdx.x == 0) scan[0] = atomicAdd(rb.nitems2, all);
    __syncthreads();
    const int at = scan[0];
    if (at + all > rb.item_cap) {
      if (threadIdx.x == 0) atomicCAS(&m.work->err, 0, 5 /* SGPU_ERR_BOUNDS */);
      return;
    }
    for (int k = k1 + static_cast<int>(threadIdx.x); k < cnt; k += kRayThreads) {
      const int sl = s_order[k];
      const int c = (leaf_units(m, rb.slot_leaf[base + sl]) + kRayChunk - 1) / kRayChunk;
      for (int j = 0; j < c; j++) rb.items2[at + off + j] = make_int2(ray * L + sl, j);
      off += c;
    }
    return;
  }
  if (threadIdx.x != 0) return;
  if (round == 0) rb.st_win[ray] = make_int4(-1, -1, -1, -1);  // settled
  if constexpr (kNear) {
    ray_write_near(m, rb, ray, o, d, s_depth, s_win_slot, s_win_pos, s_win_tri);
  } else {
    ray_write_result(m, rb, ray, o, d, rt, s_depth, s_win_slot, s_win_pos, s_win_tri);
  }
}

}  // namespace

size_t ray_leaves_smem(const DevMesh& m) {
  return sizeof(float) * m.totnode + sizeof(int) * m.totnode + sizeof(float) * m.nleaf +
         static_cast<size_t>(m.totnode) + 16;
}
size_t ray_finish_smem(const DevMesh& m) {
  return (sizeof(unsigned long long) + sizeof(float) + sizeof(int)) * static_cast<size_t>(m.nleaf) + 16;
}
int ray_items_per_ray(const DevMesh& m) {
  if (m.type == kFaces) return m.totlt / kRayChunk + m.nleaf;
  const long long g1 = m.grid_size - 1;
  const long long units = static_cast<long long>(m.totvert / m.grid_area) * g1 * g1;
  return static_cast<int>(units / kRayChunk) + m.nleaf;
}

template <bool kNear>
static cudaError_t configure_ray_mode(size_t leaves_smem, size_t finish_smem) {
  cudaError_t e = cudaFuncSetAttribute(k_ray_leaves<kNear>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       static_cast<int>(leaves_smem));
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(k_ray_finish<kNear>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              static_cast<int>(finish_smem));
}

cudaError_t configure_ray_kernels(size_t leaves_smem, size_t finish_smem) {
  const cudaError_t e = configure_ray_mode<false>(leaves_smem, finish_smem);
  return e != cudaSuccess ? e : configure_ray_mode<true>(leaves_smem, finish_smem);
}

template <bool kNear>
static cudaError_t launch_ray_mode(const DevMesh& m, const RayBatch& rb, int nrays, int tris_grid,
                                   cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(rb.nitems, 0, sizeof(int), s);
  if (e == cudaSuccess) e = cudaMemsetAsync(rb.nitems2, 0, sizeof(int), s);
  if (e != cudaSuccess) return e;
  k_ray_leaves<kNear><<<nrays, kRayThreads, ray_leaves_smem(m), s>>>(m, rb);
  // every leaf in round 0 settles every ray there: no second round
  const int rounds = rb.first_leaves >= m.nleaf ? 1 : 2;
  for (int round = 0; round < rounds && e == cudaSuccess; round++) {
    e = cudaGetLastError();
    if (e != cudaSuccess) break;
    k_ray_tris<kNear><<<tris_grid, kRayThreads, 0, s>>>(m, rb, round);
    e = cudaGetLastError();
    if (e != cudaSuccess) break;
    k_ray_finish<kNear><<<nrays, kRayThreads, ray_finish_smem(m), s>>>(m, rb, round);
  }
  if (e != cudaSuccess) return e;
  return cudaGetLastError();
}

cudaError_t launch_raycast(const DevMesh& m, const RayBatch& rb, int nrays, int tris_grid,
                           cudaStream_t s) {
  return rb.nearest ? launch_ray_mode<true>(m, rb, nrays, tris_grid, s)
                    : launch_ray_mode<false>(m, rb, nrays, tris_grid, s);
}

}  // namespace sgpu
