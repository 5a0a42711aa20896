// PBVH_GRIDS normal update and seam stitching, per work item; shared by the
// per-call kernels (kernels_grids.cu) and the persistent stroke kernel.
//   grid_claim_face:     a face of a flagged leaf joins the update (once per
//                        epoch) with its grids, base edges and base vertices.
//   grid_element_normal: one element of a claimed grid — the mean of the
//                        normals of the quads around it (subdiv_ccg.c:670-740).
//   grid_face_seam_item: one face-internal seam pair or one face centre
//                        (:951-984), after every inner normal is done.
//   grid_seam_item:      one boundary element index of a base edge
//                        (:1010-1048) or one base-vertex corner (:1081-1104).
// The three element passes only depend on one another in that order: inner
// normals read positions of their own grid, seams and centres touch disjoint
// elements, and the base edges and corners come last, as the reference runs
// them after every face.
#pragma once

#include "sgpu_device.cuh"

namespace sgpu {

__device__ __forceinline__ bool grid_claim(unsigned int* mark, int i, unsigned int epoch) {
  return atomicExch(&mark[i], epoch) != epoch;
}

__device__ __forceinline__ void grid_claim_face(const DevMesh& m, int grid, unsigned int epoch) {
  const int f = m.grid_face[grid];
  if (!grid_claim(m.face_mark, f, epoch)) return;
  m.face_list[atomicAdd(&m.grid_counts[0], 1)] = f;
  const int s = m.face_start[f], n = m.face_ngrids[f];
  const int gb = atomicAdd(&m.grid_counts[3], n);
  for (int c = 0; c < n; c++) m.cgrid_list[gb + c] = s + c;
  for (int c = 0; c < n; c++) {
    const int e = m.face_edges[s + c];
    const int v = m.face_verts[s + c];
    if (grid_claim(m.edge_mark, e, epoch)) m.edge_list[atomicAdd(&m.grid_counts[1], 1)] = e;
    if (grid_claim(m.bvert_mark, v, epoch)) m.bvert_list[atomicAdd(&m.grid_counts[2], 1)] = v;
  }
}

// Owner key of a claimed face in an epoch: newer epochs and smaller faces
// compare smaller.
__device__ __forceinline__ unsigned long long grid_owner_key(unsigned int epoch, int f) {
  return (static_cast<unsigned long long>(0xFFFFFFFFu - epoch) << 32) | static_cast<unsigned int>(f);
}

// The face of a grid joins the update (persistent kernel): the face and its
// grids are listed; its base edges and corners are not — each is averaged
// once, by the claimed face of least index among its faces, recorded here
// with a 64-bit minimum per edge and base vertex.
__device__ __forceinline__ void grid_claim_face_only(const DevMesh& m, int grid, unsigned int epoch) {
  // the face, its first grid and its size in one load; the corners' edges and
  // vertices are loaded alongside the claim's round trip
  const int4 gi = m.grid_info[grid];
  const int f = gi.x, s = gi.y, n = gi.z;
  if (!grid_claim(m.face_mark, f, epoch)) return;
  const int fi = atomicAdd(&m.grid_counts[0], 1);
  const int gb = atomicAdd(&m.grid_counts[3], n);
  const unsigned long long key = grid_owner_key(epoch, f);
  for (int c0 = 0; c0 < n; c0 += 4) {
    int e[4], v[4];
#pragma unroll
    for (int u = 0; u < 4; u++)
      if (c0 + u < n) {
        e[u] = m.face_edges[s + c0 + u];
        v[u] = m.face_verts[s + c0 + u];
      }
#pragma unroll
    for (int u = 0; u < 4; u++)
      if (c0 + u < n) {
        atomicMin(&m.edge_own[e[u]], key);
        atomicMin(&m.bvert_own[v[u]], key);
      }
  }
  m.face_list[fi] = f;
  m.face_info[fi] = make_int2(s, n);
  for (int c = 0; c < n; c++) m.cgrid_list[gb + c] = s + c;
}

// average_grid_element, subdiv_ccg.c:883-901
__device__ __forceinline__ void grid_avg_pair(const DevMesh& m, int a, int b) {
  const float4 ca = __ldcg(&m.co[a]), cb = __ldcg(&m.co[b]);
  const float4 na = __ldcg(&m.no[a]), nb = __ldcg(&m.no[b]);
  float4 c, n;
  c.x = (ca.x + cb.x) * 0.5f;
  c.y = (ca.y + cb.y) * 0.5f;
  c.z = (ca.z + cb.z) * 0.5f;
  c.w = ca.w;
  n.x = (na.x + nb.x) * 0.5f;
  n.y = (na.y + nb.y) * 0.5f;
  n.z = (na.z + nb.z) * 0.5f;
  n.w = 0.0f;
  m.co[a] = c;
  m.co[b] = c;
  m.no[a] = n;
  m.no[b] = n;
  if (m.mask) {
    const float mk = (__ldcg(&m.mask[a]) + __ldcg(&m.mask[b])) * 0.5f;
    m.mask[a] = mk;
    m.mask[b] = mk;
  }
}

// Averages co, no and mask over els[0..n) (in order) and stores the mean in
// every one of them (GridElementAccumulator, subdiv_ccg.c:903-949).
// Up to kAvgBatch copies (base edges: 2, quad-mesh corners: 4): every
// element index loaded first, then the copies' values (summed in copy
// order); the mean's positions are written as three scalars, so a copy's
// fourth component stays as it is without being read again.
constexpr int kAvgBatch = 4;
template <class ElemAt>
__device__ __forceinline__ void grid_average_set(const DevMesh& m, int n, ElemAt el) {
  float cx = 0.0f, cy = 0.0f, cz = 0.0f, nx = 0.0f, ny = 0.0f, nz = 0.0f, mk = 0.0f;
  if (n <= kAvgBatch) {
    int e[kAvgBatch];
#pragma unroll
    for (int f = 0; f < kAvgBatch; f++) e[f] = f < n ? el(f) : 0;
#pragma unroll
    for (int f = 0; f < kAvgBatch; f++)
      if (f < n) {
        const float4 co = __ldcg(&m.co[e[f]]), no = __ldcg(&m.no[e[f]]);
        cx += co.x, cy += co.y, cz += co.z;
        nx += no.x, ny += no.y, nz += no.z;
        if (m.mask) mk += __ldcg(&m.mask[e[f]]);
      }
    const float inv = 1.0f / (float)n;
    cx *= inv, cy *= inv, cz *= inv;
    nx *= inv, ny *= inv, nz *= inv;
    mk *= inv;
#pragma unroll
    for (int f = 0; f < kAvgBatch; f++)
      if (f < n) {
        float* c = reinterpret_cast<float*>(&m.co[e[f]]);
        c[0] = cx;
        c[1] = cy;
        c[2] = cz;
        m.no[e[f]] = make_float4(nx, ny, nz, 0.0f);
        if (m.mask) m.mask[e[f]] = mk;
      }
    return;
  }
  for (int f = 0; f < n; f++) {
    const int e = el(f);
    const float4 co = __ldcg(&m.co[e]), no = __ldcg(&m.no[e]);
    cx += co.x, cy += co.y, cz += co.z;
    nx += no.x, ny += no.y, nz += no.z;
    if (m.mask) mk += __ldcg(&m.mask[e]);
  }
  const float inv = 1.0f / (float)n;
  cx *= inv, cy *= inv, cz *= inv;
  nx *= inv, ny *= inv, nz *= inv;
  mk *= inv;
  for (int f = 0; f < n; f++) {
    const int e = el(f);
    const float4 old = __ldcg(&m.co[e]);
    m.co[e] = make_float4(cx, cy, cz, old.w);
    m.no[e] = make_float4(nx, ny, nz, 0.0f);
    if (m.mask) m.mask[e] = mk;
  }
}

// 1 / counter for the 1, 2 or 4 quads around a grid element (3 cannot occur
// in a grid; kept for completeness): the correctly rounded quotients of the
// division the element normal is defined with, without the division.
__device__ __forceinline__ float inv_count(int counter) {
  return counter == 4 ? 0.25f : counter == 2 ? 0.5f : counter == 1 ? 1.0f : 1.0f / 3.0f;
}

// Normal of element (x, y) of the grid starting at element base: the mean of
// the normals of the quads around it, added in the order of
// subdiv_ccg.c:707-737.  Quad (qx, qy) has corners (qx, qy+1), (qx+1, qy+1),
// (qx+1, qy), (qx, qy); its normal is the same normal_quad value whichever
// element evaluates it.
__device__ __forceinline__ float4 grid_element_normal(const DevMesh& m, int base, int x, int y) {
  const int gs = m.grid_size, g1 = gs - 1;
  float3 p[3][3];  // p[dy + 1][dx + 1] = position of (x + dx, y + dy)
#pragma unroll
  for (int dy = -1; dy <= 1; dy++)
#pragma unroll
    for (int dx = -1; dx <= 1; dx++) {
      const int xx = x + dx, yy = y + dy;
      p[dy + 1][dx + 1] = (xx >= 0 && xx < gs && yy >= 0 && yy < gs)
                              ? xyz(__ldcg(&m.co[base + yy * gs + xx]))
                              : make_float3(0.0f, 0.0f, 0.0f);
    }
  // quad with lower corner (x + ox, y + oy), ox, oy in {-1, 0}
  auto quad = [&](int ox, int oy) {
    return normal_quad(p[oy + 2][ox + 1], p[oy + 2][ox + 2], p[oy + 1][ox + 2], p[oy + 1][ox + 1]);
  };
  float ax = 0.0f, ay = 0.0f, az = 0.0f;
  int counter = 0;
  if (x < g1 && y < g1) {
    const float3 q = quad(0, 0);
    ax += q.x, ay += q.y, az += q.z;
    counter++;
  }
  if (x >= 1) {
    if (y < g1) {
      const float3 q = quad(-1, 0);
      ax += q.x, ay += q.y, az += q.z;
      counter++;
    }
    if (y >= 1) {
      const float3 q = quad(-1, -1);
      ax += q.x, ay += q.y, az += q.z;
      counter++;
    }
  }
  if (y >= 1 && x < g1) {
    const float3 q = quad(0, -1);
    ax += q.x, ay += q.y, az += q.z;
    counter++;
  }
  const float inv = inv_count(counter);
  return make_float4(ax * inv, ay * inv, az * inv, 0.0f);
}

// Inner-normal item it < ng * area: element it % area of claimed grid it / area.
__device__ __forceinline__ void grid_inner_item(const DevMesh& m, long long it) {
  const int area = m.grid_area, gs = m.grid_size;
  const int g = __ldcg(&m.cgrid_list[it / area]);
  const int e = static_cast<int>(it % area);
  m.no[g * area + e] = grid_element_normal(m, g * area, e % gs, e / gs);
}

// Face-seam item: it < ng * (gs-1) pairs element (i, 0) of the previous grid
// of the face with (0, i) of the claimed grid, i = 1 + it % (gs-1); the rest
// are face centres, element (0, 0) of every grid of the face.
__device__ __forceinline__ void grid_face_seam_item(const DevMesh& m, long long it, int ng) {
  const int gs = m.grid_size, g1 = gs - 1, area = m.grid_area;
  const long long pairs = (long long)ng * g1;
  if (it < pairs) {
    const int g = __ldcg(&m.cgrid_list[it / g1]);
    const int i = 1 + static_cast<int>(it % g1);
    const int f = m.grid_face[g];
    const int s = m.face_start[f], n = m.face_ngrids[f];
    const int prev = s + (g - s + n - 1) % n;
    grid_avg_pair(m, prev * area + i, g * area + i * gs);
  } else {
    const int f = __ldcg(&m.face_list[it - pairs]);
    const int s = m.face_start[f], n = m.face_ngrids[f];
    grid_average_set(m, n, [&](int c) { return (s + c) * area; });
  }
}

// One seam item: it < ne*(2gs-2) is (edge, boundary index 1..2gs-2), the rest
// are base vertices.
__device__ __forceinline__ void grid_seam_item(const DevMesh& m, long long it, int ne) {
  const int g2 = 2 * m.grid_size, inner = g2 - 2;
  const long long edge_items = (long long)ne * inner;
  if (it < edge_items) {
    const int e = m.edge_list[it / inner];
    const int i = 1 + (int)(it % inner);
    const int f0 = m.edge_off[e], f1 = m.edge_off[e + 1];
    if (f1 - f0 == 1) return;
    grid_average_set(m, f1 - f0, [&](int k) { return m.edge_elems[(long long)(f0 + k) * g2 + i]; });
  } else {
    const int v = m.bvert_list[it - edge_items];
    const int f0 = m.bvert_off[v], f1 = m.bvert_off[v + 1];
    if (f1 - f0 == 1) return;
    grid_average_set(m, f1 - f0, [&](int k) { return m.bvert_elems[f0 + k]; });
  }
}

}  // namespace sgpu
