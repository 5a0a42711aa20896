// PBVH_GRIDS normal update and seam stitching, per work item; shared by the
// per-call kernels (kernels_grids.cu) and the persistent stroke kernel.
//   grid_claim_face:   a face of a flagged leaf joins the update (once per epoch)
//                      with its base edges and base vertices.
//   grid_face_update:  one face by one CTA — inner quad normals and per-element
//                      averages of its grids (subdiv_ccg.c:670-740), then the
//                      face-internal seams and the shared centre (:951-984).
//   grid_seam_item:    one boundary element index of a base edge (:1010-1048)
//                      or one base-vertex corner (:1081-1104).
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
  for (int c = 0; c < n; c++) {
    const int e = m.face_edges[s + c];
    const int v = m.face_verts[s + c];
    if (grid_claim(m.edge_mark, e, epoch)) m.edge_list[atomicAdd(&m.grid_counts[1], 1)] = e;
    if (grid_claim(m.bvert_mark, v, epoch)) m.bvert_list[atomicAdd(&m.grid_counts[2], 1)] = v;
  }
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
template <class ElemAt>
__device__ __forceinline__ void grid_average_set(const DevMesh& m, int n, ElemAt el) {
  float cx = 0.0f, cy = 0.0f, cz = 0.0f, nx = 0.0f, ny = 0.0f, nz = 0.0f, mk = 0.0f;
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

// One face, the whole CTA; fn: shared memory for 3*(gs-1)^2 floats.
__device__ inline void grid_face_update(const DevMesh& m, int f, float* fn) {
  const int gs = m.grid_size, g1 = gs - 1, area = m.grid_area;
  const int start = m.face_start[f], n = m.face_ngrids[f];
  for (int c = 0; c < n; c++) {
    const int base = (start + c) * area;
    for (int q = threadIdx.x; q < g1 * g1; q += blockDim.x) {
      const int x = q % g1, y = q / g1;
      const float3 nq = normal_quad(xyz(__ldcg(&m.co[base + (y + 1) * gs + x])),
                                    xyz(__ldcg(&m.co[base + (y + 1) * gs + x + 1])),
                                    xyz(__ldcg(&m.co[base + y * gs + x + 1])),
                                    xyz(__ldcg(&m.co[base + y * gs + x])));
      fn[3 * q] = nq.x;
      fn[3 * q + 1] = nq.y;
      fn[3 * q + 2] = nq.z;
    }
    __syncthreads();
    for (int e = threadIdx.x; e < area; e += blockDim.x) {
      const int x = e % gs, y = e / gs;
      float ax = 0.0f, ay = 0.0f, az = 0.0f;
      int counter = 0;
      int q;
      if (x < g1 && y < g1) {
        q = y * g1 + x;
        ax += fn[3 * q], ay += fn[3 * q + 1], az += fn[3 * q + 2];
        counter++;
      }
      if (x >= 1) {
        if (y < g1) {
          q = y * g1 + (x - 1);
          ax += fn[3 * q], ay += fn[3 * q + 1], az += fn[3 * q + 2];
          counter++;
        }
        if (y >= 1) {
          q = (y - 1) * g1 + (x - 1);
          ax += fn[3 * q], ay += fn[3 * q + 1], az += fn[3 * q + 2];
          counter++;
        }
      }
      if (y >= 1 && x < g1) {
        q = (y - 1) * g1 + x;
        ax += fn[3 * q], ay += fn[3 * q + 1], az += fn[3 * q + 2];
        counter++;
      }
      const float inv = 1.0f / (float)counter;
      m.no[base + e] = make_float4(ax * inv, ay * inv, az * inv, 0.0f);
    }
    __syncthreads();
  }
  // seams between consecutive grids: prev grid (i, 0) with grid (0, i), i >= 1
  for (int w = threadIdx.x; w < n * g1; w += blockDim.x) {
    const int c = w / g1, i = 1 + w % g1;
    const int g = start + c;
    const int prev = start + (c + n - 1) % n;
    grid_avg_pair(m, prev * area + i, g * area + i * gs);
  }
  __syncthreads();
  if (threadIdx.x == 0)
    grid_average_set(m, n, [&](int c) { return (start + c) * area; });
  __syncthreads();
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
