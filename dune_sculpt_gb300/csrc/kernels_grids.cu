// PBVH_GRIDS normal update with seam stitching (multires), as the reference
// runs it after a dab: BKE_pbvh_update_normals (pbvh.c:4572-4580) ->
// BKE_pbvh_get_grid_updates (pbvh.c:3523-3566) -> KERNEL_subdiv_ccg_update_normals
// (subdiv_ccg.c:847-874).
//   k_grid_gather:  faces of flagged leaves (deduplicated), their base edges
//                   and base vertices; clears UpdateNormals.
//   k_grid_faces:   per face, inner grid normals (subdiv_ccg.c:670-740) and the
//                   face-internal seam/centre averaging (:951-984).
//   k_grid_seams:   averaging across base edges (:1010-1048) and base-vertex
//                   corners (:1081-1104); both touch disjoint elements.
// Work lists are built with atomics, so their order varies, but every list
// item writes elements no other item touches, so results do not depend on it.
#include <cuda_runtime.h>

#include "sgpu_device.cuh"
#include "sgpu_kernels.h"

namespace sgpu {

constexpr int kGThreads = 256;

__device__ __forceinline__ bool claim(unsigned int* mark, int i, unsigned int epoch) {
  return atomicExch(&mark[i], epoch) != epoch;
}

__global__ void __launch_bounds__(kGThreads) k_grid_gather(DevMesh m) {
  const unsigned int epoch = m.work->grid_epoch + 1u;
  for (int leaf = blockIdx.x; leaf < m.nleaf; leaf += gridDim.x) {
    if (!(m.leaf_flag[leaf] & kUpdateNormals)) continue;
    const int p0 = m.leaf_prim_off[leaf], p1 = m.leaf_prim_off[leaf + 1];
    for (int j = p0 + threadIdx.x; j < p1; j += blockDim.x) {
      const int f = m.grid_face[m.leaf_prims[j]];
      if (!claim(m.face_mark, f, epoch)) continue;
      m.face_list[atomicAdd(&m.grid_counts[0], 1)] = f;
      const int s = m.face_start[f], n = m.face_ngrids[f];
      for (int c = 0; c < n; c++) {
        const int e = m.face_edges[s + c];
        const int v = m.face_verts[s + c];
        if (claim(m.edge_mark, e, epoch)) m.edge_list[atomicAdd(&m.grid_counts[1], 1)] = e;
        if (claim(m.bvert_mark, v, epoch)) m.bvert_list[atomicAdd(&m.grid_counts[2], 1)] = v;
      }
    }
    __syncthreads();
    if (threadIdx.x == 0) atomicAnd(&m.leaf_flag[leaf], ~kUpdateNormals);
  }
}

__device__ __forceinline__ void avg_pair(const DevMesh& m, int a, int b) {
  float4 ca = m.co[a], cb = m.co[b];
  float4 na = m.no[a], nb = m.no[b];
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
    const float mk = (m.mask[a] + m.mask[b]) * 0.5f;
    m.mask[a] = mk;
    m.mask[b] = mk;
  }
}

// One CTA per affected face (grid-stride).  Shared memory: (gs-1)^2 quad
// normals of the grid being processed.
__global__ void __launch_bounds__(kGThreads) k_grid_faces(DevMesh m) {
  extern __shared__ float fn[];  // 3 * (gs-1)^2
  const int nf = m.grid_counts[0];
  const int gs = m.grid_size, g1 = gs - 1, area = m.grid_area;
  unsigned long long ab = 0;  // algorithmic bytes (profiling)
  for (int k = blockIdx.x; k < nf; k += gridDim.x) {
    const int f = m.face_list[k];
    const int start = m.face_start[f], n = m.face_ngrids[f];
    // co read + normal written per element; each seam pair and the centre
    // read and write co, no and mask of their elements
    if (threadIdx.x == 0) ab += 24ull * area * n + 112ull * g1 * n + 56ull * n;
    for (int c = 0; c < n; c++) {
      const int base = (start + c) * area;
      // subdiv_ccg_recalc_inner_face_normals: quad {(x,y+1),(x+1,y+1),(x+1,y),(x,y)}
      for (int q = threadIdx.x; q < g1 * g1; q += blockDim.x) {
        const int x = q % g1, y = q / g1;
        const float3 nq = normal_quad(xyz(m.co[base + (y + 1) * gs + x]),
                                      xyz(m.co[base + (y + 1) * gs + x + 1]),
                                      xyz(m.co[base + y * gs + x + 1]), xyz(m.co[base + y * gs + x]));
        fn[3 * q] = nq.x;
        fn[3 * q + 1] = nq.y;
        fn[3 * q + 2] = nq.z;
      }
      __syncthreads();
      // subdiv_ccg_average_inner_face_normals: mean of the adjacent quads
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
    // subdiv_ccg_average_inner_face_grids: seams between consecutive grids
    // (prev grid (i, 0) with grid (0, i), i >= 1; all pairs disjoint) ...
    for (int w = threadIdx.x; w < n * g1; w += blockDim.x) {
      const int c = w / g1, i = 1 + w % g1;
      const int g = start + c;
      const int prev = start + (c + n - 1) % n;
      avg_pair(m, prev * area + i, g * area + i * gs);
    }
    __syncthreads();
    // ... then the shared centre element.
    if (threadIdx.x == 0) {
      float cx = 0.0f, cy = 0.0f, cz = 0.0f, nx = 0.0f, ny = 0.0f, nz = 0.0f, mk = 0.0f;
      for (int c = 0; c < n; c++) {
        const int e = (start + c) * area;
        const float4 co = m.co[e], no = m.no[e];
        cx += co.x, cy += co.y, cz += co.z;
        nx += no.x, ny += no.y, nz += no.z;
        if (m.mask) mk += m.mask[e];
      }
      const float inv = 1.0f / (float)n;
      cx *= inv, cy *= inv, cz *= inv;
      nx *= inv, ny *= inv, nz *= inv;
      mk *= inv;
      for (int c = 0; c < n; c++) {
        const int e = (start + c) * area;
        const float4 old = m.co[e];
        m.co[e] = make_float4(cx, cy, cz, old.w);
        m.no[e] = make_float4(nx, ny, nz, 0.0f);
        if (m.mask) m.mask[e] = mk;
      }
    }
    __syncthreads();
  }
  prof_add(m, kKGridFaces, ab);
}

// Edges: one thread per (edge, boundary index 1 .. 2gs-2); corners: one thread
// per base vertex.  The last CTA resets the lists for the next update.
__global__ void __launch_bounds__(kGThreads) k_grid_seams(DevMesh m) {
  __shared__ bool am_last;
  const int ne = m.grid_counts[1], nv = m.grid_counts[2];
  const int g2 = 2 * m.grid_size, inner = g2 - 2;
  const long long edge_items = (long long)ne * inner;
  const long long total = edge_items + nv;
  unsigned long long ab = 0;  // algorithmic bytes (profiling)
  for (long long it = (long long)blockIdx.x * blockDim.x + threadIdx.x; it < total;
       it += (long long)gridDim.x * blockDim.x) {
    if (it < edge_items) {
      const int e = m.edge_list[it / inner];
      const int i = 1 + (int)(it % inner);
      const int f0 = m.edge_off[e], f1 = m.edge_off[e + 1];
      const int nfe = f1 - f0;
      if (nfe == 1) continue;
      ab += 56ull * nfe;  // co, no, mask read and written per adjacent face
      float cx = 0.0f, cy = 0.0f, cz = 0.0f, nx = 0.0f, ny = 0.0f, nz = 0.0f, mk = 0.0f;
      for (int f = f0; f < f1; f++) {
        const int el = m.edge_elems[(long long)f * g2 + i];
        const float4 co = m.co[el], no = m.no[el];
        cx += co.x, cy += co.y, cz += co.z;
        nx += no.x, ny += no.y, nz += no.z;
        if (m.mask) mk += m.mask[el];
      }
      const float inv = 1.0f / (float)nfe;
      cx *= inv, cy *= inv, cz *= inv;
      nx *= inv, ny *= inv, nz *= inv;
      mk *= inv;
      for (int f = f0; f < f1; f++) {
        const int el = m.edge_elems[(long long)f * g2 + i];
        const float4 old = m.co[el];
        m.co[el] = make_float4(cx, cy, cz, old.w);
        m.no[el] = make_float4(nx, ny, nz, 0.0f);
        if (m.mask) m.mask[el] = mk;
      }
    } else {
      const int v = m.bvert_list[it - edge_items];
      const int f0 = m.bvert_off[v], f1 = m.bvert_off[v + 1];
      const int nfv = f1 - f0;
      if (nfv == 1) continue;
      ab += 56ull * nfv;
      float cx = 0.0f, cy = 0.0f, cz = 0.0f, nx = 0.0f, ny = 0.0f, nz = 0.0f, mk = 0.0f;
      for (int f = f0; f < f1; f++) {
        const int el = m.bvert_elems[f];
        const float4 co = m.co[el], no = m.no[el];
        cx += co.x, cy += co.y, cz += co.z;
        nx += no.x, ny += no.y, nz += no.z;
        if (m.mask) mk += m.mask[el];
      }
      const float inv = 1.0f / (float)nfv;
      cx *= inv, cy *= inv, cz *= inv;
      nx *= inv, ny *= inv, nz *= inv;
      mk *= inv;
      for (int f = f0; f < f1; f++) {
        const int el = m.bvert_elems[f];
        const float4 old = m.co[el];
        m.co[el] = make_float4(cx, cy, cz, old.w);
        m.no[el] = make_float4(nx, ny, nz, 0.0f);
        if (m.mask) m.mask[el] = mk;
      }
    }
  }
  prof_add(m, kKGridSeams, ab);
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) {
    const unsigned int ticket = atomicAdd(&m.work->ticket_update, 1u);
    am_last = (ticket == gridDim.x - 1);
  }
  __syncthreads();
  if (!am_last) return;
  if (threadIdx.x == 0) {
    m.grid_counts[0] = 0;
    m.grid_counts[1] = 0;
    m.grid_counts[2] = 0;
    m.work->grid_epoch = m.work->grid_epoch + 1u;
    m.work->ticket_update = 0u;
  }
}

static int grids_grid() {
  static int g = 0;
  if (g == 0) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    g = sms > 0 ? 2 * sms : 264;
  }
  return g;
}

int grid_size_limit() { return 65; }

void configure_grid_kernels() {
  const int g1 = grid_size_limit() - 1;
  cudaFuncSetAttribute(k_grid_faces, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       static_cast<int>(sizeof(float) * 3 * g1 * g1));
}

cudaError_t launch_grid_gather(const DevMesh& m, cudaStream_t s) {
  const int g = grids_grid();
  int gl = m.nleaf < g ? m.nleaf : g;
  if (gl < 1) gl = 1;
  k_grid_gather<<<gl, kGThreads, 0, s>>>(m);
  return cudaGetLastError();
}

cudaError_t launch_grid_faces(const DevMesh& m, cudaStream_t s) {
  const size_t smem = sizeof(float) * 3 * (m.grid_size - 1) * (m.grid_size - 1);
  k_grid_faces<<<grids_grid(), kGThreads, smem, s>>>(m);
  return cudaGetLastError();
}

cudaError_t launch_grid_seams(const DevMesh& m, cudaStream_t s) {
  k_grid_seams<<<grids_grid(), kGThreads, 0, s>>>(m);
  return cudaGetLastError();
}

}  // namespace sgpu
