// PBVH_GRIDS normal update with seam stitching (multires), as the reference
// runs it after a dab: BKE_pbvh_update_normals (pbvh.c:4572-4580) ->
// BKE_pbvh_get_grid_updates (pbvh.c:3523-3566) -> KERNEL_subdiv_ccg_update_normals
// (subdiv_ccg.c:847-874).
//   k_grid_gather:  faces of flagged leaves (deduplicated), their base edges
//                   and base vertices; clears UpdateNormals.
//   k_grid_inner:   inner normals of every element of the claimed grids.
//   k_grid_face_seams: face-internal seam pairs and face centres.
//   k_grid_seams:   averaging across base edges and base-vertex corners; both
//                   touch disjoint elements.
// Work lists are built with atomics, so their order varies, but every list
// item writes elements no other item touches, so results do not depend on it.
#include <cuda_runtime.h>

#include "sgpu_device.cuh"
#include "sgpu_grids.cuh"
#include "sgpu_kernels.h"

namespace sgpu {

constexpr int kGThreads = 256;

__global__ void __launch_bounds__(kGThreads) k_grid_gather(DevMesh m) {
  const unsigned int epoch = m.work->grid_epoch + 1u;
  for (int leaf = blockIdx.x; leaf < m.nleaf; leaf += gridDim.x) {
    if (!(m.leaf_flag[leaf] & kUpdateNormals)) continue;
    const int p0 = m.leaf_prim_off[leaf], p1 = m.leaf_prim_off[leaf + 1];
    for (int j = p0 + threadIdx.x; j < p1; j += blockDim.x) grid_claim_face(m, m.leaf_prims[j], epoch);
    __syncthreads();
    if (threadIdx.x == 0) atomicAnd(&m.leaf_flag[leaf], ~kUpdateNormals);
  }
}

// One thread per element of the claimed grids (grid-stride).
__global__ void __launch_bounds__(kGThreads) k_grid_inner(DevMesh m) {
  const long long items = (long long)m.grid_counts[3] * m.grid_area;
  unsigned long long ab = 0;  // algorithmic bytes (profiling): co read, normal written
  for (long long it = (long long)blockIdx.x * blockDim.x + threadIdx.x; it < items;
       it += (long long)gridDim.x * blockDim.x) {
    grid_inner_item(m, it);
    ab += 24u;
  }
  prof_add(m, kKGridFaces, ab);
}

// One thread per face-internal seam pair or face centre (grid-stride).
__global__ void __launch_bounds__(kGThreads) k_grid_face_seams(DevMesh m) {
  const int ng = m.grid_counts[3], nf = m.grid_counts[0];
  const long long pairs = (long long)ng * (m.grid_size - 1);
  const long long items = pairs + nf;
  unsigned long long ab = 0;  // co, no and mask read and written per element
  for (long long it = (long long)blockIdx.x * blockDim.x + threadIdx.x; it < items;
       it += (long long)gridDim.x * blockDim.x) {
    grid_face_seam_item(m, it, ng);
    ab += it < pairs ? 112ull : 56ull * m.face_ngrids[m.face_list[it - pairs]];
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
    int nfaces;
    if (it < edge_items) {
      const int e = m.edge_list[it / inner];
      nfaces = m.edge_off[e + 1] - m.edge_off[e];
    } else {
      const int v = m.bvert_list[it - edge_items];
      nfaces = m.bvert_off[v + 1] - m.bvert_off[v];
    }
    if (nfaces > 1) ab += 56ull * nfaces;  // co, no, mask read and written per face
    grid_seam_item(m, it, ne);
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
    m.grid_counts[3] = 0;
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

void configure_grid_kernels() {}

cudaError_t launch_grid_gather(const DevMesh& m, cudaStream_t s) {
  const int g = grids_grid();
  int gl = m.nleaf < g ? m.nleaf : g;
  if (gl < 1) gl = 1;
  k_grid_gather<<<gl, kGThreads, 0, s>>>(m);
  return cudaGetLastError();
}

cudaError_t launch_grid_inner(const DevMesh& m, cudaStream_t s) {
  k_grid_inner<<<grids_grid(), kGThreads, 0, s>>>(m);
  return cudaGetLastError();
}

cudaError_t launch_grid_face_seams(const DevMesh& m, cudaStream_t s) {
  k_grid_face_seams<<<grids_grid(), kGThreads, 0, s>>>(m);
  return cudaGetLastError();
}

cudaError_t launch_grid_seams(const DevMesh& m, cudaStream_t s) {
  k_grid_seams<<<grids_grid(), kGThreads, 0, s>>>(m);
  return cudaGetLastError();
}

}  // namespace sgpu
