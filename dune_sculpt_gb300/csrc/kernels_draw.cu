// Headless PBVH draw-buffer fill: GPU_pbvh_mesh_buffers_update
// (gpu_buffers.c:174-305) and GPU_pbvh_grid_buffers_update (gpu_buffers.c:548-725)
// for every leaf flagged PBVH_UpdateDrawBuffers, as pbvh_update_draw_buffers
// (pbvh.c:3240-3290) runs them, writing the reference's interleaved vertex
// format (36 bytes: pos f32x3 at 0, nor i16x3 at 16, msk u8 at 22, ac u16x4 at
// 24, fset u8x3 at 32; the padding zero).
//
// One CTA per (leaf, chunk of 256 units): a unit is a visible looptri (3
// vertices), a grid element (1) or a flat grid quad (4).  Each thread builds
// its unit's vertices in shared memory, then the CTA writes the chunk's words
// to the leaf's contiguous range with consecutive 32-bit stores, so the 36-byte
// records (4-byte aligned only) leave the SM as full coalesced lines.  Each
// CTA ORs its part of the leaf's show_overlay (a non-zero mask byte or a
// non-default face set) into a per-leaf word; k_draw_finish then publishes
// show_overlay and clears PBVH_RebuildDrawBuffers | PBVH_UpdateDrawBuffers
// once every chunk has read the flags.
#include <cuda_runtime.h>

#include "sgpu_device.cuh"
#include "sgpu_draw.h"
#include "sgpu_kernels.h"

namespace sgpu {
namespace {

constexpr int kDrawThreads = 256;
constexpr unsigned int kWhite = 0x00ffffffu;   // fset of the default face set
constexpr int kFlatStride = 4 * kDrawWords + 1;  // odd word stride: no bank conflicts

// normal_float_to_short_v3 (math_vector_inline.c:1260-1265) for two components.
__device__ __forceinline__ unsigned int nor_pair(float a, float b) {
  const short sa = static_cast<short>(a * 32767.0f);
  const short sb = static_cast<short>(b * 32767.0f);
  return static_cast<unsigned short>(sa) |
         (static_cast<unsigned int>(static_cast<unsigned short>(sb)) << 16);
}
__device__ __forceinline__ unsigned int nor_one(float a) {
  return static_cast<unsigned short>(static_cast<short>(a * 32767.0f));
}

// (uchar)(fmask * 255): the conversion through int, as the host compilers emit it.
__device__ __forceinline__ unsigned int mask_byte(float fmask) {
  return static_cast<unsigned char>(static_cast<int>(fmask * 255.0f));
}

__device__ __forceinline__ void put_vertex(unsigned int* w, float4 co, unsigned int n01,
                                           unsigned int n2, unsigned int cm, unsigned int c0,
                                           unsigned int c1, unsigned int fset) {
  w[0] = __float_as_uint(co.x);
  w[1] = __float_as_uint(co.y);
  w[2] = __float_as_uint(co.z);
  w[3] = 0u;
  w[4] = n01;
  w[5] = n2 | (cm << 16);
  w[6] = c0;
  w[7] = c1;
  w[8] = fset & kWhite;
}

// PBVH_FACES: 3 vertices per visible looptri, in the leaf's prim order.
// 128-thread CTAs: 16 per SM, so that the gathers of more CTAs overlap.
constexpr int kFacesThreads = 128;
__global__ void __launch_bounds__(kFacesThreads) k_draw_faces(DevMesh m, DrawDev dd) {
  __shared__ unsigned int s_w[kFacesThreads * 3 * kDrawWords];
  const int leaf = blockIdx.x;
  const int c = blockIdx.y * kFacesThreads;
  if (!(m.leaf_flag[leaf] & kUpdateDrawBuffers)) return;
  const int nt = dd.leaf_tri_count[leaf];
  if (c >= nt) return;
  const int t0 = dd.leaf_tri_start[leaf];
  const bool smooth = dd.leaf_smooth[leaf] != 0;
  const long long vbase = dd.leaf_vert_off[leaf];
  int overlay = 0;
  const int t = c + static_cast<int>(threadIdx.x);
  if (t < nt) {
    const int4 tv = reinterpret_cast<const int4*>(dd.tri_v4)[t0 + t];
    unsigned int n01 = 0u, n2 = 0u, cm = 0u;
    if (!smooth) {  // the poly normal (BKE_mesh_calc_poly_normal)
      const float3 n = poly_normal(m, tv.w);
      n01 = nor_pair(n.x, n.y);
      n2 = nor_one(n.z);
      if (m.mask) cm = mask_byte((m.mask[tv.x] + m.mask[tv.y] + m.mask[tv.z]) / 3.0f);
    }
    const unsigned int fs = dd.fset ? dd.fset[tv.w] : kWhite;
    overlay |= static_cast<int>(fs >> 24);
    unsigned int* w = s_w + threadIdx.x * 3 * kDrawWords;
#pragma unroll
    for (int j = 0; j < 3; j++) {
      const int v = j == 0 ? tv.x : (j == 1 ? tv.y : tv.z);
      if (smooth) {
        const float4 n = m.no[v];
        n01 = nor_pair(n.x, n.y);
        n2 = nor_one(n.z);
        if (m.mask) cm = mask_byte(m.mask[v]);
      }
      overlay |= cm != 0u;
      unsigned int c0 = 0u, c1 = 0u;
      if (dd.col) {
        const size_t k = 2 * static_cast<size_t>(vbase + 3LL * t + j);
        c0 = dd.col[k];
        c1 = dd.col[k + 1];
      }
      put_vertex(w + j * kDrawWords, m.co[v], n01, n2, cm, c0, c1, fs);
    }
  }
  __syncthreads();
  const int words = min(kFacesThreads, nt - c) * 3 * kDrawWords;
  unsigned int* dst = dd.vbo + (vbase + 3LL * c) * kDrawWords;
  for (int i = threadIdx.x; i < words; i += kFacesThreads) dst[i] = s_w[i];
  overlay = __syncthreads_or(overlay);
  if (threadIdx.x == 0 && overlay) atomicOr(&dd.overlay_acc[leaf], 1);
}

// PBVH_GRIDS, smooth leaves: one vertex per grid element (grid, row, column
// order), two elements per thread (their loads in flight together).  The
// colour attribute is white (the update always has GPU_PBVH_BUFFERS_SHOW_VCOL).
constexpr int kSmoothUnits = 2 * kDrawThreads;

__device__ __forceinline__ void grid_smooth_vertex(const DevMesh& m, const DrawDev& dd, int g0,
                                                   int u, unsigned int* w, int& overlay) {
  const int grid = m.leaf_prims[g0 + u / m.grid_area];
  const size_t e = static_cast<size_t>(grid) * m.grid_area + u % m.grid_area;
  const float4 co = m.co[e], n = m.no[e];
  unsigned int cm = 0u;
  if (m.mask) {
    cm = mask_byte(m.mask[e]);
    overlay |= cm != 0u;
  }
  const unsigned int fs = dd.fset ? dd.fset[grid] : kWhite;
  overlay |= static_cast<int>(fs >> 24);
  put_vertex(w, co, nor_pair(n.x, n.y), nor_one(n.z), cm, 0xffffffffu, 0xffffffffu, fs);
}

__global__ void __launch_bounds__(kDrawThreads) k_draw_grids_smooth(DevMesh m, DrawDev dd) {
  __shared__ unsigned int s_w[kSmoothUnits * kDrawWords];
  const int leaf = blockIdx.x;
  const int c = blockIdx.y * kSmoothUnits;
  if (!(m.leaf_flag[leaf] & kUpdateDrawBuffers) || !dd.leaf_smooth[leaf]) return;
  const int g0 = m.leaf_prim_off[leaf], ng = m.leaf_prim_off[leaf + 1] - g0;
  const int units = ng * m.grid_area;
  if (c >= units) return;
  int overlay = 0;
  const int u0 = c + static_cast<int>(threadIdx.x), u1 = u0 + kDrawThreads;
  if (u0 < units) grid_smooth_vertex(m, dd, g0, u0, s_w + threadIdx.x * kDrawWords, overlay);
  if (u1 < units)
    grid_smooth_vertex(m, dd, g0, u1, s_w + (threadIdx.x + kDrawThreads) * kDrawWords, overlay);
  __syncthreads();
  const int words = min(kSmoothUnits, units - c) * kDrawWords;
  unsigned int* dst = dd.vbo + (dd.leaf_vert_off[leaf] + c) * kDrawWords;
  for (int i = threadIdx.x; i < words; i += kDrawThreads) dst[i] = s_w[i];
  overlay = __syncthreads_or(overlay);
  if (threadIdx.x == 0 && overlay) atomicOr(&dd.overlay_acc[leaf], 1);
}

// PBVH_GRIDS, flat leaves: four vertices per grid quad with the quad's normal
// (normal_quad_v3 of the corners in reverse order) and mean mask.
__global__ void __launch_bounds__(kDrawThreads) k_draw_grids_flat(DevMesh m, DrawDev dd) {
  __shared__ unsigned int s_w[kDrawThreads * kFlatStride];
  const int leaf = blockIdx.x;
  const int c = blockIdx.y * kDrawThreads;
  if (!(m.leaf_flag[leaf] & kUpdateDrawBuffers) || dd.leaf_smooth[leaf]) return;
  const int g0 = m.leaf_prim_off[leaf], ng = m.leaf_prim_off[leaf + 1] - g0;
  const int gs = m.grid_size, area = m.grid_area, g1 = gs - 1, nq = g1 * g1;
  const int units = ng * nq;
  if (c >= units) return;
  int overlay = 0;
  const int u = c + static_cast<int>(threadIdx.x);
  if (u < units) {
    const int grid = m.leaf_prims[g0 + u / nq];
    const int r = u % nq, y = r / g1, x = r % g1;
    const size_t e0 = static_cast<size_t>(grid) * area + y * gs + x;
    const size_t e1 = e0 + 1, e2 = e0 + gs + 1, e3 = e0 + gs;
    const float4 c0 = m.co[e0], c1 = m.co[e1], c2 = m.co[e2], c3 = m.co[e3];
    const float3 n = normal_quad(xyz(c3), xyz(c2), xyz(c1), xyz(c0));
    unsigned int cm = 0u;
    if (m.mask) {
      cm = mask_byte((m.mask[e0] + m.mask[e1] + m.mask[e2] + m.mask[e3]) * 0.25f);
      overlay |= cm != 0u;
    }
    const unsigned int fs = dd.fset ? dd.fset[grid] : kWhite;
    overlay |= static_cast<int>(fs >> 24);
    const unsigned int n01 = nor_pair(n.x, n.y), n2 = nor_one(n.z);
    unsigned int* w = s_w + threadIdx.x * kFlatStride;
    put_vertex(w, c0, n01, n2, cm, 0xffffffffu, 0xffffffffu, fs);
    put_vertex(w + kDrawWords, c1, n01, n2, cm, 0xffffffffu, 0xffffffffu, fs);
    put_vertex(w + 2 * kDrawWords, c2, n01, n2, cm, 0xffffffffu, 0xffffffffu, fs);
    put_vertex(w + 3 * kDrawWords, c3, n01, n2, cm, 0xffffffffu, 0xffffffffu, fs);
  }
  __syncthreads();
  const int n_units = min(kDrawThreads, units - c);
  unsigned int* dst = dd.vbo + (dd.leaf_vert_off[leaf] + 4LL * c) * kDrawWords;
  for (int i = threadIdx.x; i < n_units * 4 * kDrawWords; i += kDrawThreads)
    dst[i] = s_w[(i / (4 * kDrawWords)) * kFlatStride + i % (4 * kDrawWords)];
  overlay = __syncthreads_or(overlay);
  if (threadIdx.x == 0 && overlay) atomicOr(&dd.overlay_acc[leaf], 1);
}

// After every chunk: show_overlay of the refilled leaves, the draw flags
// cleared on every leaf (pbvh_update_draw_buffers, pbvh.c:3280-3289).
__global__ void k_draw_finish(DevMesh m, DrawDev dd) {
  const int leaf = blockIdx.x * blockDim.x + threadIdx.x;
  if (leaf >= m.nleaf) return;
  const int f = m.leaf_flag[leaf];
  if (!(f & (kUpdateDrawBuffers | kRebuildDrawBuffers))) return;
  if (f & kUpdateDrawBuffers) {
    dd.overlay[leaf] = dd.overlay_acc[leaf];
    dd.overlay_acc[leaf] = 0;
  }
  m.leaf_flag[leaf] = f & ~(kUpdateDrawBuffers | kRebuildDrawBuffers);
}

}  // namespace

cudaError_t launch_draw_fill(const DevMesh& m, const DrawDev& dd, int max_units_smooth,
                             int max_units_flat, cudaStream_t s) {
  if (m.nleaf <= 0) return cudaSuccess;
  if (m.type == kFaces) {
    if (max_units_flat + max_units_smooth > 0) {
      const int units = max(max_units_flat, max_units_smooth);
      k_draw_faces<<<dim3(m.nleaf, (units + kFacesThreads - 1) / kFacesThreads), kFacesThreads,
                     0, s>>>(m, dd);
    }
  } else {
    if (max_units_smooth > 0)
      k_draw_grids_smooth<<<dim3(m.nleaf, (max_units_smooth + kSmoothUnits - 1) / kSmoothUnits),
                            kDrawThreads, 0, s>>>(m, dd);
    if (max_units_flat > 0)
      k_draw_grids_flat<<<dim3(m.nleaf, (max_units_flat + kDrawThreads - 1) / kDrawThreads),
                          kDrawThreads, 0, s>>>(m, dd);
  }
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  k_draw_finish<<<(m.nleaf + 255) / 256, 256, 0, s>>>(m, dd);
  return cudaGetLastError();
}

}  // namespace sgpu
