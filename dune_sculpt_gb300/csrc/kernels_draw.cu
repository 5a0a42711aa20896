// Headless PBVH draw-buffer fill: GPU_pbvh_mesh_buffers_update
// (gpu_buffers.c:174-305) and GPU_pbvh_grid_buffers_update (gpu_buffers.c:548-725)
// for every leaf flagged PBVH_UpdateDrawBuffers, as pbvh_update_draw_buffers
// (pbvh.c:3240-3290) runs them, writing the reference's interleaved vertex
// format (36 bytes: pos f32x3 at 0, nor i16x3 at 16, msk u8 at 22, ac u16x4 at
// 24, fset u8x3 at 32; the padding zero).
//
// One CTA per leaf.  Each thread builds the vertices of one unit (a visible
// looptri: 3 vertices; a grid element: 1; a flat grid quad: 4) in shared
// memory, then the CTA writes the chunk's words to the leaf's contiguous range
// with consecutive 32-bit stores, so the 36-byte records (4-byte aligned only)
// leave the SM as full coalesced lines.  The CTA also reduces the leaf's
// show_overlay (a non-zero mask byte or a non-default face set) and clears
// PBVH_RebuildDrawBuffers | PBVH_UpdateDrawBuffers.
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
__global__ void __launch_bounds__(kDrawThreads) k_draw_faces(DevMesh m, DrawDev dd) {
  __shared__ unsigned int s_w[kDrawThreads * 3 * kDrawWords];
  const int leaf = blockIdx.x;
  const int f = m.leaf_flag[leaf];
  if (!(f & (kUpdateDrawBuffers | kRebuildDrawBuffers))) return;
  int overlay = 0;
  if (f & kUpdateDrawBuffers) {
    const int t0 = dd.leaf_tri_start[leaf], nt = dd.leaf_tri_count[leaf];
    const bool smooth = dd.leaf_smooth[leaf] != 0;
    const long long vbase = dd.leaf_vert_off[leaf];
    unsigned int* out = dd.vbo + vbase * kDrawWords;
    for (int c = 0; c < nt; c += kDrawThreads) {
      const int t = c + static_cast<int>(threadIdx.x);
      if (t < nt) {
        const int4 tv = m.lt_v4[dd.tris[t0 + t]];
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
      const int words = min(kDrawThreads, nt - c) * 3 * kDrawWords;
      unsigned int* dst = out + static_cast<size_t>(c) * 3 * kDrawWords;
      for (int i = threadIdx.x; i < words; i += kDrawThreads) dst[i] = s_w[i];
      __syncthreads();
    }
  }
  overlay = __syncthreads_or(overlay);
  if (threadIdx.x == 0) {
    if (f & kUpdateDrawBuffers) dd.overlay[leaf] = overlay;
    atomicAnd(&m.leaf_flag[leaf], ~(kUpdateDrawBuffers | kRebuildDrawBuffers));
  }
}

// PBVH_GRIDS: smooth leaves one vertex per grid element (grid, row, column
// order); flat leaves four per grid quad with the quad's normal
// (normal_quad_v3 of the corners in reverse order) and mean mask.  The colour
// attribute is white (the update always has GPU_PBVH_BUFFERS_SHOW_VCOL).
__global__ void __launch_bounds__(kDrawThreads) k_draw_grids(DevMesh m, DrawDev dd) {
  __shared__ unsigned int s_w[kDrawThreads * kFlatStride];
  const int leaf = blockIdx.x;
  const int f = m.leaf_flag[leaf];
  if (!(f & (kUpdateDrawBuffers | kRebuildDrawBuffers))) return;
  int overlay = 0;
  if (f & kUpdateDrawBuffers) {
    const int g0 = m.leaf_prim_off[leaf], ng = m.leaf_prim_off[leaf + 1] - g0;
    const int gs = m.grid_size, area = m.grid_area, g1 = gs - 1, nq = g1 * g1;
    const bool smooth = dd.leaf_smooth[leaf] != 0;
    const int vpu = smooth ? 1 : 4;  // vertices per unit
    const int units = ng * (smooth ? area : nq);
    unsigned int* out = dd.vbo + dd.leaf_vert_off[leaf] * kDrawWords;
    for (int c = 0; c < units; c += kDrawThreads) {
      const int u = c + static_cast<int>(threadIdx.x);
      if (u < units) {
        if (smooth) {
          const int grid = m.leaf_prims[g0 + u / area];
          const size_t e = static_cast<size_t>(grid) * area + u % area;
          const float4 n = m.no[e];
          unsigned int cm = 0u;
          if (m.mask) {
            cm = mask_byte(m.mask[e]);
            overlay |= cm != 0u;
          }
          const unsigned int fs = dd.fset ? dd.fset[grid] : kWhite;
          overlay |= static_cast<int>(fs >> 24);
          put_vertex(s_w + threadIdx.x * kDrawWords, m.co[e], nor_pair(n.x, n.y), nor_one(n.z),
                     cm, 0xffffffffu, 0xffffffffu, fs);
        } else {
          const int grid = m.leaf_prims[g0 + u / nq];
          const int r = u % nq, y = r / g1, x = r % g1;
          const size_t e0 = static_cast<size_t>(grid) * area + y * gs + x;
          const size_t e[4] = {e0, e0 + 1, e0 + gs + 1, e0 + gs};
          const float4 c0 = m.co[e[0]], c1 = m.co[e[1]], c2 = m.co[e[2]], c3 = m.co[e[3]];
          const float3 n = normal_quad(xyz(c3), xyz(c2), xyz(c1), xyz(c0));
          unsigned int cm = 0u;
          if (m.mask) {
            cm = mask_byte((m.mask[e[0]] + m.mask[e[1]] + m.mask[e[2]] + m.mask[e[3]]) * 0.25f);
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
      }
      __syncthreads();
      const int n_units = min(kDrawThreads, units - c);
      unsigned int* dst = out + static_cast<size_t>(c) * vpu * kDrawWords;
      if (smooth) {
        for (int i = threadIdx.x; i < n_units * kDrawWords; i += kDrawThreads) dst[i] = s_w[i];
      } else {
        for (int i = threadIdx.x; i < n_units * 4 * kDrawWords; i += kDrawThreads)
          dst[i] = s_w[(i / (4 * kDrawWords)) * kFlatStride + i % (4 * kDrawWords)];
      }
      __syncthreads();
    }
  }
  overlay = __syncthreads_or(overlay);
  if (threadIdx.x == 0) {
    if (f & kUpdateDrawBuffers) dd.overlay[leaf] = overlay;
    atomicAnd(&m.leaf_flag[leaf], ~(kUpdateDrawBuffers | kRebuildDrawBuffers));
  }
}

}  // namespace

cudaError_t launch_draw_fill(const DevMesh& m, const DrawDev& dd, cudaStream_t s) {
  if (m.nleaf <= 0) return cudaSuccess;
  if (m.type == kFaces)
    k_draw_faces<<<m.nleaf, kDrawThreads, 0, s>>>(m, dd);
  else
    k_draw_grids<<<m.nleaf, kDrawThreads, 0, s>>>(m, dd);
  return cudaGetLastError();
}

}  // namespace sgpu
