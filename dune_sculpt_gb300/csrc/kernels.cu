// Per-call CUDA kernels of libsculptgpu: node culling, area normal/centre
// reduction, the four brushes, the FACES normal update and the bounding-box
// refit with its bottom-up flush.  Each kernel is one phase of the reference's
// per-dab call sequence; they read their work sizes (culled leaf count, vertex
// prefix) from device memory, so a whole stroke can be captured in one CUDA
// graph without host round trips.
#include <cuda_runtime.h>

#include "sgpu_device.cuh"
#include "sgpu_kernels.h"

namespace sgpu {

constexpr int kCullThreads = 1024;
constexpr int kThreads = 256;

// ---------------------------------------------------------------------------
// Block-wide exclusive scan of ints (blockDim.x a multiple of 32, <= 1024).
__device__ int block_exclusive_scan(int v, int* total, int* smem32) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nwarps = blockDim.x >> 5;
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
    smem32[lane] = w;  // inclusive prefix of warp totals
  }
  __syncthreads();
  const int warp_base = warp > 0 ? smem32[warp - 1] : 0;
  *total = smem32[nwarps - 1];
  __syncthreads();
  return warp_base + x - v;
}

// Sphere callback of the spec (closest point of the box; strict "<").
__device__ __forceinline__ bool sphere_hits(float4 mn, float4 mx, const float* c, float rsq) {
  float t[3];
  const float bmin[3] = {mn.x, mn.y, mn.z};
  const float bmax[3] = {mx.x, mx.y, mx.z};
#pragma unroll
  for (int i = 0; i < 3; i++) {
    float nearest;
    if (bmin[i] > c[i]) {
      nearest = bmin[i];
    } else if (bmax[i] < c[i]) {
      nearest = bmax[i];
    } else {
      nearest = c[i];
    }
    t[i] = c[i] - nearest;
  }
  return (t[0] * t[0] + t[1] * t[1] + t[2] * t[2]) < rsq;
}

// BKE_pbvh_search_gather with the sphere callback (pbvh.c:2622-2767).  A leaf
// is gathered when it and every ancestor pass the callback (the DFS prunes a
// failing internal node's subtree).  Leaves are numbered by their left-first
// DFS rank, so emitting passing leaves in rank order reproduces the
// reference's output order.  One CTA; per-node results in shared memory.
__global__ void __launch_bounds__(kCullThreads) k_cull(DevMesh m, PassParams pp) {
  extern __shared__ unsigned char pass[];
  __shared__ int smem32[32];
  __shared__ int run_cnt, run_verts;
  const float4* bb = pp.original ? m.orig_vb : m.vb;
  for (int n = threadIdx.x; n < m.totnode; n += blockDim.x)
    pass[n] = sphere_hits(bb[2 * n], bb[2 * n + 1], pp.loc, pp.cull_radius_sq) ? 1 : 0;
  if (threadIdx.x == 0) {
    run_cnt = 0;
    run_verts = 0;
  }
  __syncthreads();
  for (int base = 0; base < m.nleaf; base += blockDim.x) {
    const int id = base + threadIdx.x;
    int ok = 0, nv = 0;
    if (id < m.nleaf) {
      int node = m.leaf_node[id];
      ok = pass[node];
      int p = m.node_parent[node];
      while (ok && p >= 0) {
        ok = pass[p];
        p = m.node_parent[p];
      }
      nv = ok ? leaf_nverts(m, id) : 0;
    }
    int tot_ok, tot_nv;
    const int pos = block_exclusive_scan(ok, &tot_ok, smem32);
    const int voff = block_exclusive_scan(nv, &tot_nv, smem32);
    if (ok) {
      m.cull_list[run_cnt + pos] = id;
      m.cull_off[run_cnt + pos] = run_verts + voff;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      run_cnt += tot_ok;
      run_verts += tot_nv;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    m.work->cull_count = run_cnt;
    m.cull_off[run_cnt] = run_verts;
  }
  // 24 B per node box tested, 8 B per leaf emitted (id + vertex offset).
  prof_add(m, kKCull, threadIdx.x == 0 ? 24ull * m.totnode + 8ull * run_cnt : 0ull);
}

// Host-provided node list: node indices -> leaf ids and vertex prefix.
__global__ void __launch_bounds__(kCullThreads) k_set_list(DevMesh m, const int* nodes,
                                                           int totnode) {
  __shared__ int smem32[32];
  __shared__ int run_verts;
  if (threadIdx.x == 0) run_verts = 0;
  __syncthreads();
  for (int base = 0; base < totnode; base += blockDim.x) {
    const int k = base + threadIdx.x;
    int nv = 0, id = -1;
    if (k < totnode) {
      const int node = nodes[k];
      if (node < 0 || node >= m.totnode || m.node_leaf[node] < 0) {
        set_err(m, SGPU_ERR_INVALID_ARG);
      } else {
        id = m.node_leaf[node];
        nv = leaf_nverts(m, id);
      }
    }
    int tot_nv;
    const int voff = block_exclusive_scan(nv, &tot_nv, smem32);
    if (k < totnode) {
      m.cull_list[k] = id < 0 ? 0 : id;
      m.cull_off[k] = run_verts + voff;
    }
    __syncthreads();
    if (threadIdx.x == 0) run_verts += tot_nv;
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    m.work->cull_count = totnode;
    m.cull_off[totnode] = run_verts;
  }
}

// ---------------------------------------------------------------------------
// Area normal / centre (spec): each culled leaf in blocks of kAreaBlock
// visited vertices (area_blocks per leaf, the empty ones zero); in a block,
// lane t (of 256) sums its elements t, t+256, ... with compensated sums;
// lanes merge pairwise (t, t+s) for s = 128 .. 1; the block partials then
// merge pairwise over (culled-list index, block) in order, (i, i+s),
// s = 1, 2, 4, ...  The last CTA to finish performs that final tree.

__global__ void __launch_bounds__(kThreads) k_area(DevMesh m, DevBrush b, PassParams pp) {
  __shared__ Lane sl[kThreads];
  __shared__ bool am_last;
  const int cnt = m.work->cull_count;
  const float rn = b.radius * b.normal_radius_factor;
  const float ra = b.radius * b.area_radius_factor;
  const float rn2 = rn * rn, ra2 = ra * ra;
  const int t = threadIdx.x;
  unsigned long long ab = 0;  // algorithmic bytes (profiling)
  const int nb = m.area_blocks;
  const int nparts = cnt * nb;
  for (int k = blockIdx.x; k < nparts; k += gridDim.x) {
    const int leaf = m.cull_list[k / nb];
    const int i0 = (k % nb) * kAreaBlock;
    const int nv = min(leaf_nverts(m, leaf), i0 + kAreaBlock);
    Lane l;
#pragma unroll
    for (int q = 0; q < 6; q++) l.v[q].s = l.v[q].e = 0.0f;
    l.n_no = l.n_co = 0;
    for (int i = i0 + t; i < nv; i += kThreads) {
      const int v = leaf_vert(m, leaf, i);
      const float4 co = m.co[v];
      const float d2 = dist_sq(co, pp.loc);
      ab += (m.type == kFaces ? 4u : 0u) + 24u;  // index, co, no
      if (d2 <= rn2) {
        const float4 no = m.no[v];
        cs_add(l.v[0], no.x);
        cs_add(l.v[1], no.y);
        cs_add(l.v[2], no.z);
        l.n_no++;
      }
      if (d2 <= ra2) {
        cs_add(l.v[3], co.x);
        cs_add(l.v[4], co.y);
        cs_add(l.v[5], co.z);
        l.n_co++;
      }
    }
    sl[t] = l;
    __syncthreads();
    for (int s = kThreads / 2; s >= 32; s >>= 1) {
      if (t < s) {
        Lane a = sl[t];
        lane_merge(a, sl[t + s]);
        sl[t] = a;
      }
      __syncthreads();
    }
    if (t < 32) {
      Lane a = sl[t];
      for (int s = 16; s >= 1; s >>= 1) {
        const Lane o = lane_shfl_down(a, s);
        lane_merge(a, o);
      }
      if (t == 0) part_store(&m.parts[k], a);
    }
    __syncthreads();
  }
  prof_add(m, kKArea, ab);
  __threadfence();
  __syncthreads();
  if (t == 0) {
    const unsigned int ticket = atomicAdd(&m.work->ticket_area, 1u);
    am_last = (ticket == gridDim.x - 1);
  }
  __syncthreads();
  if (!am_last) return;
  __threadfence();
  for (int s = 1; s < nparts; s <<= 1) {
    for (int i = t * 2 * s; i + s < nparts; i += kThreads * 2 * s) {
      Lane a = part_load(&m.parts[i]);
      lane_merge(a, part_load(&m.parts[i + s]));
      part_store(&m.parts[i], a);
    }
    __threadfence_block();
    __syncthreads();
  }
  if (t == 0) {
    Lane tot;
    if (nparts > 0) {
      tot = part_load(&m.parts[0]);
    } else {
#pragma unroll
      for (int q = 0; q < 6; q++) tot.v[q].s = tot.v[q].e = 0.0f;
      tot.n_no = tot.n_co = 0;
    }
    float nx = tot.v[0].s + tot.v[0].e;
    float ny = tot.v[1].s + tot.v[1].e;
    float nz = tot.v[2].s + tot.v[2].e;
    normalize3(nx, ny, nz);
    float cx, cy, cz;
    if (tot.n_co > 0) {
      const float inv = 1.0f / (float)tot.n_co;
      cx = (tot.v[3].s + tot.v[3].e) * inv;
      cy = (tot.v[4].s + tot.v[4].e) * inv;
      cz = (tot.v[5].s + tot.v[5].e) * inv;
    } else {
      cx = pp.loc[0];
      cy = pp.loc[1];
      cz = pp.loc[2];
    }
    Work* w = m.work;
    w->area_no[0] = nx;
    w->area_no[1] = ny;
    w->area_no[2] = nz;
    w->area_co[0] = cx;
    w->area_co[1] = cy;
    w->area_co[2] = cz;
    w->area_n_co = tot.n_co;
    w->ticket_area = 0u;
  }
}

// ---------------------------------------------------------------------------
// Brushes.  Work item i in [0, cull_off[cnt]) is vertex (i - cull_off[k]) of
// culled leaf k, found by binary search over cull_off.

__device__ __forceinline__ int find_slot(const int* off, int cnt, int i) {
  int lo = 0, hi = cnt;  // off[lo] <= i < off[hi]
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (__ldg(&off[mid]) <= i) {
      lo = mid;
    } else {
      hi = mid;
    }
  }
  return lo;
}

__device__ __forceinline__ void count_displaced(const DevMesh& m, bool moved) {
  const unsigned int bal = __ballot_sync(0xffffffffu, moved);
  if ((threadIdx.x & 31) == 0 && bal) atomicAdd(&m.work->displaced, (unsigned long long)__popc(bal));
}

__device__ __forceinline__ void mark_culled(const DevMesh& m, int cnt) {
  if (blockIdx.x == 0)
    for (int k = threadIdx.x; k < cnt; k += blockDim.x) atomicOr(&m.leaf_flag[m.cull_list[k]], kMarkUpdate);
}

__device__ __forceinline__ void load_curve(const DevBrush& b, float* y) {
  for (int i = threadIdx.x; i <= kCurveTable; i += blockDim.x) y[i] = b.y[i];
  __syncthreads();
}

// ---------------------------------------------------------------------------
// Original-data brushes (grab, elastic deform): one dab over all its passes.

// Leaves whose orig_vb box (and every ancestor's) meets any pass sphere, or
// every leaf (all != 0), in left-first order: the union of the passes' lists
// (a box meeting a sphere implies its ancestors' boxes meet it).
__global__ void __launch_bounds__(kCullThreads) k_cull_dab(DevMesh m, DabPasses dp,
                                                           float radius_sq, int all) {
  extern __shared__ unsigned char pass[];
  __shared__ int smem32[32];
  __shared__ int run_cnt, run_verts;
  for (int n = threadIdx.x; n < m.totnode; n += blockDim.x) {
    int ok = all;
    for (int p = 0; p < dp.npass && !ok; p++)
      ok = sphere_hits(m.orig_vb[2 * n], m.orig_vb[2 * n + 1], dp.loc[p], radius_sq) ? 1 : 0;
    pass[n] = static_cast<unsigned char>(ok);
  }
  if (threadIdx.x == 0) {
    run_cnt = 0;
    run_verts = 0;
  }
  __syncthreads();
  for (int base = 0; base < m.nleaf; base += blockDim.x) {
    const int id = base + threadIdx.x;
    int ok = 0, nv = 0;
    if (id < m.nleaf) {
      int node = m.leaf_node[id];
      ok = pass[node];
      int p = m.node_parent[node];
      while (ok && p >= 0) {
        ok = pass[p];
        p = m.node_parent[p];
      }
      nv = ok ? leaf_nverts(m, id) : 0;
    }
    int tot_ok, tot_nv;
    const int pos = block_exclusive_scan(ok, &tot_ok, smem32);
    const int voff = block_exclusive_scan(nv, &tot_nv, smem32);
    if (ok) {
      m.cull_list[run_cnt + pos] = id;
      m.cull_off[run_cnt + pos] = run_verts + voff;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      run_cnt += tot_ok;
      run_verts += tot_nv;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    m.work->cull_count = run_cnt;
    m.cull_off[run_cnt] = run_verts;
  }
  prof_add(m, kKCull, threadIdx.x == 0 ? 24ull * m.totnode + 8ull * run_cnt : 0ull);
}

// One dab of grab / elastic deform over the gathered leaves (orig_vertex).
__global__ void __launch_bounds__(kThreads) k_orig_dab(DevMesh m, DevBrush b, DabPasses dp) {
  __shared__ float ys[kCurveTable + 1];
  load_curve(b, ys);
  const int cnt = m.work->cull_count;
  const int total = m.cull_off[cnt];
  mark_culled(m, cnt);
  unsigned long long ab = 0;
  const int stride = gridDim.x * blockDim.x;
  for (int base = blockIdx.x * blockDim.x; base < total; base += stride) {
    const int i = base + threadIdx.x;
    unsigned int moved = 0u;
    if (i < total) {
      const int k = find_slot(m.cull_off, cnt, i);
      const int v = leaf_vert(m, m.cull_list[k], i - m.cull_off[k]);
      float4 co = m.co[v];
      moved = orig_vertex(m, b, ys, dp, v, co);
      m.co[v] = co;
      if (m.type == kFaces) m.vtag[v] = 1;
      // index, original position (+ normal for the front face), mask, automask; position write
      ab += (m.type == kFaces ? 4u : 0u) + 12u + ((b.flag & kBrushFrontFace) ? 12u : 0u) +
            (m.mask ? 4u : 0u) + (m.automask ? 4u : 0u) + 12u;
    }
    const unsigned int sum = __reduce_add_sync(0xffffffffu, moved);
    if ((threadIdx.x & 31) == 0 && sum) atomicAdd(&m.work->displaced, (unsigned long long)sum);
  }
  prof_add(m, kKBrush, ab);
}

// Draw, inflate and clay strips (one pass each; positions written in place,
// each vertex by exactly one thread since leaves expose unique vertices).
__global__ void __launch_bounds__(kThreads) k_brush(DevMesh m, DevBrush b, PassParams pp) {
  __shared__ float ys[kCurveTable + 1];
  load_curve(b, ys);
  const int cnt = m.work->cull_count;
  const int total = m.cull_off[cnt];
  float area_no[3] = {0.0f, 0.0f, 0.0f}, area_co[3] = {0.0f, 0.0f, 0.0f};
  if (uses_area(b.tool)) {
    for (int k = 0; k < 3; k++) {
      area_no[k] = __ldcg(&m.work->area_no[k]);
      area_co[k] = __ldcg(&m.work->area_co[k]);
    }
  }
  BrushFrame f;
  if (!make_frame(b, pp, area_no, area_co, f)) return;
  mark_culled(m, cnt);
  unsigned long long ab = 0;  // algorithmic bytes (profiling)
  const int stride = gridDim.x * blockDim.x;
  for (int base = blockIdx.x * blockDim.x; base < total; base += stride) {
    const int i = base + threadIdx.x;
    bool moved = false;
    if (i < total) {
      const int k = find_slot(m.cull_off, cnt, i);
      const int v = leaf_vert(m, m.cull_list[k], i - m.cull_off[k]);
      float4 co = m.co[v];
      const bool hit = b.tool == kToolLayer ? layer_vertex(m, b, ys, pp, v, co, moved)
                                            : brush_vertex(m, b, ys, pp, f, v, co, moved);
      if (hit) {
        m.co[v] = co;
        if (m.type == kFaces) m.vtag[v] = 1;
      }
      // index, co, mask, automask, normal (inflate / front-face); co write on a hit
      ab += (m.type == kFaces ? 4u : 0u) + 12u + (m.mask ? 4u : 0u) + (m.automask ? 4u : 0u) +
            ((b.tool == kToolInflate || (b.flag & kBrushFrontFace)) ? 12u : 0u) + (hit ? 12u : 0u);
    }
    count_displaced(m, moved);
  }
  prof_add(m, kKBrush, ab);
}

// Smooth, one Jacobi sweep in two launches: compute new positions from the
// sweep-start state into scratch (w = 1 marks a hit), then write them back.
__global__ void __launch_bounds__(kThreads) k_smooth_compute(DevMesh m, DevBrush b,
                                                             PassParams pp) {
  __shared__ float ys[kCurveTable + 1];
  load_curve(b, ys);
  const int cnt = m.work->cull_count;
  const int total = m.cull_off[cnt];
  if (pp.iteration == 0) mark_culled(m, cnt);
  unsigned long long ab = 0;  // algorithmic bytes (profiling)
  const int stride = gridDim.x * blockDim.x;
  for (int base = blockIdx.x * blockDim.x; base < total; base += stride) {
    const int i = base + threadIdx.x;
    bool moved = false;
    if (i < total) {
      const int k = find_slot(m.cull_off, cnt, i);
      const int v = leaf_vert(m, m.cull_list[k], i - m.cull_off[k]);
      const float4 co = m.co[v];
      float4 out = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
      bool mv = false;
      if (smooth_vertex(m, b, ys, pp, v, co, out, mv)) {
        out.w = 1.0f;
        moved = (pp.iteration == 0) && mv;
        const int valence = m.type == kFaces ? m.nb_off[v + 1] - m.nb_off[v] : 4;
        ab += (m.type == kFaces ? 8u : 0u) + 16ull * valence;  // ring range, ring ids + co
      } else {
        out = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
      }
      m.scratch[i] = out;
      ab += (m.type == kFaces ? 4u : 0u) + 12u + (m.mask ? 4u : 0u) + 16u;  // idx, co, mask, out
    }
    count_displaced(m, moved);
  }
  prof_add(m, kKSmoothCompute, ab);
}

__global__ void __launch_bounds__(kThreads) k_smooth_apply(DevMesh m) {
  const int cnt = m.work->cull_count;
  const int total = m.cull_off[cnt];
  const int stride = gridDim.x * blockDim.x;
  unsigned long long ab = 0;  // algorithmic bytes (profiling)
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += stride) {
    const float4 s = m.scratch[i];
    ab += 16u;
    if (s.w == 0.0f) continue;
    const int k = find_slot(m.cull_off, cnt, i);
    const int v = leaf_vert(m, m.cull_list[k], i - m.cull_off[k]);
    float4 co = m.co[v];
    co.x = s.x;
    co.y = s.y;
    co.z = s.z;
    m.co[v] = co;
    if (m.type == kFaces) m.vtag[v] = 1;
    ab += (m.type == kFaces ? 4u : 0u) + 12u;
  }
  prof_add(m, kKSmoothApply, ab);
}

// ---------------------------------------------------------------------------
// FACES normal update (gather form of pbvh.c:2912-3036) fused with the leaf
// bounding-box refit (update_node_vb over PBVH_ITER_ALL, pbvh.c:2026-2046;
// pbvh_update_BB_redraw, pbvh.c:3124-3160).  The last CTA clears the
// UpdateNormals flags and runs the bottom-up flush (pbvh_flush_bb,
// pbvh.c:3287-3317) level by level.


__device__ void leaf_refit(const DevMesh& m, int leaf, float* red /* 6*kThreads/32 */,
                           unsigned long long& ab) {
  float mn[3] = {FLT_MAX, FLT_MAX, FLT_MAX};
  float mx[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
  (void)red;
  const int nv = leaf_nverts_all(m, leaf);
  // co of every leaf vertex (+ its index for FACES); the node box written once
  if (threadIdx.x < nv)
    ab += (m.type == kFaces ? 16ull : 12ull) * ((nv - threadIdx.x + blockDim.x - 1) / blockDim.x);
  if (threadIdx.x == 0) ab += 24u;
  // chunk boxes (one warp per chunk of kChunk entries), then their union
  const int nch = m.leaf_chunk_off[leaf + 1] - m.leaf_chunk_off[leaf];
  for (int c = threadIdx.x >> 5; c < nch; c += blockDim.x >> 5) chunk_refit_warp(m, leaf, c, mn, mx);
  __syncthreads();
  if (threadIdx.x < 32) leaf_box_from_chunks(m, leaf);
  __syncthreads();
}

// Chunk boxes of every leaf (mesh creation, positions replaced): one warp per
// chunk, grid-stride over all chunks.
__global__ void __launch_bounds__(kThreads) k_chunk_boxes_all(DevMesh m, int nchunks) {
  float mn[3], mx[3];
  const int warps = gridDim.x * (blockDim.x >> 5);
  for (int id = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); id < nchunks; id += warps) {
    int lo = 0, hi = m.nleaf;  // leaf_chunk_off[lo] <= id < leaf_chunk_off[hi]
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if (m.leaf_chunk_off[mid] <= id) {
        lo = mid;
      } else {
        hi = mid;
      }
    }
    chunk_refit_warp(m, lo, id - m.leaf_chunk_off[lo], mn, mx);
  }
}

cudaError_t launch_chunk_boxes_all(const DevMesh& m, int nchunks, cudaStream_t s) {
  int g = (nchunks + (kThreads / 32) - 1) / (kThreads / 32);
  if (g > 4096) g = 4096;
  if (g < 1) g = 1;
  k_chunk_boxes_all<<<g, kThreads, 0, s>>>(m, nchunks);
  return cudaGetLastError();
}

__device__ void faces_leaf_normals(const DevMesh& m, int leaf, unsigned long long& ab) {
  const int off = m.leaf_vert_off[leaf];
  const int nu = m.leaf_uniq[leaf];
  for (int i = threadIdx.x; i < nu; i += blockDim.x) {
    const int v = m.leaf_verts[off + i];
    if (!m.vtag[v]) continue;
    float4 n;
    const int used = vertex_normal(m, v, n);
    // the vertex's co read and normal written; one looptri record per face used
    ab += 24u + 16u * used;
    m.no[v] = n;
    m.vtag[v] = 0;
  }
}

// Bottom-up flush of updated boxes, run by one CTA.
__device__ void flush_bounds(const DevMesh& m, int flag) {
  const int bits = flag & (kUpdateBB | kUpdateOriginalBB);
  for (int leaf = threadIdx.x; leaf < m.nleaf; leaf += blockDim.x) {
    const int node = m.leaf_node[leaf];
    const int f = m.leaf_flag[leaf];
    m.node_upd[node] = (unsigned char)(f & bits);
    if (f & bits) m.leaf_flag[leaf] = f & ~bits;
  }
  __syncthreads();
  for (int l = 0; l < m.nlevels; l++) {
    const int b0 = m.level_off[l], b1 = m.level_off[l + 1];
    for (int j = b0 + threadIdx.x; j < b1; j += blockDim.x) {
      const int node = m.level_nodes[j];
      const int c = m.node_child[node];
      const int u = m.node_upd[c] | m.node_upd[c + 1];
      m.node_upd[node] = (unsigned char)u;
      if (u & kUpdateBB) {
        const float4 a0 = m.vb[2 * c], a1 = m.vb[2 * c + 1];
        const float4 c0 = m.vb[2 * (c + 1)], c1 = m.vb[2 * (c + 1) + 1];
        float4 mn, mx;
        mn.x = fmin_ref(fmin_ref(FLT_MAX, a0.x), c0.x);
        mn.y = fmin_ref(fmin_ref(FLT_MAX, a0.y), c0.y);
        mn.z = fmin_ref(fmin_ref(FLT_MAX, a0.z), c0.z);
        mx.x = fmax_ref(fmax_ref(-FLT_MAX, a1.x), c1.x);
        mx.y = fmax_ref(fmax_ref(-FLT_MAX, a1.y), c1.y);
        mx.z = fmax_ref(fmax_ref(-FLT_MAX, a1.z), c1.z);
        mn.w = mx.w = 0.0f;
        m.vb[2 * node] = mn;
        m.vb[2 * node + 1] = mx;
      }
      if (u & kUpdateOriginalBB) {
        m.orig_vb[2 * node] = m.vb[2 * node];
        m.orig_vb[2 * node + 1] = m.vb[2 * node + 1];
      }
    }
    __syncthreads();
  }
}

__global__ void __launch_bounds__(kThreads) k_update_faces(DevMesh m, int do_normals,
                                                           int bounds_flag) {
  __shared__ float red[6 * (kThreads / 32)];
  __shared__ bool am_last;
  unsigned long long ab = 0;  // algorithmic bytes (profiling)
  for (int leaf = blockIdx.x; leaf < m.nleaf; leaf += gridDim.x) {
    const int f = m.leaf_flag[leaf];
    if (do_normals && m.type == kFaces && (f & kUpdateNormals)) faces_leaf_normals(m, leaf, ab);
    if ((bounds_flag & kUpdateBB) && (f & kUpdateBB)) leaf_refit(m, leaf, red, ab);
    if (threadIdx.x == 0) {
      const int node = m.leaf_node[leaf];
      if ((bounds_flag & kUpdateOriginalBB) && (f & kUpdateOriginalBB)) {
        m.orig_vb[2 * node] = m.vb[2 * node];
        m.orig_vb[2 * node + 1] = m.vb[2 * node + 1];
      }
      if ((bounds_flag & kUpdateRedraw) && (f & kUpdateRedraw))
        atomicAnd(&m.leaf_flag[leaf], ~kUpdateRedraw);
    }
  }
  prof_add(m, kKUpdate, ab);
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) {
    const unsigned int ticket = atomicAdd(&m.work->ticket_update, 1u);
    am_last = (ticket == gridDim.x - 1);
  }
  __syncthreads();
  if (!am_last) return;
  __threadfence();
  if (do_normals && m.type == kFaces) {
    for (int leaf = threadIdx.x; leaf < m.nleaf; leaf += blockDim.x)
      m.leaf_flag[leaf] &= ~kUpdateNormals;
    __syncthreads();
  }
  if (bounds_flag & (kUpdateBB | kUpdateOriginalBB)) flush_bounds(m, bounds_flag);
  if (threadIdx.x == 0) m.work->ticket_update = 0u;
}

__global__ void k_mark_all(DevMesh m, int bits) {
  for (int leaf = blockIdx.x * blockDim.x + threadIdx.x; leaf < m.nleaf;
       leaf += gridDim.x * blockDim.x)
    atomicOr(&m.leaf_flag[leaf], bits);
}

cudaError_t launch_mark_all(const DevMesh& m, int bits, cudaStream_t s) {
  k_mark_all<<<(m.nleaf + kThreads - 1) / kThreads, kThreads, 0, s>>>(m, bits);
  return cudaGetLastError();
}

__global__ void k_mark_node(DevMesh m, int node) {
  if (node >= 0 && node < m.totnode && m.node_leaf[node] >= 0)
    atomicOr(&m.leaf_flag[m.node_leaf[node]], kMarkUpdate);
}

// ---------------------------------------------------------------------------
// Launchers

static int g_grid = 0;

static int work_grid() {
  if (g_grid == 0) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    g_grid = sms > 0 ? 2 * sms : 264;
  }
  return g_grid;
}

cudaError_t launch_cull(const DevMesh& m, const PassParams& pp, cudaStream_t s) {
  const size_t smem = (static_cast<size_t>(m.totnode) + 15) & ~static_cast<size_t>(15);
  k_cull<<<1, kCullThreads, smem, s>>>(m, pp);
  return cudaGetLastError();
}

cudaError_t launch_cull_dab(const DevMesh& m, const DabPasses& dp, float radius_sq, int all,
                           cudaStream_t s) {
  const size_t smem = (static_cast<size_t>(m.totnode) + 15) & ~static_cast<size_t>(15);
  k_cull_dab<<<1, kCullThreads, smem, s>>>(m, dp, radius_sq, all);
  return cudaGetLastError();
}

cudaError_t launch_orig_dab(const DevMesh& m, const DevBrush& b, const DabPasses& dp,
                            cudaStream_t s) {
  k_orig_dab<<<work_grid(), kThreads, 0, s>>>(m, b, dp);
  return cudaGetLastError();
}

cudaError_t launch_set_list(const DevMesh& m, const int* dev_nodes, int totnode,
                            cudaStream_t s) {
  k_set_list<<<1, kCullThreads, 0, s>>>(m, dev_nodes, totnode);
  return cudaGetLastError();
}

cudaError_t launch_area(const DevMesh& m, const DevBrush& b, const PassParams& pp,
                        cudaStream_t s) {
  const int items = m.nleaf * m.area_blocks;
  int g = items < work_grid() ? items : work_grid();
  if (g < 1) g = 1;
  k_area<<<g, kThreads, 0, s>>>(m, b, pp);
  return cudaGetLastError();
}

cudaError_t launch_brush(const DevMesh& m, const DevBrush& b, const PassParams& pp,
                         cudaStream_t s) {
  k_brush<<<work_grid(), kThreads, 0, s>>>(m, b, pp);
  return cudaGetLastError();
}

cudaError_t launch_smooth_compute(const DevMesh& m, const DevBrush& b, const PassParams& pp,
                                  cudaStream_t s) {
  k_smooth_compute<<<work_grid(), kThreads, 0, s>>>(m, b, pp);
  return cudaGetLastError();
}

cudaError_t launch_smooth_apply(const DevMesh& m, cudaStream_t s) {
  k_smooth_apply<<<work_grid(), kThreads, 0, s>>>(m);
  return cudaGetLastError();
}

__global__ void k_l2_flush(uint4* buf, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    buf[i] = make_uint4((unsigned)i, 0u, 0u, 0u);
}

// Reads a buffer larger than L2, so that the dirty lines the write left are
// written back now and L2 holds clean lines of an unrelated buffer.
__global__ void k_l2_read(const uint4* buf, size_t n, unsigned int* sink) {
  unsigned int acc = 0u;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    const uint4 v = __ldcg(&buf[i]);
    acc ^= v.x ^ v.y ^ v.z ^ v.w;
  }
  if (acc == 0x9e3779b9u) sink[0] = acc;  // keeps the loads
}

cudaError_t launch_l2_flush(void* buf, size_t bytes, cudaStream_t s) {
  // write the first half, then read the second half (written once at allocation)
  const size_t half = bytes / 2;
  k_l2_flush<<<work_grid() * 4, kThreads, 0, s>>>(static_cast<uint4*>(buf), half / 16);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  k_l2_read<<<work_grid() * 4, kThreads, 0, s>>>(
      reinterpret_cast<const uint4*>(static_cast<char*>(buf) + half), half / 16,
      static_cast<unsigned int*>(buf));
  return cudaGetLastError();
}

cudaError_t launch_update_faces(const DevMesh& m, int do_normals, int bounds_flag,
                                cudaStream_t s) {
  int g = m.nleaf < work_grid() ? m.nleaf : work_grid();
  if (g < 1) g = 1;
  k_update_faces<<<g, kThreads, 0, s>>>(m, do_normals, bounds_flag);
  return cudaGetLastError();
}

cudaError_t launch_mark_node(const DevMesh& m, int node, cudaStream_t s) {
  k_mark_node<<<1, 1, 0, s>>>(m, node);
  return cudaGetLastError();
}

// Conversions between a caller's vertex order and the device order:
// out[i] = in[idx[i]] (whole float4 or one float).
__global__ void k_gather_f4(float4* out, const float4* in, const int* idx, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) out[i] = in[idx[i]];
}
__global__ void k_gather_f1(float* out, const float* in, const int* idx, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) out[i] = in[idx[i]];
}

// Packed xyz (3 floats per vertex, the caller's layout) to and from the
// float4 device arrays, through an optional order map (idx, nullable).
__global__ void k_xyz_to_f4(float4* out, const float* in3, const int* idx, int n, int keep_w) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const size_t j = 3 * static_cast<size_t>(idx ? idx[i] : i);
    out[i] = make_float4(in3[j], in3[j + 1], in3[j + 2], keep_w ? out[i].w : 0.0f);
  }
}
__global__ void k_f4_to_xyz(float* out3, const float4* in, const int* idx, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float4 a = in[idx ? idx[i] : i];
    const size_t j = 3 * static_cast<size_t>(i);
    out3[j] = a.x;
    out3[j + 1] = a.y;
    out3[j + 2] = a.z;
  }
}

// The positions of a GRIDS stroke back into the caller's page-locked output
// (out3, 3 floats per element, mapped into the device's address space): a
// grid whose positions equal the stroke's input (in3, the same layout) bit for
// bit is not written (the host copied the input there); a changed grid is
// written whole.  One CTA per grid at a time.
__global__ void k_grid_writeback(float* out3, const float4* co, const float* in3, int ngrids, int area) {
  for (int g = blockIdx.x; g < ngrids; g += gridDim.x) {
    const size_t e0 = static_cast<size_t>(g) * area;
    int diff = 0;
    for (int i = threadIdx.x; i < area; i += blockDim.x) {
      const float4 a = co[e0 + i];
      const float* b = in3 + 3 * (e0 + i);
      diff |= (__float_as_uint(a.x) != __float_as_uint(b[0])) | (__float_as_uint(a.y) != __float_as_uint(b[1])) |
              (__float_as_uint(a.z) != __float_as_uint(b[2]));
    }
    if (__syncthreads_or(diff)) {
      for (int i = threadIdx.x; i < area; i += blockDim.x) {
        const float4 a = co[e0 + i];
        float* o = out3 + 3 * (e0 + i);
        o[0] = a.x;
        o[1] = a.y;
        o[2] = a.z;
      }
    }
  }
}

// The same for a FACES stroke: the caller's vertex order (co[idx[i]] is its
// vertex i; records of 16 bytes, the MVert layout), blocks of blockDim.x
// vertices compared bitwise with the input (in) and written whole when changed.
__global__ void k_vert_writeback(float4* out, const float4* co, const int* idx, const float4* in, int n) {
  for (int b0 = blockIdx.x * blockDim.x; b0 < n; b0 += gridDim.x * blockDim.x) {
    const int i = b0 + threadIdx.x;
    float4 a = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    int diff = 0;
    if (i < n) {
      a = co[idx[i]];
      const float4 c = in[i];
      diff = (__float_as_uint(a.x) != __float_as_uint(c.x)) | (__float_as_uint(a.y) != __float_as_uint(c.y)) |
             (__float_as_uint(a.z) != __float_as_uint(c.z)) | (__float_as_uint(a.w) != __float_as_uint(c.w));
    }
    if (__syncthreads_or(diff) && i < n) out[i] = a;
  }
}

static int gather_grid(int n) {
  const int g = (n + kThreads - 1) / kThreads;
  const int cap = 4 * work_grid();
  return g < 1 ? 1 : (g > cap ? cap : g);
}

cudaError_t launch_gather_f4(float4* out, const float4* in, const int* idx, int n, cudaStream_t s) {
  k_gather_f4<<<gather_grid(n), kThreads, 0, s>>>(out, in, idx, n);
  return cudaGetLastError();
}
cudaError_t launch_gather_f1(float* out, const float* in, const int* idx, int n, cudaStream_t s) {
  k_gather_f1<<<gather_grid(n), kThreads, 0, s>>>(out, in, idx, n);
  return cudaGetLastError();
}
cudaError_t launch_xyz_to_f4(float4* out, const float* in3, const int* idx, int n, bool keep_w,
                             cudaStream_t s) {
  k_xyz_to_f4<<<gather_grid(n), kThreads, 0, s>>>(out, in3, idx, n, keep_w ? 1 : 0);
  return cudaGetLastError();
}
cudaError_t launch_f4_to_xyz(float* out3, const float4* in, const int* idx, int n, cudaStream_t s) {
  k_f4_to_xyz<<<gather_grid(n), kThreads, 0, s>>>(out3, in, idx, n);
  return cudaGetLastError();
}
cudaError_t launch_vert_writeback(float4* out, const float4* co, const int* idx, const float4* in, int n,
                                  cudaStream_t s) {
  k_vert_writeback<<<gather_grid(n), kThreads, 0, s>>>(out, co, idx, in, n);
  return cudaGetLastError();
}
cudaError_t launch_grid_writeback(float* out3, const float4* co, const float* in3, int ngrids, int area,
                                  cudaStream_t s) {
  const int cap = 8 * work_grid();
  k_grid_writeback<<<ngrids < cap ? (ngrids > 0 ? ngrids : 1) : cap, 128, 0, s>>>(out3, co, in3, ngrids, area);
  return cudaGetLastError();
}

int cull_smem_limit() { return 200 * 1024; }

void configure_kernels() {
  cudaFuncSetAttribute(k_cull, cudaFuncAttributeMaxDynamicSharedMemorySize, cull_smem_limit());
}

}  // namespace sgpu
