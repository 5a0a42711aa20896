// Persistent stroke kernel of libsculptgpu (device code).  kernels_team.cu
// launches it as cluster teams, kernels_wide.cu as one team over the whole
// GPU.
//
// One launch runs whole strokes.  A team (a thread-block cluster of C CTAs of
// 256 threads, C chosen by the autotuner, or every CTA of a cooperative launch
// with one CTA per SM) takes a mesh's stroke and runs every dab of it: per
// symmetry pass the node search, the area normal/centre, the brush (smooth as
// Jacobi sweeps over a compacted list of vertices inside the sphere), then
// the normal update and the bounding-box refit with its flush;
// UpdateOriginalBB at the end of the stroke.  Phases are separated by team
// barriers: barrier.cluster arrive.release / wait.acquire for a cluster, a
// counter in global memory (release add, bounded wait, acquire fence) for the
// whole GPU, so no phase waits for a kernel boundary.  Cluster teams take
// meshes from a work queue (an atomic job counter); meshes are independent,
// teams never wait for one another, and a team that starts late simply finds
// fewer jobs.  The whole-GPU team runs its jobs in order.
//
// The arithmetic is the same device code as the per-call kernels
// (sgpu_device.cuh), so results are bit-identical to them and to the FP32
// restatement of the reference.
#pragma once

#include <algorithm>
#include <map>
#include <mutex>
#include <tuple>
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include "sgpu_device.cuh"
#include "sgpu_grids.cuh"
#include "sgpu_kernels.h"
#include "sgpu_team.h"

namespace cg = cooperative_groups;

namespace sgpu {

constexpr int kTeamThreads = 256;
// Shared staging region at the start of the dynamic shared memory: the smooth
// neighbour tables, the area stage, or a claimed face's grids (never live at
// the same time).
constexpr size_t kStageBytes = 40960;
static_assert(sizeof(float4) * kNbCache * kTeamThreads <= kStageBytes, "smooth tables");

struct TeamShared {
  DevMesh m;
  TeamJob job;
  int jobid;
  int cnt, total;
  int scan[32];
  unsigned long long scan64[32];
  int nh;                  // smooth hits of this CTA in the current pass
  int hv[kTeamThreads];    // their vertices and positions (first kTeamThreads)
  float4 hco[kTeamThreads];
  float area[6];
  int nmark;
  int bar_ok;    // outcome of the whole-GPU team barrier's wait
  DabPasses dp;  // passes of a grab / elastic deform dab
  // node search, second level: descendant ranges of the passing split-depth
  // nodes (at most 2^6) and their prefix
  int nrange;
  int2 crange[64];
  int croff[65];
  // both passes of a single-axis symmetry searched at once (team_cull_pair):
  // split = first list entry of the second pass when they run as one (joint;
  // the list's length otherwise); held = entries of the second pass's list
  // stored behind the first one's (-1: none), with its vertex total, first
  // entry and first offset; live1 = the joint second pass has a frame
  int split, joint, held, held_total, held_base, held_off, live1, pair_ovl;
  PassParams mpp[2];    // the passes' parameters and frames read by the area
  BrushFrame mframe[2]; // blocks and the sweep (one pass, or a joint pair)
};

// Block-wide exclusive scan (kTeamThreads threads).
static __device__ int team_block_scan(int v, int* total, int* smem32) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  constexpr int nwarps = kTeamThreads / 32;
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
  const int warp_base = warp > 0 ? smem32[warp - 1] : 0;
  *total = smem32[nwarps - 1];
  __syncthreads();
  return warp_base + x - v;
}

__device__ __forceinline__ bool box_hits(float4 mn, float4 mx, const float* c, float rsq) {
  const float bmin[3] = {mn.x, mn.y, mn.z};
  const float bmax[3] = {mx.x, mx.y, mx.z};
  float t[3];
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

__device__ __forceinline__ int smem_find_slot(const int* off, int cnt, int i) {
  int lo = 0, hi = cnt;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (off[mid] <= i) {
      lo = mid;
    } else {
      hi = mid;
    }
  }
  return lo;
}

// Appends v to list (counter cnt) with one atomic per coalesced group.
__device__ __forceinline__ void append(int* list, int* cnt, int v) {
  cg::coalesced_group g = cg::coalesced_threads();
  int base = 0;
  if (g.thread_rank() == 0) base = atomicAdd(cnt, static_cast<int>(g.size()));
  base = g.shfl(base, 0);
  list[base + g.thread_rank()] = v;
}

__device__ __forceinline__ void tag_vertex(const DevMesh& m, int v, int* tag_cnt) {
  if (atomicExch(&m.vtag[v], 1u) == 0u) append(m.tag_list, tag_cnt, v);
}

// Block-wide exclusive scan of 64-bit values (kTeamThreads threads).
static __device__ unsigned long long team_block_scan64(unsigned long long v, unsigned long long* total,
                                                unsigned long long* smem32) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  constexpr int nwarps = kTeamThreads / 32;
  unsigned long long x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned long long y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) smem32[warp] = x;
  __syncthreads();
  if (warp == 0) {
    unsigned long long w = lane < nwarps ? smem32[lane] : 0ull;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned long long y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    smem32[lane] = w;
  }
  __syncthreads();
  const unsigned long long warp_base = warp > 0 ? smem32[warp - 1] : 0ull;
  *total = smem32[nwarps - 1];
  __syncthreads();
  return warp_base + x - v;
}

// Per-job tables of the node search in shared memory (any type with the same
// two indexable members serves).
struct CullTabs {
  const unsigned short* lnode;  // leaf -> node
  const int* lnv;               // leaf -> brush-visible vertex count
};

// Node search of one pass into this CTA's shared memory (every CTA of the team
// computes the same list).  Same result and order as k_cull: a leaf is listed
// when its box and the boxes of all its ancestors pass.  Node boxes are
// tested in two levels: every node down to the mesh's split depth, then the
// descendants of the split-depth nodes that passed (kBox loads in flight per
// thread); a failing internal node covers the leaf-id range of its subtree
// (left-first DFS ranks), recorded as +1/-1 in a difference array; a running
// sum over the leaves then says which leaves lie under a failing ancestor.  Each thread owns a run of consecutive
// leaves (at most 64: the team kernel takes at most 64 * 256 leaves); block
// scans give the coverage entering the run and the list positions.  s_coff
// doubles as the difference array.
//
// kPair: two spheres at once (the two passes of a single-axis symmetry);
// hits returns a pass mask (bit p: the box meets sphere p), the difference
// array counts pass 0 in its low 16 bits and pass 1 above (coverage is at
// most the tree depth), and the lists are written one after the other:
// pass 0's at [0, sh.split), pass 1's behind it with its vertex offsets
// continuing from pass 0's total — when both fit the list arrays (cap
// entries; cap 0: one sphere, bit 1 never set).  Then: lists without a
// common leaf under a joinable tool (joinable 1; 2: and without a pair of
// leaves joined by a mesh edge, for the smooth brush's rings) make one list
// of both (sh.joint, sh.cnt and sh.total over both); otherwise sh.cnt and
// sh.total are pass 0's and sh.held counts pass 1's stored entries (-1 when
// they did not fit).
template <int kBox, bool kTwoLevel, bool kPair = false, class Hit, class Tabs>
__device__ __forceinline__ void team_cull_by(const DevMesh& m, const float4* bb, Hit hits,
                                             unsigned char* s_pass, int* s_cl, int* s_coff,
                                             const Tabs& ct, TeamShared& sh, int cap = 0,
                                             int joinable = 0, const int4* top = nullptr) {
  const int L = m.nleaf;
  for (int i = threadIdx.x; i <= L; i += kTeamThreads) s_coff[i] = 0;
  // one-level search (cull_ntop 0): the second level's single range is every node
  if (kTwoLevel && threadIdx.x == 0) {
    sh.nrange = m.cull_ntop == 0 ? 1 : 0;
    sh.crange[0] = make_int2(0, m.totnode);
  }
  if (kPair && threadIdx.x == 0) sh.pair_ovl = 0;
  __syncthreads();
  // A failing internal node marks its leaves' id range in the difference
  // array; every tested node records its outcome.
  auto outcome = [&](int n, unsigned hit, int llo, int lhi) {
    s_pass[n] = static_cast<unsigned char>(hit);
    if constexpr (kPair) {
      const int inc = ((hit & 1u) ? 0 : 1) + ((cap > 0 && !(hit & 2u)) ? 65536 : 0);
      if (inc != 0 && lhi - llo > 1) {
        atomicAdd(&s_coff[llo], inc);
        atomicAdd(&s_coff[lhi], -inc);
      }
    } else if (!hit && lhi - llo > 1) {  // internal node (leaves own a range of one)
      atomicAdd(&s_coff[llo], 1);
      atomicAdd(&s_coff[lhi], -1);
    }
  };
  if constexpr (!kTwoLevel) {
    // the build without the two-level code: every node box tested directly
    // (the same outcomes; launches whose trees are all small take it)
    for (int n0 = threadIdx.x; n0 < m.totnode; n0 += kBox * kTeamThreads) {
      float4 lo[kBox], hi[kBox];
      int llo[kBox], lhi[kBox];
#pragma unroll
      for (int j = 0; j < kBox; j++) {
        const int n = n0 + j * kTeamThreads;
        if (n < m.totnode) {
          lo[j] = __ldcg(&bb[2 * n]);
          hi[j] = __ldcg(&bb[2 * n + 1]);
          llo[j] = m.node_leaf_lo[n];
          lhi[j] = m.node_leaf_hi[n];
        }
      }
#pragma unroll
      for (int j = 0; j < kBox; j++) {
        const int n = n0 + j * kTeamThreads;
        if (n < m.totnode) outcome(n, hits(lo[j], hi[j]), llo[j], lhi[j]);
      }
    }
  } else {
  // First level: every node down to the split depth; a passing internal node
  // at the split depth lists its descendants' range for the second level.
  const int4* tops = top ? top : m.cull_top;  // (a copy on chip, when given)
  for (int k = threadIdx.x; k < m.cull_ntop; k += kTeamThreads) {
    const int4 e = tops[k];
    const float4 lo = __ldcg(&bb[2 * e.x]), hi = __ldcg(&bb[2 * e.x + 1]);
    const unsigned hit = hits(lo, hi);
    outcome(e.x, hit, m.node_leaf_lo[e.x], m.node_leaf_hi[e.x]);
    if (hit && e.y >= 0) sh.crange[atomicAdd(&sh.nrange, 1)] = make_int2(e.y, e.z);
  }
  __syncthreads();
  // Second level: the listed ranges, every node tested (kBox loads in flight
  // per thread).  Nodes under a failing split-depth node are not tested: its
  // mark covers their leaves, and the leaf pass below reads no outcome there.
  const int R = sh.nrange;
  if (threadIdx.x < 32) {
    int a = 2 * threadIdx.x < R ? sh.crange[2 * threadIdx.x].y - sh.crange[2 * threadIdx.x].x : 0;
    int b = 2 * threadIdx.x + 1 < R
                ? sh.crange[2 * threadIdx.x + 1].y - sh.crange[2 * threadIdx.x + 1].x : 0;
    int x = a + b;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, x, o);
      if (static_cast<int>(threadIdx.x) >= o) x += y;
    }
    sh.croff[2 * threadIdx.x] = x - a - b;
    sh.croff[2 * threadIdx.x + 1] = x - b;
    if (threadIdx.x == 31) sh.croff[64] = x;
  }
  __syncthreads();
  const int T2 = sh.croff[64];
  for (int i0 = threadIdx.x; i0 < T2; i0 += kBox * kTeamThreads) {
    float4 lo[kBox], hi[kBox];
    int nn[kBox], llo[kBox], lhi[kBox];
#pragma unroll
    for (int j = 0; j < kBox; j++) {
      const int i = i0 + j * kTeamThreads;
      nn[j] = -1;
      if (i < T2) {
        const int r = smem_find_slot(sh.croff, R, i);
        const int n = sh.crange[r].x + (i - sh.croff[r]);
        nn[j] = n;
        lo[j] = __ldcg(&bb[2 * n]);
        hi[j] = __ldcg(&bb[2 * n + 1]);
        llo[j] = m.node_leaf_lo[n];
        lhi[j] = m.node_leaf_hi[n];
      }
    }
#pragma unroll
    for (int j = 0; j < kBox; j++)
      if (nn[j] >= 0) outcome(nn[j], hits(lo[j], hi[j]), llo[j], lhi[j]);
  }
  }
  __syncthreads();
  const int seg = (L + kTeamThreads - 1) / kTeamThreads;
  const int l0 = min(L, static_cast<int>(threadIdx.x) * seg), l1 = min(L, l0 + seg);
  int dsum = 0;
  for (int id = l0; id < l1; id++) dsum += s_coff[id];
  int dtot;
  int cov = team_block_scan(dsum, &dtot, sh.scan);
  unsigned long long okmask = 0ull;
  unsigned long long cnt = 0ull, nvs = 0ull;
  if constexpr (!kPair) {
    for (int id = l0; id < l1; id++) {
      cov += s_coff[id];
      if (cov == 0 && s_pass[ct.lnode[id]]) {
        cnt++;
        nvs += static_cast<unsigned long long>(ct.lnv[id]);
        okmask |= 1ull << (id - l0);
      }
    }
  } else {
    unsigned long long okmask1 = 0ull, cnt1 = 0ull, nvs1 = 0ull;
    const bool two = cap > 0;
    for (int id = l0; id < l1; id++) {
      cov += s_coff[id];
      const bool in0 = (cov & 0xFFFF) == 0, in1 = two && (cov >> 16) == 0;
      if (!in0 && !in1) continue;  // under a failing ancestor of every sphere
      const unsigned pm = s_pass[ct.lnode[id]];
      if (in0 && (pm & 1u)) {
        cnt++;
        nvs += static_cast<unsigned long long>(ct.lnv[id]);
        okmask |= 1ull << (id - l0);
      }
      if (in1 && (pm & 2u)) {
        cnt1++;
        nvs1 += static_cast<unsigned long long>(ct.lnv[id]);
        okmask1 |= 1ull << (id - l0);
      }
    }
    if (okmask & okmask1) sh.pair_ovl = 1;
    unsigned long long total0, total1 = 0ull, excl1 = 0ull;
    const unsigned long long excl0 = team_block_scan64((nvs << 24) | cnt, &total0, sh.scan64);
    if (cap > 0) excl1 = team_block_scan64((nvs1 << 24) | cnt1, &total1, sh.scan64);
    const int c0 = static_cast<int>(total0 & 0xFFFFFFull), t0 = static_cast<int>(total0 >> 24);
    const int c1 = static_cast<int>(total1 & 0xFFFFFFull), t1 = static_cast<int>(total1 >> 24);
    const bool both = cap > 0 && c0 + c1 <= cap;  // (cap 0: one sphere)
    int pos = static_cast<int>(excl0 & 0xFFFFFFull), voff = static_cast<int>(excl0 >> 24);
    int pos1 = c0 + static_cast<int>(excl1 & 0xFFFFFFull), voff1 = t0 + static_cast<int>(excl1 >> 24);
    for (int id = l0; id < l1; id++) {
      const bool w0 = (okmask >> (id - l0)) & 1ull, w1 = both && ((okmask1 >> (id - l0)) & 1ull);
      if (!w0 && !w1) continue;
      const int nv = ct.lnv[id];
      if (w0) {
        s_cl[pos] = id;
        s_coff[pos] = voff;
        pos++;
        voff += nv;
      }
      if (w1) {
        s_cl[pos1] = id;
        s_coff[pos1] = voff1;
        pos1++;
        voff1 += nv;
      }
    }
    // joinable 2: pass 1's leaves in a bitmap over the leaves (the node marks
    // are read; their bytes hold it), then pass 0's leaves' neighbours looked up
    bool joined = false;
    if (joinable == 2 && both && !sh.pair_ovl) {
      unsigned int* bits = reinterpret_cast<unsigned int*>(s_pass);
      __syncthreads();  // the lists are written
      for (int i = threadIdx.x; i < (L + 31) / 32; i += kTeamThreads) bits[i] = 0u;
      __syncthreads();
      for (int k = threadIdx.x; k < c1; k += kTeamThreads) {
        const int leaf = s_cl[c0 + k];
        atomicOr(&bits[leaf >> 5], 1u << (leaf & 31));
      }
      __syncthreads();
      int hit = 0;
      for (int k = threadIdx.x; k < c0 && !hit; k += kTeamThreads) {
        const int leaf = s_cl[k];
        for (int j = m.leaf_adj_off[leaf]; j < m.leaf_adj_off[leaf + 1] && !hit; j++) {
          const int o = m.leaf_adj[j];
          hit = (bits[o >> 5] >> (o & 31)) & 1u;
        }
      }
      joined = __syncthreads_or(hit) != 0;
    }
    if (threadIdx.x == 0) {
      const bool joint = both && joinable != 0 && !sh.pair_ovl && !joined;
      sh.joint = joint ? 1 : 0;
      sh.split = c0;
      sh.cnt = joint ? c0 + c1 : c0;
      sh.total = joint ? t0 + t1 : t0;
      sh.held = (both && !joint) ? c1 : -1;
      sh.held_total = t1;
      sh.held_base = c0;
      sh.held_off = t0;
      s_coff[c0] = t0;
      if (both) s_coff[c0 + c1] = t0 + t1;
    }
    __syncthreads();
    return;
  }
  // (vertex count << 24) | leaf count: leaves < 2^24, vertices < 2^31
  unsigned long long total;
  const unsigned long long excl = team_block_scan64((nvs << 24) | cnt, &total, sh.scan64);
  // the scan's barriers separate the reads of s_coff above from the writes below
  int pos = static_cast<int>(excl & 0xFFFFFFull);
  int voff = static_cast<int>(excl >> 24);
  for (int id = l0; id < l1; id++) {
    if (!((okmask >> (id - l0)) & 1ull)) continue;
    s_cl[pos] = id;
    s_coff[pos] = voff;
    pos++;
    voff += ct.lnv[id];
  }
  if (threadIdx.x == 0) {
    sh.cnt = static_cast<int>(total & 0xFFFFFFull);
    sh.total = static_cast<int>(total >> 24);
    s_coff[sh.cnt] = sh.total;
  }
  __syncthreads();
}

// The sweep of one grab / elastic deform dab over the gathered leaves (every
// CTA of the team, strided by GT threads); returns the algorithmic bytes.
__device__ __forceinline__ unsigned long long team_orig_sweep(const DevMesh& m, const DevBrush& b,
                                                           const DabPasses& dp, const int* s_cl,
                                                           const int* s_coff, int cnt, int total,
                                                           int gt, int GT, int* tag_cnt) {
  // index, original position (+ normal for the front face), mask, automask; position write
  const unsigned vbytes = (m.type == kFaces ? 4u : 0u) + 12u +
                          ((b.flag & kBrushFrontFace) ? 12u : 0u) + (m.mask ? 4u : 0u) +
                          (m.automask ? 4u : 0u) + 12u;
  const int lane = threadIdx.x & 31;
  unsigned long long ab = 0;
  for (int base = gt - lane; base < total; base += GT) {
    const int i = base + lane;
    unsigned int moved = 0u;
    if (i < total) {
      const int k = smem_find_slot(s_coff, cnt, i);
      const int v = leaf_vert(m, s_cl[k], i - s_coff[k]);
      float4 co = __ldcg(&m.co[v]);
      moved = orig_vertex(m, b, b.y, dp, v, co);
      m.co[v] = co;
      ab += vbytes;
      if (m.type == kFaces) tag_vertex(m, v, tag_cnt);
    }
    const unsigned int sum = __reduce_add_sync(0xffffffffu, moved);
    if (lane == 0 && sum) atomicAdd(&m.work->displaced, (unsigned long long)sum);
  }
  return ab;
}

// The node search of one pass (sphere at the pass location).
template <int kBox, bool kTwoLevel, class Tabs>
__device__ void team_cull(const DevMesh& m, const PassParams& pp, unsigned char* s_pass,
                          int* s_cl, int* s_coff, const Tabs& ct, TeamShared& sh,
                          const int4* top = nullptr) {
  team_cull_by<kBox, kTwoLevel>(
      m, pp.original ? m.orig_vb : m.vb,
      [&](float4 lo, float4 hi) { return box_hits(lo, hi, pp.loc, pp.cull_radius_sq) ? 1u : 0u; },
      s_pass, s_cl, s_coff, ct, sh, 0, 0, top);
}

// The node searches of both passes of a single-axis symmetry in one (the
// spheres at loc0 and loc1, the same radius and boxes); cap bounds the
// entries of the two lists together.
template <int kBox, bool kTwoLevel, class Tabs>
__device__ void team_cull_pair(const DevMesh& m, const PassParams& pp, const float* loc1, bool pair,
                               unsigned char* s_pass, int* s_cl, int* s_coff, const Tabs& ct,
                               TeamShared& sh, int cap, int joinable, const int4* top) {
  team_cull_by<kBox, kTwoLevel, true>(
      m, pp.original ? m.orig_vb : m.vb,
      [&](float4 lo, float4 hi) {
        unsigned h = box_hits(lo, hi, pp.loc, pp.cull_radius_sq) ? 1u : 0u;
        if (pair && box_hits(lo, hi, loc1, pp.cull_radius_sq)) h |= 2u;
        return h;
      },
      s_pass, s_cl, s_coff, ct, sh, pair ? cap : 0, joinable, top);
}

// The gather of one grab / elastic deform dab (k_cull_dab): orig_vb boxes that
// meet any pass sphere, or every leaf (all != 0).
template <bool kTwoLevel>
__device__ __forceinline__ void team_cull_union(const DevMesh& m, const DabPasses& dp, float rsq,
                                             int all, unsigned char* s_pass, int* s_cl,
                                             int* s_coff, const CullTabs& ct, TeamShared& sh,
                                             const int4* top) {
  team_cull_by<2, kTwoLevel>(
      m, m.orig_vb,
      [&](float4 lo, float4 hi) {
        bool ok = all != 0;
        for (int p = 0; p < dp.npass && !ok; p++) ok = box_hits(lo, hi, dp.loc[p], rsq);
        return ok ? 1u : 0u;
      },
      s_pass, s_cl, s_coff, ct, sh, 0, 0, top);
}

// The second pass's list of a pair search, stored behind the first one's
// (sh.held entries from sh.held_base, offsets from sh.held_off), moved to
// the front of the list arrays with offsets from 0; sets sh.cnt, sh.total
// and sh.split to its own.  Rounds of kTeamThreads entries read before they
// write; later rounds read at or above base + their start.
__device__ __forceinline__ void team_list_to_front(int* s_cl, int* s_coff, TeamShared& sh) {
  const int base = sh.held_base, n = sh.held, off = sh.held_off;
  __syncthreads();
  if (threadIdx.x == 0) {
    sh.cnt = sh.split = n;
    sh.total = sh.held_total;
    sh.held = -1;
  }
  for (int k0 = 0; k0 <= n; k0 += kTeamThreads) {
    const int k = k0 + static_cast<int>(threadIdx.x);
    int leaf = 0, o = 0;
    if (k <= n) {
      if (k < n) leaf = s_cl[base + k];
      o = s_coff[base + k] - off;
    }
    __syncthreads();
    if (k <= n) {
      if (k < n) s_cl[k] = leaf;
      s_coff[k] = o;
    }
    __syncthreads();
  }
}

// How two passes over disjoint leaves can run as one: 1 for the tools whose
// sweep reads and writes only the vertex itself (and the pass's frame); 2
// for smooth, whose hits read their one-ring (the lists must also have no
// pair of leaves joined by a mesh edge); 0 otherwise.
__device__ __forceinline__ int pair_tool(int tool) {
  return (tool == kToolDraw || tool == kToolInflate || tool == kToolPinch || tool == kToolCrease ||
          tool == kToolClayStrips)
             ? 1
             : tool == kToolSmooth ? 2 : 0;
}

constexpr int kFlushTab = 128;  // ancestors whose boxes stay on chip
constexpr unsigned short kNoPos = 0xFFFFu;

constexpr int kFlushTouch = 128;  // touched leaves whose flush data is staged

// Flush tables (CTA 0): new boxes of the first kFlushTab listed ancestors,
// the new boxes of their children that are touched leaves, and per touched
// leaf (first kFlushTouch) its slot in kid (or -1) and its chunk range.
struct FlushSmem {
  float4 own[2 * kFlushTab];
  float4 kid[4 * kFlushTab];
  int kslot[kFlushTouch];
  int2 kco[kFlushTouch];
};

// One listed ancestor per thread (fast path): its node, depth, and per child
// the source of the child's box: 0 = unchanged (a/b registers), 1 = touched
// leaf (fs.kid), 2 = listed ancestor at list position p0/p1 (fs.own).
struct FlushState {
  int node, dep;
  int k0, k1, p0, p1;
  float4 a0, a1, b0, b1;
};

__device__ __forceinline__ bool bit_set(const unsigned int* bits, int i) {
  return (bits[i >> 5] >> (i & 31)) & 1u;
}

// Flush, first half (CTA 0 while the other CTAs refit): every ancestor of a
// touched leaf is listed once (claimed in a bitmap over the nodes, which also
// marks the touched leaf nodes) and s_idx[node] = its list position; with at
// most kFlushTab ancestors, each thread takes one and loads the boxes of its
// children that the update leaves unchanged.  touched: the touched leaves.
template <class LeafNode>
static __device__ void team_flush_mark(const DevMesh& m, int ntouch, const int* touched, const LeafNode* lnode,
                                const int* s_par,
                                unsigned int* bits, int* s_list, unsigned short* s_idx,
                                FlushSmem& fs, TeamShared& sh, FlushState& f) {
  for (int i = threadIdx.x; i < (m.totnode + 31) / 32; i += kTeamThreads) bits[i] = 0u;
  if (threadIdx.x == 0) sh.nmark = 0;
  __syncthreads();
  for (int k = threadIdx.x; k < ntouch; k += kTeamThreads) {
    const int leaf_node = static_cast<int>(lnode[touched[k]]);
    atomicOr(&bits[leaf_node >> 5], 1u << (leaf_node & 31));
    int p = s_par[leaf_node];
    while (p >= 0) {
      const unsigned int bit = 1u << (p & 31);
      if (atomicOr(&bits[p >> 5], bit) & bit) break;  // claimed: so are its ancestors
      s_list[atomicAdd(&sh.nmark, 1)] = p;
      p = s_par[p];
    }
  }
  __syncthreads();
  const int nm = sh.nmark;
  for (int t = threadIdx.x; t < nm; t += kTeamThreads) s_idx[s_list[t]] = static_cast<unsigned short>(t);
  __syncthreads();
  for (int k = threadIdx.x; k < min(ntouch, kFlushTouch); k += kTeamThreads) {
    const int leaf = touched[k];
    const int node = static_cast<int>(lnode[leaf]);
    const int p = s_par[node];
    const int pos = p >= 0 ? s_idx[p] : kNoPos;
    fs.kslot[k] = pos < kFlushTab ? 2 * pos + (node - m.node_child[p]) : -1;
    fs.kco[k] = make_int2(m.leaf_chunk_off[leaf], m.leaf_chunk_off[leaf + 1]);
  }
  f.node = -1;
  f.dep = -1;
  if (nm <= kFlushTab && static_cast<int>(threadIdx.x) < nm) {
    f.node = s_list[threadIdx.x];
    f.dep = m.node_depth[f.node];
    const int c = m.node_child[f.node];
    f.p0 = s_idx[c];
    f.p1 = s_idx[c + 1];
    f.k0 = f.p0 != kNoPos ? 2 : (bit_set(bits, c) ? 1 : 0);
    f.k1 = f.p1 != kNoPos ? 2 : (bit_set(bits, c + 1) ? 1 : 0);
    if (f.k0 == 0) {
      f.a0 = __ldcg(&m.vb[2 * c]);
      f.a1 = __ldcg(&m.vb[2 * c + 1]);
    }
    if (f.k1 == 0) {
      f.b0 = __ldcg(&m.vb[2 * c + 2]);
      f.b1 = __ldcg(&m.vb[2 * c + 3]);
    }
  }
}

__device__ __forceinline__ void box_union(const float4& a0, const float4& a1, const float4& b0,
                                          const float4& b1, float4& mn, float4& mx) {
  mn.x = fmin_ref(fmin_ref(FLT_MAX, a0.x), b0.x);
  mn.y = fmin_ref(fmin_ref(FLT_MAX, a0.y), b0.y);
  mn.z = fmin_ref(fmin_ref(FLT_MAX, a0.z), b0.z);
  mx.x = fmax_ref(fmax_ref(-FLT_MAX, a1.x), b1.x);
  mx.y = fmax_ref(fmax_ref(-FLT_MAX, a1.y), b1.y);
  mx.z = fmax_ref(fmax_ref(-FLT_MAX, a1.z), b1.z);
  mn.w = mx.w = 0.0f;
}

// Flush, second half (CTA 0, after the refit): the touched leaf boxes from
// their chunk boxes (one warp per leaf; also handed to the parent's thread in
// fs.kid), then each listed ancestor becomes the union of its two children
// (update_node_vb, pbvh.c:2026-2046), deepest level first as pbvh_flush_bb
// (pbvh.c:3287-3317) orders it.  Resets s_idx to kNoPos.
template <class LeafNode>
static __device__ void team_flush_levels(const DevMesh& m, int ntouch, const int* touched, const LeafNode* lnode,
                                  const int* s_par, const int* s_list, unsigned short* s_idx,
                                  FlushSmem& fs, TeamShared& sh, FlushState& f,
                                  unsigned long long& ab) {
  const int nm = sh.nmark;
  const int lane = threadIdx.x & 31;
  for (int k = threadIdx.x >> 5; k < ntouch; k += kTeamThreads / 32) {
    int2 co;
    int slot;
    if (k < kFlushTouch) {
      co = fs.kco[k];
      slot = fs.kslot[k];
    } else {
      const int leaf = touched[k];
      co = make_int2(m.leaf_chunk_off[leaf], m.leaf_chunk_off[leaf + 1]);
      const int node = static_cast<int>(lnode[leaf]);
      const int p = s_par[node];
      const int pos = p >= 0 ? s_idx[p] : kNoPos;
      slot = pos < kFlushTab ? 2 * pos + (node - m.node_child[p]) : -1;
    }
    float mn[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, mx[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    for (int id = co.x + lane; id < co.y; id += 32) {
      const float4 c0 = __ldcg(&m.chunk_box[2 * id]), c1 = __ldcg(&m.chunk_box[2 * id + 1]);
      mn[0] = fmin_ref(mn[0], c0.x);
      mn[1] = fmin_ref(mn[1], c0.y);
      mn[2] = fmin_ref(mn[2], c0.z);
      mx[0] = fmax_ref(mx[0], c1.x);
      mx[1] = fmax_ref(mx[1], c1.y);
      mx[2] = fmax_ref(mx[2], c1.z);
    }
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1)
#pragma unroll
      for (int q = 0; q < 3; q++) {
        mn[q] = fmin_ref(mn[q], __shfl_xor_sync(0xffffffffu, mn[q], o));
        mx[q] = fmax_ref(mx[q], __shfl_xor_sync(0xffffffffu, mx[q], o));
      }
    if (lane == 0) {
      const float4 bmn = make_float4(mn[0], mn[1], mn[2], 0.0f);
      const float4 bmx = make_float4(mx[0], mx[1], mx[2], 0.0f);
      const int node = static_cast<int>(lnode[touched[k]]);
      m.vb[2 * node] = bmn;
      m.vb[2 * node + 1] = bmx;
      if (slot >= 0) {
        fs.kid[2 * slot] = bmn;
        fs.kid[2 * slot + 1] = bmx;
      }
      ab += 32ull * (co.y - co.x + 1);  // chunk boxes read, leaf box written
    }
  }
  __syncthreads();
  if (nm <= 32) {
    // one warp: each lane keeps one ancestor's box in registers and hands it
    // to its parent's lane by shuffle
    if (threadIdx.x < 32) {
      const int t = lane;
      float own[6] = {FLT_MAX, FLT_MAX, FLT_MAX, -FLT_MAX, -FLT_MAX, -FLT_MAX};
      if (f.node >= 0) ab += 72u;
      for (int dd = m.max_depth; dd >= 0; dd--) {
        float c0[6], c1[6];
#pragma unroll
        for (int q = 0; q < 6; q++) {
          c0[q] = __shfl_sync(0xffffffffu, own[q], f.p0 & 31);
          c1[q] = __shfl_sync(0xffffffffu, own[q], f.p1 & 31);
        }
        if (f.dep == dd) {
          if (f.k0 == 2) {
            f.a0 = make_float4(c0[0], c0[1], c0[2], 0.0f);
            f.a1 = make_float4(c0[3], c0[4], c0[5], 0.0f);
          } else if (f.k0 == 1) {
            f.a0 = fs.kid[4 * t];
            f.a1 = fs.kid[4 * t + 1];
          }
          if (f.k1 == 2) {
            f.b0 = make_float4(c1[0], c1[1], c1[2], 0.0f);
            f.b1 = make_float4(c1[3], c1[4], c1[5], 0.0f);
          } else if (f.k1 == 1) {
            f.b0 = fs.kid[4 * t + 2];
            f.b1 = fs.kid[4 * t + 3];
          }
          float4 mn, mx;
          box_union(f.a0, f.a1, f.b0, f.b1, mn, mx);
          own[0] = mn.x, own[1] = mn.y, own[2] = mn.z;
          own[3] = mx.x, own[4] = mx.y, own[5] = mx.z;
          m.vb[2 * f.node] = mn;
          m.vb[2 * f.node + 1] = mx;
        }
      }
    }
    __syncthreads();
  } else if (nm <= kFlushTab) {
    const int t = threadIdx.x;
    if (f.node >= 0) ab += 72u;  // two child boxes read, one box written
    for (int dd = m.max_depth; dd >= 0; dd--) {
      if (f.dep == dd) {
        if (f.k0 == 2) {
          f.a0 = fs.own[2 * f.p0];
          f.a1 = fs.own[2 * f.p0 + 1];
        } else if (f.k0 == 1) {
          f.a0 = fs.kid[4 * t];
          f.a1 = fs.kid[4 * t + 1];
        }
        if (f.k1 == 2) {
          f.b0 = fs.own[2 * f.p1];
          f.b1 = fs.own[2 * f.p1 + 1];
        } else if (f.k1 == 1) {
          f.b0 = fs.kid[4 * t + 2];
          f.b1 = fs.kid[4 * t + 3];
        }
        float4 mn, mx;
        box_union(f.a0, f.a1, f.b0, f.b1, mn, mx);
        fs.own[2 * t] = mn;
        fs.own[2 * t + 1] = mx;
        m.vb[2 * f.node] = mn;
        m.vb[2 * f.node + 1] = mx;
      }
      __syncthreads();
    }
  } else {
    // many ancestors: per level, every thread scans the list; child boxes
    // come from fs.own (first kFlushTab list positions) or global memory
    for (int dd = m.max_depth; dd >= 0; dd--) {
      for (int t = threadIdx.x; t < nm; t += kTeamThreads) {
        const int node = s_list[t];
        if (m.node_depth[node] != dd) continue;
        const int c = m.node_child[node];
        float4 box[2][2];
        for (int h = 0; h < 2; h++) {
          const int pc = s_idx[c + h];
          if (pc < kFlushTab) {
            box[h][0] = fs.own[2 * pc];
            box[h][1] = fs.own[2 * pc + 1];
          } else {
            box[h][0] = __ldcg(&m.vb[2 * (c + h)]);
            box[h][1] = __ldcg(&m.vb[2 * (c + h) + 1]);
          }
        }
        float4 mn, mx;
        box_union(box[0][0], box[0][1], box[1][0], box[1][1], mn, mx);
        if (t < kFlushTab) {
          fs.own[2 * t] = mn;
          fs.own[2 * t + 1] = mx;
        }
        m.vb[2 * node] = mn;
        m.vb[2 * node + 1] = mx;
        ab += 72u;
      }
      __syncthreads();
    }
  }
  for (int t = threadIdx.x; t < nm; t += kTeamThreads) s_idx[s_list[t]] = kNoPos;
  __syncthreads();
}

// Compensated area partial of one block (at most kAreaBlock visited
// vertices) of a culled leaf by the CTA: the lane structure of k_area.  The
// block's positions and normals are staged in shared memory kAreaStage at a
// time with cp.async (16 bytes each, no register holds them in flight), in
// two buffers, so that the copies of the next round are in flight while the
// current round is summed; lane t adds its elements t, t+256, ... of each
// round in order, so the sums are those of the one-round form.
constexpr int kAreaStage = 512;  // staged vertices per round and buffer: 16 KB
static_assert(4 * kAreaStage * sizeof(float4) <= kStageBytes, "the area stage");
static __device__ void team_area_block(const DevMesh& m, const float* c, float rn2,
                                       float ra2, int leaf, int blk, float4* s_stage, Lane* sl,
                                       AreaPart* out) {
  const int t = threadIdx.x;
  const int i0 = blk * kAreaBlock;
  const int i1 = min(leaf_nverts(m, leaf), i0 + kAreaBlock);
  auto issue = [&](int r0, int buf) {
    float4* s_co = s_stage + 2 * buf * kAreaStage;
    float4* s_no = s_co + kAreaStage;
    const int r1 = min(i1, r0 + kAreaStage);
    for (int i = r0 + t; i < r1; i += kTeamThreads) {
      const int v = leaf_vert(m, leaf, i);
      cp_async16(&s_co[i - r0], &m.co[v]);
      cp_async16(&s_no[i - r0], &m.no[v]);
    }
    cp_async_commit();
  };
  Lane l;
#pragma unroll
  for (int q = 0; q < 6; q++) l.v[q].s = l.v[q].e = 0.0f;
  l.n_no = l.n_co = 0;
  if (i0 < i1) issue(i0, 0);
  int buf = 0;
  for (int r0 = i0; r0 < i1; r0 += kAreaStage, buf ^= 1) {
    // the other buffer was summed before the last barrier: refill it
    if (r0 + kAreaStage < i1) {
      issue(r0 + kAreaStage, buf ^ 1);
      cp_async_wait_group1();
    } else {
      cp_async_wait_group0();
    }
    __syncthreads();
    const float4* s_co = s_stage + 2 * buf * kAreaStage;
    const float4* s_no = s_co + kAreaStage;
    const int r1 = min(i1, r0 + kAreaStage);
    for (int i = r0 + t; i < r1; i += kTeamThreads) {
      const float4 co = s_co[i - r0];
      const float d2 = dist_sq(co, c);
      if (d2 <= rn2) {
        const float4 no = s_no[i - r0];
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
    __syncthreads();  // this buffer is free for the round after next
  }
  sl[t] = l;
  __syncthreads();
  for (int s = kTeamThreads / 2; s >= 32; s >>= 1) {
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
    if (t == 0) part_store(out, a);
  }
  __syncthreads();
}

// Final pairwise tree over the leaf partials (i, i+s), s = 1, 2, 4, ... by one
// CTA in shared memory; writes area normal and centre into sh.area.
constexpr int kTeamMaxChunks = 64;  // area partials per pass <= 64 * 256

static __device__ void team_area_final(const DevMesh& m, const PassParams& pp, int cnt, Lane* sl,
                                Lane* chunks, TeamShared& sh, int first = 0) {
  // Partials are staged in shared memory in chunks of kTeamThreads (a power of
  // two, so each chunk is a complete subtree of the pairwise tree); the chunk
  // totals then merge with the same pairwise rule, which completes the tree.
  const int nchunks = (cnt + kTeamThreads - 1) / kTeamThreads;
  for (int c = 0; c < nchunks; c++) {
    const int c0 = c * kTeamThreads;
    const int n = min(kTeamThreads, cnt - c0);
    if (threadIdx.x < n) sl[threadIdx.x] = part_load(&m.parts[first + c0 + threadIdx.x]);
    __syncthreads();
    for (int s = 1; s < n; s <<= 1) {
      const int i = threadIdx.x * 2 * s;
      if (i + s < n) {
        Lane a = sl[i];
        lane_merge(a, sl[i + s]);
        sl[i] = a;
      }
      __syncthreads();
    }
    if (threadIdx.x == 0) chunks[c] = sl[0];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    for (int s = 1; s < nchunks; s <<= 1)
      for (int i = 0; i + s < nchunks; i += 2 * s) lane_merge(chunks[i], chunks[i + s]);
    Lane acc;
    if (nchunks > 0) {
      acc = chunks[0];
    } else {
#pragma unroll
      for (int q = 0; q < 6; q++) acc.v[q].s = acc.v[q].e = 0.0f;
      acc.n_no = acc.n_co = 0;
    }
    float nx = acc.v[0].s + acc.v[0].e, ny = acc.v[1].s + acc.v[1].e, nz = acc.v[2].s + acc.v[2].e;
    normalize3(nx, ny, nz);
    sh.area[0] = nx;
    sh.area[1] = ny;
    sh.area[2] = nz;
    if (acc.n_co > 0) {
      const float inv = 1.0f / (float)acc.n_co;
      sh.area[3] = (acc.v[3].s + acc.v[3].e) * inv;
      sh.area[4] = (acc.v[4].s + acc.v[4].e) * inv;
      sh.area[5] = (acc.v[5].s + acc.v[5].e) * inv;
    } else {
      sh.area[3] = pp.loc[0];
      sh.area[4] = pp.loc[1];
      sh.area[5] = pp.loc[2];
    }
  }
  __syncthreads();
}

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// The faces of leaves that a dab marks join the dab's GRIDS normal update
// (grid_claim_face, once per epoch): CTA r claims for the leaves k = r, r+C,
// ... of list[0..n).  Called where the leaves are marked, so the claims
// complete with the phase that marks them.
__device__ __forceinline__ void team_claim_faces(const DevMesh& m, const int* list, int n,
                                                 unsigned rank, unsigned C, unsigned int epoch) {
  for (int k = static_cast<int>(rank); k < n; k += static_cast<int>(C)) {
    const int leaf = list[k];
    const int p0 = m.leaf_prim_off[leaf], p1 = m.leaf_prim_off[leaf + 1];
    for (int j = p0 + threadIdx.x; j < p1; j += kTeamThreads)
      grid_claim_face_only(m, m.leaf_prims[j], epoch);
  }
}

// Grids of one face staged on chip at a time: positions (float4), masks and
// quad normals (float3); the largest group of at most 4 grids whose tables
// fit in bytes.
__host__ __device__ __forceinline__ size_t face_group_bytes(int grid_size, int group) {
  const size_t area = static_cast<size_t>(grid_size) * grid_size;
  const size_t quads = static_cast<size_t>(grid_size - 1) * (grid_size - 1);
  return group * (16u * area + 4u * area + 12u * quads);
}
__host__ __device__ __forceinline__ int face_grid_group(int grid_size, size_t bytes) {
  int g = 4;
  while (g > 0 && face_group_bytes(grid_size, g) > bytes) g--;
  return g;
}

// Normal of staged element i (grid i / area of the stage): the mean of the
// staged normals of the quads around it, added in the order of
// grid_element_normal (subdiv_ccg.c:707-737).
// Element (x, y) of staged grid c.
__device__ __forceinline__ float3 staged_normal_at(const float3* s_q, int c, int x, int y, int g1) {
  const float3* q = s_q + c * g1 * g1;
  float ax = 0.0f, ay = 0.0f, az = 0.0f;
  int counter = 0;
  auto add = [&](const float3& v) {
    ax += v.x, ay += v.y, az += v.z;
    counter++;
  };
  if (x < g1 && y < g1) add(q[y * g1 + x]);
  if (x >= 1) {
    if (y < g1) add(q[y * g1 + x - 1]);
    if (y >= 1) add(q[(y - 1) * g1 + x - 1]);
  }
  if (y >= 1 && x < g1) add(q[(y - 1) * g1 + x]);
  return make_float3(ax * inv_count(counter), ay * inv_count(counter), az * inv_count(counter));
}

// The owner records of face f's corners for the dab of this epoch (threads
// t_begin, t_begin + t_step, ...): corner c's base edge and base vertex are
// averaged by the first of their faces (slot order) claimed in the epoch
// (subdiv_ccg.c:1010-1048, 1081-1104 average each once) — the claimed face of
// least index, whose key the claims left in edge_own / bvert_own; the
// owner's record holds the element slots and face count, the others' a count
// of 0.  Needs the epoch's claims complete.
__device__ __forceinline__ void grid_corner_owners(const DevMesh& m, int f, int s, int n,
                                                   unsigned int epoch, int t_begin, int t_step) {
  const unsigned long long key = grid_owner_key(epoch, f);
  for (int t = t_begin; t < 2 * n; t += t_step) {
    const bool edge = t < n;
    const int c = edge ? t : t - n;
    const int id = edge ? m.face_edges[s + c] : m.face_verts[s + c];
    const int* off = edge ? m.edge_off : m.bvert_off;
    const unsigned long long own = __ldcg(edge ? &m.edge_own[id] : &m.bvert_own[id]);
    const int f0 = off[id], f1 = off[id + 1];
    m.corner_own[2 * (s + c) + (edge ? 0 : 1)] =
        make_int2(f0, (own == key && f1 - f0 > 1) ? f1 - f0 : 0);
  }
}

// Inner normals, face-internal seams and the centre of one claimed face by
// one CTA (subdiv_ccg.c:670-740 and 951-984).  The face's grids are staged in
// shared memory with cp.async (positions and masks), the normal_quad of every
// quad is computed once (the per-element form evaluates a quad up to four
// times with the same corners and the same result), and each element normal
// is the mean of its staged quad normals, added in the order of
// grid_element_normal.  The seam pairs and the centre then average the staged
// positions and masks and the new normals, as the reference averages after
// every inner normal; pairs and the centre touch disjoint elements, so each
// reads the values the inner-normal step left.  Faces are independent here:
// a face's grids hold their own copies of the base-edge elements, which the
// base-edge pass averages afterwards.  GRIDS positions carry w = 0.
// The owner records of the face's corners are written while the first
// stage is in flight (grid_corner_owners); with kSplitOwners and at most
// kTeamThreads records, one thread per record loads its corner's id before
// the stage, the owner key and face range after it, and writes the record
// once the face is done, so that the dependent loads overlap the normals.
// The cluster builds and the builds that pair mirror passes keep the first
// form: the split costs them registers.
// kPrefetch (with kSplitOwners): when the face's base-edge and corner items
// (team_grid_face_boundary) fit one per thread and their tables fit the stage
// after the grids, the records also go to shared memory after the quad
// normals, each item's thread loads the element indices of its set during the
// element normals, and the face returns true: the boundary phase of this face
// on this CTA then reads the indices from boundary_prefetch(...) instead of
// walking record -> index -> element after the team barrier.
__host__ __device__ __forceinline__ size_t boundary_prefetch_offset(int grid_size, int group) {
  return (face_group_bytes(grid_size, group) + 15u) & ~static_cast<size_t>(15);
}
// The 2n records (int2, first: 8-byte aligned), then per item the set's size
// (0: not the owner; -1: larger than kAvgBatch, read the record) and its
// kAvgBatch element indices.
__host__ __device__ __forceinline__ size_t boundary_prefetch_bytes(int items, int n) {
  return 16u * n + static_cast<size_t>(items) * 4u * (1 + kAvgBatch);
}
template <bool kSplitOwners = true, bool kPrefetch = false>
static __device__ bool team_grid_face(const DevMesh& m, int f, int s, int n, unsigned char* stage,
                                      int group, unsigned int epoch) {
  const int gs = m.grid_size, g1 = gs - 1, area = m.grid_area, qa = g1 * g1;
  float4* s_co = reinterpret_cast<float4*>(stage);
  float* s_mk = reinterpret_cast<float*>(s_co + group * area);
  float3* s_q = reinterpret_cast<float3*>(s_mk + group * area);  // quad normals
  const bool whole = n <= group;  // the seams below read the stage
  const bool split_owners = kSplitOwners && 2 * n <= kTeamThreads;
  const int ot = static_cast<int>(threadIdx.x);
  const bool oedge = ot < n;
  const int oc = oedge ? ot : ot - n;
  int oid = -1, of0 = 0, of1 = 0;
  unsigned long long own = 0ull;
  if (split_owners && ot < 2 * n) oid = oedge ? m.face_edges[s + oc] : m.face_verts[s + oc];
  const int g2 = 2 * gs, per_corner = g2 - 1, items = n * per_corner;
  const size_t pre_off = boundary_prefetch_offset(gs, group);
  const bool pre = kPrefetch && split_owners && whole && items <= kTeamThreads &&
                   pre_off + boundary_prefetch_bytes(items, n) <= kStageBytes;
  int2* p_rec = reinterpret_cast<int2*>(stage + pre_off);
  int* p_cnt = reinterpret_cast<int*>(p_rec + 2 * n);
  int* p_idx = p_cnt + items;
  int pidx[kAvgBatch];
  int pcnt = 0;
  for (int c0 = 0; c0 < n; c0 += group) {
    const int nc = min(group, n - c0);
    for (int i = threadIdx.x; i < nc * area; i += kTeamThreads) {
      const size_t e = static_cast<size_t>(s + c0) * area + i;
      cp_async16(&s_co[i], &m.co[e]);
      if (m.mask) cp_async4(&s_mk[i], &m.mask[e]);
    }
    if (c0 == 0 && !split_owners) grid_corner_owners(m, f, s, n, epoch, threadIdx.x, kTeamThreads);
    cp_async_wait_all();
    __syncthreads();
    if (c0 == 0 && oid >= 0) {
      own = __ldcg(oedge ? &m.edge_own[oid] : &m.bvert_own[oid]);
      const int* off = oedge ? m.edge_off : m.bvert_off;
      of0 = off[oid];
      of1 = off[oid + 1];
    }
    // each thread keeps one quad (element) position and walks the grids
    for (int q = threadIdx.x; q < qa; q += kTeamThreads) {
      const int qy = q / g1, qx = q - qy * g1;
      for (int c = 0; c < nc; c++) {
        const float4* p = s_co + c * area;
        // quad (qx, qy): corners (qx, qy+1), (qx+1, qy+1), (qx+1, qy), (qx, qy)
        s_q[c * qa + q] = normal_quad(xyz(p[(qy + 1) * gs + qx]), xyz(p[(qy + 1) * gs + qx + 1]),
                                      xyz(p[qy * gs + qx + 1]), xyz(p[qy * gs + qx]));
      }
    }
    if (pre && oid >= 0)
      p_rec[ot] = make_int2(of0, (own == grid_owner_key(epoch, f) && of1 - of0 > 1) ? of1 - of0 : 0);
    __syncthreads();
    if (pre && ot < items) {
      const int c = ot / per_corner, j = ot - c * per_corner;
      const bool edge = j < g2 - 2;
      const int2 r = p_rec[edge ? c : n + c];
      pcnt = r.y > kAvgBatch ? -1 : r.y;
#pragma unroll
      for (int k = 0; k < kAvgBatch; k++)
        if (k < pcnt) pidx[k] = edge ? m.edge_elems[(long long)(r.x + k) * g2 + j + 1] : m.bvert_elems[r.x + k];
    }
    // (grid, element) items dealt flat over the CTA: 4 grids of 289 elements
    // take at most 5 normals a thread instead of 2 elements x 4 grids
    for (int i = threadIdx.x; i < nc * area; i += kTeamThreads) {
      const int c = static_cast<int>(div_invariant(static_cast<unsigned int>(i), m.area_mul, m.area_shift));
      const int e = i - c * area;
      const int y = static_cast<int>(div_invariant(static_cast<unsigned int>(e), m.size_mul, m.size_shift));
      const int x = e - y * gs;
      const float3 nv = staged_normal_at(s_q, c, x, y, g1);
      m.no[static_cast<size_t>(s + c0 + c) * area + e] = make_float4(nv.x, nv.y, nv.z, 0.0f);
    }
    if (pre && ot < items) {
      p_cnt[ot] = pcnt;
#pragma unroll
      for (int k = 0; k < kAvgBatch; k++)
        if (k < pcnt) p_idx[kAvgBatch * ot + k] = pidx[k];
    }
    __syncthreads();  // a next group restages after this barrier
  }
  const int pairs = n * g1;
  if (whole) {
    // pairs and the centre from the stage
    // element (i, 0) of grid ca and element (0, i) of grid cb
    auto avg_pair = [&](int ga_, int gb_, int i) {
      const int ia = ga_ * area + i, ib = gb_ * area + i * gs;
      const float4 ca = s_co[ia], cb = s_co[ib];
      const float3 na = staged_normal_at(s_q, ga_, i, 0, g1), nb = staged_normal_at(s_q, gb_, 0, i, g1);
      float4 c;
      c.x = (ca.x + cb.x) * 0.5f;
      c.y = (ca.y + cb.y) * 0.5f;
      c.z = (ca.z + cb.z) * 0.5f;
      c.w = ca.w;
      const float4 nn = make_float4((na.x + nb.x) * 0.5f, (na.y + nb.y) * 0.5f,
                                    (na.z + nb.z) * 0.5f, 0.0f);
      const size_t ga = static_cast<size_t>(s) * area + ia, gb = static_cast<size_t>(s) * area + ib;
      m.co[ga] = c;
      m.co[gb] = c;
      m.no[ga] = nn;
      m.no[gb] = nn;
      if (m.mask) {
        const float mk = (s_mk[ia] + s_mk[ib]) * 0.5f;
        m.mask[ga] = mk;
        m.mask[gb] = mk;
      }
    };
    for (int it = threadIdx.x; it <= pairs; it += kTeamThreads) {
      if (it < pairs) {
        const int c = it / g1, i = 1 + (it - c * g1);
        const int prev = c == 0 ? n - 1 : c - 1;
        avg_pair(prev, c, i);
      } else {
        // GridElementAccumulator over element 0 of every grid, in grid order
        float cx = 0.0f, cy = 0.0f, cz = 0.0f, nx = 0.0f, ny = 0.0f, nz = 0.0f, mk = 0.0f;
        for (int c = 0; c < n; c++) {
          const float4 co = s_co[c * area];
          const float3 no = staged_normal_at(s_q, c, 0, 0, g1);
          cx += co.x, cy += co.y, cz += co.z;
          nx += no.x, ny += no.y, nz += no.z;
          if (m.mask) mk += s_mk[c * area];
        }
        const float inv = 1.0f / (float)n;
        cx *= inv, cy *= inv, cz *= inv;
        nx *= inv, ny *= inv, nz *= inv;
        mk *= inv;
        for (int c = 0; c < n; c++) {
          const size_t e = static_cast<size_t>(s + c) * area;
          m.co[e] = make_float4(cx, cy, cz, s_co[c * area].w);
          m.no[e] = make_float4(nx, ny, nz, 0.0f);
          if (m.mask) m.mask[e] = mk;
        }
      }
    }
  } else {
    // more grids than one stage holds: the seams from global memory (the
    // normals written above are visible to the CTA after the barrier)
    for (int it = threadIdx.x; it <= pairs; it += kTeamThreads) {
      if (it < pairs) {
        const int c = it / g1, i = 1 + (it - c * g1);
        const int g = s + c, prev = s + (c + n - 1) % n;
        grid_avg_pair(m, prev * area + i, g * area + i * gs);
      } else {
        grid_average_set(m, n, [&](int c) { return (s + c) * area; });
      }
    }
  }
  if (oid >= 0)
    m.corner_own[2 * (s + oc) + (oedge ? 0 : 1)] =
        make_int2(of0, (own == grid_owner_key(epoch, f) && of1 - of0 > 1) ? of1 - of0 : 0);
  __syncthreads();  // the stage is read: the CTA's next face may restage it
  return pre;
}

// Base edges and corners of one claimed face by one CTA: each base edge and
// base vertex is averaged once, by the first of its faces (slot order) that
// is claimed in this epoch (subdiv_ccg.c:1010-1048, 1081-1104).  With
// records (the face went through team_grid_face this dab) the owner
// decisions are read from corner_own; without (the unstaged path) they are
// made here first, one thread per corner record.
// pre: the tables team_grid_face<true, true> left for this face (null when
// it left none; records first, then the item tables).
static __device__ void team_grid_face_boundary(const DevMesh& m, int f, int s, int n,
                                               unsigned int epoch, bool records,
                                               const unsigned char* pre = nullptr) {
  const int g2 = 2 * m.grid_size, per_corner = g2 - 1;
  if (!records) {
    grid_corner_owners(m, f, s, n, epoch, threadIdx.x, kTeamThreads);
    __syncthreads();  // the CTA's own records (global memory, CTA barrier)
  }
  for (int it = threadIdx.x; it < n * per_corner; it += kTeamThreads) {
    if (pre) {
      const int* p_cnt = reinterpret_cast<const int*>(pre + 16 * n);
      const int cnt = p_cnt[it];
      if (cnt == 0) continue;
      if (cnt > 0) {
        const int* idx = p_cnt + n * per_corner + kAvgBatch * it;
        grid_average_set(m, cnt, [&](int k) { return idx[k]; });
        continue;
      }
    }
    const int c = it / per_corner, j = it - c * per_corner;
    if (j < g2 - 2) {
      const int2 e = __ldcg(&m.corner_own[2 * (s + c)]);
      if (e.y == 0) continue;
      const int i = j + 1;
      grid_average_set(m, e.y, [&](int k) { return m.edge_elems[(long long)(e.x + k) * g2 + i]; });
    } else {
      const int2 v = __ldcg(&m.corner_own[2 * (s + c) + 1]);
      if (v.y == 0) continue;
      grid_average_set(m, v.y, [&](int k) { return m.bvert_elems[v.x + k]; });
    }
  }
}

// Team barrier.  A cluster team uses barrier.cluster (cluster.sync():
// arrive.release, wait.acquire).  The whole-GPU team (every CTA of a
// cooperative launch, so all of them are resident) counts arrivals in global
// memory: after a CTA barrier, thread 0 adds one to the counter (acquire and
// release semantics) and polls it with acquire loads until it reaches the CTA
// count times the barrier's ordinal, before the CTA barrier that lets its
// threads go on (the adds form one release sequence, so the load or add that
// sees the full count synchronizes with every CTA's arrival).  The wait is bounded by a time limit and an
// iteration cap; a CTA that gives up records SGPU_ERR_TIMEOUT in *status and
// sets the counter's abort bit, and every CTA that sees the bit returns false
// (the kernel then leaves).  extra: arrivals the barrier waits for beyond the
// CTAs of the launch (0; a host-side test hook makes it 1 so that the wait
// runs out).
constexpr unsigned int kBarAbort = 0x80000000u;

__device__ __forceinline__ unsigned int ld_acquire_gpu(const unsigned int* p) {
  unsigned int v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

template <bool kWide>
struct TeamBarrier {
  unsigned int C;
  unsigned int* count;
  unsigned int target;
  unsigned long long limit_ns;
  int* status;
  int* s_ok;  // shared: the wait's outcome for the CTA
  unsigned int extra;

  __device__ __forceinline__ bool sync() {
    if constexpr (!kWide) {
      if (C > 1) {
        cg::this_cluster().sync();
      } else {
        __syncthreads();
      }
      return true;
    } else {
      __syncthreads();
      target += C + extra;
      if (threadIdx.x == 0) {
        unsigned int v;
        asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], 1;"
                     : "=r"(v)
                     : "l"(count)
                     : "memory");
        v += 1u;
        int ok = 1;
        unsigned long long t0 = 0ull;
        for (unsigned int it = 1;; it++) {
          if (v & kBarAbort) {
            ok = 0;
            break;
          }
          if (v >= target) break;
          if ((it & 1023u) == 0u) {
            const unsigned long long now = global_ns();
            if (t0 == 0ull) {
              t0 = now;
            } else if (now - t0 > limit_ns || it >= (1u << 28)) {
              atomicCAS(status, 0, SGPU_ERR_TIMEOUT);
              atomicOr(count, kBarAbort);
              ok = 0;
              break;
            }
          }
          v = ld_acquire_gpu(count);
        }
        *s_ok = ok;
      }
      __syncthreads();
      return *s_ok != 0;
    }
  }
};

// Profiling helpers: algorithmic bytes (warp-aggregated, converged code) and
// per-phase time measured by the team's first thread.
__device__ __forceinline__ void team_bytes(const TeamArgs& a, int phase, unsigned long long b) {
  if (!a.prof_bytes) return;
#pragma unroll
  for (int o = 16; o >= 1; o >>= 1) b += __shfl_xor_sync(0xffffffffu, b, o);
  if ((threadIdx.x & 31) == 0 && b) atomicAdd(&a.prof_bytes[phase], b);
}

struct PhaseClock {
  unsigned long long last;
  __device__ __forceinline__ void mark(const TeamArgs& a, unsigned rank, int phase) {
    if (!a.phase_ns || rank != 0 || threadIdx.x != 0) return;
    const unsigned long long now = global_ns();
    atomicAdd(&a.phase_ns[phase], now - last);
    last = now;
  }
};

// Two builds of the kernel: one CTA per SM with the full register file (the
// fastest single strokes), or two CTAs per SM (twice the teams for batches).
// kOrig: the build that also runs grab, elastic deform and layer dabs (the
// other build carries none of their code).
// kWide: the whole-GPU team (cooperative launch, one CTA per SM), which runs
// the jobs one after another.
template <int kMinBlocks, bool kOrig, bool kWide, bool kTwoLevel = false, bool kSym = false>
__global__ void __launch_bounds__(kTeamThreads, kMinBlocks) k_team_stroke(TeamArgs a) {
  unsigned C, rank;
  if constexpr (kWide) {
    C = gridDim.x;
    rank = blockIdx.x;
  } else {
    const cg::cluster_group cluster = cg::this_cluster();
    C = cluster.num_blocks();
    rank = cluster.block_rank();
  }
  // Item lists are dealt to the team in warp-sized blocks, round-robin over
  // the CTAs (block b goes to CTA b % C), so that a short list still spreads
  // its scattered loads over every SM of the cluster.
  const int lane = threadIdx.x & 31;
  const int gt = 32 * ((threadIdx.x >> 5) * static_cast<int>(C) + static_cast<int>(rank)) + lane;
  const int GT = C * kTeamThreads;
  __shared__ TeamShared sh;
  // area lanes and flush tables are never live at the same time
  union Scratch {
    Lane lanes[kTeamThreads];
    FlushSmem flush;
  };
  static_assert(sizeof(FlushSmem) <= sizeof(Lane) * kTeamThreads, "flush tables exceed the lanes");
  __shared__ Scratch s_scr;
  Lane* s_lanes = s_scr.lanes;
  __shared__ Lane s_chunks[kTeamMaxChunks];
  __shared__ int4 s_top[kCullTopMax];  // the node search's first level (cull_top)
  extern __shared__ __align__(16) unsigned char dyn[];
  float4* s_nbc = reinterpret_cast<float4*>(dyn);  // smooth neighbour tables
  int* s_par = reinterpret_cast<int*>(dyn + kStageBytes);
  int* s_cl = s_par + a.max_nodes;
  int* s_coff = s_cl + a.max_leaves + 1;
  int* s_lnv = s_coff + a.max_leaves + 2;
  unsigned short* s_idx = reinterpret_cast<unsigned short*>(s_lnv + a.max_leaves);
  unsigned short* s_lnode = s_idx + ((a.max_nodes + 1) & ~1);
  // node marks; also the flush's claim bitmap (32-bit words): the ushort
  // arrays before it have even lengths, so this starts 4-byte aligned
  unsigned char* s_pass = reinterpret_cast<unsigned char*>(s_lnode + ((a.max_leaves + 1) & ~1));
  const CullTabs ct{s_lnode, s_lnv};
  PhaseClock clk;
  clk.last = a.phase_ns ? global_ns() : 0ull;
  TeamBarrier<kWide> bar{C, a.bar, 0u, a.wait_ns, a.status, &sh.bar_ok,
                         static_cast<unsigned int>(a.bar_extra)};
#define TEAM_SYNC()          \
  do {                       \
    if (!bar.sync()) return; \
  } while (0)

  int next_wide = 0;
  for (;;) {
    int jid;
    if constexpr (kWide) {
      jid = next_wide++;
    } else {
      if (rank == 0 && threadIdx.x == 0) sh.jobid = atomicAdd(a.next_job, 1);
      TEAM_SYNC();
      jid = (C > 1) ? *cg::this_cluster().map_shared_rank(&sh.jobid, 0) : sh.jobid;
      TEAM_SYNC();
    }
    if (jid >= a.njobs) return;
    {
      const int* src = reinterpret_cast<const int*>(&a.jobs[jid]);
      int* dst = reinterpret_cast<int*>(&sh.job);
      for (int i = threadIdx.x; i < static_cast<int>(sizeof(TeamJob) / 4); i += kTeamThreads)
        dst[i] = src[i];
    }
    __syncthreads();
    {
      const int* src = reinterpret_cast<const int*>(&a.meshes[sh.job.mesh]);
      int* dst = reinterpret_cast<int*>(&sh.m);
      for (int i = threadIdx.x; i < static_cast<int>(sizeof(DevMesh) / 4); i += kTeamThreads)
        dst[i] = src[i];
    }
    __syncthreads();
    const DevMesh& m = sh.m;
    DevBrush& b = sh.job.brush;
    Work* w = m.work;
    for (int i = threadIdx.x; i < m.totnode; i += kTeamThreads) {
      s_par[i] = m.node_parent[i];
      s_idx[i] = kNoPos;
    }
    for (int k = threadIdx.x; k < m.nleaf; k += kTeamThreads) {
      s_lnode[k] = static_cast<unsigned short>(m.leaf_node[k]);
      s_lnv[k] = leaf_nverts(m, k);
    }
    for (int k = threadIdx.x; k < m.cull_ntop; k += kTeamThreads) s_top[k] = m.cull_top[k];
    // GRIDS work-list stamps: dab d uses epoch grid_epoch0 + d + 1
    const unsigned int grid_epoch0 = __ldcg(&w->grid_epoch);
    TEAM_SYNC();
    if (rank == 0 && threadIdx.x == 0) {
      for (int k = 0; k < 3; k++) w->hit_count[k] = 0;
      w->tag_count[0] = w->tag_count[1] = 0;
      w->touch_count[0] = w->touch_count[1] = 0;
      if (m.type == kGrids) m.grid_counts[0] = m.grid_counts[1] = m.grid_counts[2] = m.grid_counts[3] = 0;
    }
    TEAM_SYNC();
    // Leaves flagged and vertices tagged before the stroke (by per-call entry
    // points) join the first dab's update, as they would in the per-call path.
    if (rank == 0)
      for (int leaf = threadIdx.x; leaf < m.nleaf; leaf += kTeamThreads) {
        const int f = __ldcg(&m.leaf_flag[leaf]);
        if (!(f & (kUpdateNormals | kUpdateBB))) continue;
        append(m.touch_list, &w->touch_count[0], leaf);
        if (m.type == kGrids)  // the first dab's normal update takes its faces
          for (int j = m.leaf_prim_off[leaf]; j < m.leaf_prim_off[leaf + 1]; j++)
            grid_claim_face_only(m, m.leaf_prims[j], grid_epoch0 + 1u);
        if ((f & kUpdateNormals) && m.type == kFaces) {
          const int off = m.leaf_vert_off[leaf];
          for (int i = 0; i < m.leaf_uniq[leaf]; i++) {
            const int v = m.leaf_verts[off + i];
            if (__ldcg(&m.vtag[v])) m.tag_list[atomicAdd(&w->tag_count[0], 1)] = v;
          }
        }
      }
    TEAM_SYNC();
    clk.mark(a, rank, kPhJob);
    const int default_tool = b.tool;
    int q = 0;  // smooth sweep counter (hit-list rotation)
    for (int d = 0; d < sh.job.ndabs; d++) {
      const int par = d & 1;
      if (rank == 0 && threadIdx.x == 0) {
        w->tag_count[par ^ 1] = 0;
        w->touch_count[par ^ 1] = 0;
      }
      const int tool = sh.job.tools ? sh.job.tools[d] : default_tool;
      __syncthreads();
      if (threadIdx.x == 0) b.tool = tool;
      __syncthreads();
      const float scale = (tool == kToolClayStrips) ? 1.41421356237309504880f : 1.0f;
      const float r = b.radius * scale;
      int* tag_cnt = &w->tag_count[par];
      int* touch_cnt = &w->touch_count[par];
      // GRIDS work-list stamp of this dab
      const unsigned int epoch = grid_epoch0 + static_cast<unsigned int>(d) + 1u;
      if (kOrig && uses_original(tool)) {
        // grab / elastic deform: one gather over all passes, then each vertex
        // rebuilt from its stroke-start position (k_cull_dab, k_orig_dab)
        if (threadIdx.x == 0) {
          DabPasses& dp = sh.dp;
          dp.npass = 0;
          for (int pass = 0; pass < 8; pass++) {
            if ((pass & ~sh.job.symmetry) != 0) continue;
            for (int k = 0; k < 3; k++) {
              const float sgn = (pass & (1 << k)) ? -1.0f : 1.0f;
              dp.loc[dp.npass][k] = sgn * sh.job.dabs[6 * d + k];
              dp.delta[dp.npass][k] = sgn * sh.job.dabs[6 * d + 3 + k];
              dp.view[dp.npass][k] = sgn * sh.job.view[k];
            }
            dp.npass++;
          }
          // the Kelvinlet force of the dab (BKE_kelvinlet_init_params,
          // kelvinlet.c:6-21): |grab delta| * strength
          const float* gd = &sh.job.dabs[6 * d + 3];
          b.kl_f = sqrtf(gd[0] * gd[0] + gd[1] * gd[1] + gd[2] * gd[2]) * b.strength;
        }
        __syncthreads();
        team_cull_union<kTwoLevel>(m, sh.dp, b.radius * b.radius, tool == kToolElasticDeform ? 1 : 0, s_pass,
                        s_cl, s_coff, ct, sh, s_top);
        const int cnt = sh.cnt, total = sh.total;
        team_bytes(a, kPhCull, (rank == 0 && threadIdx.x == 0) ? 24ull * m.totnode + 8ull * cnt : 0ull);
        clk.mark(a, rank, kPhCull);
        if (rank == 0)
          for (int k = threadIdx.x; k < cnt; k += kTeamThreads) {
            const int leaf = s_cl[k];
            const int old = atomicOr(&m.leaf_flag[leaf], kMarkUpdate);
            if (!(old & kUpdateNormals)) append(m.touch_list, touch_cnt, leaf);
          }
        if (m.type == kGrids) team_claim_faces(m, s_cl, cnt, rank, C, epoch);
        team_bytes(a, kPhBrush, team_orig_sweep(m, b, sh.dp, s_cl, s_coff, cnt, total, gt, GT, tag_cnt));
        TEAM_SYNC();
        clk.mark(a, rank, kPhBrush);
      }
      // kSym builds, single-axis symmetry: one node search gives both passes'
      // lists (boxes change only at the end of the dab, so the second pass's
      // list is the one a search after the first pass would give).  When the
      // lists share no leaf and the tool reads and writes only the vertex
      // itself, the two passes commute and run as one (joint): one area phase
      // with a pairwise tree per pass, one sweep with each vertex under its
      // own pass's frame.  The pair's state stays in shared memory (sh.split,
      // sh.joint, sh.held).
      for (int pass = 0; pass < 8 && !(kOrig && uses_original(tool)); pass++) {
        if ((pass & ~sh.job.symmetry) != 0) continue;
        if constexpr (kSym) {
          if (pass != 0 && sh.joint) break;  // the second pass ran with the first
        }
        PassParams pp;
        for (int k = 0; k < 3; k++) {
          const float sgn = (pass & (1 << k)) ? -1.0f : 1.0f;
          pp.loc[k] = sgn * sh.job.dabs[6 * d + k];
          pp.delta[k] = sgn * sh.job.dabs[6 * d + 3 + k];
          pp.view[k] = sgn * sh.job.view[k];
        }
        pp.cull_radius_sq = r * r;
        pp.original = sh.job.use_orig || (kOrig && tool == kToolLayer);  // layer: stroke-start boxes
        pp.iter_strength = 1.0f;
        pp.iteration = 0;
        if constexpr (!kSym) {
          team_cull<kMinBlocks == 1 ? 8 : 2, kTwoLevel>(m, pp, s_pass, s_cl, s_coff, ct, sh, s_top);
          // 24 B per node box tested, 8 B per leaf emitted (counted once per team)
          team_bytes(a, kPhCull, (rank == 0 && threadIdx.x == 0) ? 24ull * m.totnode + 8ull * sh.cnt : 0ull);
        } else {
          const int sym = sh.job.symmetry;
          const bool pair = pass == 0 && (sym == 1 || sym == 2 || sym == 4);
          if (pass != 0 && sh.held >= 0) {
            if (threadIdx.x == 0) sh.mpp[0] = pp;
            team_list_to_front(s_cl, s_coff, sh);
          } else {
            // (sh.mpp is read after the search's barriers)
            float loc1[3];
            for (int k = 0; k < 3; k++) loc1[k] = ((sym >> k) & 1) ? -pp.loc[k] : pp.loc[k];
            if (threadIdx.x == 0) {
              sh.mpp[0] = pp;
              PassParams p1 = pp;
              for (int k = 0; k < 3; k++) {
                p1.loc[k] = loc1[k];
                if ((sym >> k) & 1) {
                  p1.delta[k] = -pp.delta[k];
                  p1.view[k] = -pp.view[k];
                }
              }
              sh.mpp[1] = p1;
            }
            team_cull_pair<kMinBlocks == 1 ? 8 : 2, kTwoLevel>(m, pp, loc1, pair, s_pass, s_cl, s_coff, ct,
                                                               sh, a.max_leaves + 1, pair_tool(tool), s_top);
            // node boxes tested once for the pass or pair, 8 B per leaf emitted
            team_bytes(a, kPhCull, (rank == 0 && threadIdx.x == 0)
                                       ? 24ull * m.totnode + 8ull * (sh.held >= 0 ? sh.cnt + sh.held : sh.cnt)
                                       : 0ull);
          }
        }
        const int cnt = sh.cnt, total = sh.total;
        clk.mark(a, rank, kPhCull);
        float area_no[3] = {0.0f, 0.0f, 0.0f}, area_co[3] = {0.0f, 0.0f, 0.0f};
        if (uses_area(tool)) {
          const float rn = b.radius * b.normal_radius_factor;
          const float ra = b.radius * b.area_radius_factor;
          unsigned long long ab = 0;
          const int nb = m.area_blocks;
          for (int k = rank; k < cnt * nb; k += C) {
            const int leaf = s_cl[k / nb], blk = k % nb;
            if constexpr (!kSym) {
              team_area_block(m, pp.loc, rn * rn, ra * ra, leaf, blk, s_nbc, s_lanes, &m.parts[k]);
            } else {
              const bool second = k / nb >= sh.split;
              float c[3];
              for (int q = 0; q < 3; q++) c[q] = second ? sh.mpp[1].loc[q] : pp.loc[q];
              team_area_block(m, c, rn * rn, ra * ra, leaf, blk, s_nbc, s_lanes, &m.parts[k]);
            }
            const int nv = min(leaf_nverts(m, leaf) - blk * kAreaBlock, kAreaBlock);
            if (static_cast<int>(threadIdx.x) < nv)
              ab += ((m.type == kFaces ? 4ull : 0ull) + 24ull) *
                    ((nv - threadIdx.x + kTeamThreads - 1) / kTeamThreads);
          }
          team_bytes(a, kPhArea, ab);
          TEAM_SYNC();
          if (kSym && sh.joint) {
            // the second pass's tree over its own partials, and its frame
            team_area_final(m, sh.mpp[1], (cnt - sh.split) * nb, s_lanes, s_chunks, sh, sh.split * nb);
            BrushFrame f1;
            const bool ok1 = make_frame(b, sh.mpp[1], sh.area, sh.area + 3, f1);
            __syncthreads();  // sh.area read
            if (threadIdx.x == 0) {
              sh.live1 = ok1 ? 1 : 0;
              if (ok1) sh.mframe[1] = f1;
            }
          }
          team_area_final(m, pp, (kSym ? sh.split : cnt) * nb, s_lanes, s_chunks, sh);
          for (int k = 0; k < 3; k++) {
            area_no[k] = sh.area[k];
            area_co[k] = sh.area[3 + k];
          }
          clk.mark(a, rank, kPhArea);
        } else if (kSym && sh.joint && threadIdx.x == 0) {
          BrushFrame f1;
          sh.live1 = make_frame(b, sh.mpp[1], area_no, area_co, f1) ? 1 : 0;
          sh.mframe[1] = f1;
        }
        BrushFrame f;
        int lo = 0, hi = cnt;  // the leaves of the passes with a frame
        bool joint = false;
        if constexpr (!kSym) {
          if (!make_frame(b, pp, area_no, area_co, f)) continue;
        } else {
          const bool ok0 = make_frame(b, pp, area_no, area_co, f);
          joint = sh.joint != 0;
          if (joint) __syncthreads();  // sh.live1
          // (a pass without a frame marks nothing)
          const bool ok1 = joint && sh.live1;
          if (!ok0 && !ok1) continue;
          if (joint && threadIdx.x == 0) sh.mframe[0] = f;
          lo = ok0 ? 0 : sh.split;
          hi = (!joint || ok1) ? cnt : sh.split;
        }
        if (rank == 0)
          for (int k = lo + static_cast<int>(threadIdx.x); k < hi; k += kTeamThreads) {
            const int leaf = s_cl[k];
            const int old = atomicOr(&m.leaf_flag[leaf], kMarkUpdate);
            if (!(old & kUpdateNormals)) append(m.touch_list, touch_cnt, leaf);
          }
        if (m.type == kGrids) team_claim_faces(m, s_cl + lo, hi - lo, rank, C, epoch);
        if (tool != kToolSmooth) {
          unsigned long long ab = 0;
          const unsigned vbytes = (m.type == kFaces ? 4u : 0u) + 12u + (m.mask ? 4u : 0u) +
                                  (m.automask ? 4u : 0u) +
                                  ((tool == kToolInflate || (b.flag & kBrushFrontFace)) ? 12u : 0u);
          if (!joint) {
            for (int base = gt - lane; base < total; base += GT) {
              const int i = base + lane;
              bool moved = false;
              if (i < total) {
                const int k = smem_find_slot(s_coff, cnt, i);
                const int v = leaf_vert(m, s_cl[k], i - s_coff[k]);
                float4 co = __ldcg(&m.co[v]);
                ab += vbytes;
                const bool hit = (kOrig && tool == kToolLayer) ? layer_vertex(m, b, b.y, pp, v, co, moved)
                                                    : brush_vertex(m, b, b.y, pp, f, v, co, moved);
                if (hit) {
                  m.co[v] = co;
                  ab += 12u;
                  if (m.type == kFaces) tag_vertex(m, v, tag_cnt);
                }
              }
              const unsigned bal = __ballot_sync(0xffffffffu, moved);
              if ((threadIdx.x & 31) == 0 && bal) atomicAdd(&w->displaced, (unsigned long long)__popc(bal));
            }
          } else if constexpr (kSym) {
            // the joint pair: each vertex under its own pass's parameters and
            // frame (in shared memory), the passes' vertices [vlo, vhi)
            const int vlo = s_coff[lo], vhi = s_coff[hi], split = sh.split;
            __syncthreads();  // the frames in shared memory
            for (int base = vlo + gt - lane; base < vhi; base += GT) {
              const int i = base + lane;
              bool moved = false;
              if (i < vhi) {
                const int k = smem_find_slot(s_coff, cnt, i);
                const int v = leaf_vert(m, s_cl[k], i - s_coff[k]);
                float4 co = __ldcg(&m.co[v]);
                ab += vbytes;
                const int pk = k >= split ? 1 : 0;
                if (brush_vertex(m, b, b.y, sh.mpp[pk], sh.mframe[pk], v, co, moved)) {
                  m.co[v] = co;
                  ab += 12u;
                  if (m.type == kFaces) tag_vertex(m, v, tag_cnt);
                }
              }
              const unsigned bal = __ballot_sync(0xffffffffu, moved);
              if ((threadIdx.x & 31) == 0 && bal) atomicAdd(&w->displaced, (unsigned long long)__popc(bal));
            }
          }
          team_bytes(a, kPhBrush, ab);
          TEAM_SYNC();
          clk.mark(a, rank, kPhBrush);
        } else {
          float st = b.strength;
          if (st < 0.0f) st = 0.0f;
          if (st > 1.0f) st = 1.0f;
          const int count = (int)(st * 4.0f);
          const float last = 4.0f * (st - (float)count * 0.25f);
          // Jacobi sweeps over slots.  CTA r gives its hits the slots
          // [r * R, r * R + nh) (R bounds its share of the candidates), so no
          // slot counter is shared.  The thread that runs a hit's first sweep
          // keeps it for the later ones; its first hit keeps vertex, value and
          // ring table on chip.  The last sweep writes the positions.  The two
          // slot maps alternate by pass, so a pass clears its entries while
          // the next one fills the other map.
          int* const smap = m.slot_map[q & 1];
          q++;
          // kSym builds: a hit's slot record holds its pass in the top bit (a
          // joint pair's hits carry their own pass's parameters, kept in
          // shared memory with the sweep's strength)
          auto hit_v = [](int x) { return kSym ? (x & 0x7FFFFFFF) : x; };
          auto hit_p = [](int x) { return kSym ? static_cast<int>(static_cast<unsigned int>(x) >> 31) : 0; };
          auto pass_of = [&](int pk) -> const PassParams& {
            if constexpr (kSym) {
              return sh.mpp[pk];
            } else {
              (void)pk;
              return pp;
            }
          };
          const int split = kSym ? sh.split : cnt;
          int* const slot_v = m.hit_list[0];
          float4* const val[2] = {m.scratch, m.scratch2};
          const int R = 32 * ((total + 32 * static_cast<int>(C) - 1) / (32 * static_cast<int>(C)));
          const int sbase = static_cast<int>(rank) * R;
          pp.iter_strength = (count != 0) ? 1.0f : last;
          pp.iteration = 0;
          if (threadIdx.x == 0) {
            sh.nh = 0;
            if constexpr (kSym)
              for (int k = 0; k < 2; k++) {
                sh.mpp[k].iter_strength = pp.iter_strength;
                sh.mpp[k].iteration = 0;
              }
          }
          __syncthreads();
          // first sweep, stage 1: distance test of this CTA's candidates
          const float rr = b.radius * b.radius;
          unsigned long long ab = 0;
          constexpr int kCand = 4;
          for (int base = gt - lane; base < total; base += kCand * GT) {
            int vv[kCand];
            float4 cc[kCand];
            unsigned int pm = 0u;  // the candidates of a joint pair's second pass
#pragma unroll
            for (int j = 0; j < kCand; j++) {
              const int i = base + j * GT + lane;
              vv[j] = -1;
              if (i < total) {
                const int k = smem_find_slot(s_coff, cnt, i);
                vv[j] = leaf_vert(m, s_cl[k], i - s_coff[k]);
                if (kSym && k >= split) pm |= 1u << j;
              }
            }
#pragma unroll
            for (int j = 0; j < kCand; j++)
              if (vv[j] >= 0) cc[j] = __ldcg(&m.co[vv[j]]);
#pragma unroll
            for (int j = 0; j < kCand; j++) {
              if (vv[j] < 0) continue;
              ab += 16u;  // vertex id, co
              const int pk = static_cast<int>((pm >> j) & 1u);
              if (!(dist_sq(cc[j], pass_of(pk).loc) <= rr)) continue;
              cg::coalesced_group g = cg::coalesced_threads();
              int h = 0;
              if (g.thread_rank() == 0) h = atomicAdd(&sh.nh, static_cast<int>(g.size()));
              h = g.shfl(h, 0) + g.thread_rank();
              const int rec = kSym ? (vv[j] | (pk << 31)) : vv[j];
              slot_v[sbase + h] = rec;
              if (h < kTeamThreads) {
                sh.hv[h] = rec;
                sh.hco[h] = cc[j];
              }
            }
          }
          __syncthreads();
          const int nh = sh.nh;
          // stage 2: the first sweep of the hits
          int v0 = -1, n0 = -1, p0 = 0;
          float4 own = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
          for (int hb = threadIdx.x - lane; hb < nh; hb += kTeamThreads) {
            const int h = hb + lane;
            bool moved = false;
            if (h < nh) {
              const int x = h < kTeamThreads ? sh.hv[h] : __ldcg(&slot_v[sbase + h]);
              const int v = hit_v(x), pk = hit_p(x);
              const float4 co = h < kTeamThreads ? sh.hco[h] : __ldcg(&m.co[v]);
              float4 out;
              int nr = -1;
              if (h == static_cast<int>(threadIdx.x)) {
                out = smooth_first(m, b, pass_of(pk), v, co, s_nbc + threadIdx.x, kTeamThreads, &nr, moved);
                v0 = v;
                n0 = nr;
                p0 = pk;
                own = out;
              } else {
                smooth_vertex(m, b, b.y, pass_of(pk), v, co, out, moved);
              }
              val[0][sbase + h] = out;
              smap[v] = sbase + h;
              if (m.type == kFaces) tag_vertex(m, v, tag_cnt);
              const int valence = m.type == kFaces ? m.nb_off[v + 1] - m.nb_off[v] : 4;
              // mask, ring range and ring (id + co) reads; value, map and slot written
              ab += (m.mask ? 4ull : 0ull) + (m.type == kFaces ? 8ull : 0ull) + 16ull * valence + 24ull;
            }
            const unsigned bal = __ballot_sync(0xffffffffu, moved);
            if (lane == 0 && bal) atomicAdd(&w->displaced, (unsigned long long)__popc(bal));
          }
          team_bytes(a, kPhBrush, ab);
          TEAM_SYNC();
          clk.mark(a, rank, kPhBrush);
          if (count == 0) {
            for (int h = threadIdx.x; h < nh; h += kTeamThreads) {
              const int v = h == static_cast<int>(threadIdx.x) ? v0 : hit_v(__ldcg(&slot_v[sbase + h]));
              m.co[v] = h == static_cast<int>(threadIdx.x) ? own : __ldcg(&val[0][sbase + h]);
            }
          }
          for (int it = 1; it <= count; it++) {
            pp.iter_strength = (it != count) ? 1.0f : last;
            pp.iteration = it;
            if constexpr (kSym) {
              // (the last sweep's reads ended at its team barrier)
              if (threadIdx.x == 0)
                for (int k = 0; k < 2; k++) {
                  sh.mpp[k].iter_strength = pp.iter_strength;
                  sh.mpp[k].iteration = it;
                }
              __syncthreads();
            }
            const float4* src = val[(it - 1) & 1];
            float4* dst = val[it & 1];
            ab = 0;
            for (int h = threadIdx.x; h < nh; h += kTeamThreads) {
              float4 out;
              int v, nring;
              if (h == static_cast<int>(threadIdx.x) && n0 >= 0) {
                if (it == 1) smooth_resolve(s_nbc + threadIdx.x, kTeamThreads, n0, smap);
                out = smooth_slot_cached(m, b, pass_of(p0), v0, own, n0, s_nbc + threadIdx.x, kTeamThreads,
                                         src);
                v = v0;
                nring = n0;
              } else {
                const bool first = h == static_cast<int>(threadIdx.x);
                const int x = first ? 0 : __ldcg(&slot_v[sbase + h]);
                v = first ? v0 : hit_v(x);
                const int pk = first ? p0 : hit_p(x);
                out = smooth_slot(m, b, pass_of(pk), v, first ? own : __ldcg(&src[sbase + h]), src, smap);
                nring = m.type == kFaces ? m.nb_off[v + 1] - m.nb_off[v] : 4;
              }
              if (h == static_cast<int>(threadIdx.x)) own = out;
              if (it == count) {
                m.co[v] = out;
              } else {
                dst[sbase + h] = out;
              }
              // value and mask read, ring values read, value written
              ab += 16ull + (m.mask ? 4ull : 0ull) + 16ull * nring + 16ull;
            }
            team_bytes(a, kPhApply, ab);
            TEAM_SYNC();
            clk.mark(a, rank, kPhApply);
          }
          if (count == 0) {
            TEAM_SYNC();
            clk.mark(a, rank, kPhApply);
          }
          // clear this pass's map entries; the map is next filled two smooth
          // passes later, after at least one more team barrier
          for (int h = threadIdx.x; h < nh; h += kTeamThreads)
            smap[h == static_cast<int>(threadIdx.x) ? v0 : hit_v(__ldcg(&slot_v[sbase + h]))] = -1;
        }
      }
      // End of the dab.  FACES: refit of the touched leaves, then the flush
      // (CTA 0) alongside the normal update of the tagged vertices (the other
      // CTAs): normals read positions and leaf flags, the flush reads chunk
      // boxes and writes node boxes.  GRIDS: the normal update moves seam
      // positions, so it runs first, then refit and flush.
      const int ntag = __ldcg(tag_cnt);
      const int ntouch = __ldcg(touch_cnt);
      unsigned long long ab = 0;
      FlushState fst;
      if (m.type == kGrids) {
        // GRIDS: the faces of the dab's leaves (claimed where the leaves were
        // marked): inner normals, face seams and centres, one CTA per face;
        // then the base edges and corners (positions move at the seams, so
        // the refit below follows).
        const int nf = __ldcg(&m.grid_counts[0]);
        const int group = face_grid_group(m.grid_size, kStageBytes);
        int pre_fi = -1;  // the face whose boundary item tables the stage holds
        if (group > 0) {
          for (int fi = static_cast<int>(rank); fi < nf; fi += static_cast<int>(C)) {
            const int f = __ldcg(&m.face_list[fi]);
            const int2 fs = __ldcg(&m.face_info[fi]);
            pre_fi = team_grid_face<kWide && !kSym, kWide && !kSym>(m, f, fs.x, fs.y, dyn, group, epoch)
                         ? fi
                         : -1;
            if (threadIdx.x == 0) {
              const int n = fs.y;
              // positions read, normals written; the seam pairs and the
              // centre read and write co, no and mask
              ab += 24ull * n * m.grid_area + 112ull * n * (m.grid_size - 1) + 56ull * n;
            }
          }
          team_bytes(a, kPhGridFaces, ab);
          ab = 0;
          TEAM_SYNC();
          clk.mark(a, rank, kPhGridFaces);
        } else {
          // grids too large to stage: one item per element, then the seams
          const int ng = __ldcg(&m.grid_counts[3]);
          const long long inner = (long long)ng * m.grid_area;
          for (long long it = gt; it < inner; it += GT) {
            grid_inner_item(m, it);
            ab += 24u;  // co read, normal written
          }
          TEAM_SYNC();
          const long long pairs = (long long)ng * (m.grid_size - 1);
          for (long long it = gt; it < pairs + nf; it += GT) {
            grid_face_seam_item(m, it, ng);
            ab += it < pairs ? 112ull : 56ull * m.face_ngrids[__ldcg(&m.face_list[it - pairs])];
          }
          TEAM_SYNC();
        }
        for (int fi = static_cast<int>(rank); fi < nf; fi += static_cast<int>(C))
          {
            const int2 fs = __ldcg(&m.face_info[fi]);
            team_grid_face_boundary(
                m, __ldcg(&m.face_list[fi]), fs.x, fs.y, epoch, group > 0,
                fi == pre_fi ? dyn + boundary_prefetch_offset(m.grid_size, group) : nullptr);
          }
        TEAM_SYNC();
        clk.mark(a, rank, kPhGridSeams);
        if (rank == 0 && threadIdx.x == 0)
          m.grid_counts[0] = m.grid_counts[1] = m.grid_counts[2] = m.grid_counts[3] = 0;
      }
      // refit: the chunk boxes of the touched leaves, one warp per chunk
      // across the team (chunk offsets of the touched leaves in s_coff)
      {
        const int seg = (ntouch + kTeamThreads - 1) / kTeamThreads;
        const int t0 = min(ntouch, static_cast<int>(threadIdx.x) * seg), t1 = min(ntouch, t0 + seg);
        int nc = 0;
        for (int k = t0; k < t1; k++) {
          const int leaf = __ldcg(&m.touch_list[k]);
          s_cl[k] = leaf;
          nc += m.leaf_chunk_off[leaf + 1] - m.leaf_chunk_off[leaf];
        }
        int nchunk;
        int off = team_block_scan(nc, &nchunk, sh.scan);
        for (int k = t0; k < t1; k++) {
          s_coff[k] = off;
          off += m.leaf_chunk_off[s_cl[k] + 1] - m.leaf_chunk_off[s_cl[k]];
        }
        __syncthreads();
        // chunks dealt over CTAs 1..C-1 while CTA 0 lists the ancestors to flush
        const int wpc = kTeamThreads / 32;
        const int rc = C > 1 ? static_cast<int>(C) - 1 : 1;
        const int rr = C > 1 ? static_cast<int>(rank) - 1 : 0;
        const unsigned idb = (m.type == kFaces ? 4u : 0u) + 12u;  // vertex id, position
        if (rank != 0 || C == 1) {
          for (int j = (threadIdx.x >> 5) * rc + rr; j < nchunk; j += rc * wpc) {
            const int k = smem_find_slot(s_coff, ntouch, j);
            const int leaf = s_cl[k], c = j - s_coff[k];
            float mn[3], mx[3];
            chunk_refit_warp(m, leaf, c, mn, mx);
            if (lane == 0)
              ab += 32ull + idb * static_cast<unsigned long long>(min(kChunk, leaf_nverts_all(m, leaf) - c * kChunk));
          }
        }
        if (rank == 0)
          team_flush_mark(m, ntouch, s_cl, s_lnode, s_par, reinterpret_cast<unsigned int*>(s_pass), s_coff, s_idx,
                          s_scr.flush, sh, fst);
      }
      team_bytes(a, kPhUpdate, ab);
      TEAM_SYNC();
      clk.mark(a, rank, kPhUpdate);
      // flush by CTA 0: the listed ancestors bottom-up
      unsigned long long fb = 0;
      if (rank == 0) team_flush_levels(m, ntouch, s_cl, s_lnode, s_par, s_coff, s_idx, s_scr.flush, sh, fst, fb);
      team_bytes(a, kPhFlush, fb);
      if (m.type == kFaces && (rank != 0 || C == 1)) {
        // normals over CTAs 1..C-1 (all of the team when it is one CTA)
        const int nc = C > 1 ? static_cast<int>(C) - 1 : 1;
        const int cr = C > 1 ? static_cast<int>(rank) - 1 : 0;
        ab = 0;
        for (int j = 32 * ((threadIdx.x >> 5) * nc + cr) + lane; j < ntag; j += nc * kTeamThreads) {
          const int v = __ldcg(&m.tag_list[j]);
          float4 n;
          const int used = vertex_normal(m, v, n);
          m.no[v] = n;
          m.vtag[v] = 0u;
          ab += 24ull + 16ull * used;
        }
        team_bytes(a, kPhUpdate, ab);
      }
      TEAM_SYNC();
      clk.mark(a, rank, kPhFlush);
      // the touched leaves' update flags clear once both have read them
      if (rank == 0)
        for (int k = threadIdx.x; k < ntouch; k += kTeamThreads)
          atomicAnd(&m.leaf_flag[__ldcg(&m.touch_list[k])], ~(kUpdateNormals | kUpdateBB));
    }
    // end of stroke: BKE_pbvh_update_bounds(UpdateOriginalBB)
    for (int i = threadIdx.x; i < m.totnode; i += kTeamThreads) s_pass[i] = 0;
    __syncthreads();
    for (int leaf = threadIdx.x; leaf < m.nleaf; leaf += kTeamThreads) {
      if (!(__ldcg(&m.leaf_flag[leaf]) & kUpdateOriginalBB)) continue;
      int n = m.leaf_node[leaf];
      s_pass[n] = 1;
      n = s_par[n];
      while (n >= 0 && !s_pass[n]) {
        s_pass[n] = 1;
        n = s_par[n];
      }
    }
    __syncthreads();
    for (int n = gt; n < m.totnode; n += GT)
      if (s_pass[n]) {
        m.orig_vb[2 * n] = __ldcg(&m.vb[2 * n]);
        m.orig_vb[2 * n + 1] = __ldcg(&m.vb[2 * n + 1]);
      }
    TEAM_SYNC();
    for (int leaf = gt; leaf < m.nleaf; leaf += GT) atomicAnd(&m.leaf_flag[leaf], ~kUpdateOriginalBB);
    if (rank == 0 && threadIdx.x == 0 && m.type == kGrids)
      w->grid_epoch = grid_epoch0 + static_cast<unsigned int>(sh.job.ndabs);
    TEAM_SYNC();
    clk.mark(a, rank, kPhJob);
  }
}
#undef TEAM_SYNC

}  // namespace sgpu
