// Lockstep batch launch of the persistent stroke kernel: a node-level work
// queue over every mesh of a batch.
//
// One cooperative launch, one CTA per SM.  All CTAs step through the batch's
// strokes together, dab by dab (dab d of every stroke that has one), and
// every phase of a dab pools the work items of all meshes:
//
//   cull         one CTA per mesh: the node search of the pass (the same
//                code and order as the team kernel), published as the mesh's
//                culled-leaf list; brushes without an area normal also build
//                their frame and mark the leaves here;
//   area         (mesh, culled leaf, block of 4096 visited vertices) items,
//                one per CTA; the CTA that finishes a mesh's last item reduces
//                the partials (the same pairwise tree), builds the frame and
//                marks the leaves;
//   brush        (mesh, culled leaf, run of 32 visited vertices) items, one
//                per warp; smooth tests the sphere, takes a slot from the
//                mesh's hit counter and runs the first Jacobi sweep;
//   smooth       (mesh, hit) items per later sweep, one per thread;
//   GRIDS faces  (mesh, claimed face) items, one per CTA: inner normals, face
//                seams and centre, then the base edges and corners;
//   refit        (mesh, touched leaf, refit chunk) items, one per warp;
//   flush        one CTA per mesh (ancestor boxes bottom-up), while the other
//                CTAs take (mesh, tagged vertex) normal items.
//
// Item spaces are prefix sums over the meshes of per-mesh counts, computed
// identically by every CTA in shared memory; an item finds its mesh by a
// binary search there, and runs of a leaf are padded to the mesh's largest
// leaf so that no per-leaf prefix is needed.  Phases are separated by the
// whole-GPU barrier of the team kernel (release add, bounded acquire wait,
// SGPU_ERR_TIMEOUT when a wait runs out).  Every item runs the same device
// code as the single-mesh paths, so each mesh's result is bit-identical to
// its own stroke.
#include <map>
#include <mutex>
#include <tuple>
#include <utility>
#include <cuda_runtime.h>

#include "team_kernel.cuh"

namespace sgpu {

namespace {

// Leaf tables of the node search read from the mesh in global memory.
struct LockTabs {
  struct Node {
    const int* p;
    __device__ __forceinline__ int operator[](int i) const { return p[i]; }
  } lnode;
  struct Verts {
    const DevMesh* m;
    __device__ __forceinline__ int operator[](int i) const { return leaf_nverts(*m, i); }
  } lnv;
};

// Dynamic shared memory: the stage, the per-job tables, then the node search
// and flush tables of the mesh a CTA works on.
struct LockLayout {
  size_t P, ep0, tool, sym, q, cl, coff, idx, par, pass, total;
  __host__ __device__ LockLayout(int max_nodes, int max_leaves) {
    auto up = [](size_t x) { return (x + 15) & ~static_cast<size_t>(15); };
    P = kStageBytes;
    ep0 = up(P + sizeof(int) * (kLockMaxJobs + 1));
    tool = up(ep0 + sizeof(unsigned int) * kLockMaxJobs);
    sym = up(tool + kLockMaxJobs);
    q = up(sym + kLockMaxJobs);
    cl = up(q + kLockMaxJobs);
    coff = up(cl + sizeof(int) * (max_leaves + 1));
    idx = up(coff + sizeof(int) * (max_leaves + 2));
    par = up(idx + sizeof(unsigned short) * max_nodes);
    pass = up(par + sizeof(int) * max_nodes);
    const size_t bits = 4 * static_cast<size_t>((max_nodes + 31) / 32);
    total = up(pass + (bits > static_cast<size_t>(max_nodes) ? bits : max_nodes));
  }
};

// Exclusive prefix over the jobs of count(j) into s_P[0..J] (s_P[J] = total),
// the same in every CTA.  Starts with a CTA barrier: warps may still be
// finding jobs in the previous prefix.
template <class F>
__device__ int lock_prefix(int J, int* s_P, int* scan32, F count) {
  __syncthreads();
  const int seg = (J + kTeamThreads - 1) / kTeamThreads;
  const int j0 = min(J, static_cast<int>(threadIdx.x) * seg), j1 = min(J, j0 + seg);
  int sum = 0;
  for (int j = j0; j < j1; j++) {
    const int c = count(j);
    s_P[j] = c;
    sum += c;
  }
  int total;
  int off = team_block_scan(sum, &total, scan32);
  for (int j = j0; j < j1; j++) {
    const int c = s_P[j];
    s_P[j] = off;
    off += c;
  }
  if (threadIdx.x == 0) s_P[J] = total;
  __syncthreads();
  return total;
}

// Smooth sweeps of a stroke strength (do_smooth_brush): count full sweeps and
// the strength of the last one.
__device__ __forceinline__ int smooth_count(float strength, float* last) {
  float st = strength;
  if (st < 0.0f) st = 0.0f;
  if (st > 1.0f) st = 1.0f;
  const int count = (int)(st * 4.0f);
  *last = 4.0f * (st - (float)count * 0.25f);
  return count;
}

// The leaves of a pass are marked for the update (BKE_pbvh_node_mark_update)
// and, GRIDS, their faces claimed for the dab's normal update; by one CTA.
__device__ void lock_mark(const DevMesh& m, const int* list, int cnt, int* touch_cnt,
                          unsigned int epoch) {
  for (int k = threadIdx.x; k < cnt; k += kTeamThreads) {
    const int leaf = list[k];
    const int old = atomicOr(&m.leaf_flag[leaf], kMarkUpdate);
    if (!(old & kUpdateNormals)) append(m.touch_list, touch_cnt, leaf);
  }
  if (m.type == kGrids) team_claim_faces(m, list, cnt, 0u, 1u, epoch);
}

// The update flags of a dab's touched leaves clear once its normal update and
// flush are done (by one CTA).
__device__ void lock_clear_touched(const DevMesh& m, int par) {
  const int nt = __ldcg(&m.work->touch_count[par]);
  for (int k = threadIdx.x; k < nt; k += kTeamThreads)
    atomicAnd(&m.leaf_flag[__ldcg(&m.touch_list[k])], ~(kUpdateNormals | kUpdateBB));
}

// End of a job's stroke by one CTA (after its last dab's flush):
// BKE_pbvh_update_bounds(UpdateOriginalBB) over the flagged leaves and their
// ancestors, and the GRIDS work-list stamp.
__device__ void lock_finish_job(const DevMesh& m, const TeamJob& jb, unsigned int ep0,
                                unsigned char* s_pass) {
  for (int i = threadIdx.x; i < m.totnode; i += kTeamThreads) s_pass[i] = 0;
  __syncthreads();
  for (int leaf = threadIdx.x; leaf < m.nleaf; leaf += kTeamThreads) {
    if (!(__ldcg(&m.leaf_flag[leaf]) & kUpdateOriginalBB)) continue;
    int n = m.leaf_node[leaf];
    s_pass[n] = 1;
    n = m.node_parent[n];
    while (n >= 0 && !s_pass[n]) {
      s_pass[n] = 1;
      n = m.node_parent[n];
    }
  }
  __syncthreads();
  for (int n = threadIdx.x; n < m.totnode; n += kTeamThreads)
    if (s_pass[n]) {
      m.orig_vb[2 * n] = __ldcg(&m.vb[2 * n]);
      m.orig_vb[2 * n + 1] = __ldcg(&m.vb[2 * n + 1]);
    }
  __syncthreads();
  for (int leaf = threadIdx.x; leaf < m.nleaf; leaf += kTeamThreads)
    atomicAnd(&m.leaf_flag[leaf], ~kUpdateOriginalBB);
  if (threadIdx.x == 0 && m.type == kGrids)
    m.work->grid_epoch = ep0 + static_cast<unsigned int>(jb.ndabs);
  __syncthreads();
}

// Brush items: runs of 32 visited vertices of one culled leaf, kRuns per item.
constexpr int kRuns = 4;
__device__ __forceinline__ int lock_groups(const DevMesh& m) {
  return ((m.max_leaf_verts + 31) / 32 + kRuns - 1) / kRuns;
}

// Brings a vertex's brush inputs (mask, automask, normal) into L1 ahead of
// the brush arithmetic that reads them.
__device__ __forceinline__ void prefetch_l1(const void* p) {
  asm volatile("prefetch.global.L1 [%0];" ::"l"(p));
}
__device__ __forceinline__ void lock_prefetch(const DevMesh& m, int v, bool normal) {
  if (m.mask) prefetch_l1(&m.mask[v]);
  if (m.automask) prefetch_l1(&m.automask[v]);
  if (normal) prefetch_l1(&m.no[v]);
}

// FACES: the item's moved vertices join the dab's normal update once each
// (vert_bitmap): all exchanges issued together, then one list append for the
// warp.
__device__ __forceinline__ void lock_tag(const DevMesh& m, const int* vv, const bool* tag,
                                         int* tag_cnt) {
  const int lane = threadIdx.x & 31;
  unsigned int old[kRuns], bal[kRuns];
#pragma unroll
  for (int u = 0; u < kRuns; u++) old[u] = tag[u] ? atomicExch(&m.vtag[vv[u]], 1u) : 1u;
  int total = 0;
#pragma unroll
  for (int u = 0; u < kRuns; u++) {
    bal[u] = __ballot_sync(0xffffffffu, old[u] == 0u);
    total += __popc(bal[u]);
  }
  if (total == 0) return;
  int base = 0;
  if (lane == 0) base = atomicAdd(tag_cnt, total);
  base = __shfl_sync(0xffffffffu, base, 0);
  const unsigned int below = (1u << lane) - 1u;
#pragma unroll
  for (int u = 0; u < kRuns; u++) {
    if (old[u] == 0u) m.tag_list[base + __popc(bal[u] & below)] = vv[u];
    base += __popc(bal[u]);
  }
}

// The flush of a dab by the job's home CTA (the parents staged on chip), the
// same two halves as the team kernel's (mark the ancestors, then unite the
// boxes bottom-up).  Runs before the home CTA's next node search of the job,
// the only reader of the boxes in between.
__device__ void lock_flush(const DevMesh& m, int par, int* s_par, unsigned char* s_pass,
                           int* s_list, unsigned short* s_idx, FlushSmem& fs, TeamShared& sh) {
  for (int i = threadIdx.x; i < m.totnode; i += kTeamThreads) s_par[i] = m.node_parent[i];
  __syncthreads();
  const int ntouch = __ldcg(&m.work->touch_count[par]);
  FlushState fst;
  unsigned long long fb = 0;
  team_flush_mark(m, ntouch, m.touch_list, m.leaf_node, s_par, reinterpret_cast<unsigned int*>(s_pass), s_list,
                  s_idx, fs, sh, fst);
  __syncthreads();
  team_flush_levels(m, ntouch, m.touch_list, m.leaf_node, s_par, s_list, s_idx, fs, sh, fst, fb);
}

// Refit of chunks c0 .. c0+n-1 (n <= kRuns) of a leaf by one warp: every
// position load issued first, then each chunk's box reduced exactly as
// chunk_refit_warp does (lane pairs, then the xor tree) and stored.
__device__ void lock_refit_chunks(const DevMesh& m, int leaf, int c0, int n) {
  const int lane = threadIdx.x & 31;
  const int nv = leaf_nverts_all(m, leaf);
  int v0[kRuns], v1[kRuns];
  float4 p0[kRuns], p1[kRuns];
#pragma unroll
  for (int u = 0; u < kRuns; u++) {
    const int c = c0 + u;
    const int i0 = c * kChunk + lane, i1 = i0 + 32;
    const int e = min(nv, (c + 1) * kChunk);
    v0[u] = (u < n && i0 < e) ? leaf_vert_all(m, leaf, i0) : -1;
    v1[u] = (u < n && i1 < e) ? leaf_vert_all(m, leaf, i1) : -1;
  }
#pragma unroll
  for (int u = 0; u < kRuns; u++) {
    p0[u] = v0[u] >= 0 ? __ldcg(&m.co[v0[u]]) : make_float4(FLT_MAX, FLT_MAX, FLT_MAX, 0.0f);
    p1[u] = v1[u] >= 0 ? __ldcg(&m.co[v1[u]]) : p0[u];
  }
#pragma unroll
  for (int u = 0; u < kRuns; u++) {
    if (u >= n) break;  // warp-uniform
    const float a[3] = {p0[u].x, p0[u].y, p0[u].z}, b[3] = {p1[u].x, p1[u].y, p1[u].z};
    float mn[3], mx[3];
    for (int k = 0; k < 3; k++) {
      mn[k] = v0[u] >= 0 ? ((a[k] < b[k]) ? a[k] : b[k]) : FLT_MAX;
      mx[k] = v0[u] >= 0 ? ((a[k] > b[k]) ? a[k] : b[k]) : -FLT_MAX;
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
      const int id = m.leaf_chunk_off[leaf] + c0 + u;
      m.chunk_box[2 * id] = make_float4(mn[0], mn[1], mn[2], 0.0f);
      m.chunk_box[2 * id + 1] = make_float4(mx[0], mx[1], mx[2], 0.0f);
    }
  }
}

__device__ __forceinline__ PassParams pass_params(const TeamJob& jb, const DevBrush& b, int d,
                                                  int pass, int tool) {
  PassParams pp;
  for (int k = 0; k < 3; k++) {
    const float sgn = (pass & (1 << k)) ? -1.0f : 1.0f;
    pp.loc[k] = sgn * jb.dabs[6 * d + k];
    pp.delta[k] = sgn * jb.dabs[6 * d + 3 + k];
    pp.view[k] = sgn * jb.view[k];
  }
  const float r = b.radius * ((tool == kToolClayStrips) ? 1.41421356237309504880f : 1.0f);
  pp.cull_radius_sq = r * r;
  pp.original = jb.use_orig;
  pp.iter_strength = 1.0f;
  pp.iteration = 0;
  return pp;
}

}  // namespace

// Two builds: one CTA per SM (255 registers per thread) or two (128: twice
// the warps in flight for the latency-bound item loops).
template <int kMinBlocks>
__global__ void __launch_bounds__(kTeamThreads, kMinBlocks) k_lock_stroke(TeamArgs a) {
  const unsigned C = gridDim.x, rank = blockIdx.x;
  constexpr int kWarps = kTeamThreads / 32;
  const int lane = threadIdx.x & 31;
  // warps and threads interleaved over the CTAs (item b goes to CTA b % C)
  const int gw = (threadIdx.x >> 5) * static_cast<int>(C) + static_cast<int>(rank);
  const int GW = kWarps * static_cast<int>(C);
  const int gt = 32 * gw + lane;
  const int GT = static_cast<int>(C) * kTeamThreads;
  const int J = a.njobs;
  __shared__ TeamShared sh;
  union Scratch {
    Lane lanes[kTeamThreads];
    FlushSmem flush;
  };
  __shared__ Scratch s_scr;
  __shared__ Lane s_chunks[kTeamMaxChunks];
  __shared__ int s_flags[8];
  extern __shared__ __align__(16) unsigned char dyn[];
  const LockLayout lay(a.max_nodes, a.max_leaves);
  float4* s_stage = reinterpret_cast<float4*>(dyn);
  int* s_P = reinterpret_cast<int*>(dyn + lay.P);
  unsigned int* s_ep0 = reinterpret_cast<unsigned int*>(dyn + lay.ep0);
  signed char* s_tool = reinterpret_cast<signed char*>(dyn + lay.tool);
  unsigned char* s_sym = dyn + lay.sym;
  unsigned char* s_q = dyn + lay.q;
  int* s_cl = reinterpret_cast<int*>(dyn + lay.cl);
  int* s_coff = reinterpret_cast<int*>(dyn + lay.coff);
  unsigned short* s_idx = reinterpret_cast<unsigned short*>(dyn + lay.idx);
  int* s_par = reinterpret_cast<int*>(dyn + lay.par);
  unsigned char* s_pass = dyn + lay.pass;
  PhaseClock clk;
  clk.last = a.phase_ns ? global_ns() : 0ull;
  TeamBarrier<true> bar{C, a.bar, 0u, a.wait_ns, a.status, &sh.bar_ok,
                        static_cast<unsigned int>(a.bar_extra)};
  // (phase marks before a barrier time the phase's work in CTA 0; the wait
  // at the barrier goes to the job bucket)
#define LOCK_SYNC()                \
  do {                             \
    if (!bar.sync()) return;       \
    clk.mark(a, rank, kPhJob);     \
  } while (0)

  auto mesh_of = [&](int j) -> const DevMesh& { return a.meshes[a.jobs[j].mesh]; };
  auto find_job = [&](int i) { return smem_find_slot(s_P, J, i); };

  // ---- set-up: per-job tables, the longest stroke, each job's start
  if (threadIdx.x == 0) s_flags[0] = 0;
  for (int i = threadIdx.x; i < a.max_nodes; i += kTeamThreads) s_idx[i] = kNoPos;
  __syncthreads();
  for (int j = threadIdx.x; j < J; j += kTeamThreads) {
    const TeamJob& jb = a.jobs[j];
    s_ep0[j] = __ldcg(&mesh_of(j).work->grid_epoch);
    s_sym[j] = static_cast<unsigned char>(jb.symmetry & 7);
    s_q[j] = 0;
    atomicMax(&s_flags[0], jb.ndabs);
  }
  __syncthreads();
  const int maxd = s_flags[0];
  for (int j = static_cast<int>(rank); j < J; j += static_cast<int>(C)) {
    const DevMesh& m = mesh_of(j);
    Work* w = m.work;
    if (threadIdx.x == 0) {
      for (int k = 0; k < 3; k++) w->hit_count[k] = 0;
      w->tag_count[0] = w->tag_count[1] = 0;
      w->touch_count[0] = w->touch_count[1] = 0;
      if (m.type == kGrids) m.grid_counts[0] = m.grid_counts[1] = m.grid_counts[2] = m.grid_counts[3] = 0;
    }
    __syncthreads();
    // leaves flagged and vertices tagged before the stroke join the first
    // dab's update, as in the team kernel
    for (int leaf = threadIdx.x; leaf < m.nleaf; leaf += kTeamThreads) {
      const int f = __ldcg(&m.leaf_flag[leaf]);
      if (!(f & (kUpdateNormals | kUpdateBB))) continue;
      append(m.touch_list, &w->touch_count[0], leaf);
      if (m.type == kGrids)
        for (int k = m.leaf_prim_off[leaf]; k < m.leaf_prim_off[leaf + 1]; k++)
          grid_claim_face_only(m, m.leaf_prims[k], s_ep0[j] + 1u);
      if ((f & kUpdateNormals) && m.type == kFaces) {
        const int off = m.leaf_vert_off[leaf];
        for (int i = 0; i < m.leaf_uniq[leaf]; i++) {
          const int v = m.leaf_verts[off + i];
          if (__ldcg(&m.vtag[v])) m.tag_list[atomicAdd(&w->tag_count[0], 1)] = v;
        }
      }
    }
    __syncthreads();
  }
  clk.mark(a, rank, kPhJob);
  LOCK_SYNC();

  for (int d = 0; d < maxd; d++) {
    const int par = d & 1;
    for (int j = threadIdx.x; j < J; j += kTeamThreads) {
      const TeamJob& jb = a.jobs[j];
      s_tool[j] = static_cast<signed char>(d < jb.ndabs ? (jb.tools ? jb.tools[d] : jb.brush.tool) : -1);
    }
    __syncthreads();
    // ---- dab start, by each job's home CTA (rank j % C): the previous dab's
    // flush and flags, this dab's counters reset, the dab's tool set;
    // strokes that ended with the previous dab finish
    for (int j = static_cast<int>(rank); j < J; j += static_cast<int>(C)) {
      const TeamJob& jb = a.jobs[j];
      const DevMesh& m = mesh_of(j);
      if (d > jb.ndabs) continue;
      if (d > 0) {
        lock_flush(m, par ^ 1, s_par, s_pass, s_coff, s_idx, s_scr.flush, sh);
        lock_clear_touched(m, par ^ 1);
      }
      if (d == jb.ndabs) {
        __syncthreads();
        lock_finish_job(m, jb, s_ep0[j], s_pass);
        continue;
      }
      __syncthreads();
      if (threadIdx.x == 0) {
        m.work->tag_count[par ^ 1] = 0;
        m.work->touch_count[par ^ 1] = 0;
        a.lbrush[j].tool = s_tool[j];
      }
      __syncthreads();
    }
    clk.mark(a, rank, kPhFlush);
    auto active = [&](int j, int pass) { return s_tool[j] >= 0 && (pass & ~s_sym[j]) == 0; };

    for (int pass = 0; pass < 8; pass++) {
      // which phases this pass has (the same in every CTA); the first barrier
      // ends the reads of the previous pass's flags
      __syncthreads();
      if (threadIdx.x == 0) s_flags[1] = 0;
      __syncthreads();
      int f_any = 0, f_area = 0, f_smooth = 0, f_zero = 0;
      for (int j = threadIdx.x; j < J; j += kTeamThreads) {
        if (!active(j, pass)) continue;
        f_any = 1;
        const int tool = s_tool[j];
        if (uses_area(tool)) f_area = 1;
        if (tool == kToolSmooth) {
          f_smooth = 1;
          float last;
          const int c = smooth_count(a.jobs[j].brush.strength, &last);
          if (c == 0) f_zero = 1;
          atomicMax(&s_flags[1], c);
        }
      }
      const bool any = __syncthreads_or(f_any);
      const bool any_area = __syncthreads_or(f_area);
      const bool any_smooth = __syncthreads_or(f_smooth);
      const bool any_zero = __syncthreads_or(f_zero);
      const int max_count = s_flags[1];
      if (!any) continue;

      // ---- cull, one CTA per job; brushes without an area normal mark here
      for (int j = static_cast<int>(rank); j < J; j += static_cast<int>(C)) {
        if (!active(j, pass)) continue;
        const TeamJob& jb = a.jobs[j];
        const DevMesh& m = mesh_of(j);
        const DevBrush& b = a.lbrush[j];
        LockJob& L = a.lock[j];
        const int tool = s_tool[j];
        const PassParams pp = pass_params(jb, b, d, pass, tool);
        const LockTabs tabs{{m.leaf_node}, {&m}};
        team_cull<8, kMinBlocks == 1>(m, pp, s_pass, s_cl, s_coff, tabs, sh);
        const int cnt = sh.cnt, total = sh.total;
        for (int k = threadIdx.x; k < cnt; k += kTeamThreads) {
          m.cull_list[k] = s_cl[k];
          m.cull_off[k] = s_coff[k];
        }
        bool go = false;
        BrushFrame f;
        if (cnt > 0 && !uses_area(tool)) {
          const float zero[3] = {0.0f, 0.0f, 0.0f};
          go = make_frame(b, pp, zero, zero, f);
          if (go) lock_mark(m, s_cl, cnt, &m.work->touch_count[par], s_ep0[j] + d + 1u);
        }
        if (tool == kToolSmooth && threadIdx.x == 0) {
          // the counter of the job's next smooth pass (last used two smooth
          // passes ago, cleared since)
          L.nh[(s_q[j] + 1) % 3] = 0;
        }
        if (threadIdx.x == 0) {
          m.cull_off[cnt] = total;
          L.pp = pp;
          L.cnt = cnt;
          L.total = total;
          L.ticket = 0u;
          if (go) L.frame = f;
          L.go = go ? 1 : 0;
        }
        __syncthreads();  // the CTA's tables serve its next job
      }
      clk.mark(a, rank, kPhCull);
      LOCK_SYNC();

      // ---- area normal and centre: (job, leaf, block) items, one per CTA
      if (any_area) {
        const int NA = lock_prefix(J, s_P, sh.scan, [&](int j) {
          if (!active(j, pass) || !uses_area(s_tool[j])) return 0;
          return __ldcg(&a.lock[j].cnt) * mesh_of(j).area_blocks;
        });
        for (int it = static_cast<int>(rank); it < NA; it += static_cast<int>(C)) {
          const int j = find_job(it);
          const int k = it - s_P[j];
          const int nitems = s_P[j + 1] - s_P[j];
          const DevMesh& m = mesh_of(j);
          const DevBrush& b = a.lbrush[j];
          LockJob& L = a.lock[j];
          const PassParams pp = L.pp;
          const int nb = m.area_blocks;
          const float rn = b.radius * b.normal_radius_factor;
          const float ra = b.radius * b.area_radius_factor;
          team_area_block(m, pp.loc, rn * rn, ra * ra, __ldcg(&m.cull_list[k / nb]), k % nb, s_stage,
                          s_scr.lanes, &m.parts[k]);
          if (threadIdx.x == 0) {
            __threadfence();
            sh.nmark = (atomicAdd(&L.ticket, 1u) + 1u == static_cast<unsigned int>(nitems)) ? 1 : 0;
            if (sh.nmark) __threadfence();
          }
          __syncthreads();
          if (sh.nmark) {
            // the job's last item: reduce, frame, mark
            team_area_final(m, pp, nitems, s_scr.lanes, s_chunks, sh);
            BrushFrame f;
            const bool go = make_frame(b, pp, sh.area, sh.area + 3, f);
            if (go)
              lock_mark(m, m.cull_list, __ldcg(&L.cnt), &m.work->touch_count[par],
                        s_ep0[j] + d + 1u);
            if (threadIdx.x == 0) {
              if (go) L.frame = f;
              L.go = go ? 1 : 0;
            }
          }
          __syncthreads();
        }
        clk.mark(a, rank, kPhArea);
        LOCK_SYNC();
      }

      // ---- brush: (job, leaf, kRuns runs of 32 visited vertices) items, one
      // per warp; the runs' positions are loaded together and their
      // per-vertex inputs prefetched, so one item's latency covers kRuns runs
      {
        const int NB = lock_prefix(J, s_P, sh.scan, [&](int j) {
          if (!active(j, pass) || !__ldcg(&a.lock[j].go)) return 0;
          return __ldcg(&a.lock[j].cnt) * lock_groups(mesh_of(j));
        });
        int cj = -1;
        PassParams pp;
        BrushFrame f;
        float rr = 0.0f;
        bool inflate = false;
        for (int it = gw; it < NB; it += GW) {
          const int j = find_job(it);
          const DevMesh& m = mesh_of(j);
          const DevBrush& b = a.lbrush[j];
          const int tool = s_tool[j];
          if (j != cj) {
            cj = j;
            pp = a.lock[j].pp;
            inflate = tool == kToolInflate || (b.flag & kBrushFrontFace);
            if (tool == kToolSmooth) {
              float last;
              pp.iter_strength = smooth_count(b.strength, &last) != 0 ? 1.0f : last;
              rr = b.radius * b.radius;
            } else {
              f = a.lock[j].frame;
            }
          }
          const int G = lock_groups(m);
          const int k = it - s_P[j];
          const int slot = k / G, grp = k - slot * G;
          const int leaf = __ldcg(&m.cull_list[slot]);
          const int nv = __ldcg(&m.cull_off[slot + 1]) - __ldcg(&m.cull_off[slot]);
          const int base = grp * kRuns * 32;
          if (base >= nv) continue;  // padding (warp-uniform)
          int vv[kRuns];
          float4 cc[kRuns];
#pragma unroll
          for (int u = 0; u < kRuns; u++) {
            const int i = base + u * 32 + lane;
            vv[u] = i < nv ? leaf_vert(m, leaf, i) : -1;
          }
#pragma unroll
          for (int u = 0; u < kRuns; u++)
            if (vv[u] >= 0) cc[u] = __ldcg(&m.co[vv[u]]);
#pragma unroll
          for (int u = 0; u < kRuns; u++)
            if (vv[u] >= 0) lock_prefetch(m, vv[u], inflate);
          bool tag[kRuns];
          unsigned int moved_n = 0u;
          if (tool != kToolSmooth) {
#pragma unroll
            for (int u = 0; u < kRuns; u++) {
              bool moved = false;
              tag[u] = false;
              if (vv[u] >= 0 && brush_vertex(m, b, b.y, pp, f, vv[u], cc[u], moved)) {
                m.co[vv[u]] = cc[u];
                tag[u] = true;
              }
              moved_n += __popc(__ballot_sync(0xffffffffu, moved));
            }
          } else {
            // the sphere test, slots from the job's hit counter (one add per
            // item), and the first Jacobi sweep into the slots (positions are
            // not written until the sweeps are done)
            const int q = s_q[j];
            int* const smap = m.slot_map[q & 1];
            unsigned int bl[kRuns];
            int tot = 0;
#pragma unroll
            for (int u = 0; u < kRuns; u++) {
              tag[u] = vv[u] >= 0 && dist_sq(cc[u], pp.loc) <= rr;
              bl[u] = __ballot_sync(0xffffffffu, tag[u]);
              tot += __popc(bl[u]);
            }
            int hb = 0;
            if (lane == 0 && tot > 0) hb = atomicAdd(&a.lock[j].nh[q % 3], tot);
            hb = __shfl_sync(0xffffffffu, hb, 0);
            const unsigned int below = (1u << lane) - 1u;
#pragma unroll
            for (int u = 0; u < kRuns; u++) {
              bool moved = false;
              if (tag[u]) {
                const int h = hb + __popc(bl[u] & below);
                float4 out;
                smooth_vertex(m, b, b.y, pp, vv[u], cc[u], out, moved);
                m.hit_list[0][h] = vv[u];
                m.scratch[h] = out;
                smap[vv[u]] = h;
              }
              hb += __popc(bl[u]);
              moved_n += __popc(__ballot_sync(0xffffffffu, moved));
            }
          }
          if (m.type == kFaces) lock_tag(m, vv, tag, &m.work->tag_count[par]);
          if (lane == 0 && moved_n) atomicAdd(&m.work->displaced, (unsigned long long)moved_n);
        }
        clk.mark(a, rank, kPhBrush);
        LOCK_SYNC();
      }

      // ---- smooth: the later Jacobi sweeps, (job, hit) items, one per thread
      if (any_smooth) {
        auto smooth_job = [&](int j) {
          return active(j, pass) && s_tool[j] == kToolSmooth && __ldcg(&a.lock[j].go);
        };
        auto hits = [&](int j) { return __ldcg(&a.lock[j].nh[s_q[j] % 3]); };
        if (any_zero) {
          // strength below a quarter: the first sweep is the result
          const int NH = lock_prefix(J, s_P, sh.scan, [&](int j) {
            if (!smooth_job(j)) return 0;
            float last;
            return smooth_count(a.lbrush[j].strength, &last) == 0 ? hits(j) : 0;
          });
          for (int it = gt; it < NH; it += GT) {
            const int j = find_job(it);
            const DevMesh& m = mesh_of(j);
            const int h = it - s_P[j];
            m.co[__ldcg(&m.hit_list[0][h])] = __ldcg(&m.scratch[h]);
          }
          clk.mark(a, rank, kPhApply);
          LOCK_SYNC();
        }
        for (int sweep = 1; sweep <= max_count; sweep++) {
          const int NH = lock_prefix(J, s_P, sh.scan, [&](int j) {
            if (!smooth_job(j)) return 0;
            float last;
            return sweep <= smooth_count(a.lbrush[j].strength, &last) ? hits(j) : 0;
          });
          int cj = -1;
          PassParams pp;
          int count = 0;
          for (int it = gt; it < NH; it += GT) {
            const int j = find_job(it);
            const DevMesh& m = mesh_of(j);
            const DevBrush& b = a.lbrush[j];
            if (j != cj) {
              cj = j;
              pp = a.lock[j].pp;
              float last;
              count = smooth_count(b.strength, &last);
              pp.iter_strength = (sweep != count) ? 1.0f : last;
              pp.iteration = sweep;
            }
            const int h = it - s_P[j];
            const float4* vsrc = ((sweep - 1) & 1) ? m.scratch2 : m.scratch;
            float4* vdst = (sweep & 1) ? m.scratch2 : m.scratch;
            const int v = __ldcg(&m.hit_list[0][h]);
            const float4 out =
                smooth_slot(m, b, pp, v, __ldcg(&vsrc[h]), vsrc, m.slot_map[s_q[j] & 1]);
            if (sweep == count) {
              m.co[v] = out;
            } else {
              vdst[h] = out;
            }
          }
          clk.mark(a, rank, kPhApply);
          LOCK_SYNC();
        }
        // the pass's map entries clear; the map is next filled two smooth
        // passes of the job later, after more barriers
        const int NH = lock_prefix(J, s_P, sh.scan, [&](int j) { return smooth_job(j) ? hits(j) : 0; });
        for (int it = gt; it < NH; it += GT) {
          const int j = find_job(it);
          const DevMesh& m = mesh_of(j);
          m.slot_map[s_q[j] & 1][__ldcg(&m.hit_list[0][it - s_P[j]])] = -1;
        }
        __syncthreads();
        for (int j = threadIdx.x; j < J; j += kTeamThreads)
          if (active(j, pass) && s_tool[j] == kToolSmooth) s_q[j] = static_cast<unsigned char>((s_q[j] + 1) % 6);
        __syncthreads();
      }
    }

    // ---- end of the dab
    auto in_dab = [&](int j) { return s_tool[j] >= 0; };
    int f_grids = 0;
    for (int j = threadIdx.x; j < J; j += kTeamThreads)
      if (in_dab(j) && mesh_of(j).type == kGrids) f_grids = 1;
    if (__syncthreads_or(f_grids)) {
      // GRIDS: the claimed faces, one per CTA; then their base edges and corners
      const int NF = lock_prefix(J, s_P, sh.scan, [&](int j) {
        return in_dab(j) && mesh_of(j).type == kGrids ? __ldcg(&mesh_of(j).grid_counts[0]) : 0;
      });
      int pre_it = -1;  // the face whose boundary item tables the stage holds
      for (int it = static_cast<int>(rank); it < NF; it += static_cast<int>(C)) {
        const int j = find_job(it);
        const DevMesh& m = mesh_of(j);
        const int2 fs = __ldcg(&m.face_info[it - s_P[j]]);
        pre_it = team_grid_face<true, true>(m, __ldcg(&m.face_list[it - s_P[j]]), fs.x, fs.y, dyn,
                                            face_grid_group(m.grid_size, kStageBytes),
                                            s_ep0[j] + d + 1u)
                     ? it
                     : -1;
      }
      clk.mark(a, rank, kPhGridFaces);
      LOCK_SYNC();
      for (int it = static_cast<int>(rank); it < NF; it += static_cast<int>(C)) {
        const int j = find_job(it);
        const DevMesh& m = mesh_of(j);
        const int2 fs = __ldcg(&m.face_info[it - s_P[j]]);
        team_grid_face_boundary(
            m, __ldcg(&m.face_list[it - s_P[j]]), fs.x, fs.y, s_ep0[j] + d + 1u, true,
            it == pre_it
                ? dyn + boundary_prefetch_offset(m.grid_size, face_grid_group(m.grid_size, kStageBytes))
                : nullptr);
      }
      clk.mark(a, rank, kPhGridSeams);
      LOCK_SYNC();
    }
    // refit ((job, touched leaf, kRuns chunks) items, one per warp) and
    // FACES normals ((job, tagged vertex) items, one per thread): both only
    // read positions; the flush follows at the next dab start
    {
      const int NR = lock_prefix(J, s_P, sh.scan, [&](int j) {
        if (!in_dab(j)) return 0;
        const DevMesh& m = mesh_of(j);
        return __ldcg(&m.work->touch_count[par]) * ((m.max_leaf_chunks + kRuns - 1) / kRuns);
      });
      for (int it = gw; it < NR; it += GW) {
        const int j = find_job(it);
        const DevMesh& m = mesh_of(j);
        const int G = (m.max_leaf_chunks + kRuns - 1) / kRuns;
        const int k = it - s_P[j];
        const int slot = k / G, c0 = (k - slot * G) * kRuns;
        const int leaf = __ldcg(&m.touch_list[slot]);
        const int nch = m.leaf_chunk_off[leaf + 1] - m.leaf_chunk_off[leaf];
        if (c0 >= nch) continue;  // padding (warp-uniform)
        lock_refit_chunks(m, leaf, c0, min(kRuns, nch - c0));
      }
      clk.mark(a, rank, kPhUpdate);
      const int NT = lock_prefix(J, s_P, sh.scan, [&](int j) {
        if (!in_dab(j)) return 0;
        const DevMesh& m = mesh_of(j);
        return m.type == kFaces ? __ldcg(&m.work->tag_count[par]) : 0;
      });
      for (int it = gt; it < NT; it += GT) {
        const int j = find_job(it);
        const DevMesh& m = mesh_of(j);
        const int v = __ldcg(&m.tag_list[it - s_P[j]]);
        float4 n;
        vertex_normal(m, v, n);
        m.no[v] = n;
        m.vtag[v] = 0u;
      }
      // the GRIDS work lists of the dab are consumed
      for (int j = static_cast<int>(rank); j < J; j += static_cast<int>(C)) {
        const DevMesh& m = mesh_of(j);
        if (in_dab(j) && m.type == kGrids && threadIdx.x == 0)
          m.grid_counts[0] = m.grid_counts[1] = m.grid_counts[2] = m.grid_counts[3] = 0;
      }
      clk.mark(a, rank, kPhUpdate);
      LOCK_SYNC();
    }
  }
  // strokes that end with the batch's last dab: its flush, then the end
  for (int j = static_cast<int>(rank); j < J; j += static_cast<int>(C)) {
    const TeamJob& jb = a.jobs[j];
    if (jb.ndabs != maxd) continue;
    const DevMesh& m = mesh_of(j);
    if (maxd > 0) {
      lock_flush(m, (maxd - 1) & 1, s_par, s_pass, s_coff, s_idx, s_scr.flush, sh);
      lock_clear_touched(m, (maxd - 1) & 1);
      __syncthreads();
    }
    lock_finish_job(m, jb, s_ep0[j], s_pass);
  }
  clk.mark(a, rank, kPhFlush);
}
#undef LOCK_SYNC

bool lock_grids_fit(int grid_size) { return face_grid_group(grid_size, kStageBytes) > 0; }

size_t lock_smem_bytes(int max_nodes, int max_leaves) {
  return LockLayout(max_nodes, max_leaves).total;
}

int lock_ctas(int max_nodes, int max_leaves, int per_sm) {
  static std::mutex mu;
  static std::map<std::tuple<int, size_t, int>, int> cache;
  static std::map<int, size_t> configured;  // per device: largest smem set so far
  if (per_sm != 1 && per_sm != 2) return 0;
  const size_t smem = lock_smem_bytes(max_nodes, max_leaves);
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  std::lock_guard<std::mutex> lock(mu);
  const auto key = std::make_tuple(dev, smem, per_sm);
  auto it = cache.find(key);
  if (it != cache.end() && configured[dev] >= smem) return it->second;
  int coop = 0, sms = 0;
  if (cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev) != cudaSuccess || !coop)
    return 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
  const size_t want = std::max(smem, configured[dev]);
  if (cudaFuncSetAttribute(k_lock_stroke<1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           static_cast<int>(want)) != cudaSuccess ||
      cudaFuncSetAttribute(k_lock_stroke<2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           static_cast<int>(want)) != cudaSuccess)
    return 0;
  configured[dev] = want;
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(
          &n, per_sm == 1 ? k_lock_stroke<1> : k_lock_stroke<2>, kTeamThreads, smem) != cudaSuccess)
    return 0;
  const int ctas = n >= per_sm ? std::min(sms * per_sm, kTeamMaxWideCtas) : 0;
  cache[key] = ctas;
  return ctas;
}

cudaError_t launch_lock_stroke(const TeamArgs& a, int nctas, int per_sm, cudaStream_t s) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(static_cast<unsigned>(nctas));
  cfg.blockDim = dim3(kTeamThreads);
  cfg.dynamicSmemBytes = lock_smem_bytes(a.max_nodes, a.max_leaves);
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return per_sm == 2 ? cudaLaunchKernelEx(&cfg, k_lock_stroke<2>, a)
                     : cudaLaunchKernelEx(&cfg, k_lock_stroke<1>, a);
}

}  // namespace sgpu
