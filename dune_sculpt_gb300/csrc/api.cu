// C ABI of libsculptgpu (include/sculpt_gpu.h): mesh upload and device mirror
// of the PBVH, the per-call entry points that replace the reference's
// BKE_pbvh_* / do_*_brush calls, and whole strokes (eager or CUDA graph).
#include <cuda_runtime.h>

#include <cstdarg>
#include <cstddef>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "../../include/sculpt_gpu.h"
#include "sgpu_device.cuh"
#include "sgpu_draw.h"
#include "sgpu_host.h"
#include "sgpu_kernels.h"
#include "sgpu_ray.h"
#include "sgpu_team.h"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <map>
#include <mutex>
#include <thread>
#include <tuple>

using namespace sgpu;

namespace {

thread_local std::string g_err;

int fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_err = buf;
  return code;
}

int cuda_fail(cudaError_t e, const char* what) {
  if (e == cudaErrorMemoryAllocation)
    return fail(SGPU_ERR_OOM, "%s: %s", what, cudaGetErrorString(e));
  return fail(SGPU_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

#define CK(expr, what)                              \
  do {                                              \
    cudaError_t _e = (expr);                        \
    if (_e != cudaSuccess) return cuda_fail(_e, what); \
  } while (0)
// The same inside a mesh-creation function: frees the partial mesh (bail).
#define CK_BAIL(expr, what)                                   \
  do {                                                        \
    cudaError_t _e = (expr);                                  \
    if (_e != cudaSuccess) return bail(cuda_fail(_e, what));  \
  } while (0)

// Host-side test hooks (sgpu_debug_inject).  g_inject_alloc > 0: the mesh
// allocation that brings it to zero fails as out of memory.  g_wait_ns: the
// whole-GPU team's barrier wait limit.  g_bar_extra: arrivals its barriers
// wait for beyond the launch's CTAs (1 makes every wait run out).
constexpr unsigned long long kDefaultWaitNs = 2000000000ull;
std::atomic<long long> g_inject_alloc{0};
std::atomic<unsigned long long> g_wait_ns{kDefaultWaitNs};
std::atomic<int> g_bar_extra{0};
// Test hook: CTAs per SM of every lockstep launch (0: the team shape's).
std::atomic<int> g_lock_per_sm{0};

bool injected_alloc_failure() {
  long long n = g_inject_alloc.load();
  while (n > 0) {
    if (g_inject_alloc.compare_exchange_weak(n, n - 1)) return n == 1;
  }
  return false;
}

}  // namespace

namespace sgpu {
void set_error_message(const std::string& msg) { g_err = msg; }
}  // namespace sgpu

struct sgpu_mesh {
  HostMesh host;
  DevMesh dev{};
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  cudaEvent_t ev_h0 = nullptr, ev_h1 = nullptr;  // host-buffer path
  std::vector<void*> allocs;
  int* d_nodes_tmp = nullptr;
  bool has_mask = false;
  // FACES device vertex order (see sgpu_mesh_create_faces): caller index ->
  // device index and back; empty / null for GRIDS (element order kept).
  std::vector<int> o2n;
  const int* d_o2n = nullptr;
  const int* d_n2o = nullptr;
  // stroke graph cache
  cudaGraphExec_t gexec = nullptr;
  std::vector<unsigned char> gkey;
  int g_nodes = 0;
  int g_launches = 0;
  // profiling: event pool and (kind, start, end) marks of the current stroke
  bool profiling = false;
  std::vector<cudaEvent_t> ev_pool;
  size_t ev_used = 0;
  struct Mark {
    int kind;
    cudaEvent_t a, b;
  };
  std::vector<Mark> prof_marks;
  // snapshot (per-stroke restore) and L2 flush buffers
  float4* snap_co = nullptr;
  float4* snap_no = nullptr;
  float* snap_mask = nullptr;
  float4* snap_vb = nullptr;
  float4* snap_orig_vb = nullptr;
  int* snap_flag = nullptr;
  void* flush_buf = nullptr;
  // persistent stroke kernel: cluster size and device staging of the job
  int team_cluster = 8;
  int team_build = 0;     // CTAs per SM of the cluster build: 0 auto, 1, 2
  bool team_set = false;  // set by sgpu_mesh_set_team or the autotuner
  int nchunks = 0;  // refit chunks over all leaves
  DevMesh* t_meshes = nullptr;
  TeamJob* t_jobs = nullptr;
  float* t_dabs = nullptr;
  int* t_tools = nullptr;
  int* t_counter = nullptr;
  LockJob* t_lock = nullptr;     // lockstep launch: per-job state
  DevBrush* t_lbrush = nullptr;  // and per-job brushes
  size_t t_dab_cap = 0, t_tool_cap = 0, t_mesh_cap = 0, t_job_cap = 0, t_counter_cap = 0;
  size_t t_lock_cap = 0, t_lbrush_cap = 0;
  float* t_keep = nullptr;  // host-buffer GRIDS stroke: the positions input, kept
  size_t t_keep_cap = 0;
  // page-locked displaced counters of the last persistent launch
  unsigned long long* h_disp = nullptr;
  size_t h_disp_cap = 0;
  // ray-cast batch buffers (grown to the largest batch; see sgpu_raycast):
  // one device block and one page-locked host block with the same layout,
  // 7 floats in per ray (start, direction, length), 4 floats and 3 ints out
  // per ray (depth, face normal; hit, active vertex, active face), then the
  // error word
  RayBatch ray{};
  unsigned char* ray_dev = nullptr;
  unsigned char* ray_host = nullptr;
  size_t ray_cap = 0;
  bool ray_configured = false;
  // the captured call (copies in, kernels, copies out) for (rays, original)
  cudaGraphExec_t ray_graph = nullptr;
  int ray_graph_n = -1, ray_graph_orig = -1, ray_graph_near = -1;
  // stroke-start positions and normals stored (grab, elastic deform)
  bool orig_stored = false;
  // headless draw buffers (sgpu_draw_buffers_build): host layout, device view
  // and its allocations
  DrawLayout draw;
  DrawDev draw_dev{};
  std::vector<void*> draw_allocs;
  bool draw_built = false;

  void free_draw() {
    for (void* p : draw_allocs) cudaFree(p);
    draw_allocs.clear();
    draw_dev = DrawDev{};
    draw = DrawLayout{};
    draw_built = false;
  }

  cudaEvent_t prof_event() {
    if (ev_used == ev_pool.size()) {
      cudaEvent_t e = nullptr;
      if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
      ev_pool.push_back(e);
    }
    return ev_pool[ev_used++];
  }

  template <class T>
  int alloc(T** out, size_t count) {
    void* p = nullptr;
    const size_t bytes = (count > 0 ? count : 1) * sizeof(T);
    if (injected_alloc_failure())
      return fail(SGPU_ERR_OOM, "cudaMalloc: injected allocation failure (test hook)");
    cudaError_t e = cudaMalloc(&p, bytes);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc");
    allocs.push_back(p);
    e = cudaMemsetAsync(p, 0, bytes, stream);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemsetAsync");
    *out = static_cast<T*>(p);
    return SGPU_OK;
  }
  template <class T>
  int upload(const T** out, const std::vector<T>& v) {
    T* p = nullptr;
    int rc = alloc(&p, v.size());
    if (rc) return rc;
    if (!v.empty()) {
      cudaError_t e = cudaMemcpyAsync(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice,
                                      stream);
      if (e != cudaSuccess) return cuda_fail(e, "upload");
    }
    *out = p;
    return SGPU_OK;
  }
  template <class T>
  int upload_to(T* dst, const std::vector<T>& v) {
    cudaError_t e = cudaMemcpyAsync(dst, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice,
                                    stream);
    if (e != cudaSuccess) return cuda_fail(e, "upload");
    e = cudaStreamSynchronize(stream);
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamSynchronize");
    return SGPU_OK;
  }
  template <class T>
  int upload_mut(T** out, const std::vector<T>& v) {
    const T* p = nullptr;
    int rc = upload(&p, v);
    *out = const_cast<T*>(p);
    return rc;
  }
  void release() {
    if (gexec) cudaGraphExecDestroy(gexec);
    gexec = nullptr;
    if (stream) cudaStreamSynchronize(stream);
    for (void* p : allocs) cudaFree(p);
    allocs.clear();
    for (void* p : {static_cast<void*>(t_meshes), static_cast<void*>(t_jobs),
                    static_cast<void*>(t_dabs), static_cast<void*>(t_tools),
                    static_cast<void*>(t_counter), static_cast<void*>(t_lock),
                    static_cast<void*>(t_lbrush), static_cast<void*>(t_keep)})
      if (p) cudaFree(p);
    t_keep = nullptr;
    t_keep_cap = 0;
    t_lock = nullptr;
    t_lbrush = nullptr;
    t_lock_cap = t_lbrush_cap = 0;
    t_meshes = nullptr;
    t_jobs = nullptr;
    t_dabs = nullptr;
    t_tools = nullptr;
    t_counter = nullptr;
    if (h_disp) cudaFreeHost(h_disp);
    h_disp = nullptr;
    h_disp_cap = 0;
    if (ray_graph) cudaGraphExecDestroy(ray_graph);
    ray_graph = nullptr;
    for (void* p : {static_cast<void*>(ray_dev), static_cast<void*>(ray.count),
                    static_cast<void*>(ray.slot_leaf), static_cast<void*>(ray.slot_tmin),
                    static_cast<void*>(ray.slot_order), static_cast<void*>(ray.slot_key),
                    static_cast<void*>(ray.items), static_cast<void*>(ray.nitems),
                    static_cast<void*>(ray.slot_special), static_cast<void*>(ray.items2),
                    static_cast<void*>(ray.nitems2), static_cast<void*>(ray.st_depth),
                    static_cast<void*>(ray.st_run), static_cast<void*>(ray.st_win)})
      if (p) cudaFree(p);
    if (ray_host) cudaFreeHost(ray_host);
    free_draw();
    ray = RayBatch{};
    ray_dev = ray_host = nullptr;
    ray_cap = 0;
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
    if (ev_h0) cudaEventDestroy(ev_h0);
    if (ev_h1) cudaEventDestroy(ev_h1);
    for (cudaEvent_t e : ev_pool) cudaEventDestroy(e);
    ev_pool.clear();
    if (stream) cudaStreamDestroy(stream);
    stream = nullptr;
  }
};

namespace {

bool g_configured = false;

int ensure_device() {
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0)
    return fail(SGPU_ERR_CUDA, "no CUDA device available (%s)", cudaGetErrorString(e));
  if (!g_configured) {
    configure_kernels();
    configure_grid_kernels();
    g_configured = true;
  }
  return SGPU_OK;
}

// Mirrors the host PBVH and work areas to the device.
int upload_pbvh(sgpu_mesh* m) {
  HostMesh& h = m->host;
  DevMesh& d = m->dev;
  const int N = h.totnode, L = static_cast<int>(h.leaf_nodes.size());
  d.totnode = N;
  d.nleaf = L;
  d.max_leaf_verts = d.max_leaf_chunks = 0;
  d.nlevels = static_cast<int>(h.level_off.size()) - 1;
  std::vector<float4> vb(2 * static_cast<size_t>(N));
  for (int n = 0; n < N; n++) {
    const float* b = &h.vb[6 * static_cast<size_t>(n)];
    vb[2 * n] = make_float4(b[0], b[1], b[2], 0.0f);
    vb[2 * n + 1] = make_float4(b[3], b[4], b[5], 0.0f);
  }
  int rc;
  if ((rc = m->upload_mut(&d.vb, vb))) return rc;
  if ((rc = m->upload_mut(&d.orig_vb, vb))) return rc;
  if ((rc = m->upload(&d.node_child, h.children))) return rc;
  if ((rc = m->upload(&d.node_parent, h.parent))) return rc;
  if ((rc = m->upload(&d.node_leaf, h.node_leaf))) return rc;
  if ((rc = m->upload(&d.leaf_node, h.leaf_nodes))) return rc;
  std::vector<int> vert_off(L + 1, 0), uniq(L, 0), ubase(L, 0), verts, prim_off(L + 1, 0), prims,
      lflag(L);
  int unext = 0;
  for (int k = 0; k < L; k++) {
    const int node = h.leaf_nodes[k];
    lflag[k] = h.flag[node];
    prim_off[k + 1] = prim_off[k] + h.totprim[node];
    for (int i = 0; i < h.totprim[node]; i++) prims.push_back(h.prim_indices[h.prim_off[node] + i]);
    if (h.type == kFaces) {
      const int tot = h.uniq[node] + h.face_verts_n[node];
      uniq[k] = h.uniq[node];
      ubase[k] = unext;
      vert_off[k + 1] = vert_off[k] + tot;
      for (int i = 0; i < tot; i++) {
        const int v = m->o2n[h.vert_indices[h.vert_off[node] + i]];
        // the unique vertices of the leaf are consecutive in device order
        if (i < h.uniq[node] && v != unext + i)
          return fail(SGPU_ERR_INVALID_ARG, "leaf %d owns vertex %d twice", k, v);
        verts.push_back(v);
      }
      unext += h.uniq[node];
    }
  }
  // FACES: leaves joined by a mesh edge (a one-ring neighbour owned by
  // another leaf); the smooth brush's two mirror passes commute when no leaf
  // of one is joined to a leaf of the other
  std::vector<int> adj_off(L + 1, 0), adj;
  if (h.type == kFaces && h.nb_off.size() > 1) {
    const int V = static_cast<int>(h.nb_off.size()) - 1;
    std::vector<int> vleaf(V, -1);
    for (int k = 0; k < L; k++)
      for (int i = 0; i < uniq[k]; i++) vleaf[ubase[k] + i] = k;
    std::vector<std::vector<int>> sets(L);
    for (int v = 0; v < V; v++) {
      const int lv = vleaf[m->o2n[v]];
      if (lv < 0) continue;
      for (int q = h.nb_off[v]; q < h.nb_off[v + 1]; q++) {
        const int lu = vleaf[m->o2n[h.nb_idx[q]]];
        if (lu >= 0 && lu != lv) sets[lv].push_back(lu);
      }
    }
    for (int k = 0; k < L; k++) {
      std::sort(sets[k].begin(), sets[k].end());
      sets[k].erase(std::unique(sets[k].begin(), sets[k].end()), sets[k].end());
      adj_off[k + 1] = adj_off[k] + static_cast<int>(sets[k].size());
      adj.insert(adj.end(), sets[k].begin(), sets[k].end());
    }
  }
  if ((rc = m->upload(&d.leaf_adj_off, adj_off))) return rc;
  if ((rc = m->upload(&d.leaf_adj, adj))) return rc;
  if ((rc = m->upload(&d.leaf_vert_off, vert_off))) return rc;
  if ((rc = m->upload(&d.leaf_uniq, uniq))) return rc;
  if ((rc = m->upload(&d.leaf_ubase, ubase))) return rc;
  if ((rc = m->upload(&d.leaf_verts, verts))) return rc;
  if ((rc = m->upload(&d.leaf_prim_off, prim_off))) return rc;
  if ((rc = m->upload(&d.leaf_prims, prims))) return rc;
  if ((rc = m->upload_mut(&d.leaf_flag, lflag))) return rc;
  if ((rc = m->upload(&d.level_off, h.level_off))) return rc;
  if ((rc = m->upload(&d.level_nodes, h.level_nodes))) return rc;
  if ((rc = m->upload(&d.node_leaf_lo, h.leaf_lo))) return rc;
  if ((rc = m->upload(&d.node_leaf_hi, h.leaf_hi))) return rc;
  if ((rc = m->upload(&d.node_depth, h.depth))) return rc;
  {
    // two-level node search: nodes of depth <= split, and the descendant
    // range of each internal node at the split depth; without contiguous
    // ranges every node goes in the first level
    std::vector<int> dlo(N, -1), dhi(N, -1), size(N, 1);
    for (int n = N - 1; n >= 0; n--) {
      const int c = h.children[n];
      if (c < 0) continue;
      size[n] = 1 + size[c] + size[c + 1];
      dlo[n] = c;
      dhi[n] = std::max(std::max(c + 2, dhi[c]), dhi[c + 1]);
    }
    bool contiguous = true;
    for (int n = 0; n < N; n++)
      if (h.children[n] >= 0 && dhi[n] - dlo[n] != size[n] - 1) contiguous = false;
    // up to 4096 nodes (two rounds of batched box loads) the one-level
    // search over every node is as short: no first-level list then
    const int split = contiguous ? std::min(h.max_depth, 6) : h.max_depth;
    const bool two_level = contiguous && N > 4096;
    std::vector<int4> top;
    for (int n = 0; n < N; n++) {
      if (h.depth[n] > split) continue;
      const bool ranged = h.depth[n] == split && h.children[n] >= 0;
      top.push_back(make_int4(n, ranged ? dlo[n] : -1, ranged ? dhi[n] : -1, 0));
    }
    const bool fits = top.size() <= static_cast<size_t>(kCullTopMax);
    if (!two_level || !fits) top.assign(1, make_int4(0, -1, -1, 0));
    d.cull_ntop = two_level && fits ? static_cast<int>(top.size()) : 0;
    if ((rc = m->upload(&d.cull_top, top))) return rc;
  }
  d.max_depth = h.max_depth;
  if (h.max_depth >= 256)
    return fail(SGPU_ERR_UNSUPPORTED, "PBVH depth %d above 255", h.max_depth);
  {
    std::vector<int> choff(L + 1, 0);
    for (int k = 0; k < L; k++) {
      const int node = h.leaf_nodes[k];
      const int nall = h.type == kFaces ? h.uniq[node] + h.face_verts_n[node]
                                        : h.totprim[node] * h.grid_area;
      choff[k + 1] = choff[k] + (nall + kChunk - 1) / kChunk;
      d.max_leaf_chunks = std::max(d.max_leaf_chunks, choff[k + 1] - choff[k]);
    }
    if ((rc = m->upload(&d.leaf_chunk_off, choff))) return rc;
    if ((rc = m->alloc(&d.chunk_box, 2 * static_cast<size_t>(choff[L]) + 2))) return rc;
    m->nchunks = choff[L];
  }
  // smooth slot arrays: the persistent kernel's per-CTA slot ranges may end
  // up to 32 entries per CTA of the team past the vertex count
  const size_t nslot = static_cast<size_t>(h.totvert) + 32 * static_cast<size_t>(kTeamMaxWideCtas);
  if ((rc = m->alloc(&d.hit_list[0], nslot))) return rc;
  if ((rc = m->alloc(&d.hit_list[1], static_cast<size_t>(h.totvert)))) return rc;
  if ((rc = m->alloc(&d.tag_list, static_cast<size_t>(h.totvert)))) return rc;
  // a leaf flagged before a stroke (update pending) is listed at the stroke
  // start and may be listed again when the first dab marks it
  if ((rc = m->alloc(&d.touch_list, 2 * static_cast<size_t>(L) + 2))) return rc;
  if ((rc = m->alloc(&d.work, 1))) return rc;
  if ((rc = m->alloc(&d.cull_list, L + 1))) return rc;
  if ((rc = m->alloc(&d.cull_off, L + 2))) return rc;
  {
    int blocks = 1;
    for (int k = 0; k < L; k++) {
      const int node = h.leaf_nodes[k];
      const int nv = h.type == kFaces ? h.uniq[node] : h.totprim[node] * h.grid_area;
      blocks = std::max(blocks, (nv + kAreaBlock - 1) / kAreaBlock);
      d.max_leaf_verts = std::max(d.max_leaf_verts, nv);
    }
    d.area_blocks = blocks;
  }
  if ((rc = m->alloc(&d.parts, static_cast<size_t>(L) * d.area_blocks + 1))) return rc;
  if ((rc = m->alloc(&d.scratch, nslot))) return rc;
  if ((rc = m->alloc(&d.scratch2, nslot))) return rc;
  for (int k = 0; k < 2; k++) {
    if ((rc = m->alloc(&d.slot_map[k], static_cast<size_t>(h.totvert)))) return rc;
    CK(cudaMemsetAsync(d.slot_map[k], 0xFF, sizeof(int) * static_cast<size_t>(h.totvert), m->stream),
       "slot map init");
  }
  if ((rc = m->alloc(&d.node_upd, N))) return rc;
  if ((rc = m->alloc(&m->d_nodes_tmp, L + 1))) return rc;
  if (N > cull_smem_limit())
    return fail(SGPU_ERR_UNSUPPORTED, "PBVH has %d nodes; the node search holds at most %d", N,
                cull_smem_limit());
  CK(launch_chunk_boxes_all(d, m->nchunks, m->stream), "chunk box kernel");
  return SGPU_OK;
}

int create_common(sgpu_mesh* m) {
  CK(cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking), "cudaStreamCreate");
  CK(cudaEventCreate(&m->ev0), "cudaEventCreate");
  CK(cudaEventCreate(&m->ev1), "cudaEventCreate");
  return SGPU_OK;
}

int check_mesh(const sgpu_mesh* m) {
  if (!m) return fail(SGPU_ERR_INVALID_ARG, "mesh handle is NULL");
  return SGPU_OK;
}

int device_err(sgpu_mesh* m) {
  int err = 0;
  CK(cudaMemcpyAsync(&err, &m->dev.work->err, sizeof(int), cudaMemcpyDeviceToHost, m->stream),
     "read error word");
  CK(cudaStreamSynchronize(m->stream), "cudaStreamSynchronize");
  if (err) {
    const int zero = 0;
    cudaMemcpy(&m->dev.work->err, &zero, sizeof(int), cudaMemcpyHostToDevice);
    return fail(err, "a kernel reported error code %d (invalid node list or bounds)", err);
  }
  return SGPU_OK;
}

bool make_brush(const SGPU_Brush* b, int tool, DevBrush* out) {
  std::memset(out, 0, sizeof(*out));
  Curve c;
  if (!build_curve(b->curve_preset, &c)) return false;
  out->tool = tool;
  out->flag = b->flag;
  out->radius = b->radius;
  out->strength = b->strength;
  out->normal_radius_factor = b->normal_radius_factor;
  out->area_radius_factor = b->area_radius_factor;
  out->plane_offset = b->plane_offset;
  out->crease_pinch_factor = b->crease_pinch_factor;
  out->elastic_type = b->elastic_deform_type;
  out->height = b->height;
  out->x_first = c.x_first;
  out->x_last = c.x_last;
  out->mintable = c.mintable;
  out->range = c.range;
  std::memcpy(out->y, c.y, sizeof(out->y));
  return true;
}

bool tool_ok(int tool) {
  return tool == kToolDraw || tool == kToolSmooth || tool == kToolInflate ||
         tool == kToolClayStrips || tool == kToolPinch || tool == kToolCrease ||
         tool == kToolGrab || tool == kToolElasticDeform || tool == kToolLayer;
}

// Elastic deform moves every vertex of the mesh in every dab: the per-call
// kernels spread that sweep over the whole GPU, a cluster team over one
// cluster (measured about 8x slower on a 655k-vertex mesh), so single-mesh
// strokes with such dabs on a cluster team take the graph path; the
// whole-GPU team keeps them.
bool stroke_has_whole_mesh(const SGPU_Brush* brush, const int* dab_tools, int ndabs) {
  for (int d = 0; d < ndabs; d++)
    if ((dab_tools ? dab_tools[d] : brush->sculpt_tool) == kToolElasticDeform) return true;
  return false;
}

bool stroke_has_original(const SGPU_Brush* brush, const int* dab_tools, int ndabs) {
  for (int d = 0; d < ndabs; d++)
    if (needs_stroke_start(dab_tools ? dab_tools[d] : brush->sculpt_tool)) return true;
  return false;
}

// Device buffers of the stroke-start positions and normals (allocated once,
// outside any stream capture).
int ensure_original(sgpu_mesh* m) {
  if (m->dev.orig_co) return SGPU_OK;
  float4 *a = nullptr, *b = nullptr;
  float* l = nullptr;
  int rc;
  if ((rc = m->alloc(&a, m->dev.totvert)) || (rc = m->alloc(&b, m->dev.totvert)) ||
      (rc = m->alloc(&l, m->dev.totvert)))
    return rc;
  m->dev.orig_co = a;
  m->dev.orig_no = b;
  m->dev.layer_disp = l;
  return SGPU_OK;
}

// The undo push of the stroke start: positions and normals kept as originals
// (stream-ordered, capturable).
int copy_original(sgpu_mesh* m, cudaStream_t s) {
  const size_t bytes = sizeof(float4) * m->dev.totvert;
  CK(cudaMemcpyAsync(m->dev.orig_co, m->dev.co, bytes, cudaMemcpyDeviceToDevice, s),
     "copy original positions");
  CK(cudaMemcpyAsync(m->dev.orig_no, m->dev.no, bytes, cudaMemcpyDeviceToDevice, s),
     "copy original normals");
  CK(cudaMemsetAsync(m->dev.layer_disp, 0, sizeof(float) * m->dev.totvert, s),
     "reset layer heights");
  m->orig_stored = true;
  return SGPU_OK;
}

// The symmetry passes of one dab.
DabPasses dab_passes(const SGPU_Brush* brush, const float loc[3], const float delta[3]) {
  DabPasses dp{};
  for (int pass = 0; pass < 8; pass++) {
    if ((pass & ~brush->symmetry) != 0) continue;
    for (int k = 0; k < 3; k++) {
      const float sgn = (pass & (1 << k)) ? -1.0f : 1.0f;
      dp.loc[dp.npass][k] = sgn * loc[k];
      dp.delta[dp.npass][k] = sgn * delta[k];
      dp.view[dp.npass][k] = sgn * brush->view_normal[k];
    }
    dp.npass++;
  }
  return dp;
}

// BKE_kelvinlet_init_params (kelvinlet.c:6-21) with shear modulus 1 and the
// force |grab_delta| * strength (the mouse-direction sign taken as +1).
void kelvinlet_params(DevBrush* b, const float delta[3], float poisson) {
  const float len = sqrtf(delta[0] * delta[0] + delta[1] * delta[1] + delta[2] * delta[2]);
  b->kl_a = 1.0f / (4.0f * 3.14159265358979323846f * 1.0f);
  b->kl_b = b->kl_a / (4.0f * (1.0f - poisson));
  b->kl_c = 2.0f * (3.0f * b->kl_a - 2.0f * b->kl_b);
  b->kl_f = len * b->strength;
  b->kl_rs[0] = b->radius * 1.0f;
  b->kl_rs[1] = b->kl_rs[0] * 2.0f;
  b->kl_rs[2] = b->kl_rs[1] * 2.0f;
}

// Launch bookkeeping: counts launches and, while profiling, brackets each one
// with CUDA events on the mesh stream.
struct Launcher {
  sgpu_mesh* m;
  int launches = 0;
  template <class F>
  int run(int kind, const char* what, F&& f) {
    cudaEvent_t a = nullptr;
    if (m->profiling) {
      a = m->prof_event();
      if (!a) return fail(SGPU_ERR_CUDA, "cudaEventCreate failed");
      cudaEventRecord(a, m->stream);
    }
    const cudaError_t e = f();
    if (e != cudaSuccess) return cuda_fail(e, what);
    if (m->profiling) {
      cudaEvent_t b = m->prof_event();
      if (!b) return fail(SGPU_ERR_CUDA, "cudaEventCreate failed");
      cudaEventRecord(b, m->stream);
      m->prof_marks.push_back({kind, a, b});
    }
    launches++;
    return SGPU_OK;
  }
};

#define LAUNCH(L, kind, what, expr)                                \
  do {                                                             \
    const int _rc = (L).run((kind), (what), [&] { return (expr); }); \
    if (_rc) return _rc;                                           \
  } while (0)

// Launches the brush of one pass over the current device node list.
int launch_tool(Launcher& L, const DevBrush& b, PassParams pp) {
  const DevMesh& d = L.m->dev;
  cudaStream_t s = L.m->stream;
  if (uses_area(b.tool)) {
    LAUNCH(L, kKArea, "area kernel", launch_area(d, b, pp, s));
    LAUNCH(L, kKBrush, "brush kernel", launch_brush(d, b, pp, s));
  } else if (b.tool == kToolInflate || b.tool == kToolLayer) {
    LAUNCH(L, kKBrush, "brush kernel", launch_brush(d, b, pp, s));
  } else {
    // Smooth: 4 sub-steps per unit strength, the last one fractional.
    float st = b.strength;
    if (st < 0.0f) st = 0.0f;
    if (st > 1.0f) st = 1.0f;
    const int count = (int)(st * 4.0f);
    const float last = 4.0f * (st - (float)count * 0.25f);
    for (int it = 0; it <= count; it++) {
      pp.iter_strength = (it != count) ? 1.0f : last;
      pp.iteration = it;
      LAUNCH(L, kKSmoothCompute, "smooth kernel", launch_smooth_compute(d, b, pp, s));
      LAUNCH(L, kKSmoothApply, "smooth kernel", launch_smooth_apply(d, s));
    }
  }
  return SGPU_OK;
}

// One dab of grab / elastic deform: the union gather, then the dab.
int launch_orig_tool(Launcher& L, DevBrush b, const SGPU_Brush* brush, const float loc[3],
                     const float delta[3]) {
  const DevMesh& d = L.m->dev;
  cudaStream_t s = L.m->stream;
  const DabPasses dp = dab_passes(brush, loc, delta);
  const bool elastic = b.tool == kToolElasticDeform;
  if (elastic) kelvinlet_params(&b, delta, brush->elastic_deform_volume_preservation);
  LAUNCH(L, kKCull, "cull kernel", launch_cull_dab(d, dp, b.radius * b.radius, elastic ? 1 : 0, s));
  LAUNCH(L, kKBrush, "brush kernel", launch_orig_dab(d, b, dp, s));
  return SGPU_OK;
}

int launch_update_normals(Launcher& L, int bounds_flag) {
  const DevMesh& d = L.m->dev;
  cudaStream_t s = L.m->stream;
  if (d.type == kFaces) {
    LAUNCH(L, kKUpdate, "update kernel", launch_update_faces(d, 1, bounds_flag, s));
  } else {
    LAUNCH(L, kKGridGather, "grid gather kernel", launch_grid_gather(d, s));
    LAUNCH(L, kKGridFaces, "grid inner-normal kernel", launch_grid_inner(d, s));
    LAUNCH(L, kKGridFaces, "grid face-seam kernel", launch_grid_face_seams(d, s));
    LAUNCH(L, kKGridSeams, "grid seam kernel", launch_grid_seams(d, s));
    if (bounds_flag) LAUNCH(L, kKUpdate, "bounds kernel", launch_update_faces(d, 0, bounds_flag, s));
  }
  return SGPU_OK;
}

// Enqueues a whole stroke on the mesh stream.
int enqueue_stroke(Launcher& L, const SGPU_Brush* brush, const SGPU_Dab* dabs, int ndabs,
                   const int* dab_tools) {
  sgpu_mesh* m = L.m;
  DevBrush base;
  if (!make_brush(brush, brush->sculpt_tool, &base))
    return fail(SGPU_ERR_INVALID_ARG, "unknown curve preset %d", brush->curve_preset);
  CK(cudaMemsetAsync(&m->dev.work->displaced, 0, sizeof(unsigned long long), m->stream),
     "reset counter");
  if (stroke_has_original(brush, dab_tools, ndabs)) {
    const int rc = copy_original(m, m->stream);
    if (rc) return rc;
  }
  for (int d = 0; d < ndabs; d++) {
    const int tool = dab_tools ? dab_tools[d] : brush->sculpt_tool;
    base.tool = tool;
    if (uses_original(tool)) {
      int rc = launch_orig_tool(L, base, brush, dabs[d].location, dabs[d].grab_delta);
      if (rc) return rc;
      if ((rc = launch_update_normals(L, kUpdateBB))) return rc;
      continue;
    }
    const float scale = (tool == kToolClayStrips) ? 1.41421356237309504880f : 1.0f;
    const float r = brush->radius * scale;
    for (int pass = 0; pass < 8; pass++) {
      if ((pass & ~brush->symmetry) != 0) continue;
      PassParams pp{};
      for (int k = 0; k < 3; k++) {
        const float sgn = (pass & (1 << k)) ? -1.0f : 1.0f;
        pp.loc[k] = sgn * dabs[d].location[k];
        pp.delta[k] = sgn * dabs[d].grab_delta[k];
        pp.view[k] = sgn * brush->view_normal[k];
      }
      pp.cull_radius_sq = r * r;
      pp.original = brush->use_original_bb || tool == kToolLayer;  // layer: original bounds
      pp.iter_strength = 1.0f;
      LAUNCH(L, kKCull, "cull kernel", launch_cull(m->dev, pp, m->stream));
      const int rc = launch_tool(L, base, pp);
      if (rc) return rc;
    }
    const int rc = launch_update_normals(L, kUpdateBB);
    if (rc) return rc;
  }
  LAUNCH(L, kKUpdate, "bounds kernel", launch_update_faces(m->dev, 0, kUpdateOriginalBB, m->stream));
  return SGPU_OK;
}

int run_stroke(sgpu_mesh* mesh, const SGPU_Brush* brush, const SGPU_Dab* dabs, int ndabs,
               const int* dab_tools, int mode, int* launches_out);
int finish_stroke(sgpu_mesh* mesh, int mode, int launches, SGPU_StrokeStats* stats);
// wait = false: enqueue only (launch, then the displaced counters into the
// first mesh's h_disp); the caller synchronizes and reads them.
// Team of the persistent stroke kernel: cluster size (1..16) or
// SGPU_TEAM_GRID, and the CTAs per SM of the cluster build (0 auto, 1, 2).
struct TeamShape {
  int cluster;
  int ctas_per_sm;
};
int team_batch(sgpu_mesh** meshes, int n, const SGPU_Brush* brushes, const SGPU_Dab* dabs,
               const int* offs, const int* tools, TeamShape shape, cudaStream_t s,
               SGPU_StrokeStats* stats, float* total_ms, bool wait = true);

// Autotuner results, process-wide: a single-mesh stroke is keyed by (mesh
// type, log2 of its vertex count, the set of tools of the stroke, symmetry
// passes); a batch by (its mesh count, log2 of its total vertex count, the
// set of tools).  A mesh whose team was not set explicitly strokes with the
// cached shape of its key; sgpu_batch_stroke with cluster_size 0 with the
// cached shape of its batch key.
struct TuneKey {
  int batch, type, size_class, passes, nmesh;
  unsigned tools;
  bool operator<(const TuneKey& o) const {
    return std::tie(batch, type, size_class, passes, nmesh, tools) <
           std::tie(o.batch, o.type, o.size_class, o.passes, o.nmesh, o.tools);
  }
};
std::mutex g_tune_mu;
std::map<TuneKey, TeamShape> g_tune;

int size_class(long long n) {
  int c = 0;
  while (n > 1) {
    n >>= 1;
    c++;
  }
  return c;
}

unsigned tools_mask(const SGPU_Brush* b, const int* tools, int ndabs) {
  unsigned m = 0;
  for (int d = 0; d < ndabs; d++) m |= 1u << ((tools ? tools[d] : b->sculpt_tool) & 31);
  if (ndabs == 0) m = 1u << (b->sculpt_tool & 31);
  return m;
}

TuneKey stroke_key(const sgpu_mesh* m, const SGPU_Brush* b, const int* tools, int ndabs);
TuneKey batch_key(sgpu_mesh* const* meshes, int n, const SGPU_Brush* brushes, const int* offs,
                  const int* tools);
// The team a single-mesh stroke runs on: the mesh's explicit setting, else
// the autotuner's cached shape for the stroke's key, else 8 CTAs.
TeamShape mesh_team(const sgpu_mesh* m, const SGPU_Brush* b, const int* tools, int ndabs);
// Profiling counters handed to the next persistent launch (nullptr otherwise).
thread_local unsigned long long* g_team_prof_bytes = nullptr;
thread_local unsigned long long* g_team_phase_ns = nullptr;
int validate_stroke(sgpu_mesh* mesh, const SGPU_Brush* brush, const SGPU_Dab* dabs, int ndabs,
                    const int* dab_tools);

int upload_node_list(sgpu_mesh* m, const int* nodes, int totnode) {
  if (totnode < 0 || totnode > m->dev.nleaf)
    return fail(SGPU_ERR_INVALID_ARG, "node count %d out of range", totnode);
  // Each leaf at most once: a repeated leaf would move its vertices twice and
  // overrun the per-pass scratch sized to one entry per vertex.
  std::vector<unsigned char> seen(m->dev.totnode, 0);
  for (int k = 0; k < totnode; k++) {
    if (nodes[k] < 0 || nodes[k] >= m->dev.totnode || m->host.node_leaf[nodes[k]] < 0)
      return fail(SGPU_ERR_INVALID_ARG, "node %d is not a leaf of this PBVH", nodes[k]);
    if (seen[nodes[k]]++)
      return fail(SGPU_ERR_INVALID_ARG, "node %d appears twice in the node list", nodes[k]);
  }
  if (totnode > 0)
    CK(cudaMemcpyAsync(m->d_nodes_tmp, nodes, sizeof(int) * totnode, cudaMemcpyHostToDevice,
                       m->stream),
       "upload node list");
  CK(launch_set_list(m->dev, m->d_nodes_tmp, totnode, m->stream), "node list kernel");
  CK(cudaStreamSynchronize(m->stream), "cudaStreamSynchronize");
  return SGPU_OK;
}

int do_brush_tool(sgpu_mesh* m, const SGPU_Brush* brush, int tool, const float location[3],
                  const float grab_delta[3], const int* nodes, int totnode) {
  int rc = check_mesh(m);
  if (rc) return rc;
  if (!brush || !location || !grab_delta) return fail(SGPU_ERR_INVALID_ARG, "NULL argument");
  if (!tool_ok(tool)) return fail(SGPU_ERR_INVALID_ARG, "unsupported sculpt tool %d", tool);
  if (!(brush->radius > 0.0f)) return fail(SGPU_ERR_INVALID_ARG, "radius must be positive");
  if (needs_stroke_start(tool) && !m->orig_stored)
    return fail(SGPU_ERR_INVALID_ARG, "no stroke-start positions (sgpu_mesh_store_original)");
  if (uses_original(tool)) {
    if (nodes) return fail(SGPU_ERR_INVALID_ARG, "grab / elastic deform gather their own leaves");
    if (!m->orig_stored)
      return fail(SGPU_ERR_INVALID_ARG, "no stroke-start positions (sgpu_mesh_store_original)");
    if (brush->elastic_deform_type < 0 || brush->elastic_deform_type > 4)
      return fail(SGPU_ERR_INVALID_ARG, "elastic deform type out of range");
  }
  if (nodes && (rc = upload_node_list(m, nodes, totnode))) return rc;
  DevBrush b;
  if (!make_brush(brush, tool, &b))
    return fail(SGPU_ERR_INVALID_ARG, "unknown curve preset %d", brush->curve_preset);
  if (uses_original(tool)) {
    Launcher L{m};
    if ((rc = launch_orig_tool(L, b, brush, location, grab_delta))) return rc;
    return device_err(m);
  }
  PassParams pp{};
  for (int k = 0; k < 3; k++) {
    pp.loc[k] = location[k];
    pp.delta[k] = grab_delta[k];
    pp.view[k] = brush->view_normal[k];
  }
  pp.iter_strength = 1.0f;
  Launcher L{m};
  rc = launch_tool(L, b, pp);
  if (rc) return rc;
  return device_err(m);
}

template <class T>
int ensure_dev(T** p, size_t* cap, size_t n);

// The device address of a page-locked host buffer mapped into the device's
// address space, else null (pageable or unknown memory).
float* mapped_host_ptr(void* p) {
  cudaPointerAttributes pa;
  if (cudaPointerGetAttributes(&pa, p) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  if (pa.type != cudaMemoryTypeHost || !pa.devicePointer) return nullptr;
  return static_cast<float*>(pa.devicePointer);
}

// A host copy split over a few threads, running while the device works;
// joined before anything else writes the destination (and on every return).
struct HostCopy {
  std::vector<std::thread> threads;
  void start(void* dst, const void* src, size_t bytes) {
    const unsigned hw = std::thread::hardware_concurrency();
    const size_t k = std::max<size_t>(1, std::min<size_t>(8, hw > 1 ? hw / 2 : 1));
    const size_t chunk = ((bytes + k - 1) / k + 4095) & ~static_cast<size_t>(4095);
    char* d = static_cast<char*>(dst);
    const char* s = static_cast<const char*>(src);
    for (size_t off = 0; off < bytes; off += chunk) {
      const size_t n = std::min(chunk, bytes - off);
      try {
        threads.emplace_back([=] { std::memcpy(d + off, s + off, n); });
      } catch (...) {
        std::memcpy(d + off, s + off, n);  // no thread to run it: copy here
      }
    }
  }
  void join() {
    for (std::thread& t : threads)
      if (t.joinable()) t.join();
    threads.clear();
  }
  ~HostCopy() { join(); }
};

// The host-buffer stroke around the upload and download of one mesh type:
// upload, refit of every leaf box, the stroke (mode as in sgpu_stroke),
// download, all between two events on the mesh stream.
template <class Up, class Down>
int stroke_host_run(sgpu_mesh* mesh, const SGPU_Brush* brush, const SGPU_Dab* dabs, int ndabs,
                    const int* dab_tools, int mode, Up upload, Down download, int& launches,
                    SGPU_StrokeStats* stats) {
  int rc;
  if (mode != SGPU_STROKE_EAGER && mode != SGPU_STROKE_GRAPH && mode != SGPU_STROKE_TEAM)
    return fail(SGPU_ERR_INVALID_ARG, "unknown stroke mode %d", mode);
  const TeamShape team = mesh_team(mesh, brush, dab_tools, ndabs);
  if (mode == SGPU_STROKE_TEAM && team.cluster != SGPU_TEAM_GRID &&
      stroke_has_whole_mesh(brush, dab_tools, ndabs))
    mode = SGPU_STROKE_GRAPH;
  if (!mesh->ev_h0) {
    CK(cudaEventCreate(&mesh->ev_h0), "cudaEventCreate");
    CK(cudaEventCreate(&mesh->ev_h1), "cudaEventCreate");
  }
  DevMesh& d = mesh->dev;
  CK(cudaEventRecord(mesh->ev_h0, mesh->stream), "event");
  if ((rc = upload())) return rc;
  // New positions: every leaf box is refit and flushed before the stroke.
  CK(launch_mark_all(d, kUpdateBB | kUpdateOriginalBB, mesh->stream), "mark kernel");
  CK(launch_update_faces(d, 0, kUpdateBB | kUpdateOriginalBB, mesh->stream), "bounds kernel");
  launches += 2;
  SGPU_StrokeStats inner;
  std::memset(&inner, 0, sizeof(inner));
  if (mode == SGPU_STROKE_TEAM) {
    const int offs[2] = {0, ndabs};
    sgpu_mesh* one[1] = {mesh};
    float total = 0.0f;
    if ((rc = team_batch(one, 1, brush, dabs, offs, dab_tools, team, mesh->stream, &inner,
                         &total, false)))
      return rc;
    launches += 1;
  } else {
    if ((rc = run_stroke(mesh, brush, dabs, ndabs, dab_tools, mode, &launches))) return rc;
  }
  if ((rc = download())) return rc;
  CK(cudaEventRecord(mesh->ev_h1, mesh->stream), "event");
  unsigned long long displaced = 0;
  if (mode != SGPU_STROKE_TEAM)
    CK(cudaMemcpyAsync(&displaced, &d.work->displaced, sizeof(displaced), cudaMemcpyDeviceToHost,
                       mesh->stream),
       "read counter");
  CK(cudaStreamSynchronize(mesh->stream), "cudaStreamSynchronize");
  if (mode == SGPU_STROKE_TEAM) {
    displaced = mesh->h_disp[0];
    if (const int status = static_cast<int>(mesh->h_disp[1]))
      return fail(status, "persistent stroke kernel: a team barrier wait ran out (error %d); the "
                  "stroke is incomplete", status);
  }
  if ((rc = device_err(mesh))) return rc;
  if (stats) {
    float ms = 0.0f;
    CK(cudaEventElapsedTime(&ms, mesh->ev_h0, mesh->ev_h1), "elapsed");
    stats->verts_displaced = static_cast<int64_t>(displaced);
    stats->gpu_ms = ms;
    stats->kernel_launches = launches;
    stats->graph_nodes = mode == SGPU_STROKE_GRAPH ? mesh->g_nodes : 0;
  }
  return SGPU_OK;
}

int ray_query(sgpu_mesh* mesh, int nrays, const float* ray_starts, const float* ray_normals,
              const float* ray_lengths, int original, bool nearest, float* r_depths, int* r_hits,
              int* r_active_vertices, int* r_active_faces, float* r_face_normals,
              float* r_dist_sq);

}  // namespace

extern "C" {

const char* sgpu_version(void) { return "libsculptgpu 0.1 (sm_103a)"; }

const char* sgpu_last_error(void) { return g_err.c_str(); }

int sgpu_device_info(int* sm_count, int* cc_major, int* cc_minor) {
  int rc = ensure_device();
  if (rc) return rc;
  int dev = 0;
  CK(cudaGetDevice(&dev), "cudaGetDevice");
  if (sm_count) CK(cudaDeviceGetAttribute(sm_count, cudaDevAttrMultiProcessorCount, dev), "attr");
  if (cc_major) CK(cudaDeviceGetAttribute(cc_major, cudaDevAttrComputeCapabilityMajor, dev), "attr");
  if (cc_minor) CK(cudaDeviceGetAttribute(cc_minor, cudaDevAttrComputeCapabilityMinor, dev), "attr");
  return SGPU_OK;
}

int sgpu_mesh_create_faces(const SGPU_MVert* verts, int totvert, const SGPU_MPoly* polys,
                           int totpoly, const SGPU_MLoop* loops, int totloop,
                           const SGPU_MLoopTri* looptris, int totlooptri,
                           const float* vert_normals, const float* mask, const float* automask,
                           int leaf_limit, sgpu_mesh** r_mesh) {
  if (!r_mesh) return fail(SGPU_ERR_INVALID_ARG, "r_mesh is NULL");
  *r_mesh = nullptr;
  if (!verts || !polys || !loops || !looptris || totvert <= 0 || totpoly <= 0 || totloop <= 0 ||
      totlooptri <= 0)
    return fail(SGPU_ERR_INVALID_ARG, "empty or NULL mesh arrays");
  int rc = ensure_device();
  if (rc) return rc;
  sgpu_mesh* m = new (std::nothrow) sgpu_mesh();
  if (!m) return fail(SGPU_ERR_OOM, "host allocation failed");
  HostMesh& h = m->host;
  h.type = kFaces;
  h.totvert = totvert;
  h.totpoly = totpoly;
  h.totloop = totloop;
  h.totlt = totlooptri;
  h.leaf_limit = leaf_limit > 0 ? leaf_limit : 10000;
  h.poly_loopstart.resize(totpoly);
  h.poly_totloop.resize(totpoly);
  h.poly_mat.resize(totpoly);
  h.poly_flag.resize(totpoly);
  for (int p = 0; p < totpoly; p++) {
    h.poly_loopstart[p] = polys[p].loopstart;
    h.poly_totloop[p] = polys[p].totloop;
    h.poly_mat[p] = polys[p].mat_nr;
    h.poly_flag[p] = polys[p].flag;
  }
  h.loop_v.resize(totloop);
  for (int l = 0; l < totloop; l++) h.loop_v[l] = static_cast<int>(loops[l].v);
  h.lt_v.resize(3 * static_cast<size_t>(totlooptri));
  h.lt_loop.resize(3 * static_cast<size_t>(totlooptri));
  h.lt_poly.resize(totlooptri);
  for (int t = 0; t < totlooptri; t++) {
    for (int j = 0; j < 3; j++) {
      const unsigned int l = looptris[t].tri[j];
      if (l >= static_cast<unsigned int>(totloop)) {
        delete m;
        return fail(SGPU_ERR_INVALID_ARG, "looptri %d loop index out of range", t);
      }
      h.lt_v[3 * t + j] = h.loop_v[l];
      h.lt_loop[3 * t + j] = static_cast<int>(l);
    }
    h.lt_poly[t] = static_cast<int>(looptris[t].poly);
  }
  h.co.resize(3 * static_cast<size_t>(totvert));
  for (int v = 0; v < totvert; v++)
    for (int k = 0; k < 3; k++) h.co[3 * static_cast<size_t>(v) + k] = verts[v].co[k];
  std::string err;
  if (!build_faces(h, &err)) {
    delete m;
    return fail(SGPU_ERR_INVALID_ARG, "%s", err.c_str());
  }
  DevMesh& d = m->dev;
  d.type = kFaces;
  d.totvert = totvert;
  d.totlt = totlooptri;
  auto bail = [&](int code) {
    m->release();
    delete m;
    return code;
  };
  if ((rc = create_common(m))) return bail(rc);
  // Device vertex order: the unique vertices of each leaf, leaf by leaf in
  // left-first order and in the order of the leaf's vertex list, then the
  // vertices no leaf owns.  A leaf's brush-visible vertices are then one
  // contiguous range, and one-ring and face neighbours mostly share cache
  // lines.  Every order the results depend on (leaf vertex lists, one-rings,
  // vertex looptri lists) is kept as an explicit list, so the relabelling
  // does not change any result; entry points taking or returning per-vertex
  // arrays convert at the boundary.
  std::vector<int> n2o(totvert);
  {
    std::vector<int>& o2n = m->o2n;
    o2n.assign(totvert, -1);
    int c = 0;
    for (int node : h.leaf_nodes)
      for (int i = 0; i < h.uniq[node]; i++) {
        const int v = h.vert_indices[h.vert_off[node] + i];
        if (o2n[v] < 0) {
          o2n[v] = c;
          n2o[c++] = v;
        }
      }
    for (int v = 0; v < totvert; v++)
      if (o2n[v] < 0) {
        o2n[v] = c;
        n2o[c++] = v;
      }
    if ((rc = m->upload(&m->d_o2n, o2n))) return bail(rc);
    if ((rc = m->upload(&m->d_n2o, n2o))) return bail(rc);
  }
  const std::vector<int>& o2n = m->o2n;
  if ((rc = m->alloc(&d.co, totvert))) return bail(rc);
  if ((rc = m->alloc(&d.no, totvert))) return bail(rc);
  static_assert(sizeof(SGPU_MVert) == sizeof(float4), "MVert is 16 bytes");
  {
    std::vector<float4> co4(totvert);
    for (int n = 0; n < totvert; n++) std::memcpy(&co4[n], &verts[n2o[n]], sizeof(float4));
    CK(cudaMemcpyAsync(d.co, co4.data(), sizeof(float4) * totvert, cudaMemcpyHostToDevice,
                       m->stream),
       "upload verts");
    if (vert_normals) {
      for (int n = 0; n < totvert; n++) {
        const float* q = vert_normals + 3 * static_cast<size_t>(n2o[n]);
        co4[n] = make_float4(q[0], q[1], q[2], 0.0f);
      }
      CK(cudaMemcpyAsync(d.no, co4.data(), sizeof(float4) * totvert, cudaMemcpyHostToDevice,
                         m->stream),
         "upload normals");
    }
    CK(cudaStreamSynchronize(m->stream), "cudaStreamSynchronize");
  }
  std::vector<float> tmp1(totvert);
  if (mask) {
    float* dm = nullptr;
    if ((rc = m->alloc(&dm, totvert))) return bail(rc);
    for (int n = 0; n < totvert; n++) tmp1[n] = mask[n2o[n]];
    if ((rc = m->upload_to(dm, tmp1))) return bail(rc);
    d.mask = dm;
    m->has_mask = true;
  }
  if (automask) {
    float* da = nullptr;
    if ((rc = m->alloc(&da, totvert))) return bail(rc);
    for (int n = 0; n < totvert; n++) tmp1[n] = automask[n2o[n]];
    if ((rc = m->upload_to(da, tmp1))) return bail(rc);
    d.automask = da;
  }
  std::vector<int> loop_n(totloop);
  for (int l = 0; l < totloop; l++) loop_n[l] = o2n[h.loop_v[l]];
  std::vector<int2> pl(totpoly);
  std::vector<int4> pv(totpoly);
  for (int p = 0; p < totpoly; p++) {
    const int ls = h.poly_loopstart[p], tl = h.poly_totloop[p];
    pl[p] = make_int2(ls, tl);
    if (tl == 3) {
      pv[p] = make_int4(loop_n[ls], loop_n[ls + 1], loop_n[ls + 2], -1);
    } else if (tl == 4) {
      pv[p] = make_int4(loop_n[ls], loop_n[ls + 1], loop_n[ls + 2], loop_n[ls + 3]);
    } else {
      pv[p] = make_int4(-1, -1, -1, -1);
    }
  }
  // per-vertex lists in device order: rows moved, one-ring ids relabelled
  std::vector<int> vt_off(totvert + 1, 0), nb_off(totvert + 1, 0);
  std::vector<int2> vt_meta(h.vt_idx.size());
  std::vector<int> nb_idx(h.nb_idx.size());
  for (int n = 0; n < totvert; n++) {
    const int v = n2o[n];
    vt_off[n + 1] = vt_off[n] + (h.vt_off[v + 1] - h.vt_off[v]);
    for (int q = h.vt_off[v], o = vt_off[n]; q < h.vt_off[v + 1]; q++, o++) {
      const int t = h.vt_idx[q];
      vt_meta[o] = make_int2(h.lt_poly[t], h.lt_leaf[t]);
    }
    nb_off[n + 1] = nb_off[n] + (h.nb_off[v + 1] - h.nb_off[v]);
    for (int q = h.nb_off[v], o = nb_off[n]; q < h.nb_off[v + 1]; q++, o++) nb_idx[o] = o2n[h.nb_idx[q]];
  }
  {
    std::vector<int4> lt4(totlooptri);
    for (int t = 0; t < totlooptri; t++)
      lt4[t] = make_int4(o2n[h.lt_v[3 * t]], o2n[h.lt_v[3 * t + 1]], o2n[h.lt_v[3 * t + 2]],
                         h.lt_poly[t]);
    if ((rc = m->upload(&d.lt_v4, lt4))) return bail(rc);
  }
  if ((rc = m->upload(&d.poly, pl))) return bail(rc);
  if ((rc = m->upload(&d.poly_v4, pv))) return bail(rc);
  if ((rc = m->upload(&d.loop_v, loop_n))) return bail(rc);
  if ((rc = m->upload(&d.vt_off, vt_off))) return bail(rc);
  if ((rc = m->upload(&d.vt_meta, vt_meta))) return bail(rc);
  if ((rc = m->upload(&d.nb_off, nb_off))) return bail(rc);
  if ((rc = m->upload(&d.nb_idx, nb_idx))) return bail(rc);
  if ((rc = m->alloc(&d.vtag, totvert))) return bail(rc);
  if ((rc = upload_pbvh(m))) return bail(rc);
  if (!vert_normals) {
    // Every vertex tagged and every leaf flagged, then one normal update.
    CK(cudaMemsetAsync(d.vtag, 1, sizeof(unsigned int) * totvert, m->stream), "tag all");
    std::vector<int> lflag(d.nleaf);
    for (int k = 0; k < d.nleaf; k++) lflag[k] = h.flag[h.leaf_nodes[k]] | kUpdateNormals;
    CK_BAIL(cudaMemcpyAsync(d.leaf_flag, lflag.data(), sizeof(int) * d.nleaf,
                            cudaMemcpyHostToDevice, m->stream),
            "flag all");
    CK(launch_update_faces(d, 1, 0, m->stream), "normal kernel");
  }
  CK(cudaStreamSynchronize(m->stream), "cudaStreamSynchronize");
  h.co.clear();
  h.co.shrink_to_fit();
  *r_mesh = m;
  return SGPU_OK;
}

int sgpu_mesh_create_grids(int num_grids, int grid_size, const float* grids_co,
                           const float* grids_no, const float* grids_mask, int num_faces,
                           const int* face_start, const int* face_ngrids, const int* face_verts,
                           const int* face_edges, int num_base_verts, int num_base_edges,
                           const int* edge_verts, int leaf_limit, sgpu_mesh** r_mesh) {
  if (!r_mesh) return fail(SGPU_ERR_INVALID_ARG, "r_mesh is NULL");
  *r_mesh = nullptr;
  if (num_grids <= 0 || grid_size < 2 || !grids_co || num_faces <= 0 || !face_start ||
      !face_ngrids || !face_verts || !face_edges || !edge_verts || num_base_verts <= 0 ||
      num_base_edges <= 0)
    return fail(SGPU_ERR_INVALID_ARG, "empty or NULL grid arrays");
  const long long elems = static_cast<long long>(num_grids) * grid_size * grid_size;
  if (elems > 0x7fffffffLL) return fail(SGPU_ERR_UNSUPPORTED, "more than 2^31 grid elements");
  if (grid_size > grid_size_limit())
    return fail(SGPU_ERR_UNSUPPORTED, "grid_size %d above the supported %d", grid_size,
                grid_size_limit());
  int rc = ensure_device();
  if (rc) return rc;
  sgpu_mesh* m = new (std::nothrow) sgpu_mesh();
  if (!m) return fail(SGPU_ERR_OOM, "host allocation failed");
  HostMesh& h = m->host;
  h.type = kGrids;
  h.num_grids = num_grids;
  h.grid_size = grid_size;
  h.grid_area = grid_size * grid_size;
  h.totvert = static_cast<int>(elems);
  h.num_faces = num_faces;
  h.num_base_verts = num_base_verts;
  h.num_base_edges = num_base_edges;
  h.face_start.assign(face_start, face_start + num_faces);
  h.face_ngrids.assign(face_ngrids, face_ngrids + num_faces);
  int corners = 0;
  for (int f = 0; f < num_faces; f++) corners += face_ngrids[f] > 0 ? face_ngrids[f] : 0;
  h.face_verts.assign(face_verts, face_verts + corners);
  h.face_edges.assign(face_edges, face_edges + corners);
  h.edge_elems.assign(edge_verts, edge_verts + 2 * static_cast<size_t>(num_base_edges));
  for (int e = 0; e < 2 * num_base_edges; e++)
    if (edge_verts[e] < 0 || edge_verts[e] >= num_base_verts) {
      delete m;
      return fail(SGPU_ERR_INVALID_ARG, "edge vertex out of range");
    }
  h.leaf_limit = leaf_limit > 0 ? leaf_limit
                                : (10000 / h.grid_area > 1 ? 10000 / h.grid_area : 1);
  h.co.assign(grids_co, grids_co + 3 * static_cast<size_t>(elems));
  std::string err;
  if (!build_grids(h, &err)) {
    delete m;
    return fail(SGPU_ERR_INVALID_ARG, "%s", err.c_str());
  }
  DevMesh& d = m->dev;
  d.type = kGrids;
  d.totvert = static_cast<int>(elems);
  d.grid_size = grid_size;
  d.grid_area = h.grid_area;
  div_invariant_params(static_cast<unsigned int>(h.grid_area), &d.area_mul, &d.area_shift);
  div_invariant_params(static_cast<unsigned int>(grid_size), &d.size_mul, &d.size_shift);
  d.num_faces = num_faces;
  d.num_base_verts = num_base_verts;
  d.num_base_edges = num_base_edges;
  auto bail = [&](int code) {
    m->release();
    delete m;
    return code;
  };
  if ((rc = create_common(m))) return bail(rc);
  if ((rc = m->alloc(&d.co, elems))) return bail(rc);
  if ((rc = m->alloc(&d.no, elems))) return bail(rc);
  CK(cudaMemcpy2DAsync(d.co, sizeof(float4), grids_co, 3 * sizeof(float), 3 * sizeof(float), elems,
                       cudaMemcpyHostToDevice, m->stream),
     "upload grid positions");
  if (grids_no)
    CK(cudaMemcpy2DAsync(d.no, sizeof(float4), grids_no, 3 * sizeof(float), 3 * sizeof(float),
                         elems, cudaMemcpyHostToDevice, m->stream),
       "upload grid normals");
  if (grids_mask) {
    float* dm = nullptr;
    if ((rc = m->alloc(&dm, elems))) return bail(rc);
    CK(cudaMemcpyAsync(dm, grids_mask, sizeof(float) * elems, cudaMemcpyHostToDevice, m->stream),
       "upload grid mask");
    d.mask = dm;
    m->has_mask = true;
  }
  if ((rc = m->upload(&d.grid_face, h.grid_face))) return bail(rc);
  {
    std::vector<int4> info(num_grids);
    for (int gi = 0; gi < num_grids; gi++) {
      const int f = h.grid_face[gi];
      info[gi] = make_int4(f, h.face_start[f], h.face_ngrids[f], 0);
    }
    if ((rc = m->upload(&d.grid_info, info))) return bail(rc);
  }
  if ((rc = m->upload(&d.face_start, h.face_start))) return bail(rc);
  if ((rc = m->upload(&d.face_ngrids, h.face_ngrids))) return bail(rc);
  if ((rc = m->upload(&d.face_verts, h.face_verts))) return bail(rc);
  if ((rc = m->upload(&d.face_edges, h.face_edges))) return bail(rc);
  if ((rc = m->upload(&d.edge_off, h.edge_off))) return bail(rc);
  if ((rc = m->upload(&d.edge_elems, h.edge_elems))) return bail(rc);
  if ((rc = m->upload(&d.bvert_off, h.bvert_off))) return bail(rc);
  if ((rc = m->upload(&d.bvert_elems, h.bvert_elems))) return bail(rc);
  if ((rc = m->upload(&d.edge_face, h.edge_face))) return bail(rc);
  if ((rc = m->upload(&d.bvert_face, h.bvert_face))) return bail(rc);
  d.max_face_corners = h.max_face_corners;
  if ((rc = m->alloc(&d.face_list, num_faces))) return bail(rc);
  if ((rc = m->alloc(&d.face_info, num_faces))) return bail(rc);
  if ((rc = m->alloc(&d.cgrid_list, num_grids))) return bail(rc);
  if ((rc = m->alloc(&d.edge_list, num_base_edges))) return bail(rc);
  if ((rc = m->alloc(&d.bvert_list, num_base_verts))) return bail(rc);
  if ((rc = m->alloc(&d.face_mark, num_faces))) return bail(rc);
  if ((rc = m->alloc(&d.edge_mark, num_base_edges))) return bail(rc);
  if ((rc = m->alloc(&d.bvert_mark, num_base_verts))) return bail(rc);
  if ((rc = m->alloc(&d.grid_counts, 4))) return bail(rc);
  if ((rc = m->alloc(&d.corner_own, 2 * static_cast<size_t>(num_grids)))) return bail(rc);
  if ((rc = m->alloc(&d.edge_own, num_base_edges))) return bail(rc);
  if ((rc = m->alloc(&d.bvert_own, num_base_verts))) return bail(rc);
  CK_BAIL(cudaMemsetAsync(d.edge_own, 0xFF, sizeof(unsigned long long) * num_base_edges, m->stream),
          "owner keys");
  CK_BAIL(cudaMemsetAsync(d.bvert_own, 0xFF, sizeof(unsigned long long) * num_base_verts, m->stream),
          "owner keys");
  if ((rc = upload_pbvh(m))) return bail(rc);
  if (!grids_no) {
    std::vector<int> lflag(d.nleaf);
    for (int k = 0; k < d.nleaf; k++) lflag[k] = h.flag[h.leaf_nodes[k]] | kUpdateNormals;
    CK_BAIL(cudaMemcpyAsync(d.leaf_flag, lflag.data(), sizeof(int) * d.nleaf,
                            cudaMemcpyHostToDevice, m->stream),
            "flag all");
    Launcher L{m};
    if ((rc = launch_update_normals(L, 0))) return bail(rc);
  }
  CK(cudaStreamSynchronize(m->stream), "cudaStreamSynchronize");
  h.co.clear();
  h.co.shrink_to_fit();
  *r_mesh = m;
  return SGPU_OK;
}

int sgpu_mesh_destroy(sgpu_mesh* mesh) {
  if (!mesh) return fail(SGPU_ERR_INVALID_ARG, "mesh handle is NULL");
  mesh->release();
  delete mesh;
  return SGPU_OK;
}

int sgpu_mesh_info(const sgpu_mesh* mesh, SGPU_MeshInfo* r_info) {
  int rc = check_mesh(mesh);
  if (rc) return rc;
  if (!r_info) return fail(SGPU_ERR_INVALID_ARG, "r_info is NULL");
  const HostMesh& h = mesh->host;
  r_info->type = h.type;
  r_info->totvert = h.totvert;
  r_info->totnode = h.totnode;
  r_info->totleaf = static_cast<int>(h.leaf_nodes.size());
  r_info->leaf_limit = h.leaf_limit;
  r_info->totprim = static_cast<int>(h.prim_indices.size());
  r_info->leaf_vert_entries = static_cast<int>(h.vert_indices.size());
  r_info->grid_size = h.grid_size;
  return SGPU_OK;
}

int sgpu_mesh_sync(sgpu_mesh* mesh) {
  int rc = check_mesh(mesh);
  if (rc) return rc;
  CK(cudaStreamSynchronize(mesh->stream), "cudaStreamSynchronize");
  return SGPU_OK;
}

void* sgpu_mesh_stream(sgpu_mesh* mesh) { return mesh ? static_cast<void*>(mesh->stream) : nullptr; }

int sgpu_search_sphere(sgpu_mesh* mesh, const float center[3], float radius_sq, int original,
                       int* r_nodes, int* r_tot) {
  int rc = check_mesh(mesh);
  if (rc) return rc;
  if (!center) return fail(SGPU_ERR_INVALID_ARG, "center is NULL");
  PassParams pp{};
  for (int k = 0; k < 3; k++) pp.loc[k] = center[k];
  pp.cull_radius_sq = radius_sq;
  pp.original = original;
  CK(launch_cull(mesh->dev, pp, mesh->stream), "cull kernel");
  if (r_nodes || r_tot) {
    int cnt = 0;
    CK(cudaMemcpyAsync(&cnt, &mesh->dev.work->cull_count, sizeof(int), cudaMemcpyDeviceToHost,
                       mesh->stream),
       "read count");
    CK(cudaStreamSynchronize(mesh->stream), "cudaStreamSynchronize");
    if (r_nodes && cnt > 0) {
      std::vector<int> ids(cnt);
      CK(cudaMemcpy(ids.data(), mesh->dev.cull_list, sizeof(int) * cnt, cudaMemcpyDeviceToHost),
         "read list");
      for (int k = 0; k < cnt; k++) r_nodes[k] = mesh->host.leaf_nodes[ids[k]];
    }
    if (r_tot) *r_tot = cnt;
  }
  return SGPU_OK;
}

int sgpu_do_draw_brush(sgpu_mesh* mesh, const SGPU_Brush* brush, const float location[3],
                       const float grab_delta[3], const int* nodes, int totnode) {
  return do_brush_tool(mesh, brush, kToolDraw, location, grab_delta, nodes, totnode);
}
int sgpu_do_smooth_brush(sgpu_mesh* mesh, const SGPU_Brush* brush, const float location[3],
                         const float grab_delta[3], const int* nodes, int totnode) {
  return do_brush_tool(mesh, brush, kToolSmooth, location, grab_delta, nodes, totnode);
}
int sgpu_do_inflate_brush(sgpu_mesh* mesh, const SGPU_Brush* brush, const float location[3],
                          const float grab_delta[3], const int* nodes, int totnode) {
  return do_brush_tool(mesh, brush, kToolInflate, location, grab_delta, nodes, totnode);
}
int sgpu_do_clay_strips_brush(sgpu_mesh* mesh, const SGPU_Brush* brush, const float location[3],
                              const float grab_delta[3], const int* nodes, int totnode) {
  return do_brush_tool(mesh, brush, kToolClayStrips, location, grab_delta, nodes, totnode);
}
int sgpu_do_pinch_brush(sgpu_mesh* mesh, const SGPU_Brush* brush, const float location[3],
                        const float grab_delta[3], const int* nodes, int totnode) {
  return do_brush_tool(mesh, brush, kToolPinch, location, grab_delta, nodes, totnode);
}
int sgpu_do_crease_brush(sgpu_mesh* mesh, const SGPU_Brush* brush, const float location[3],
                         const float grab_delta[3], const int* nodes, int totnode) {
  return do_brush_tool(mesh, brush, kToolCrease, location, grab_delta, nodes, totnode);
}
int sgpu_do_layer_brush(sgpu_mesh* mesh, const SGPU_Brush* brush, const float location[3],
                        const float grab_delta[3], const int* nodes, int totnode) {
  return do_brush_tool(mesh, brush, kToolLayer, location, grab_delta, nodes, totnode);
}
int sgpu_do_grab_brush(sgpu_mesh* mesh, const SGPU_Brush* brush, const float location[3],
                       const float grab_delta[3], const int* nodes, int totnode) {
  return do_brush_tool(mesh, brush, kToolGrab, location, grab_delta, nodes, totnode);
}
int sgpu_do_elastic_deform_brush(sgpu_mesh* mesh, const SGPU_Brush* brush,
                                 const float location[3], const float grab_delta[3],
                                 const int* nodes, int totnode) {
  return do_brush_tool(mesh, brush, kToolElasticDeform, location, grab_delta, nodes, totnode);
}
int sgpu_mesh_store_original(sgpu_mesh* mesh) {
  int rc = check_mesh(mesh);
  if (rc) return rc;
  if ((rc = ensure_original(mesh)) || (rc = copy_original(mesh, mesh->stream))) return rc;
  CK(cudaStreamSynchronize(mesh->stream), "cudaStreamSynchronize");
  return SGPU_OK;
}
int sgpu_do_brush(sgpu_mesh* mesh, const SGPU_Brush* brush, const float location[3],
                  const float grab_delta[3], const int* nodes, int totnode) {
  if (!brush) return fail(SGPU_ERR_INVALID_ARG, "brush is NULL");
  return do_brush_tool(mesh, brush, brush->sculpt_tool, location, grab_delta, nodes, totnode);
}

int sgpu_calc_area_normal_and_center(sgpu_mesh* mesh, const SGPU_Brush* brush,
                                     const float location[3], const int* nodes, int totnode,
                                     float r_area_no[3], float r_area_co[3]) {
  int rc = check_mesh(mesh);
  if (rc) return rc;
  if (!brush || !location || !r_area_no || !r_area_co)
    return fail(SGPU_ERR_INVALID_ARG, "NULL argument");
  if (!(brush->radius > 0.0f)) return fail(SGPU_ERR_INVALID_ARG, "radius must be positive");
  if (nodes && (rc = upload_node_list(mesh, nodes, totnode))) return rc;
  DevBrush b;
  if (!make_brush(brush, kToolDraw, &b))
    return fail(SGPU_ERR_INVALID_ARG, "unknown curve preset %d", brush->curve_preset);
  PassParams pp{};
  for (int k = 0; k < 3; k++) pp.loc[k] = location[k];
  pp.iter_strength = 1.0f;
  CK(launch_area(mesh->dev, b, pp, mesh->stream), "area kernel");
  float out[6];
  static_assert(offsetof(Work, area_co) == offsetof(Work, area_no) + 3 * sizeof(float),
                "area normal and centre are adjacent");
  CK(cudaMemcpyAsync(out, mesh->dev.work->area_no, sizeof(out), cudaMemcpyDeviceToHost,
                     mesh->stream),
     "read area");
  if ((rc = device_err(mesh))) return rc;
  for (int k = 0; k < 3; k++) {
    r_area_no[k] = out[k];
    r_area_co[k] = out[3 + k];
  }
  return SGPU_OK;
}

int sgpu_pbvh_update_normals(sgpu_mesh* mesh) {
  int rc = check_mesh(mesh);
  if (rc) return rc;
  Launcher L{mesh};
  if ((rc = launch_update_normals(L, 0))) return rc;
  return device_err(mesh);
}

int sgpu_pbvh_update_bounds(sgpu_mesh* mesh, int flag) {
  int rc = check_mesh(mesh);
  if (rc) return rc;
  CK(launch_update_faces(mesh->dev, 0, flag, mesh->stream), "bounds kernel");
  return device_err(mesh);
}

int sgpu_pbvh_node_mark_update(sgpu_mesh* mesh, int node) {
  int rc = check_mesh(mesh);
  if (rc) return rc;
  if (node < 0 || node >= mesh->dev.totnode || mesh->host.node_leaf[node] < 0)
    return fail(SGPU_ERR_INVALID_ARG, "node %d is not a leaf", node);
  CK(launch_mark_node(mesh->dev, node, mesh->stream), "mark kernel");
  return SGPU_OK;
}

int sgpu_stroke(sgpu_mesh* mesh, const SGPU_Brush* brush, const SGPU_Dab* dabs, int ndabs,
                const int* dab_tools, int mode, SGPU_StrokeStats* stats) {
  int rc = check_mesh(mesh);
  if (rc) return rc;
  if (!brush || (!dabs && ndabs > 0) || ndabs < 0)
    return fail(SGPU_ERR_INVALID_ARG, "NULL brush or dabs");
  if (!(brush->radius > 0.0f)) return fail(SGPU_ERR_INVALID_ARG, "radius must be positive");
  for (int d = 0; d < ndabs; d++) {
    const int tool = dab_tools ? dab_tools[d] : brush->sculpt_tool;
    if (!tool_ok(tool)) return fail(SGPU_ERR_INVALID_ARG, "unsupported sculpt tool %d", tool);
  }
  if (brush->symmetry < 0 || brush->symmetry > 7)
    return fail(SGPU_ERR_INVALID_ARG, "symmetry flags out of range");
  const TeamShape team = mesh_team(mesh, brush, dab_tools, ndabs);
  if (mode == SGPU_STROKE_TEAM && team.cluster != SGPU_TEAM_GRID &&
      stroke_has_whole_mesh(brush, dab_tools, ndabs))
    mode = SGPU_STROKE_GRAPH;
  if (mode == SGPU_STROKE_TEAM) {
    const int offs[2] = {0, ndabs};
    sgpu_mesh* one[1] = {mesh};
    float total_ms = 0.0f;
    rc = team_batch(one, 1, brush, dabs, offs, dab_tools, team, mesh->stream, stats, &total_ms);
    return rc;
  }
  CK(cudaEventRecord(mesh->ev0, mesh->stream), "event");
  int launches = 0;
  if ((rc = run_stroke(mesh, brush, dabs, ndabs, dab_tools, mode, &launches))) return rc;
  CK(cudaEventRecord(mesh->ev1, mesh->stream), "event");
  return finish_stroke(mesh, mode, launches, stats);
}

// Strokes of one batch run concurrently: a mesh may appear once.
static int check_distinct(sgpu_mesh* const* meshes, int n) {
  std::vector<const sgpu_mesh*> v(meshes, meshes + n);
  std::sort(v.begin(), v.end());
  for (int i = 0; i < n; i++) {
    if (!v[i]) return fail(SGPU_ERR_INVALID_ARG, "NULL mesh in the batch");
    if (i > 0 && v[i] == v[i - 1]) return fail(SGPU_ERR_INVALID_ARG, "a mesh appears twice in the batch");
  }
  return SGPU_OK;
}

// One persistent launch with the phase counters armed; fills out.
static int profiled_team_batch(sgpu_mesh** meshes, int n, const SGPU_Brush* brushes,
                               const SGPU_Dab* dabs, const int* offs, const int* tools,
                               TeamShape shape, SGPU_TeamProfile* out, SGPU_StrokeStats* stats) {
  unsigned long long* counters = nullptr;
  cudaStream_t s = meshes[0]->stream;
  CK(cudaMalloc(&counters, sizeof(unsigned long long) * 2 * kTeamPhases), "cudaMalloc");
  CK(cudaMemsetAsync(counters, 0, sizeof(unsigned long long) * 2 * kTeamPhases, s), "memset");
  g_team_prof_bytes = counters;
  g_team_phase_ns = counters + kTeamPhases;
  float total = 0.0f;
  int rc = team_batch(meshes, n, brushes, dabs, offs, tools, shape, s, stats, &total);
  g_team_prof_bytes = nullptr;
  g_team_phase_ns = nullptr;
  unsigned long long host[2 * kTeamPhases] = {};
  if (!rc) cudaMemcpy(host, counters, sizeof(host), cudaMemcpyDeviceToHost);
  cudaFree(counters);
  if (rc) return rc;
  std::memset(out, 0, sizeof(*out));
  out->total_ms = total;
  for (int k = 0; k < kTeamPhases && k < SGPU_TEAM_PHASES; k++) {
    out->phase_bytes[k] = static_cast<double>(host[k]);
    out->phase_ms[k] = static_cast<double>(host[kTeamPhases + k]) * 1e-6;
  }
  return SGPU_OK;
}

int sgpu_stroke_team_profile(sgpu_mesh* mesh, const SGPU_Brush* brush, const SGPU_Dab* dabs,
                             int ndabs, const int* dab_tools, SGPU_TeamProfile* out,
                             SGPU_StrokeStats* stats) {
  int rc = validate_stroke(mesh, brush, dabs, ndabs, dab_tools);
  if (rc) return rc;
  if (!out) return fail(SGPU_ERR_INVALID_ARG, "NULL profile");
  const int offs[2] = {0, ndabs};
  sgpu_mesh* one[1] = {mesh};
  SGPU_StrokeStats st;
  rc = profiled_team_batch(one, 1, brush, dabs, offs, dab_tools,
                           mesh_team(mesh, brush, dab_tools, ndabs), out, &st);
  if (rc) return rc;
  if (stats) *stats = st;
  return SGPU_OK;
}

int sgpu_batch_team_profile(sgpu_mesh** meshes, int nmesh, const SGPU_Brush* brushes,
                            const SGPU_Dab* dabs, const int* dab_offsets, const int* dab_tools,
                            int cluster_size, SGPU_TeamProfile* out, SGPU_StrokeStats* stats) {
  if (!meshes || nmesh <= 0 || !brushes || !dab_offsets)
    return fail(SGPU_ERR_INVALID_ARG, "NULL or empty batch");
  if (!out) return fail(SGPU_ERR_INVALID_ARG, "NULL profile");
  if (int rc = check_distinct(meshes, nmesh)) return rc;
  for (int i = 0; i < nmesh; i++) {
    const int nd = dab_offsets[i + 1] - dab_offsets[i];
    int rc = validate_stroke(meshes[i], &brushes[i], dabs + dab_offsets[i], nd,
                             dab_tools ? dab_tools + dab_offsets[i] : nullptr);
    if (rc) return rc;
  }
  for (int i = 0; i < nmesh; i++) CK(cudaStreamSynchronize(meshes[i]->stream), "sync");
  TeamShape shape{cluster_size, 0};
  if (cluster_size == 0) {
    shape = TeamShape{meshes[0]->team_cluster, meshes[0]->team_build};
    std::lock_guard<std::mutex> lock(g_tune_mu);
    const auto it = g_tune.find(batch_key(meshes, nmesh, brushes, dab_offsets, dab_tools));
    if (it != g_tune.end()) shape = it->second;
  }
  return profiled_team_batch(meshes, nmesh, brushes, dabs, dab_offsets, dab_tools, shape, out,
                             stats);
}

int sgpu_mesh_set_team(sgpu_mesh* mesh, int cluster_size) {
  int rc = check_mesh(mesh);
  if (rc) return rc;
  if (cluster_size != 1 && cluster_size != 2 && cluster_size != 4 && cluster_size != 8 &&
      cluster_size != 16 && cluster_size != SGPU_TEAM_GRID)
    return fail(SGPU_ERR_INVALID_ARG, "cluster size must be 1, 2, 4, 8, 16 or SGPU_TEAM_GRID");
  mesh->team_cluster = cluster_size;
  mesh->team_build = 0;
  mesh->team_set = true;
  return SGPU_OK;
}

int sgpu_debug_inject(int what, int64_t value) {
  switch (what) {
    case SGPU_INJECT_ALLOC_FAIL:
      if (value < 0) return fail(SGPU_ERR_INVALID_ARG, "allocation count must be >= 0");
      g_inject_alloc.store(value);
      return SGPU_OK;
    case SGPU_INJECT_WAIT_NS:
      if (value < 0) return fail(SGPU_ERR_INVALID_ARG, "wait limit must be >= 0");
      g_wait_ns.store(value > 0 ? static_cast<unsigned long long>(value) : kDefaultWaitNs);
      return SGPU_OK;
    case SGPU_INJECT_BARRIER_EXTRA:
      if (value < 0 || value > 1) return fail(SGPU_ERR_INVALID_ARG, "barrier extra must be 0 or 1");
      g_bar_extra.store(static_cast<int>(value));
      return SGPU_OK;
    case SGPU_DEBUG_LOCKSTEP_PER_SM:
      if (value < 0 || value > 2) return fail(SGPU_ERR_INVALID_ARG, "CTAs per SM must be 0, 1 or 2");
      g_lock_per_sm.store(static_cast<int>(value));
      return SGPU_OK;
    default:
      return fail(SGPU_ERR_INVALID_ARG, "unknown injection hook %d", what);
  }
}

int sgpu_mesh_get_team(const sgpu_mesh* mesh, int* cluster_size) {
  int rc = check_mesh(mesh);
  if (rc) return rc;
  if (cluster_size) *cluster_size = mesh->team_cluster;
  return SGPU_OK;
}

int sgpu_autotune_team(sgpu_mesh* mesh, const SGPU_Brush* brush, const SGPU_Dab* dabs,
                       int ndabs, const int* dab_tools, int* r_cluster, float* r_ms) {
  int rc = validate_stroke(mesh, brush, dabs, ndabs, dab_tools);
  if (rc) return rc;
  if ((rc = sgpu_mesh_snapshot(mesh))) return rc;
  const int sizes[SGPU_AUTOTUNE_CANDIDATES] = {SGPU_TEAM_GRID, 1, 2, 4, 8, 16};
  const bool whole = stroke_has_whole_mesh(brush, dab_tools, ndabs);
  TeamShape best{mesh->team_cluster, 0};
  float best_ms = -1.0f;
  for (int k = 0; k < SGPU_AUTOTUNE_CANDIDATES; k++) {
    float ms = -1.0f;
    const TeamShape shape{sizes[k], 1};
    const bool ok = shape.cluster == SGPU_TEAM_GRID
                        ? team_wide_ctas(mesh->dev.totnode, mesh->dev.nleaf) > 0
                        : !whole && team_max_active_clusters(shape.cluster, mesh->dev.totnode,
                                                             mesh->dev.nleaf) > 0;
    if (ok) {
      const int offs[2] = {0, ndabs};
      sgpu_mesh* one[1] = {mesh};
      // two trials, keep the second (the first pays one-time setup)
      for (int trial = 0; trial < 2; trial++) {
        if ((rc = sgpu_mesh_restore(mesh))) return rc;
        SGPU_StrokeStats st;
        float total = 0.0f;
        if ((rc = team_batch(one, 1, brush, dabs, offs, dab_tools, shape, mesh->stream, &st,
                             &total)))
          return rc;
        ms = total;
      }
      if (best_ms < 0.0f || ms < best_ms) {
        best_ms = ms;
        best = shape;
      }
    }
    if (r_ms) r_ms[k] = ms;
  }
  if ((rc = sgpu_mesh_restore(mesh))) return rc;
  mesh->team_cluster = best.cluster;
  mesh->team_build = best.ctas_per_sm;
  mesh->team_set = true;
  {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    g_tune[stroke_key(mesh, brush, dab_tools, ndabs)] = best;
  }
  if (r_cluster) *r_cluster = best.cluster;
  return SGPU_OK;
}

int sgpu_autotune_batch(sgpu_mesh** meshes, int nmesh, const SGPU_Brush* brushes,
                        const SGPU_Dab* dabs, const int* dab_offsets, const int* dab_tools,
                        int* r_cluster, int* r_ctas_per_sm, float* r_ms) {
  if (!meshes || nmesh <= 0 || !brushes || !dab_offsets)
    return fail(SGPU_ERR_INVALID_ARG, "NULL or empty batch");
  if (int rc = check_distinct(meshes, nmesh)) return rc;
  for (int i = 0; i < nmesh; i++) {
    const int nd = dab_offsets[i + 1] - dab_offsets[i];
    int rc = validate_stroke(meshes[i], &brushes[i], dabs + dab_offsets[i], nd,
                             dab_tools ? dab_tools + dab_offsets[i] : nullptr);
    if (rc) return rc;
  }
  int rc;
  for (int i = 0; i < nmesh; i++)
    if ((rc = sgpu_mesh_snapshot(meshes[i]))) return rc;
  int max_nodes = 0, max_leaves = 0;
  for (int i = 0; i < nmesh; i++) {
    max_nodes = std::max(max_nodes, meshes[i]->dev.totnode);
    max_leaves = std::max(max_leaves, meshes[i]->dev.nleaf);
  }
  const TeamShape cand[SGPU_AUTOTUNE_BATCH_CANDIDATES] = {
      {16, 1}, {8, 1}, {8, 2}, {4, 1}, {4, 2}, {2, 2}, {SGPU_TEAM_GRID, 1}, {SGPU_TEAM_LOCKSTEP, 1},
      {SGPU_TEAM_LOCKSTEP, 2}};
  TeamShape best{8, 0};
  float best_ms = -1.0f;
  auto restore_all = [&]() -> int {
    for (int i = 0; i < nmesh; i++) {
      const int r = sgpu_mesh_restore(meshes[i]);
      if (r) return r;
    }
    return SGPU_OK;
  };
  for (int k = 0; k < SGPU_AUTOTUNE_BATCH_CANDIDATES; k++) {
    const TeamShape& c = cand[k];
    float ms = -1.0f;
    const bool ok = c.cluster == SGPU_TEAM_GRID       ? team_wide_ctas(max_nodes, max_leaves) > 0
                    : c.cluster == SGPU_TEAM_LOCKSTEP ? lock_ctas(max_nodes, max_leaves, c.ctas_per_sm) > 0
                    : team_max_active_clusters(c.cluster, max_nodes, max_leaves) > 0;
    if (ok) {
      for (int trial = 0; trial < 2; trial++) {
        if ((rc = restore_all())) return rc;
        float total = 0.0f;
        rc = team_batch(meshes, nmesh, brushes, dabs, dab_offsets, dab_tools, c,
                        meshes[0]->stream, nullptr, &total);
        if (rc == SGPU_ERR_CUDA && c.cluster > 0) {
          ms = -1.0f;  // this build holds no team of this size on the device
          break;
        }
        if (rc == SGPU_ERR_UNSUPPORTED && c.cluster == SGPU_TEAM_LOCKSTEP) {
          ms = -1.0f;  // the batch has dabs or grids the lockstep launch does not take
          break;
        }
        if (rc) return rc;
        ms = total;
      }
      if (ms > 0.0f && (best_ms < 0.0f || ms < best_ms)) {
        best_ms = ms;
        best = c;
      }
    }
    if (r_ms) r_ms[k] = ms;
  }
  if ((rc = restore_all())) return rc;
  {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    g_tune[batch_key(meshes, nmesh, brushes, dab_offsets, dab_tools)] = best;
  }
  if (r_cluster) *r_cluster = best.cluster;
  if (r_ctas_per_sm) *r_ctas_per_sm = best.ctas_per_sm;
  return SGPU_OK;
}

int sgpu_batch_stroke(sgpu_mesh** meshes, int nmesh, const SGPU_Brush* brushes,
                      const SGPU_Dab* dabs, const int* dab_offsets, const int* dab_tools,
                      int mode, int cluster_size, SGPU_StrokeStats* stats, float* r_total_ms) {
  if (!meshes || nmesh <= 0 || !brushes || !dab_offsets)
    return fail(SGPU_ERR_INVALID_ARG, "NULL or empty batch");
  if (int rc = check_distinct(meshes, nmesh)) return rc;
  for (int i = 0; i < nmesh; i++) {
    const int nd = dab_offsets[i + 1] - dab_offsets[i];
    int rc = validate_stroke(meshes[i], &brushes[i], dabs + dab_offsets[i], nd,
                             dab_tools ? dab_tools + dab_offsets[i] : nullptr);
    if (rc) return rc;
  }
  for (int i = 0; i < nmesh; i++) CK(cudaStreamSynchronize(meshes[i]->stream), "sync");
  if (mode == SGPU_BATCH_TEAM) {
    TeamShape shape{cluster_size, 0};
    if (cluster_size == 0) {
      shape = TeamShape{meshes[0]->team_cluster, meshes[0]->team_build};
      std::lock_guard<std::mutex> lock(g_tune_mu);
      const auto it = g_tune.find(batch_key(meshes, nmesh, brushes, dab_offsets, dab_tools));
      if (it != g_tune.end()) shape = it->second;
    }
    float total = 0.0f;
    int rc = team_batch(meshes, nmesh, brushes, dabs, dab_offsets, dab_tools, shape,
                        meshes[0]->stream, stats, &total);
    if (r_total_ms) *r_total_ms = total;
    return rc;
  }
  if (mode != SGPU_BATCH_SEQUENTIAL) return fail(SGPU_ERR_INVALID_ARG, "unknown batch mode");
  // one plain graph-mode stroke per mesh, one after another on the first
  // mesh's timeline (each waits for the previous one to finish)
  cudaEvent_t t0 = meshes[0]->ev0, t1 = nullptr;
  CK(cudaEventRecord(t0, meshes[0]->stream), "event");
  float sum = 0.0f;
  for (int i = 0; i < nmesh; i++) {
    const int nd = dab_offsets[i + 1] - dab_offsets[i];
    SGPU_StrokeStats st;
    int rc = sgpu_stroke(meshes[i], &brushes[i], dabs + dab_offsets[i], nd,
                         dab_tools ? dab_tools + dab_offsets[i] : nullptr, SGPU_STROKE_GRAPH, &st);
    if (rc) return rc;
    if (stats) stats[i] = st;
    sum += st.gpu_ms;
  }
  (void)t1;
  if (r_total_ms) *r_total_ms = sum;
  return SGPU_OK;
}

}  // extern "C"

namespace {

int validate_stroke(sgpu_mesh* mesh, const SGPU_Brush* brush, const SGPU_Dab* dabs, int ndabs,
                    const int* dab_tools) {
  int rc = check_mesh(mesh);
  if (rc) return rc;
  if (!brush || (!dabs && ndabs > 0) || ndabs < 0)
    return fail(SGPU_ERR_INVALID_ARG, "NULL brush or dabs");
  if (!(brush->radius > 0.0f)) return fail(SGPU_ERR_INVALID_ARG, "radius must be positive");
  for (int d = 0; d < ndabs; d++) {
    const int tool = dab_tools ? dab_tools[d] : brush->sculpt_tool;
    if (!tool_ok(tool)) return fail(SGPU_ERR_INVALID_ARG, "unsupported sculpt tool %d", tool);
  }
  if (brush->symmetry < 0 || brush->symmetry > 7)
    return fail(SGPU_ERR_INVALID_ARG, "symmetry flags out of range");
  return SGPU_OK;
}

}  // namespace

extern "C" {

int sgpu_stroke_host(sgpu_mesh* mesh, const SGPU_Brush* brush, const SGPU_Dab* dabs, int ndabs,
                     const int* dab_tools, const SGPU_MVert* verts_in,
                     const float* vert_normals_in, SGPU_MVert* verts_out, int mode,
                     SGPU_StrokeStats* stats) {
  int rc = validate_stroke(mesh, brush, dabs, ndabs, dab_tools);
  if (rc) return rc;
  if (mesh->dev.type != kFaces) return fail(SGPU_ERR_INVALID_ARG, "not a FACES mesh");
  if (!verts_in || !verts_out) return fail(SGPU_ERR_INVALID_ARG, "NULL host buffers");
  DevMesh& d = mesh->dev;
  int launches = 0;
  const size_t bytes = sizeof(float4) * static_cast<size_t>(d.totvert);
  // A page-locked, mapped output takes the changed blocks of vertices from
  // the device; host threads copy the input into it meanwhile (as for GRIDS).
  float4* d_out = reinterpret_cast<float4*>(mapped_host_ptr(verts_out));
  HostCopy host_copy;
  if (d_out && (rc = ensure_dev(&mesh->t_keep, &mesh->t_keep_cap, 4 * static_cast<size_t>(d.totvert))))
    return rc;
  float4* verts_dev = d_out ? reinterpret_cast<float4*>(mesh->t_keep) : d.scratch;
  auto upload = [&]() -> int {
    // host buffers in the caller's vertex order, converted on the device
    CK(cudaMemcpyAsync(verts_dev, verts_in, bytes, cudaMemcpyHostToDevice, mesh->stream), "upload verts");
    CK(launch_gather_f4(d.co, verts_dev, mesh->d_n2o, d.totvert, mesh->stream), "gather kernel");
    launches++;
    if (vert_normals_in) {
      float* flat = reinterpret_cast<float*>(d.scratch2);
      CK(cudaMemcpyAsync(flat, vert_normals_in, 3 * sizeof(float) * d.totvert,
                         cudaMemcpyHostToDevice, mesh->stream),
         "upload normals");
      CK(launch_xyz_to_f4(d.no, flat, mesh->d_n2o, d.totvert, true, mesh->stream), "gather kernel");
      launches++;
    }
    // (after the first event and the queued copies: inside the timed call)
    if (d_out && static_cast<const void*>(verts_out) != static_cast<const void*>(verts_in))
      host_copy.start(verts_out, verts_in, bytes);
    return SGPU_OK;
  };
  auto download = [&]() -> int {
    if (d_out) {
      host_copy.join();  // before the device writes the output
      CK(launch_vert_writeback(d_out, d.co, mesh->d_o2n, reinterpret_cast<const float4*>(mesh->t_keep),
                               d.totvert, mesh->stream),
         "write-back kernel");
      launches++;
      return SGPU_OK;
    }
    CK(launch_gather_f4(d.scratch, d.co, mesh->d_o2n, d.totvert, mesh->stream), "gather kernel");
    launches++;
    CK(cudaMemcpyAsync(verts_out, d.scratch, bytes, cudaMemcpyDeviceToHost, mesh->stream),
       "download verts");
    return SGPU_OK;
  };
  return stroke_host_run(mesh, brush, dabs, ndabs, dab_tools, mode, upload, download, launches,
                         stats);
}

int sgpu_stroke_host_grids(sgpu_mesh* mesh, const SGPU_Brush* brush, const SGPU_Dab* dabs,
                           int ndabs, const int* dab_tools, const float* grids_co_in,
                           const float* grids_no_in, float* grids_co_out, int mode,
                           SGPU_StrokeStats* stats) {
  int rc = validate_stroke(mesh, brush, dabs, ndabs, dab_tools);
  if (rc) return rc;
  if (mesh->dev.type != kGrids) return fail(SGPU_ERR_INVALID_ARG, "not a GRIDS mesh");
  if (!grids_co_in || !grids_co_out) return fail(SGPU_ERR_INVALID_ARG, "NULL host buffers");
  DevMesh& d = mesh->dev;
  int launches = 0;
  float* flat = reinterpret_cast<float*>(d.scratch);
  const size_t bytes = 3 * sizeof(float) * static_cast<size_t>(d.totvert);
  // A page-locked, mapped output takes the changed grids straight from the
  // device; the host threads copy the input into it meanwhile (grids the
  // stroke leaves bit-identical).  Any other output gets every position back
  // through the copy engine.
  float* d_out = mapped_host_ptr(grids_co_out);
  HostCopy host_copy;
  if (d_out && (rc = ensure_dev(&mesh->t_keep, &mesh->t_keep_cap, 3 * static_cast<size_t>(d.totvert))))
    return rc;
  float* pos_in = d_out ? mesh->t_keep : flat;
  auto upload = [&]() -> int {
    CK(cudaMemcpyAsync(pos_in, grids_co_in, bytes, cudaMemcpyHostToDevice, mesh->stream),
       "upload grid positions");
    CK(launch_xyz_to_f4(d.co, pos_in, nullptr, d.totvert, false, mesh->stream), "expand kernel");
    launches++;
    if (grids_no_in) {
      CK(cudaMemcpyAsync(flat, grids_no_in, bytes, cudaMemcpyHostToDevice, mesh->stream),
         "upload grid normals");
      CK(launch_xyz_to_f4(d.no, flat, nullptr, d.totvert, false, mesh->stream), "expand kernel");
      launches++;
    }
    // (after the first event and the queued copies: inside the timed call)
    if (d_out && grids_co_out != grids_co_in) host_copy.start(grids_co_out, grids_co_in, bytes);
    return SGPU_OK;
  };
  auto download = [&]() -> int {
    if (d_out) {
      host_copy.join();  // before the device writes the output
      CK(launch_grid_writeback(d_out, d.co, mesh->t_keep, d.totvert / d.grid_area, d.grid_area,
                               mesh->stream),
         "write-back kernel");
      launches++;
      return SGPU_OK;
    }
    CK(launch_f4_to_xyz(flat, d.co, nullptr, d.totvert, mesh->stream), "pack kernel");
    launches++;
    CK(cudaMemcpyAsync(grids_co_out, flat, bytes, cudaMemcpyDeviceToHost, mesh->stream),
       "download grid positions");
    return SGPU_OK;
  };
  return stroke_host_run(mesh, brush, dabs, ndabs, dab_tools, mode, upload, download, launches,
                         stats);
}

int sgpu_stroke_profile(sgpu_mesh* mesh, const SGPU_Brush* brush, const SGPU_Dab* dabs,
                        int ndabs, const int* dab_tools, SGPU_KernelProfile* out,
                        SGPU_StrokeStats* stats) {
  int rc = validate_stroke(mesh, brush, dabs, ndabs, dab_tools);
  if (rc) return rc;
  if (!out) return fail(SGPU_ERR_INVALID_ARG, "NULL profile table");
  static const char* names[SGPU_KERNEL_KINDS] = {
      "k_cull", "k_set_list", "k_area", "k_brush", "k_smooth_compute",
      "k_smooth_apply", "k_update_faces", "k_grid_gather", "k_grid_faces", "k_grid_seams"};
  unsigned long long* counters = nullptr;
  CK(cudaMalloc(&counters, sizeof(unsigned long long) * kKindCount), "cudaMalloc");
  CK(cudaMemsetAsync(counters, 0, sizeof(unsigned long long) * kKindCount, mesh->stream),
     "memset");
  mesh->dev.prof = counters;
  mesh->profiling = true;
  mesh->ev_used = 0;
  mesh->prof_marks.clear();
  CK(cudaEventRecord(mesh->ev0, mesh->stream), "event");
  int launches = 0;
  rc = run_stroke(mesh, brush, dabs, ndabs, dab_tools, SGPU_STROKE_EAGER, &launches);
  mesh->profiling = false;
  mesh->dev.prof = nullptr;
  if (rc) {
    cudaFree(counters);
    return rc;
  }
  cudaEventRecord(mesh->ev1, mesh->stream);
  unsigned long long host_counters[kKindCount];
  cudaMemcpyAsync(host_counters, counters, sizeof(host_counters), cudaMemcpyDeviceToHost,
                  mesh->stream);
  rc = finish_stroke(mesh, SGPU_STROKE_EAGER, launches, stats);
  cudaFree(counters);
  if (rc) return rc;
  for (int k = 0; k < SGPU_KERNEL_KINDS; k++) {
    std::memset(&out[k], 0, sizeof(out[k]));
    std::snprintf(out[k].name, sizeof(out[k].name), "%s", names[k]);
    out[k].alg_bytes = static_cast<double>(host_counters[k]);
  }
  for (const auto& mk : mesh->prof_marks) {
    float ms = 0.0f;
    CK(cudaEventElapsedTime(&ms, mk.a, mk.b), "elapsed");
    out[mk.kind].launches++;
    out[mk.kind].total_ms += ms;
  }
  mesh->prof_marks.clear();
  return SGPU_OK;
}

int sgpu_mesh_snapshot(sgpu_mesh* mesh) {
  int rc = check_mesh(mesh);
  if (rc) return rc;
  DevMesh& d = mesh->dev;
  const size_t V = static_cast<size_t>(d.totvert), N2 = 2 * static_cast<size_t>(d.totnode);
  if (!mesh->snap_co) {
    if ((rc = mesh->alloc(&mesh->snap_co, V))) return rc;
    if ((rc = mesh->alloc(&mesh->snap_no, V))) return rc;
    if (d.mask && (rc = mesh->alloc(&mesh->snap_mask, V))) return rc;
    if ((rc = mesh->alloc(&mesh->snap_vb, N2))) return rc;
    if ((rc = mesh->alloc(&mesh->snap_orig_vb, N2))) return rc;
    if ((rc = mesh->alloc(&mesh->snap_flag, static_cast<size_t>(d.nleaf)))) return rc;
  }
  cudaStream_t s = mesh->stream;
  CK(cudaMemcpyAsync(mesh->snap_co, d.co, sizeof(float4) * V, cudaMemcpyDeviceToDevice, s), "snap");
  CK(cudaMemcpyAsync(mesh->snap_no, d.no, sizeof(float4) * V, cudaMemcpyDeviceToDevice, s), "snap");
  if (d.mask)
    CK(cudaMemcpyAsync(mesh->snap_mask, d.mask, sizeof(float) * V, cudaMemcpyDeviceToDevice, s),
       "snap");
  CK(cudaMemcpyAsync(mesh->snap_vb, d.vb, sizeof(float4) * N2, cudaMemcpyDeviceToDevice, s), "snap");
  CK(cudaMemcpyAsync(mesh->snap_orig_vb, d.orig_vb, sizeof(float4) * N2, cudaMemcpyDeviceToDevice,
                     s),
     "snap");
  CK(cudaMemcpyAsync(mesh->snap_flag, d.leaf_flag, sizeof(int) * d.nleaf, cudaMemcpyDeviceToDevice,
                     s),
     "snap");
  CK(cudaStreamSynchronize(s), "cudaStreamSynchronize");
  return SGPU_OK;
}

int sgpu_mesh_restore(sgpu_mesh* mesh) {
  int rc = check_mesh(mesh);
  if (rc) return rc;
  if (!mesh->snap_co) return fail(SGPU_ERR_INVALID_ARG, "no snapshot taken");
  DevMesh& d = mesh->dev;
  const size_t V = static_cast<size_t>(d.totvert), N2 = 2 * static_cast<size_t>(d.totnode);
  cudaStream_t s = mesh->stream;
  CK(cudaMemcpyAsync(d.co, mesh->snap_co, sizeof(float4) * V, cudaMemcpyDeviceToDevice, s), "restore");
  CK(cudaMemcpyAsync(d.no, mesh->snap_no, sizeof(float4) * V, cudaMemcpyDeviceToDevice, s), "restore");
  if (d.mask)
    CK(cudaMemcpyAsync(d.mask, mesh->snap_mask, sizeof(float) * V, cudaMemcpyDeviceToDevice, s),
       "restore");
  CK(cudaMemcpyAsync(d.vb, mesh->snap_vb, sizeof(float4) * N2, cudaMemcpyDeviceToDevice, s),
     "restore");
  CK(cudaMemcpyAsync(d.orig_vb, mesh->snap_orig_vb, sizeof(float4) * N2, cudaMemcpyDeviceToDevice,
                     s),
     "restore");
  CK(cudaMemcpyAsync(d.leaf_flag, mesh->snap_flag, sizeof(int) * d.nleaf, cudaMemcpyDeviceToDevice,
                     s),
     "restore");
  CK(launch_chunk_boxes_all(d, mesh->nchunks, s), "chunk box kernel");
  CK(cudaStreamSynchronize(s), "cudaStreamSynchronize");
  return SGPU_OK;
}

int sgpu_mesh_flush_l2(sgpu_mesh* mesh) {
  int rc = check_mesh(mesh);
  if (rc) return rc;
  // 256 MiB written, then another 256 MiB read (the dirty lines the write left
  // are written back before the next timed kernel)
  const size_t bytes = 512ull << 20;
  if (!mesh->flush_buf) {
    void* p = nullptr;
    if ((rc = mesh->alloc(reinterpret_cast<char**>(&p), bytes))) return rc;
    mesh->flush_buf = p;
  }
  CK(launch_l2_flush(mesh->flush_buf, bytes, mesh->stream), "flush kernel");
  CK(cudaStreamSynchronize(mesh->stream), "cudaStreamSynchronize");
  return SGPU_OK;
}

void* sgpu_host_alloc(size_t bytes) {
  void* p = nullptr;
  if (cudaMallocHost(&p, bytes) != cudaSuccess) {
    fail(SGPU_ERR_OOM, "cudaMallocHost(%zu) failed", bytes);
    return nullptr;
  }
  return p;
}

int sgpu_host_free(void* ptr) {
  if (!ptr) return SGPU_OK;
  CK(cudaFreeHost(ptr), "cudaFreeHost");
  return SGPU_OK;
}

}  // extern "C"

namespace {

// Enqueues the stroke eagerly or through the per-mesh cached CUDA graph.
int run_stroke(sgpu_mesh* mesh, const SGPU_Brush* brush, const SGPU_Dab* dabs, int ndabs,
               const int* dab_tools, int mode, int* launches_out) {
  int rc;
  if (stroke_has_original(brush, dab_tools, ndabs) && (rc = ensure_original(mesh))) return rc;
  Launcher L{mesh};
  int& launches = *launches_out;
  if (mode == SGPU_STROKE_GRAPH) {
    // Key: everything the captured launches depend on.
    std::vector<unsigned char> key(sizeof(SGPU_Brush) + sizeof(SGPU_Dab) * ndabs +
                                   sizeof(int) * (dab_tools ? ndabs : 0) + sizeof(int));
    unsigned char* p = key.data();
    std::memcpy(p, brush, sizeof(SGPU_Brush));
    p += sizeof(SGPU_Brush);
    if (ndabs) std::memcpy(p, dabs, sizeof(SGPU_Dab) * ndabs);
    p += sizeof(SGPU_Dab) * ndabs;
    if (dab_tools) std::memcpy(p, dab_tools, sizeof(int) * ndabs);
    p += sizeof(int) * (dab_tools ? ndabs : 0);
    const int nd = ndabs;
    std::memcpy(p, &nd, sizeof(int));
    if (!mesh->gexec || key != mesh->gkey) {
      if (mesh->gexec) cudaGraphExecDestroy(mesh->gexec);
      mesh->gexec = nullptr;
      cudaGraph_t graph = nullptr;
      CK(cudaStreamBeginCapture(mesh->stream, cudaStreamCaptureModeThreadLocal), "begin capture");
      rc = enqueue_stroke(L, brush, dabs, ndabs, dab_tools);
      cudaError_t ce = cudaStreamEndCapture(mesh->stream, &graph);
      if (rc) {
        if (graph) cudaGraphDestroy(graph);
        return rc;
      }
      if (ce != cudaSuccess) return cuda_fail(ce, "end capture");
      size_t nn = 0;
      cudaGraphGetNodes(graph, nullptr, &nn);
      ce = cudaGraphInstantiate(&mesh->gexec, graph, 0);
      cudaGraphDestroy(graph);
      if (ce != cudaSuccess) return cuda_fail(ce, "graph instantiate");
      mesh->gkey = key;
      mesh->g_nodes = static_cast<int>(nn);
      mesh->g_launches = L.launches;
    }
    launches += mesh->g_launches;
    CK(cudaGraphLaunch(mesh->gexec, mesh->stream), "graph launch");
  } else {
    rc = enqueue_stroke(L, brush, dabs, ndabs, dab_tools);
    if (rc) return rc;
    launches += L.launches;
  }
  return SGPU_OK;
}

// Reads the stroke's counters and error word; fills stats (events ev0..ev1).
int finish_stroke(sgpu_mesh* mesh, int mode, int launches, SGPU_StrokeStats* stats) {
  int rc;
  unsigned long long displaced = 0;
  CK(cudaMemcpyAsync(&displaced, &mesh->dev.work->displaced, sizeof(displaced),
                     cudaMemcpyDeviceToHost, mesh->stream),
     "read counter");
  if ((rc = device_err(mesh))) return rc;
  if (stats) {
    float ms = 0.0f;
    CK(cudaEventElapsedTime(&ms, mesh->ev0, mesh->ev1), "elapsed");
    stats->verts_displaced = static_cast<int64_t>(displaced);
    stats->gpu_ms = ms;
    stats->kernel_launches = launches;
    stats->graph_nodes = mode == SGPU_STROKE_GRAPH ? mesh->g_nodes : 0;
  }
  return SGPU_OK;
}

}  // namespace

extern "C" {

int sgpu_get_verts(sgpu_mesh* mesh, SGPU_MVert* out) {
  int rc = check_mesh(mesh);
  if (rc) return rc;
  if (mesh->dev.type != kFaces) return fail(SGPU_ERR_INVALID_ARG, "not a FACES mesh");
  const DevMesh& d = mesh->dev;
  CK(launch_gather_f4(d.scratch, d.co, mesh->d_o2n, d.totvert, mesh->stream), "gather kernel");
  CK(cudaMemcpyAsync(out, d.scratch, sizeof(float4) * d.totvert, cudaMemcpyDeviceToHost,
                     mesh->stream),
     "download verts");
  CK(cudaStreamSynchronize(mesh->stream), "cudaStreamSynchronize");
  return SGPU_OK;
}

int sgpu_set_verts(sgpu_mesh* mesh, const SGPU_MVert* verts) {
  int rc = check_mesh(mesh);
  if (rc) return rc;
  if (mesh->dev.type != kFaces) return fail(SGPU_ERR_INVALID_ARG, "not a FACES mesh");
  const DevMesh& d = mesh->dev;
  CK(cudaMemcpyAsync(d.scratch, verts, sizeof(float4) * d.totvert, cudaMemcpyHostToDevice,
                     mesh->stream),
     "upload verts");
  CK(launch_gather_f4(d.co, d.scratch, mesh->d_n2o, d.totvert, mesh->stream), "gather kernel");
  CK(launch_chunk_boxes_all(mesh->dev, mesh->nchunks, mesh->stream), "chunk box kernel");
  CK(cudaStreamSynchronize(mesh->stream), "cudaStreamSynchronize");
  return SGPU_OK;
}

int sgpu_get_positions(sgpu_mesh* mesh, float* out_xyz) {
  int rc = check_mesh(mesh);
  if (rc) return rc;
  const DevMesh& d = mesh->dev;
  float* flat = reinterpret_cast<float*>(d.scratch);
  CK(launch_f4_to_xyz(flat, d.co, mesh->d_o2n, d.totvert, mesh->stream), "pack kernel");
  CK(cudaMemcpyAsync(out_xyz, flat, 3 * sizeof(float) * d.totvert, cudaMemcpyDeviceToHost,
                     mesh->stream),
     "download positions");
  CK(cudaStreamSynchronize(mesh->stream), "cudaStreamSynchronize");
  return SGPU_OK;
}

int sgpu_set_positions(sgpu_mesh* mesh, const float* xyz) {
  int rc = check_mesh(mesh);
  if (rc) return rc;
  const DevMesh& d = mesh->dev;
  float* flat = reinterpret_cast<float*>(d.scratch);
  CK(cudaMemcpyAsync(flat, xyz, 3 * sizeof(float) * d.totvert, cudaMemcpyHostToDevice, mesh->stream),
     "upload positions");
  CK(launch_xyz_to_f4(d.co, flat, mesh->d_n2o, d.totvert, true, mesh->stream), "unpack kernel");
  CK(launch_chunk_boxes_all(mesh->dev, mesh->nchunks, mesh->stream), "chunk box kernel");
  CK(cudaStreamSynchronize(mesh->stream), "cudaStreamSynchronize");
  return SGPU_OK;
}

int sgpu_get_normals(sgpu_mesh* mesh, float* out_xyz) {
  int rc = check_mesh(mesh);
  if (rc) return rc;
  const DevMesh& d = mesh->dev;
  float* flat = reinterpret_cast<float*>(d.scratch);
  CK(launch_f4_to_xyz(flat, d.no, mesh->d_o2n, d.totvert, mesh->stream), "pack kernel");
  CK(cudaMemcpyAsync(out_xyz, flat, 3 * sizeof(float) * d.totvert, cudaMemcpyDeviceToHost,
                     mesh->stream),
     "download normals");
  CK(cudaStreamSynchronize(mesh->stream), "cudaStreamSynchronize");
  return SGPU_OK;
}

int sgpu_get_mask(sgpu_mesh* mesh, float* out) {
  int rc = check_mesh(mesh);
  if (rc) return rc;
  if (!mesh->dev.mask) return fail(SGPU_ERR_INVALID_ARG, "mesh has no mask");
  const DevMesh& d = mesh->dev;
  const float* src = d.mask;
  if (mesh->d_o2n) {
    float* tmp = reinterpret_cast<float*>(d.scratch);
    CK(launch_gather_f1(tmp, d.mask, mesh->d_o2n, d.totvert, mesh->stream), "gather kernel");
    src = tmp;
  }
  CK(cudaMemcpyAsync(out, src, sizeof(float) * d.totvert, cudaMemcpyDeviceToHost, mesh->stream),
     "download mask");
  CK(cudaStreamSynchronize(mesh->stream), "cudaStreamSynchronize");
  return SGPU_OK;
}

int sgpu_get_node_bbs(sgpu_mesh* mesh, float* vb, float* orig_vb) {
  int rc = check_mesh(mesh);
  if (rc) return rc;
  const int N = mesh->dev.totnode;
  std::vector<float4> a(2 * static_cast<size_t>(N)), b(2 * static_cast<size_t>(N));
  CK(cudaMemcpyAsync(a.data(), mesh->dev.vb, sizeof(float4) * 2 * N, cudaMemcpyDeviceToHost,
                     mesh->stream),
     "download vb");
  CK(cudaMemcpyAsync(b.data(), mesh->dev.orig_vb, sizeof(float4) * 2 * N, cudaMemcpyDeviceToHost,
                     mesh->stream),
     "download orig_vb");
  CK(cudaStreamSynchronize(mesh->stream), "cudaStreamSynchronize");
  for (int n = 0; n < N; n++) {
    const float4 a0 = a[2 * n], a1 = a[2 * n + 1], b0 = b[2 * n], b1 = b[2 * n + 1];
    if (vb) {
      float* o = vb + 6 * static_cast<size_t>(n);
      o[0] = a0.x, o[1] = a0.y, o[2] = a0.z, o[3] = a1.x, o[4] = a1.y, o[5] = a1.z;
    }
    if (orig_vb) {
      float* o = orig_vb + 6 * static_cast<size_t>(n);
      o[0] = b0.x, o[1] = b0.y, o[2] = b0.z, o[3] = b1.x, o[4] = b1.y, o[5] = b1.z;
    }
  }
  return SGPU_OK;
}

int sgpu_get_nodes(sgpu_mesh* mesh, int* children_offset, int* flag, int* prim_off, int* totprim,
                   int* uniq_verts, int* face_verts, int* vert_off) {
  int rc = check_mesh(mesh);
  if (rc) return rc;
  const HostMesh& h = mesh->host;
  const int N = h.totnode, L = mesh->dev.nleaf;
  std::vector<int> lflag(L);
  CK(cudaMemcpyAsync(lflag.data(), mesh->dev.leaf_flag, sizeof(int) * L, cudaMemcpyDeviceToHost,
                     mesh->stream),
     "download flags");
  CK(cudaStreamSynchronize(mesh->stream), "cudaStreamSynchronize");
  for (int n = 0; n < N; n++) {
    const bool leaf = (h.flag[n] & kLeaf) != 0;
    if (children_offset) children_offset[n] = leaf ? -1 : h.children[n];
    if (flag) flag[n] = leaf ? lflag[h.node_leaf[n]] : h.flag[n];
    if (prim_off) prim_off[n] = leaf ? h.prim_off[n] : -1;
    if (totprim) totprim[n] = leaf ? h.totprim[n] : 0;
    if (uniq_verts) uniq_verts[n] = leaf ? h.uniq[n] : 0;
    if (face_verts) face_verts[n] = leaf ? h.face_verts_n[n] : 0;
    if (vert_off) vert_off[n] = leaf ? h.vert_off[n] : -1;
  }
  return SGPU_OK;
}

int sgpu_get_prim_indices(sgpu_mesh* mesh, int* out) {
  int rc = check_mesh(mesh);
  if (rc) return rc;
  std::memcpy(out, mesh->host.prim_indices.data(), sizeof(int) * mesh->host.prim_indices.size());
  return SGPU_OK;
}

int sgpu_get_vert_indices(sgpu_mesh* mesh, int* out) {
  int rc = check_mesh(mesh);
  if (rc) return rc;
  std::memcpy(out, mesh->host.vert_indices.data(), sizeof(int) * mesh->host.vert_indices.size());
  return SGPU_OK;
}

int sgpu_curve_table(int preset, float* table_xy, float* params) {
  Curve c;
  if (!build_curve(preset, &c)) return fail(SGPU_ERR_INVALID_ARG, "unknown curve preset %d", preset);
  if (table_xy)
    for (int a = 0; a <= kCurveTable; a++) {
      table_xy[2 * a] = c.table_x[a];
      table_xy[2 * a + 1] = c.y[a];
    }
  if (params) {
    params[0] = c.mintable;
    params[1] = c.maxtable;
    params[2] = c.range;
    params[3] = c.ext_in[0];
    params[4] = c.ext_in[1];
    params[5] = c.ext_out[0];
    params[6] = c.ext_out[1];
  }
  return SGPU_OK;
}

}  // extern "C"

namespace {

template <class T>
int ensure_dev(T** p, size_t* cap, size_t n) {
  if (*p && n <= *cap) return SGPU_OK;
  if (*p) cudaFree(*p);
  *p = nullptr;
  const size_t want = n > 0 ? n : 1;
  cudaError_t e = cudaMalloc(reinterpret_cast<void**>(p), want * sizeof(T));
  if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc");
  *cap = want;
  return SGPU_OK;
}

// One persistent launch over the meshes: jobs (whole strokes) are ordered by
// estimated work, longest first, and taken by cluster teams from a counter.
TuneKey stroke_key(const sgpu_mesh* m, const SGPU_Brush* b, const int* tools, int ndabs) {
  return TuneKey{0, m->dev.type, size_class(m->dev.totvert),
                 1 << __builtin_popcount(b->symmetry & 7), 1, tools_mask(b, tools, ndabs)};
}

TuneKey batch_key(sgpu_mesh* const* meshes, int n, const SGPU_Brush* brushes, const int* offs,
                  const int* tools) {
  long long verts = 0;
  unsigned mask = 0;
  for (int i = 0; i < n; i++) {
    verts += meshes[i]->dev.totvert;
    mask |= tools_mask(&brushes[i], tools ? tools + offs[i] : nullptr, offs[i + 1] - offs[i]);
  }
  return TuneKey{1, meshes[0]->dev.type, size_class(verts), 0, n, mask};
}

TeamShape mesh_team(const sgpu_mesh* m, const SGPU_Brush* b, const int* tools, int ndabs) {
  if (m->team_set) return TeamShape{m->team_cluster, m->team_build};
  std::lock_guard<std::mutex> lock(g_tune_mu);
  const auto it = g_tune.find(stroke_key(m, b, tools, ndabs));
  return it != g_tune.end() ? it->second : TeamShape{m->team_cluster, m->team_build};
}

int team_batch(sgpu_mesh** meshes, int n, const SGPU_Brush* brushes, const SGPU_Dab* dabs,
               const int* offs, const int* tools, TeamShape shape, cudaStream_t s,
               SGPU_StrokeStats* stats, float* total_ms, bool wait) {
  const int cluster = shape.cluster;
  sgpu_mesh* m0 = meshes[0];
  // strokes with grab, elastic deform or layer dabs keep the stroke-start
  // positions (stored on the launch stream below)
  static thread_local std::vector<char> h_orig;
  h_orig.assign(n, 0);
  int rc;
  for (int i = 0; i < n; i++)
    if (stroke_has_original(&brushes[i], tools ? tools + offs[i] : nullptr, offs[i + 1] - offs[i])) {
      if ((rc = ensure_original(meshes[i]))) return rc;
      h_orig[i] = 1;
    }
  int max_nodes = 0, max_leaves = 0;
  for (int i = 0; i < n; i++) {
    max_nodes = std::max(max_nodes, meshes[i]->dev.totnode);
    max_leaves = std::max(max_leaves, meshes[i]->dev.nleaf);
  }
  int max_parts = 0;
  for (int i = 0; i < n; i++)
    max_parts = std::max(max_parts, meshes[i]->dev.nleaf * meshes[i]->dev.area_blocks);
  if (max_leaves > 64 * 256 || max_parts > 64 * 256 ||
      team_smem_bytes(max_nodes, max_leaves) > 160 * 1024)
    return fail(SGPU_ERR_UNSUPPORTED, "PBVH too large for the persistent stroke kernel");
  const bool wide = cluster == SGPU_TEAM_GRID;
  const bool lock = cluster == SGPU_TEAM_LOCKSTEP;
  int wide_ctas = 0, lock_per_sm = 1;
  if (lock) {
    if (n > kLockMaxJobs)
      return fail(SGPU_ERR_UNSUPPORTED, "the lockstep launch takes at most %d meshes", kLockMaxJobs);
    for (int i = 0; i < n; i++) {
      if (h_orig[i])
        return fail(SGPU_ERR_UNSUPPORTED,
                    "the lockstep launch runs no grab, elastic deform or layer dabs");
      const DevMesh& d = meshes[i]->dev;
      if (d.type == kGrids && !lock_grids_fit(d.grid_size))
        return fail(SGPU_ERR_UNSUPPORTED, "grids of %d x %d do not fit the lockstep launch's stage",
                    d.grid_size, d.grid_size);
    }
    // every pooled item space fits an int, even with every leaf culled
    double runs = 0.0, parts = 0.0, chunks = 0.0, verts = 0.0;
    for (int i = 0; i < n; i++) {
      const DevMesh& d = meshes[i]->dev;
      runs += static_cast<double>(d.nleaf) * ((d.max_leaf_verts + 31) / 32);
      parts += static_cast<double>(d.nleaf) * d.area_blocks;
      chunks += static_cast<double>(d.nleaf) * d.max_leaf_chunks;
      verts += static_cast<double>(d.totvert) + d.num_faces;
    }
    if (std::max(std::max(runs, parts), std::max(chunks, verts)) >= 2147483647.0)
      return fail(SGPU_ERR_UNSUPPORTED, "batch too large for one lockstep launch");
    if (shape.ctas_per_sm != 0 && shape.ctas_per_sm != 1 && shape.ctas_per_sm != 2)
      return fail(SGPU_ERR_INVALID_ARG, "CTAs per SM must be 1 or 2");
    lock_per_sm = g_lock_per_sm.load() ? g_lock_per_sm.load() : (shape.ctas_per_sm == 2 ? 2 : 1);
    wide_ctas = lock_ctas(max_nodes, max_leaves, lock_per_sm);
    if (wide_ctas <= 0)
      return fail(SGPU_ERR_UNSUPPORTED, "the lockstep launch cannot run on this device");
    // barriers: at most 8 passes of at most 8 per dab, 4 more per dab, 1 at
    // the start
    int maxd = 0;
    for (int i = 0; i < n; i++) maxd = std::max(maxd, offs[i + 1] - offs[i]);
    if ((72.0 * maxd + 8.0) * (wide_ctas + 1) >= 2147483648.0)
      return fail(SGPU_ERR_UNSUPPORTED, "too many dabs for one lockstep launch");
  } else if (wide) {
    wide_ctas = team_wide_ctas(max_nodes, max_leaves);
    if (wide_ctas <= 0)
      return fail(SGPU_ERR_UNSUPPORTED, "the whole-GPU team cannot be launched on this device");
    // the barrier counter holds (barriers so far) * CTAs below its abort bit:
    // at most 8 passes of at most 8 barriers per dab, plus 8 per stroke
    double barriers = 0.0;
    for (int i = 0; i < n; i++) barriers += 64.0 * (offs[i + 1] - offs[i]) + 8.0;
    if (barriers * (wide_ctas + 1) >= 2147483648.0)
      return fail(SGPU_ERR_UNSUPPORTED, "too many dabs for one whole-GPU launch");
  } else if (cluster < 1 || cluster > 16 || (cluster & (cluster - 1)) != 0) {
    return fail(SGPU_ERR_INVALID_ARG, "cluster size %d is not 1, 2, 4, 8 or 16", cluster);
  } else if (team_max_active_clusters(cluster, max_nodes, max_leaves) <= 0) {
    return fail(SGPU_ERR_UNSUPPORTED, "cluster size %d cannot be launched", cluster);
  }
  // staging buffers live on the first mesh; re-create when too small
  static thread_local std::vector<DevMesh> h_meshes;
  static thread_local std::vector<TeamJob> h_jobs;
  h_meshes.assign(n, DevMesh{});
  h_jobs.assign(n, TeamJob{});
  const size_t ndab = static_cast<size_t>(offs[n]);
  if ((rc = ensure_dev(&m0->t_dabs, &m0->t_dab_cap, ndab * 6))) return rc;
  if (tools && (rc = ensure_dev(&m0->t_tools, &m0->t_tool_cap, ndab))) return rc;
  if ((rc = ensure_dev(&m0->t_meshes, &m0->t_mesh_cap, static_cast<size_t>(n)))) return rc;
  if ((rc = ensure_dev(&m0->t_jobs, &m0->t_job_cap, static_cast<size_t>(n)))) return rc;
  // [0] job counter, [1] whole-GPU barrier counter, [2] status word
  if ((rc = ensure_dev(&m0->t_counter, &m0->t_counter_cap, 4))) return rc;
  if (lock) {
    if ((rc = ensure_dev(&m0->t_lock, &m0->t_lock_cap, static_cast<size_t>(n)))) return rc;
    if ((rc = ensure_dev(&m0->t_lbrush, &m0->t_lbrush_cap, static_cast<size_t>(n)))) return rc;
  }
  std::vector<int> order(n);
  std::vector<double> est(n);
  for (int i = 0; i < n; i++) {
    order[i] = i;
    const double r = brushes[i].radius;
    const int nd = offs[i + 1] - offs[i];
    const int passes = 1 << __builtin_popcount(brushes[i].symmetry & 7);
    est[i] = static_cast<double>(nd) * passes *
             (static_cast<double>(meshes[i]->dev.totvert) * r * r + 64.0 * meshes[i]->dev.nleaf);
  }
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return est[a] > est[b]; });
  for (int j = 0; j < n; j++) {
    const int i = order[j];
    h_meshes[j] = meshes[i]->dev;
    h_meshes[j].prof = nullptr;
    TeamJob& job = h_jobs[j];
    job.mesh = j;
    job.ndabs = offs[i + 1] - offs[i];
    job.symmetry = brushes[i].symmetry & 7;
    job.use_orig = brushes[i].use_original_bb;
    for (int k = 0; k < 3; k++) job.view[k] = brushes[i].view_normal[k];
    job.dabs = m0->t_dabs + static_cast<size_t>(offs[i]) * 6;
    job.tools = tools ? m0->t_tools + offs[i] : nullptr;
    if (!make_brush(&brushes[i], brushes[i].sculpt_tool, &job.brush))
      return fail(SGPU_ERR_INVALID_ARG, "unknown curve preset %d", brushes[i].curve_preset);
    // Kelvinlet constants of the stroke; the kernel sets the force per dab
    const float no_delta[3] = {0.0f, 0.0f, 0.0f};
    kelvinlet_params(&job.brush, no_delta, brushes[i].elastic_deform_volume_preservation);
  }
  CK(cudaEventRecord(m0->ev0, s), "event");
  for (int i = 0; i < n; i++)
    if (h_orig[i] && (rc = copy_original(meshes[i], s))) return rc;
  if (ndab)
    CK(cudaMemcpyAsync(m0->t_dabs, dabs, sizeof(SGPU_Dab) * ndab, cudaMemcpyHostToDevice, s),
       "upload dabs");
  if (tools && ndab)
    CK(cudaMemcpyAsync(m0->t_tools, tools, sizeof(int) * ndab, cudaMemcpyHostToDevice, s),
       "upload tools");
  CK(cudaMemcpyAsync(m0->t_meshes, h_meshes.data(), sizeof(DevMesh) * n, cudaMemcpyHostToDevice, s),
     "upload mesh table");
  CK(cudaMemcpyAsync(m0->t_jobs, h_jobs.data(), sizeof(TeamJob) * n, cudaMemcpyHostToDevice, s),
     "upload jobs");
  CK(cudaMemsetAsync(m0->t_counter, 0, 3 * sizeof(int), s), "reset job and barrier counters");
  if (lock) {
    static thread_local std::vector<DevBrush> h_lbrush;
    h_lbrush.resize(n);
    for (int j = 0; j < n; j++) h_lbrush[j] = h_jobs[j].brush;
    CK(cudaMemcpyAsync(m0->t_lbrush, h_lbrush.data(), sizeof(DevBrush) * n, cudaMemcpyHostToDevice,
                       s),
       "upload brushes");
    CK(cudaMemsetAsync(m0->t_lock, 0, sizeof(LockJob) * n, s), "reset lockstep state");
  }
  for (int i = 0; i < n; i++)
    CK(cudaMemsetAsync(&meshes[i]->dev.work->displaced, 0, sizeof(unsigned long long), s),
       "reset counter");
  TeamArgs a;
  a.meshes = m0->t_meshes;
  a.jobs = m0->t_jobs;
  a.njobs = n;
  a.next_job = m0->t_counter;
  a.orig = 0;
  for (int i = 0; i < n; i++) a.orig |= h_orig[i];
  a.two_level = 0;
  for (int i = 0; i < n; i++) a.two_level |= meshes[i]->dev.cull_ntop > 0 ? 1 : 0;
  a.sym = 0;
  for (int i = 0; i < n; i++) {
    const int sy = brushes[i].symmetry & 7;
    a.sym |= (sy == 1 || sy == 2 || sy == 4) ? 1 : 0;
  }
  a.max_nodes = max_nodes;
  a.max_leaves = max_leaves;
  a.prof_bytes = g_team_prof_bytes;
  a.phase_ns = g_team_phase_ns;
  a.bar = reinterpret_cast<unsigned int*>(m0->t_counter + 1);
  a.status = m0->t_counter + 2;
  a.wait_ns = g_wait_ns.load();
  a.bar_extra = g_bar_extra.load();
  a.lock = lock ? m0->t_lock : nullptr;
  a.lbrush = lock ? m0->t_lbrush : nullptr;
  if (lock) {
    CK(launch_lock_stroke(a, wide_ctas, lock_per_sm, s),
       "persistent stroke kernel (lockstep batch)");
  } else if (wide) {
    CK(launch_team_stroke_wide(a, wide_ctas, s), "persistent stroke kernel (whole GPU)");
  } else {
    CK(launch_team_stroke(a, cluster, s, shape.ctas_per_sm), "persistent stroke kernel");
  }
  CK(cudaEventRecord(m0->ev1, s), "event");
  // page-locked: n displaced counters, then the status word
  if (m0->h_disp_cap < static_cast<size_t>(n) + 1) {
    if (m0->h_disp) cudaFreeHost(m0->h_disp);
    m0->h_disp = nullptr;
    m0->h_disp_cap = 0;
    CK(cudaHostAlloc(reinterpret_cast<void**>(&m0->h_disp), sizeof(unsigned long long) * (n + 1),
                     cudaHostAllocDefault),
       "cudaHostAlloc");
    m0->h_disp_cap = static_cast<size_t>(n) + 1;
  }
  unsigned long long* disp = m0->h_disp;
  for (int i = 0; i < n; i++)
    CK(cudaMemcpyAsync(&disp[i], &meshes[i]->dev.work->displaced, sizeof(unsigned long long),
                       cudaMemcpyDeviceToHost, s),
       "read counter");
  disp[n] = 0ull;
  CK(cudaMemcpyAsync(&disp[n], a.status, sizeof(int), cudaMemcpyDeviceToHost, s), "read status");
  if (!wait) return SGPU_OK;
  CK(cudaStreamSynchronize(s), "cudaStreamSynchronize");
  float ms = 0.0f;
  CK(cudaEventElapsedTime(&ms, m0->ev0, m0->ev1), "elapsed");
  if (const int status = static_cast<int>(disp[n]))
    return fail(status, "persistent stroke kernel: a team barrier wait ran out (error %d); the "
                "stroke is incomplete", status);
  for (int i = 0; i < n; i++) {
    if ((rc = device_err(meshes[i]))) return rc;
    if (stats) {
      stats[i].verts_displaced = static_cast<int64_t>(disp[i]);
      stats[i].gpu_ms = ms;
      stats[i].kernel_launches = (i == 0) ? 1 : 0;
      stats[i].graph_nodes = 0;
    }
  }
  if (total_ms) *total_ms = ms;
  return SGPU_OK;
}

}  // namespace

namespace {

// Byte offsets in the ray-cast blocks for a capacity of n rays.
struct RayLayout {
  size_t in, out_f, out_i, err, total;
  explicit RayLayout(size_t n)
      : in(0), out_f(sizeof(float) * 7 * n), out_i(out_f + sizeof(float) * 4 * n),
        err(out_i + sizeof(int) * 3 * n), total(err + 16) {}
};

// Ray-cast buffers for up to n rays (grown, never shrunk; growing drops the
// captured call).
int ensure_ray_buffers(sgpu_mesh* m, int n) {
  if (static_cast<size_t>(n) <= m->ray_cap && m->ray_dev) return SGPU_OK;
  const int L = m->dev.nleaf;
  const size_t slots = static_cast<size_t>(n) * L;
  const size_t items = static_cast<size_t>(n) * ray_items_per_ray(m->dev);
  if (items > 0x7fffffffull) return fail(SGPU_ERR_UNSUPPORTED, "ray batch too large for the mesh");
  if (m->ray_graph) cudaGraphExecDestroy(m->ray_graph);
  m->ray_graph = nullptr;
  m->ray_graph_n = m->ray_graph_orig = -1;
  void* p[14] = {m->ray_dev,         m->ray.count,    m->ray.slot_leaf, m->ray.slot_tmin,
                 m->ray.slot_order,  m->ray.slot_key, m->ray.items,     m->ray.nitems,
                 m->ray.slot_special, m->ray.items2,  m->ray.nitems2,   m->ray.st_depth,
                 m->ray.st_run,      m->ray.st_win};
  for (void* q : p)
    if (q) cudaFree(q);
  if (m->ray_host) cudaFreeHost(m->ray_host);
  m->ray = RayBatch{};
  m->ray_dev = m->ray_host = nullptr;
  m->ray_cap = 0;
  const RayLayout lay(static_cast<size_t>(n));
  CK(cudaMalloc(&m->ray_dev, lay.total), "cudaMalloc");
  CK(cudaHostAlloc(reinterpret_cast<void**>(&m->ray_host), lay.total, cudaHostAllocDefault),
     "cudaHostAlloc");
  CK(cudaMalloc(&m->ray.count, sizeof(int) * n), "cudaMalloc");
  CK(cudaMalloc(&m->ray.slot_leaf, sizeof(int) * slots), "cudaMalloc");
  CK(cudaMalloc(&m->ray.slot_tmin, sizeof(float) * slots), "cudaMalloc");
  CK(cudaMalloc(&m->ray.slot_order, sizeof(int) * slots), "cudaMalloc");
  CK(cudaMalloc(&m->ray.slot_key, sizeof(unsigned long long) * slots), "cudaMalloc");
  CK(cudaMalloc(&m->ray.slot_special, sizeof(int) * slots), "cudaMalloc");
  CK(cudaMalloc(&m->ray.items, sizeof(int2) * items), "cudaMalloc");
  CK(cudaMalloc(&m->ray.nitems, sizeof(int)), "cudaMalloc");
  CK(cudaMalloc(&m->ray.items2, sizeof(int2) * items), "cudaMalloc");
  CK(cudaMalloc(&m->ray.nitems2, sizeof(int)), "cudaMalloc");
  CK(cudaMalloc(&m->ray.st_depth, sizeof(float) * n), "cudaMalloc");
  CK(cudaMalloc(&m->ray.st_run, sizeof(float) * n), "cudaMalloc");
  CK(cudaMalloc(&m->ray.st_win, sizeof(int4) * n), "cudaMalloc");
  m->ray.item_cap = static_cast<int>(items);
  m->ray_cap = static_cast<size_t>(n);
  return SGPU_OK;
}


// One batch of independent ray queries through the cached graph of its shape
// (rays, original, mode): the ray cast (nearest = false) or the nearest-to-ray
// query (starting squared distance FLT_MAX; r_dist_sq receives the result).
int ray_query(sgpu_mesh* mesh, int nrays, const float* ray_starts, const float* ray_normals,
              const float* ray_lengths, int original, bool nearest, float* r_depths, int* r_hits,
              int* r_active_vertices, int* r_active_faces, float* r_face_normals,
              float* r_dist_sq) {
  int rc = check_mesh(mesh);
  if (rc) return rc;
  if (nrays < 0) return fail(SGPU_ERR_INVALID_ARG, "negative ray count");
  if (nrays == 0) return SGPU_OK;
  if (!ray_starts || !ray_normals || !r_depths || !r_hits)
    return fail(SGPU_ERR_INVALID_ARG, "NULL ray or result array");
  if ((rc = ensure_ray_buffers(mesh, nrays))) return rc;
  DevMesh& d = mesh->dev;
  if (!mesh->ray_configured) {
    CK(configure_ray_kernels(ray_leaves_smem(d), ray_finish_smem(d)), "ray kernel attributes");
    mesh->ray_configured = true;
  }
  // inputs and outputs live at the offsets of a batch of exactly nrays rays
  const RayLayout lay(static_cast<size_t>(nrays));
  float* hin = reinterpret_cast<float*>(mesh->ray_host + lay.in);
  for (int r = 0; r < nrays; r++) {
    for (int k = 0; k < 3; k++) {
      hin[6 * r + k] = ray_starts[3 * r + k];
      hin[6 * r + 3 + k] = ray_normals[3 * r + k];
    }
    hin[6 * static_cast<size_t>(nrays) + r] = ray_lengths ? ray_lengths[r] : FLT_MAX;
  }
  cudaStream_t s = mesh->stream;
  if (!mesh->ray_graph || mesh->ray_graph_n != nrays || mesh->ray_graph_orig != original ||
      mesh->ray_graph_near != static_cast<int>(nearest)) {
    if (mesh->ray_graph) cudaGraphExecDestroy(mesh->ray_graph);
    mesh->ray_graph = nullptr;
    RayBatch rb = mesh->ray;
    float* din = reinterpret_cast<float*>(mesh->ray_dev + lay.in);
    float* dout = reinterpret_cast<float*>(mesh->ray_dev + lay.out_f);
    int* diout = reinterpret_cast<int*>(mesh->ray_dev + lay.out_i);
    rb.rays = din;
    rb.depth_in = din + 6 * static_cast<size_t>(nrays);
    rb.original = original;
    rb.nearest = nearest ? 1 : 0;
    rb.n2o = mesh->d_n2o;
    // small batches (an interactive cursor ray) in one round: the second
    // round's launches cost more latency than its saved work
    rb.first_leaves = nrays <= 64 ? d.nleaf : 2;
    rb.depth_out = dout;
    rb.face_normal = dout + nrays;
    rb.hit = diout;
    rb.active_vertex = diout + nrays;
    rb.active_face = diout + 2 * static_cast<size_t>(nrays);
    int sms = 0, dev = 0;
    CK(cudaGetDevice(&dev), "cudaGetDevice");
    CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "device attribute");
    // one graph: rays in, the three kernels, results and error word out
    cudaGraph_t graph = nullptr;
    CK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal), "begin capture");
    cudaError_t e = cudaMemcpyAsync(mesh->ray_dev + lay.in, mesh->ray_host + lay.in,
                                    lay.out_f - lay.in, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = launch_raycast(d, rb, nrays, 8 * sms, s);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(mesh->ray_host + lay.out_f, mesh->ray_dev + lay.out_f,
                          lay.err - lay.out_f, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(mesh->ray_host + lay.err, &d.work->err, sizeof(int),
                          cudaMemcpyDeviceToHost, s);
    const cudaError_t e2 = cudaStreamEndCapture(s, &graph);
    if (e == cudaSuccess) e = e2;
    if (e == cudaSuccess) e = cudaGraphInstantiate(&mesh->ray_graph, graph, 0);
    if (graph) cudaGraphDestroy(graph);
    if (e != cudaSuccess) {
      mesh->ray_graph = nullptr;
      return cuda_fail(e, "ray-query graph");
    }
    mesh->ray_graph_n = nrays;
    mesh->ray_graph_orig = original;
    mesh->ray_graph_near = static_cast<int>(nearest);
  }
  CK(cudaGraphLaunch(mesh->ray_graph, s), "ray-query graph launch");
  CK(cudaStreamSynchronize(s), "cudaStreamSynchronize");
  const int err = *reinterpret_cast<int*>(mesh->ray_host + lay.err);
  if (err) {
    CK(cudaMemsetAsync(&d.work->err, 0, sizeof(int), s), "reset error word");
    CK(cudaStreamSynchronize(s), "cudaStreamSynchronize");
    return fail(err, "a ray-query kernel reported error code %d", err);
  }
  const float* fo = reinterpret_cast<const float*>(mesh->ray_host + lay.out_f);
  const int* io = reinterpret_cast<const int*>(mesh->ray_host + lay.out_i);
  for (int r = 0; r < nrays; r++) {
    r_depths[r] = fo[r];
    r_hits[r] = io[r];
    if (r_active_vertices) r_active_vertices[r] = io[nrays + r];
    if (r_active_faces) r_active_faces[r] = io[2 * static_cast<size_t>(nrays) + r];
    if (r_face_normals)
      for (int k = 0; k < 3; k++) r_face_normals[3 * r + k] = fo[nrays + 3 * static_cast<size_t>(r) + k];
    if (r_dist_sq) r_dist_sq[r] = fo[nrays + 3 * static_cast<size_t>(r)];
  }
  return SGPU_OK;
}

}  // namespace

extern "C" {

int sgpu_raycast(sgpu_mesh* mesh, int nrays, const float* ray_starts, const float* ray_normals,
                 const float* ray_lengths, int original, float* r_depths, int* r_hits,
                 int* r_active_vertices, int* r_active_faces, float* r_face_normals) {
  return ray_query(mesh, nrays, ray_starts, ray_normals, ray_lengths, original, false, r_depths,
                   r_hits, r_active_vertices, r_active_faces, r_face_normals, nullptr);
}

int sgpu_find_nearest_to_ray(sgpu_mesh* mesh, int nrays, const float* ray_starts,
                             const float* ray_normals, int original, float* r_depths,
                             float* r_dist_sq, int* r_hits) {
  if (nrays > 0 && !r_dist_sq) return fail(SGPU_ERR_INVALID_ARG, "NULL result array");
  return ray_query(mesh, nrays, ray_starts, ray_normals, nullptr, original, true, r_depths, r_hits,
                   nullptr, nullptr, nullptr, r_dist_sq);
}

}  // extern "C"

namespace {

// One device array for the draw buffers, copied from src (count elements) or
// zeroed when src is null.
template <class T>
int draw_array(sgpu_mesh* m, T** out, const T* src, size_t count) {
  void* p = nullptr;
  const size_t bytes = (count > 0 ? count : 1) * sizeof(T);
  cudaError_t e = cudaMalloc(&p, bytes);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc (draw buffers)");
  m->draw_allocs.push_back(p);
  if (src && count > 0)
    e = cudaMemcpyAsync(p, src, count * sizeof(T), cudaMemcpyHostToDevice, m->stream);
  else
    e = cudaMemsetAsync(p, 0, bytes, m->stream);
  if (e != cudaSuccess) return cuda_fail(e, "draw buffer upload");
  *out = static_cast<T*>(p);
  return SGPU_OK;
}

}  // namespace

extern "C" {

int sgpu_draw_buffers_build(sgpu_mesh* mesh, const SGPU_DrawSetup* setup) {
  int rc = check_mesh(mesh);
  if (rc) return rc;
  HostMesh& h = mesh->host;
  DevMesh& d = mesh->dev;
  DrawInputs in;
  if (setup) {
    in.face_sets = setup->face_sets;
    in.seed = setup->face_sets_color_seed;
    in.color_default = setup->face_sets_color_default;
    in.loop_colors = h.type == kFaces ? setup->loop_colors : nullptr;
    in.vert_colors = h.type == kFaces ? setup->vert_colors : nullptr;
    in.use_vert_colors = setup->use_sculpt_vertex_colors != 0;
    in.grid_flag_mats = reinterpret_cast<const unsigned char*>(setup->grid_flag_mats);
  }
  if (h.type == kFaces) {
    // the current MVert flags (ME_HIDE) ride in the w word of the device positions
    std::vector<float4> co4(h.totvert);
    CK(cudaMemcpyAsync(co4.data(), d.co, sizeof(float4) * co4.size(), cudaMemcpyDeviceToHost,
                       mesh->stream),
       "read vertex flags");
    CK(cudaStreamSynchronize(mesh->stream), "cudaStreamSynchronize");
    in.o2n = mesh->o2n.data();
    in.vert_flag.resize(h.totvert);
    for (int v = 0; v < h.totvert; v++) {
      unsigned char b[4];
      std::memcpy(b, &co4[mesh->o2n[v]].w, 4);
      in.vert_flag[v] = b[0];
    }
  }
  mesh->free_draw();
  std::string err;
  if (!build_draw_layout(h, in, &mesh->draw, &err)) return fail(SGPU_ERR_INVALID_ARG, "%s", err.c_str());
  const DrawLayout& L = mesh->draw;
  DrawDev& dd = mesh->draw_dev;
  const size_t words = static_cast<size_t>(L.total_verts) * kDrawWords;
  if ((rc = draw_array<unsigned int>(mesh, &dd.vbo, nullptr, words))) return rc;
  long long* lvo = nullptr;
  int *lts = nullptr, *ltc = nullptr, *lsm = nullptr, *tv4 = nullptr;
  unsigned int *fset = nullptr, *col = nullptr;
  if ((rc = draw_array(mesh, &lvo, L.leaf_vert_off.data(), L.leaf_vert_off.size())) ||
      (rc = draw_array(mesh, &lts, L.leaf_tri_start.data(), L.leaf_tri_start.size())) ||
      (rc = draw_array(mesh, &ltc, L.leaf_tri_count.data(), L.leaf_tri_count.size())) ||
      (rc = draw_array(mesh, &lsm, L.leaf_smooth.data(), L.leaf_smooth.size())) ||
      (rc = draw_array(mesh, &tv4, L.tri_v4.data(), L.tri_v4.size())) ||
      (rc = draw_array<int>(mesh, &dd.overlay, nullptr, static_cast<size_t>(d.nleaf))) ||
      (rc = draw_array<int>(mesh, &dd.overlay_acc, nullptr, static_cast<size_t>(d.nleaf))))
    return rc;
  if (L.has_fset && (rc = draw_array(mesh, &fset, L.fset.data(), L.fset.size()))) return rc;
  if (L.show_vcol && (rc = draw_array(mesh, &col, L.col.data(), L.col.size()))) return rc;
  dd.leaf_vert_off = lvo;
  dd.leaf_tri_start = lts;
  dd.leaf_tri_count = ltc;
  dd.leaf_smooth = lsm;
  dd.tri_v4 = tv4;
  dd.fset = fset;
  dd.col = col;
  // every leaf rebuilt and refilled at the next update (BKE_pbvh_node_mark_rebuild_draw)
  CK(launch_mark_all(d, kRebuildDrawBuffers | kUpdateDrawBuffers, mesh->stream), "mark kernel");
  CK(cudaStreamSynchronize(mesh->stream), "cudaStreamSynchronize");
  mesh->draw_built = true;
  return SGPU_OK;
}

int sgpu_draw_buffers_update(sgpu_mesh* mesh) {
  int rc = check_mesh(mesh);
  if (rc) return rc;
  if (!mesh->draw_built) return fail(SGPU_ERR_INVALID_ARG, "draw buffers not built");
  CK(launch_draw_fill(mesh->dev, mesh->draw_dev, mesh->draw.max_units_smooth,
                      mesh->draw.max_units_flat, mesh->stream), "draw fill kernel");
  return SGPU_OK;
}

int sgpu_draw_buffers_update_timed(sgpu_mesh* mesh, int all_leaves, float* gpu_ms) {
  int rc = check_mesh(mesh);
  if (rc) return rc;
  if (!mesh->draw_built) return fail(SGPU_ERR_INVALID_ARG, "draw buffers not built");
  if (all_leaves) CK(launch_mark_all(mesh->dev, kUpdateDrawBuffers, mesh->stream), "mark kernel");
  CK(cudaEventRecord(mesh->ev0, mesh->stream), "cudaEventRecord");
  CK(launch_draw_fill(mesh->dev, mesh->draw_dev, mesh->draw.max_units_smooth,
                      mesh->draw.max_units_flat, mesh->stream), "draw fill kernel");
  CK(cudaEventRecord(mesh->ev1, mesh->stream), "cudaEventRecord");
  CK(cudaEventSynchronize(mesh->ev1), "cudaEventSynchronize");
  float ms = 0.0f;
  CK(cudaEventElapsedTime(&ms, mesh->ev0, mesh->ev1), "elapsed");
  if (gpu_ms) *gpu_ms = ms;
  return SGPU_OK;
}

int sgpu_draw_buffers_layout(sgpu_mesh* mesh, int64_t* vert_off, int* tot_tri, int* smooth,
                             int* material_index) {
  int rc = check_mesh(mesh);
  if (rc) return rc;
  if (!mesh->draw_built) return fail(SGPU_ERR_INVALID_ARG, "draw buffers not built");
  const DrawLayout& L = mesh->draw;
  const size_t n = L.node_tot_tri.size();
  if (vert_off) std::memcpy(vert_off, L.node_vert_off.data(), sizeof(int64_t) * (n + 1));
  if (tot_tri) std::memcpy(tot_tri, L.node_tot_tri.data(), sizeof(int) * n);
  if (smooth) std::memcpy(smooth, L.node_smooth.data(), sizeof(int) * n);
  if (material_index) std::memcpy(material_index, L.node_material.data(), sizeof(int) * n);
  return SGPU_OK;
}

int sgpu_draw_buffers_overlay(sgpu_mesh* mesh, int* show_overlay) {
  int rc = check_mesh(mesh);
  if (rc) return rc;
  if (!mesh->draw_built) return fail(SGPU_ERR_INVALID_ARG, "draw buffers not built");
  if (!show_overlay) return fail(SGPU_ERR_INVALID_ARG, "NULL output");
  std::vector<int> ov(mesh->dev.nleaf);
  CK(cudaMemcpyAsync(ov.data(), mesh->draw_dev.overlay, sizeof(int) * ov.size(),
                     cudaMemcpyDeviceToHost, mesh->stream),
     "read overlay flags");
  CK(cudaStreamSynchronize(mesh->stream), "cudaStreamSynchronize");
  const HostMesh& h = mesh->host;
  for (int n = 0; n < h.totnode; n++) show_overlay[n] = h.node_leaf[n] >= 0 ? ov[h.node_leaf[n]] : 0;
  return SGPU_OK;
}

int sgpu_draw_buffers_get(sgpu_mesh* mesh, void* dst, size_t bytes) {
  int rc = check_mesh(mesh);
  if (rc) return rc;
  if (!mesh->draw_built) return fail(SGPU_ERR_INVALID_ARG, "draw buffers not built");
  const size_t need = static_cast<size_t>(mesh->draw.total_verts) * SGPU_DRAW_STRIDE;
  if (!dst || bytes < need) return fail(SGPU_ERR_INVALID_ARG, "destination smaller than %zu bytes", need);
  if (need > 0)
    CK(cudaMemcpyAsync(dst, mesh->draw_dev.vbo, need, cudaMemcpyDeviceToHost, mesh->stream),
       "read draw buffers");
  CK(cudaStreamSynchronize(mesh->stream), "cudaStreamSynchronize");
  return SGPU_OK;
}

int sgpu_draw_buffers_device(sgpu_mesh* mesh, void** d_vbo, size_t* bytes) {
  int rc = check_mesh(mesh);
  if (rc) return rc;
  if (!mesh->draw_built) return fail(SGPU_ERR_INVALID_ARG, "draw buffers not built");
  if (d_vbo) *d_vbo = mesh->draw_dev.vbo;
  if (bytes) *bytes = static_cast<size_t>(mesh->draw.total_verts) * SGPU_DRAW_STRIDE;
  return SGPU_OK;
}

}  // extern "C"
