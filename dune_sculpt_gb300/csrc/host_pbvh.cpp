// Host PBVH build, topology tables and falloff curve tables of libsculptgpu.
//
// The PBVH is built once per mesh on the host, exactly as the reference builds
// it (source/dune/kernel/intern/pbvh.c:1973-2561): same split axis, same
// partition, same node numbering and the same unique/shared vertex order per
// leaf, so node lists and bounding boxes computed on the device can be compared
// bit for bit with the reference's.  Compiled with -ffp-contract=off.
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>

#include "sgpu_host.h"

namespace sgpu {
namespace {

inline float fmin_ref(float a, float b) { return (a < b) ? a : b; }  // min_ff
inline float fmax_ref(float a, float b) { return (a > b) ? a : b; }  // max_ff

struct Box {
  float mn[3], mx[3];
  void reset() {  // BB_reset, pbvh.c:1973-1977
    mn[0] = mn[1] = mn[2] = FLT_MAX;
    mx[0] = mx[1] = mx[2] = -FLT_MAX;
  }
  void expand(const float* co) {  // BB_expand, pbvh.c:1979-1985
    for (int i = 0; i < 3; i++) {
      mn[i] = fmin_ref(mn[i], co[i]);
      mx[i] = fmax_ref(mx[i], co[i]);
    }
  }
  void expand(const Box& b) {  // BB_expand_with_bb, pbvh.c:1987-1993
    for (int i = 0; i < 3; i++) {
      mn[i] = fmin_ref(mn[i], b.mn[i]);
      mx[i] = fmax_ref(mx[i], b.mx[i]);
    }
  }
  int widest_axis() const {  // BB_widest_axis, pbvh.c:1995-2016
    float d0 = mx[0] - mn[0], d1 = mx[1] - mn[1], d2 = mx[2] - mn[2];
    if (d0 > d1) return d0 > d2 ? 0 : 2;
    return d1 > d2 ? 1 : 2;
  }
};

struct PrimBox {
  Box bb;
  float c[3];  // BBC_update_centroid, pbvh.c:2018-2023
};

class Builder {
 public:
  explicit Builder(HostMesh& m) : m_(m) {}

  void run(const std::vector<PrimBox>& prims, const Box& cb) {
    prims_ = &prims;
    const int n = static_cast<int>(prims.size());
    m_.prim_indices.resize(n);
    for (int i = 0; i < n; i++) m_.prim_indices[i] = i;
    node_cap_ = 0;
    grow(100);
    m_.totnode = 1;
    if (m_.type == kFaces) {
      bitmap_.assign(m_.totvert, 0);
      stamp_.assign(m_.totvert, 0);
      value_.assign(m_.totvert, 0);
    }
    sub(0, &cb, 0, n);
    m_.children.resize(m_.totnode);
    m_.flag.resize(m_.totnode);
    m_.prim_off.resize(m_.totnode);
    m_.totprim.resize(m_.totnode);
    m_.uniq.resize(m_.totnode);
    m_.face_verts_n.resize(m_.totnode);
    m_.vert_off.resize(m_.totnode);
    m_.vb.resize(6 * static_cast<size_t>(m_.totnode));
  }

 private:
  // pbvh_grow_nodes, pbvh.c:2133-2144 (capacity growth only affects memory).
  void grow(int totnode) {
    if (totnode > node_cap_) {
      int cap = node_cap_ + node_cap_ / 3;
      if (cap < totnode) cap = totnode;
      m_.children.resize(cap, -1);
      m_.flag.resize(cap, 0);
      m_.prim_off.resize(cap, -1);
      m_.totprim.resize(cap, 0);
      m_.uniq.resize(cap, 0);
      m_.face_verts_n.resize(cap, 0);
      m_.vert_off.resize(cap, -1);
      m_.vb.resize(6 * static_cast<size_t>(cap), 0.0f);
      node_cap_ = cap;
    }
    m_.totnode = totnode;
  }

  // update_vb, pbvh.c:2240-2247: union of the primitive boxes, last to first.
  void update_vb(int node, int offset, int count) {
    Box b;
    b.reset();
    for (int i = offset + count - 1; i >= offset; i--) b.expand((*prims_)[m_.prim_indices[i]].bb);
    float* out = &m_.vb[6 * static_cast<size_t>(node)];
    for (int k = 0; k < 3; k++) {
      out[k] = b.mn[k];
      out[3 + k] = b.mx[k];
    }
  }

  bool materials_match(int pa, int pb) const {  // pbvh.c:2058-2066
    if (m_.type != kFaces) return true;
    const int a = m_.lt_poly[pa], b = m_.lt_poly[pb];
    return ((m_.poly_flag[a] & 1) == (m_.poly_flag[b] & 1)) && (m_.poly_mat[a] == m_.poly_mat[b]);
  }

  bool needs_material_split(int offset, int count) const {  // pbvh.c:2329-2362
    if (count <= 1) return false;
    const int first = m_.prim_indices[offset];
    for (int i = offset + count - 1; i > offset; i--)
      if (!materials_match(first, m_.prim_indices[i])) return true;
    return false;
  }

  // partition_indices, pbvh.c:2070-2088 (Hoare-style, first index of the right part).
  int partition(int lo, int hi, int axis, float mid) {
    int* idx = m_.prim_indices.data();
    const std::vector<PrimBox>& pb = *prims_;
    int i = lo, j = hi;
    for (;;) {
      while (pb[idx[i]].c[axis] < mid) i++;
      while (mid < pb[idx[j]].c[axis]) j--;
      if (!(i < j)) return i;
      std::swap(idx[i], idx[j]);
      i++;
    }
  }

  int partition_material(int lo, int hi) {  // pbvh.c:2091-2131
    int* idx = m_.prim_indices.data();
    const int first = idx[lo];
    int i = lo, j = hi;
    for (;;) {
      while (materials_match(first, idx[i])) i++;
      while (!materials_match(first, idx[j])) j--;
      if (!(i < j)) return i;
      std::swap(idx[i], idx[j]);
      i++;
    }
  }

  // build_mesh_leaf_node + map_insert_vert, pbvh.c:2149-2238.  A vertex is
  // unique to the first leaf (in build order) that references it; within a
  // leaf unique vertices come first, then shared ones, each in order of first
  // reference by (primitive, corner).
  void mesh_leaf(int node) {
    const int offset = m_.prim_off[node], count = m_.totprim[node];
    const int stamp = node + 1;
    int uniq = 0, shared = 0;
    for (int i = 0; i < count; i++) {
      const int lt = m_.prim_indices[offset + i];
      for (int j = 0; j < 3; j++) {
        const int v = m_.lt_v[3 * lt + j];
        if (stamp_[v] == stamp) continue;
        stamp_[v] = stamp;
        if (!bitmap_[v]) {
          bitmap_[v] = 1;
          value_[v] = uniq++;
        } else {
          value_[v] = ~shared;
          shared++;
        }
      }
    }
    const size_t base = m_.vert_indices.size();
    m_.vert_indices.resize(base + uniq + shared);
    for (int i = 0; i < count; i++) {
      const int lt = m_.prim_indices[offset + i];
      for (int j = 0; j < 3; j++) {
        const int v = m_.lt_v[3 * lt + j];
        int ndx = value_[v];
        if (ndx < 0) ndx = -ndx + uniq - 1;
        m_.vert_indices[base + ndx] = v;
      }
    }
    m_.uniq[node] = uniq;
    m_.face_verts_n[node] = shared;
    m_.vert_off[node] = static_cast<int>(base);
  }

  void leaf(int node, int offset, int count) {  // build_leaf, pbvh.c:2309-2325
    m_.flag[node] |= kLeaf;
    m_.prim_off[node] = offset;
    m_.totprim[node] = count;
    update_vb(node, offset, count);
    if (m_.type == kFaces) mesh_leaf(node);
  }

  // build_sub, pbvh.c:2372-2425
  void sub(int node, const Box* cb, int offset, int count) {
    const bool below = count <= m_.leaf_limit;
    if (below && !needs_material_split(offset, count)) {
      leaf(node, offset, count);
      return;
    }
    m_.children[node] = m_.totnode;
    grow(m_.totnode + 2);
    update_vb(node, offset, count);
    int end;
    if (!below) {
      Box local;
      if (!cb) {
        local.reset();
        for (int i = offset + count - 1; i >= offset; i--)
          local.expand((*prims_)[m_.prim_indices[i]].c);
        cb = &local;
      }
      const int axis = cb->widest_axis();
      end = partition(offset, offset + count - 1, axis, (cb->mx[axis] + cb->mn[axis]) * 0.5f);
    } else {
      end = partition_material(offset, offset + count - 1);
    }
    const int child = m_.children[node];
    sub(child, nullptr, offset, end - offset);
    sub(child + 1, nullptr, end, offset + count - end);
  }

  HostMesh& m_;
  const std::vector<PrimBox>* prims_ = nullptr;
  int node_cap_ = 0;
  std::vector<unsigned char> bitmap_;
  std::vector<int> stamp_, value_;
};

// Parent links, left-first DFS leaf ranks, depth levels for the bottom-up flush.
void derive_tables(HostMesh& m) {
  const int n = m.totnode;
  m.parent.assign(n, -1);
  for (int i = 0; i < n; i++)
    if (!(m.flag[i] & kLeaf)) {
      m.parent[m.children[i]] = i;
      m.parent[m.children[i] + 1] = i;
    }
  m.leaf_nodes.clear();
  m.node_leaf.assign(n, -1);
  std::vector<int> depth(n, 0);
  std::vector<int> stack;
  stack.push_back(0);
  int maxd = 0;
  while (!stack.empty()) {  // pbvh_iter_next order: push right, then left
    const int node = stack.back();
    stack.pop_back();
    if (m.flag[node] & kLeaf) {
      m.node_leaf[node] = static_cast<int>(m.leaf_nodes.size());
      m.leaf_nodes.push_back(node);
    } else {
      const int c = m.children[node];
      depth[c] = depth[c + 1] = depth[node] + 1;
      maxd = std::max(maxd, depth[node] + 1);
      stack.push_back(c + 1);
      stack.push_back(c);
    }
  }
  m.level_off.assign(1, 0);
  m.level_nodes.clear();
  for (int d = maxd; d >= 0; d--) {
    for (int i = 0; i < n; i++)
      if (!(m.flag[i] & kLeaf) && depth[i] == d) m.level_nodes.push_back(i);
    m.level_off.push_back(static_cast<int>(m.level_nodes.size()));
  }
  m.depth = depth;
  m.max_depth = maxd;
  // Leaves of a subtree are consecutive in left-first DFS order.
  m.leaf_lo.assign(n, 0);
  m.leaf_hi.assign(n, 0);
  for (int i = 0; i < n; i++)
    if (m.flag[i] & kLeaf) {
      m.leaf_lo[i] = m.node_leaf[i];
      m.leaf_hi[i] = m.node_leaf[i] + 1;
    }
  for (int node : m.level_nodes) {  // deepest first: children are done
    const int c = m.children[node];
    m.leaf_lo[node] = m.leaf_lo[c];
    m.leaf_hi[node] = m.leaf_hi[c + 1];
  }
}

void build_vertex_looptri(HostMesh& m) {
  const int V = m.totvert, T = m.totlt;
  m.vt_off.assign(V + 1, 0);
  for (int t = 0; t < T; t++)
    for (int j = 0; j < 3; j++) m.vt_off[m.lt_v[3 * t + j] + 1]++;
  for (int v = 0; v < V; v++) m.vt_off[v + 1] += m.vt_off[v];
  m.vt_idx.resize(static_cast<size_t>(3) * T);
  std::vector<int> fill(m.vt_off.begin(), m.vt_off.end() - 1);
  for (int t = 0; t < T; t++)
    for (int j = 0; j < 3; j++) m.vt_idx[fill[m.lt_v[3 * t + j]]++] = t;
}

// One-ring of a vertex: for each polygon using it (ascending polygon index),
// the previous then the next corner vertex, first occurrences only.
void build_one_ring(HostMesh& m) {
  const int V = m.totvert, P = m.totpoly;
  std::vector<int> pc(V + 1, 0);
  for (int p = 0; p < P; p++)
    for (int k = 0; k < m.poly_totloop[p]; k++) pc[m.loop_v[m.poly_loopstart[p] + k] + 1]++;
  for (int v = 0; v < V; v++) pc[v + 1] += pc[v];
  std::vector<int> pp(pc[V]), pk(pc[V]);
  std::vector<int> fill(pc.begin(), pc.end() - 1);
  for (int p = 0; p < P; p++)
    for (int k = 0; k < m.poly_totloop[p]; k++) {
      const int v = m.loop_v[m.poly_loopstart[p] + k];
      pp[fill[v]] = p;
      pk[fill[v]] = k;
      fill[v]++;
    }
  m.nb_off.assign(V + 1, 0);
  m.nb_idx.clear();
  m.nb_idx.reserve(static_cast<size_t>(pc[V]) * 2);
  for (int v = 0; v < V; v++) {
    m.nb_off[v] = static_cast<int>(m.nb_idx.size());
    for (int e = pc[v]; e < pc[v + 1]; e++) {
      const int p = pp[e], k = pk[e];
      const int ls = m.poly_loopstart[p], tl = m.poly_totloop[p];
      const int cand[2] = {m.loop_v[ls + (k + tl - 1) % tl], m.loop_v[ls + (k + 1) % tl]};
      for (int c : cand) {
        if (c == v) continue;
        bool dup = false;
        for (size_t q = m.nb_off[v]; q < m.nb_idx.size(); q++)
          if (m.nb_idx[q] == c) {
            dup = true;
            break;
          }
        if (!dup) m.nb_idx.push_back(c);
      }
    }
  }
  m.nb_off[V] = static_cast<int>(m.nb_idx.size());
}

}  // namespace

bool build_faces(HostMesh& m, std::string* err) {
  const int V = m.totvert, T = m.totlt;
  for (int p = 0; p < m.totpoly; p++) {
    if (m.poly_totloop[p] < 3 || m.poly_loopstart[p] < 0 ||
        m.poly_loopstart[p] + m.poly_totloop[p] > m.totloop) {
      *err = "polygon loop range out of bounds";
      return false;
    }
  }
  for (int l = 0; l < m.totloop; l++)
    if (m.loop_v[l] < 0 || m.loop_v[l] >= V) {
      *err = "loop vertex index out of range";
      return false;
    }
  for (int t = 0; t < T; t++) {
    if (m.lt_poly[t] < 0 || m.lt_poly[t] >= m.totpoly) {
      *err = "looptri polygon index out of range";
      return false;
    }
  }
  // BKE_pbvh_build_mesh, pbvh.c:2452-2514: per-looptri box and centroid.
  std::vector<PrimBox> prims(T);
  Box cb;
  cb.reset();
  for (int i = 0; i < T; i++) {
    PrimBox& pb = prims[i];
    pb.bb.reset();
    for (int j = 0; j < 3; j++) pb.bb.expand(&m.co[3 * static_cast<size_t>(m.lt_v[3 * i + j])]);
    for (int k = 0; k < 3; k++) pb.c[k] = (pb.bb.mn[k] + pb.bb.mx[k]) * 0.5f;
    cb.expand(pb.c);
  }
  if (T == 0) {
    *err = "mesh has no looptris";
    return false;
  }
  Builder(m).run(prims, cb);
  derive_tables(m);
  build_vertex_looptri(m);
  build_one_ring(m);
  m.lt_leaf.assign(T, -1);
  for (size_t k = 0; k < m.leaf_nodes.size(); k++) {
    const int node = m.leaf_nodes[k];
    for (int i = 0; i < m.totprim[node]; i++)
      m.lt_leaf[m.prim_indices[m.prim_off[node] + i]] = static_cast<int>(k);
  }
  return true;
}

bool build_grids(HostMesh& m, std::string* err) {
  const int gs = m.grid_size, area = gs * gs;
  m.grid_area = area;
  if (gs < 2 || m.num_grids <= 0) {
    *err = "grids need grid_size >= 2 and at least one grid";
    return false;
  }
  int corners = 0;
  for (int f = 0; f < m.num_faces; f++) {
    if (m.face_ngrids[f] < 3 || m.face_start[f] < 0 ||
        m.face_start[f] + m.face_ngrids[f] > m.num_grids) {
      *err = "face grid range out of bounds";
      return false;
    }
    corners += m.face_ngrids[f];
  }
  for (int c = 0; c < corners; c++)
    if (m.face_verts[c] < 0 || m.face_verts[c] >= m.num_base_verts || m.face_edges[c] < 0 ||
        m.face_edges[c] >= m.num_base_edges) {
      *err = "face corner vertex/edge out of range";
      return false;
    }
  m.grid_face.assign(m.num_grids, -1);
  for (int f = 0; f < m.num_faces; f++)
    for (int c = 0; c < m.face_ngrids[f]; c++) {
      int& owner = m.grid_face[m.face_start[f] + c];
      if (owner >= 0) {
        *err = "a grid belongs to two faces";
        return false;
      }
      owner = f;
    }
  for (int g = 0; g < m.num_grids; g++)
    if (m.grid_face[g] < 0) {
      *err = "a grid belongs to no face";
      return false;
    }
  // subdiv_ccg_init_faces_edge_neighborhood, subdiv_ccg.c:397-466
  std::vector<int> edge_verts = std::move(m.edge_elems);  // caller put edge_verts here
  m.edge_off.assign(m.num_base_edges + 1, 0);
  for (int f = 0; f < m.num_faces; f++)
    for (int c = 0; c < m.face_ngrids[f]; c++) m.edge_off[m.face_edges[m.face_start[f] + c] + 1]++;
  for (int e = 0; e < m.num_base_edges; e++) m.edge_off[e + 1] += m.edge_off[e];
  m.edge_elems.assign(static_cast<size_t>(m.edge_off[m.num_base_edges]) * 2 * gs, 0);
  std::vector<int> efill(m.edge_off.begin(), m.edge_off.end() - 1);
  auto elem = [&](int g, int x, int y) { return g * area + y * gs + x; };
  for (int f = 0; f < m.num_faces; f++) {
    const int n = m.face_ngrids[f];
    for (int corner = 0; corner < n; corner++) {
      const int vtx = m.face_verts[m.face_start[f] + corner];
      const int e = m.face_edges[m.face_start[f] + corner];
      const bool flipped = edge_verts[2 * e] != vtx;
      const int cur = m.face_start[f] + corner;
      const int next = m.face_start[f] + (corner + 1) % n;
      int* bc = &m.edge_elems[static_cast<size_t>(efill[e]++) * 2 * gs];
      int k = 0;
      if (flipped) {
        for (int i = 0; i < gs; i++) bc[k++] = elem(next, gs - i - 1, gs - 1);
        for (int i = 0; i < gs; i++) bc[k++] = elem(cur, gs - 1, i);
      } else {
        for (int i = 0; i < gs; i++) bc[k++] = elem(cur, gs - 1, gs - i - 1);
        for (int i = 0; i < gs; i++) bc[k++] = elem(next, i, gs - 1);
      }
    }
  }
  // subdiv_ccg_init_faces_vertex_neighborhood, subdiv_ccg.c:500-531
  m.bvert_off.assign(m.num_base_verts + 1, 0);
  for (int f = 0; f < m.num_faces; f++)
    for (int c = 0; c < m.face_ngrids[f]; c++) m.bvert_off[m.face_verts[m.face_start[f] + c] + 1]++;
  for (int v = 0; v < m.num_base_verts; v++) m.bvert_off[v + 1] += m.bvert_off[v];
  m.bvert_elems.assign(m.bvert_off[m.num_base_verts], 0);
  std::vector<int> vfill(m.bvert_off.begin(), m.bvert_off.end() - 1);
  for (int f = 0; f < m.num_faces; f++)
    for (int c = 0; c < m.face_ngrids[f]; c++) {
      const int g = m.face_start[f] + c;
      m.bvert_elems[vfill[m.face_verts[g]]++] = elem(g, gs - 1, gs - 1);
    }
  // the face of every edge and base-vertex slot (any element of the slot lies
  // in a grid of that face), and the most corners of a face
  m.edge_face.resize(m.edge_off[m.num_base_edges]);
  for (size_t k = 0; k < m.edge_face.size(); k++)
    m.edge_face[k] = m.grid_face[m.edge_elems[k * 2 * gs] / area];
  m.bvert_face.resize(m.bvert_off[m.num_base_verts]);
  for (size_t k = 0; k < m.bvert_face.size(); k++) m.bvert_face[k] = m.grid_face[m.bvert_elems[k] / area];
  m.max_face_corners = 0;
  for (int f = 0; f < m.num_faces; f++) m.max_face_corners = std::max(m.max_face_corners, m.face_ngrids[f]);
  // BKE_pbvh_build_grids, pbvh.c:2516-2561
  std::vector<PrimBox> prims(m.num_grids);
  Box cb;
  cb.reset();
  for (int i = 0; i < m.num_grids; i++) {
    PrimBox& pb = prims[i];
    pb.bb.reset();
    for (int j = 0; j < area; j++)
      pb.bb.expand(&m.co[3 * (static_cast<size_t>(i) * area + j)]);
    for (int k = 0; k < 3; k++) pb.c[k] = (pb.bb.mn[k] + pb.bb.mx[k]) * 0.5f;
    cb.expand(pb.c);
  }
  Builder(m).run(prims, cb);
  derive_tables(m);
  return true;
}

// ---------------------------------------------------------------------------
// Falloff curve: KERNEL_curvemap_reset (colortools.c:249-330) on the clip rect
// [0,1]^2 with negative slope, then curvemap_make_table (colortools.c:597-771)
// with auto handles and horizontal extension (CUMA_DO_CLIP only).

namespace {

struct Bez {
  float v[3][3];
};

void auto_handle(Bez& b, const Bez* prev, const Bez* next) {  // colortools.c:440-560
  const float* p1;
  const float* p3;
  float* p2 = b.v[1];
  float pt[3] = {0, 0, 0};
  if (!prev) {
    p3 = next->v[1];
    pt[0] = 2.0f * p2[0] - p3[0];
    pt[1] = 2.0f * p2[1] - p3[1];
    p1 = pt;
  } else {
    p1 = prev->v[1];
  }
  if (!next) {
    p1 = prev->v[1];
    pt[0] = 2.0f * p2[0] - p1[0];
    pt[1] = 2.0f * p2[1] - p1[1];
    p3 = pt;
  } else {
    p3 = next->v[1];
  }
  float da[2] = {p2[0] - p1[0], p2[1] - p1[1]};
  float db[2] = {p3[0] - p2[0], p3[1] - p2[1]};
  float la = std::sqrt(da[0] * da[0] + da[1] * da[1]);
  float lb = std::sqrt(db[0] * db[0] + db[1] * db[1]);
  if (la == 0.0f) la = 1.0f;
  if (lb == 0.0f) lb = 1.0f;
  float t[2] = {db[0] / lb + da[0] / la, db[1] / lb + da[1] / la};
  const float len = std::sqrt(t[0] * t[0] + t[1] * t[1]) * 2.5614f;
  if (len != 0.0f) {
    la /= len;
    b.v[0][0] = p2[0] + t[0] * -la;
    b.v[0][1] = p2[1] + t[1] * -la;
    lb /= len;
    b.v[2][0] = p2[0] + t[0] * lb;
    b.v[2][1] = p2[1] + t[1] * lb;
  }
}

void forward_diff(float q0, float q1, float q2, float q3, float* p, int it) {  // curve.cc:1710
  float f = static_cast<float>(it);
  const float rt0 = q0;
  const float rt1 = 3.0f * (q1 - q0) / f;
  f *= f;
  const float rt2 = 3.0f * (q0 - 2.0f * q1 + q2) / f;
  f *= it;
  const float rt3 = (q3 - q0 + 3.0f * (q1 - q2)) / f;
  q0 = rt0;
  q1 = rt1 + rt2 + rt3;
  q2 = 2 * rt2 + 6 * rt3;
  q3 = 6 * rt3;
  for (int a = 0; a <= it; a++) {
    *p = q0;
    p += 2;
    q0 += q1;
    q1 += q2;
    q2 += q3;
  }
}

void correct_bezpart(const float* v1, float* v2, float* v3, const float* v4) {  // fcurve.c:1407
  const float h1[2] = {v1[0] - v2[0], v1[1] - v2[1]};
  const float h2[2] = {v4[0] - v3[0], v4[1] - v3[1]};
  const float len = v4[0] - v1[0];
  const float len1 = std::fabs(h1[0]);
  const float len2 = std::fabs(h2[0]);
  if ((len1 + len2) == 0.0f) return;
  if (len1 > len) {
    const float fac = len / len1;
    v2[0] = (v1[0] - fac * h1[0]);
    v2[1] = (v1[1] - fac * h1[1]);
  }
  if (len2 > len) {
    const float fac = len / len2;
    v3[0] = (v4[0] - fac * h2[0]);
    v3[1] = (v4[1] - fac * h2[1]);
  }
}

float len3(const float* a) { return std::sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]); }

}  // namespace

bool build_curve(int preset, Curve* out) {
  float xs[4], ys[4];
  int tot;
  switch (preset) {
    case 0: xs[0] = 0, ys[0] = 1, xs[1] = 1, ys[1] = 0, tot = 2; break;
    case 1: xs[0] = 0, ys[0] = 1, xs[1] = 0.25f, ys[1] = 0.50f, xs[2] = 0.75f, ys[2] = 0.04f,
            xs[3] = 1, ys[3] = 0, tot = 4; break;
    case 2: xs[0] = 0, ys[0] = 1, xs[1] = 0.25f, ys[1] = 0.94f, xs[2] = 0.75f, ys[2] = 0.06f,
            xs[3] = 1, ys[3] = 0, tot = 4; break;
    case 3: xs[0] = 0, ys[0] = 1, xs[1] = 1, ys[1] = 1, tot = 2; break;
    case 5: xs[0] = 0, ys[0] = 1, xs[1] = 0.5f, ys[1] = 0.90f, xs[2] = 0.86f, ys[2] = 0.5f,
            xs[3] = 1, ys[3] = 0, tot = 4; break;
    case 6: xs[0] = 0, ys[0] = 1, xs[1] = 0.25f, ys[1] = 0.95f, xs[2] = 0.75f, ys[2] = 0.44f,
            xs[3] = 1, ys[3] = 0, tot = 4; break;
    default: return false;
  }
  std::memset(out, 0, sizeof(*out));
  out->mintable = 0.0f;
  out->maxtable = 1.0f;
  Bez b[4];
  std::memset(b, 0, sizeof(b));
  for (int a = 0; a < tot; a++) {
    out->mintable = fmin_ref(out->mintable, xs[a]);
    out->maxtable = fmax_ref(out->maxtable, xs[a]);
    b[a].v[1][0] = xs[a];
    b[a].v[1][1] = ys[a];
  }
  for (int a = 0; a < tot; a++)
    auto_handle(b[a], a > 0 ? &b[a - 1] : nullptr, a != tot - 1 ? &b[a + 1] : nullptr);
  if (tot > 2) {
    // First and last handles point at the nearest neighbouring handle, keeping
    // their length (colortools.c:668-709).
    for (int end = 0; end < 2; end++) {
      const int a = end == 0 ? 0 : tot - 1;
      const int own_far = end == 0 ? 2 : 0;    // handle being re-aimed
      const int own_near = end == 0 ? 0 : 2;   // mirrored handle
      const int nb = end == 0 ? 1 : tot - 2;
      const int nb_h = end == 0 ? 0 : 2;
      float d[3] = {b[a].v[1][0] - b[a].v[own_far][0], b[a].v[1][1] - b[a].v[own_far][1],
                    b[a].v[1][2] - b[a].v[own_far][2]};
      if (end == 1) {
        d[0] = b[a].v[1][0] - b[a].v[0][0];
        d[1] = b[a].v[1][1] - b[a].v[0][1];
        d[2] = b[a].v[1][2] - b[a].v[0][2];
      }
      const float hlen = len3(d);
      float vec[3] = {b[nb].v[nb_h][0], b[nb].v[nb_h][1], b[nb].v[nb_h][2]};
      if (end == 0 ? (vec[0] < b[a].v[1][0]) : (vec[0] > b[a].v[1][0])) vec[0] = b[a].v[1][0];
      for (int i = 0; i < 3; i++) vec[i] -= b[a].v[1][i];
      const float nlen = len3(vec);
      if (nlen > FLT_EPSILON) {
        for (int i = 0; i < 3; i++) vec[i] *= hlen / nlen;
        if (end == 0) {
          for (int i = 0; i < 3; i++) b[a].v[2][i] = vec[i] + b[a].v[1][i];
          for (int i = 0; i < 3; i++) b[a].v[0][i] = b[a].v[1][i] - vec[i];
        } else {
          for (int i = 0; i < 3; i++) b[a].v[0][i] = vec[i] + b[a].v[1][i];
          for (int i = 0; i < 3; i++) b[a].v[2][i] = b[a].v[1][i] - vec[i];
        }
      }
      (void)own_near;
    }
  }
  const int totpt = (tot - 1) * kCurveResol;
  std::vector<float> pts(static_cast<size_t>(totpt) * 2, 0.0f);
  for (int a = 0; a < tot - 1; a++) {
    float* p = &pts[static_cast<size_t>(a) * 2 * kCurveResol];
    correct_bezpart(b[a].v[1], b[a].v[2], b[a + 1].v[0], b[a + 1].v[1]);
    forward_diff(b[a].v[1][0], b[a].v[2][0], b[a + 1].v[0][0], b[a + 1].v[1][0], p,
                 kCurveResol - 1);
    forward_diff(b[a].v[1][1], b[a].v[2][1], b[a + 1].v[0][1], b[a + 1].v[1][1], p + 1,
                 kCurveResol - 1);
  }
  out->ext_in[0] = b[0].v[0][0] - b[0].v[1][0];
  out->ext_in[1] = b[0].v[0][1] - b[0].v[1][1];
  const float ri = std::sqrt(out->ext_in[0] * out->ext_in[0] + out->ext_in[1] * out->ext_in[1]);
  out->ext_in[0] /= ri;
  out->ext_in[1] /= ri;
  const int oa = tot - 1;
  out->ext_out[0] = b[oa].v[1][0] - b[oa].v[2][0];
  out->ext_out[1] = b[oa].v[1][1] - b[oa].v[2][1];
  const float ro =
      std::sqrt(out->ext_out[0] * out->ext_out[0] + out->ext_out[1] * out->ext_out[1]);
  out->ext_out[0] /= ro;
  out->ext_out[1] /= ro;
  const float range = (1.0f / 256.0f) * (out->maxtable - out->mintable);
  out->range = 1.0f / range;
  const float* first = pts.data();
  const float* last = pts.data() + 2 * (totpt - 1);
  const float* p = first;
  for (int a = 0; a <= kCurveTable; a++) {
    const float x = out->mintable + range * static_cast<float>(a);
    out->table_x[a] = x;
    while (x >= p[0] && p != last) p += 2;
    float y;
    if (p == first || (p == last && x >= p[0])) {
      if (std::fabs(x - p[0]) <= 1e-6f) {
        y = p[1];
      } else {  // curvemap_calc_extend without extrapolation, colortools.c:563-595
        y = (x <= first[0]) ? first[1] : ((x >= last[0]) ? last[1] : 0.0f);
      }
    } else {
      float f1 = p[0] - p[-2];
      const float f2 = p[0] - x;
      f1 = (f1 > FLT_EPSILON) ? f2 / f1 : 0.0f;
      y = f1 * p[-1] + (1.0f - f1) * p[1];
    }
    out->y[a] = y;
  }
  out->x_first = out->table_x[0];
  out->x_last = out->table_x[kCurveTable];
  return true;
}

}  // namespace sgpu
