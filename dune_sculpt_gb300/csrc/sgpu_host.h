// Host-side data model of libsculptgpu: the PBVH as built on the host (once per
// mesh) before it is mirrored to the device, plus the falloff curve.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace sgpu {

// PBVHNodeFlags (values of the reference's enum, whose header BKE_pbvh.h is absent).
constexpr int kLeaf = 1;
constexpr int kUpdateNormals = 2;
constexpr int kUpdateBB = 4;
constexpr int kUpdateOriginalBB = 8;
constexpr int kUpdateDrawBuffers = 16;
constexpr int kUpdateRedraw = 32;
// BKE_pbvh_node_mark_update, pbvh.c:3641-3645.
constexpr int kMarkUpdate =
    kUpdateNormals | kUpdateBB | kUpdateOriginalBB | kUpdateDrawBuffers | kUpdateRedraw;

constexpr int kFaces = 0;
constexpr int kGrids = 1;

constexpr int kCurveTable = 256;  // CM_TABLE, types_color.h:11-13
constexpr int kCurveResol = 32;   // CM_RESOL

// Falloff curve as evaluated on the device: the y column of the 257-entry
// table plus the scalars the evaluation reads.
struct Curve {
  float y[kCurveTable + 1];
  float x_first, x_last;  // table[0].x, table[256].x
  float mintable, maxtable, range;
  float ext_in[2], ext_out[2];
  float table_x[kCurveTable + 1];
};

// Builds the brush falloff table for a curve preset (colortools.c:249-771).
bool build_curve(int preset, Curve* out);

struct HostMesh {
  int type = kFaces;
  int totvert = 0;
  // FACES topology
  int totpoly = 0, totloop = 0, totlt = 0;
  std::vector<int> poly_loopstart, poly_totloop;
  std::vector<short> poly_mat;
  std::vector<char> poly_flag;
  std::vector<int> loop_v;
  std::vector<int> lt_v;     // 3 per looptri (vertex indices)
  std::vector<int> lt_poly;  // per looptri
  std::vector<int> lt_loop;  // 3 per looptri (loop indices)
  std::vector<int> vt_off, vt_idx;  // vertex -> looptri (ascending)
  std::vector<int> nb_off, nb_idx;  // vertex -> one-ring
  // GRIDS topology
  int num_grids = 0, grid_size = 0, grid_area = 0, num_faces = 0;
  int num_base_verts = 0, num_base_edges = 0;
  std::vector<int> face_start, face_ngrids, face_verts, face_edges;
  std::vector<int> grid_face;
  std::vector<int> edge_off, edge_elems;    // per base edge: faces * 2*grid_size elements
  std::vector<int> bvert_off, bvert_elems;  // per base vertex: one corner element per face
  std::vector<int> edge_face, bvert_face;   // the face of each edge / base-vertex slot
  int max_face_corners = 0;
  // positions used for the build (float xyz)
  std::vector<float> co;
  // PBVH (reference node numbering)
  int leaf_limit = 10000;
  int totnode = 0;
  std::vector<int> children;  // children_offset, -1 for leaves
  std::vector<int> flag;
  std::vector<int> prim_off, totprim, uniq, face_verts_n, vert_off;
  std::vector<int> prim_indices;
  std::vector<int> vert_indices;  // concatenated over leaves in build order
  std::vector<float> vb;          // 6 per node
  // derived tables for the device
  std::vector<int> parent;
  std::vector<int> leaf_nodes;  // leaf id (left-first DFS rank) -> node
  std::vector<int> node_leaf;   // node -> leaf id or -1
  std::vector<int> level_off, level_nodes;  // internal nodes by depth, deepest first
  std::vector<int> leaf_lo, leaf_hi;        // per node: leaf-id range of its subtree
  std::vector<int> depth;                   // per node, root = 0
  int max_depth = 0;
  std::vector<int> lt_leaf;                 // looptri -> leaf id
};

// BKE_pbvh_build_mesh / BKE_pbvh_build_grids and the derived tables.
// Returns false with a message on malformed input.
bool build_faces(HostMesh& m, std::string* err);
bool build_grids(HostMesh& m, std::string* err);

}  // namespace sgpu
