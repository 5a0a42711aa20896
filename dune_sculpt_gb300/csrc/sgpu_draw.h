// Headless PBVH draw buffers: the host layout (GPU_pbvh_*_buffers_build,
// gpu_buffers.c:307-400 and 727-738) and the device view the fill kernels read
// (GPU_pbvh_mesh_buffers_update / GPU_pbvh_grid_buffers_update,
// gpu_buffers.c:174-305, 548-725).
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "sgpu_host.h"

namespace sgpu {

constexpr int kRebuildDrawBuffers = 1 << 9;  // PBVH_RebuildDrawBuffers
constexpr int kMeSmooth = 1;                 // ME_SMOOTH (MPoly.flag, DMFlagMat.flag)
constexpr int kMeHide = 16;                  // ME_HIDE (MVert.flag)
constexpr int kDrawWords = 9;                // 36-byte vertex: pos 0, nor 16, msk 22, ac 24, fset 32

// What sgpu_draw_buffers_build reads besides the mesh.
struct DrawInputs {
  const int* face_sets = nullptr;
  int seed = 0, color_default = 0;
  const unsigned char* loop_colors = nullptr;
  const float* vert_colors = nullptr;
  bool use_vert_colors = false;
  const unsigned char* grid_flag_mats = nullptr;  // 4-byte DMFlagMat records
  std::vector<unsigned char> vert_flag;           // FACES: MVert.flag per vertex (caller order)
  const int* o2n = nullptr;                       // FACES: caller vertex -> device vertex
};

struct DrawLayout {
  // per node, reference order
  std::vector<int64_t> node_vert_off;  // totnode + 1
  std::vector<int> node_tot_tri, node_smooth, node_material;
  // per leaf id (the device's leaf order)
  std::vector<long long> leaf_vert_off;
  std::vector<int> leaf_tri_start, leaf_tri_count, leaf_smooth;
  std::vector<int> tris;        // FACES: visible looptris, node order
  std::vector<int> tri_v4;      // FACES: per visible looptri its device corners and poly
  std::vector<uint32_t> fset;   // per poly (FACES) / grid (GRIDS): r | g << 8 | b << 16 | nondefault << 24
  bool has_fset = false;        // face sets drawn (show_face_sets)
  std::vector<uint32_t> col;    // FACES with colours: ushort4 per vertex (2 words), buffer order
  bool show_vcol = false;
  int64_t total_verts = 0;
  int max_units_smooth = 0;     // most units of a smooth / flat leaf (looptris,
  int max_units_flat = 0;       // grid elements or grid quads)
};

// GPU_pbvh_*_buffers_build for every leaf.  Returns false with a message on
// malformed input.
bool build_draw_layout(const HostMesh& h, const DrawInputs& in, DrawLayout* out, std::string* err);

// BKE_paint_face_set_overlay_color_get (paint.c:2219-2236).
void face_set_color(int face_set, int seed, unsigned char rgb[3]);

// Device view of the draw buffers (filled by sgpu_draw_buffers_build).
struct DrawDev {
  unsigned int* vbo;              // kDrawWords words per vertex
  const long long* leaf_vert_off;  // per leaf id
  const int* leaf_tri_start;       // FACES
  const int* leaf_tri_count;       // FACES
  const int* leaf_smooth;
  const int* tri_v4;               // FACES: 4 ints per visible looptri (device corners, poly)
  const unsigned int* fset;        // per poly / grid, or null
  const unsigned int* col;         // FACES: 2 words per vertex, or null
  int* overlay;                    // per leaf id
  int* overlay_acc;                // per leaf id: OR of the chunks of the running fill
};

}  // namespace sgpu
