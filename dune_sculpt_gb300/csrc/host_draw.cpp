// Host side of the headless PBVH draw buffers: which prims each leaf draws,
// where its vertices sit in the one vertex buffer, and the per-face and
// per-vertex attributes that do not change while sculpting (face-set colours,
// vertex colours).  This is the work GPU_pbvh_mesh_buffers_build
// (gpu_buffers.c:307-400) and the set-up half of the update functions do on
// the host in the reference; the per-update fill runs on the device.
// Compiled with -ffp-contract=off.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>

#include "sgpu_draw.h"

namespace sgpu {
namespace {

// The integer hash of BLI_hash.h (not shipped with the reference; its
// BLI_hash_int_01 is called by paint.c:2225-2226): Bob Jenkins' lookup3
// final() mix over (k, 0) with the initial value 0xdeadbeef + (2 << 2) + 13,
// the same function as the two-argument hash of noise.cc:70-80.
inline uint32_t rot32(uint32_t x, int k) { return (x << k) | (x >> (32 - k)); }

uint32_t hash_int_2d(uint32_t kx, uint32_t ky) {
  uint32_t a, b, c;
  a = b = c = 0xdeadbeefu + (2u << 2) + 13u;
  a += kx;
  b += ky;
  c ^= b;
  c -= rot32(b, 14);
  a ^= c;
  a -= rot32(c, 11);
  b ^= a;
  b -= rot32(a, 25);
  c ^= b;
  c -= rot32(b, 16);
  a ^= c;
  a -= rot32(c, 4);
  b ^= a;
  b -= rot32(a, 14);
  c ^= b;
  c -= rot32(b, 24);
  return c;
}

// BLI_hash_int_01: the hash scaled to [0, 1].
float hash_int_01(uint32_t k) {
  return static_cast<float>(hash_int_2d(k, 0)) * (1.0f / static_cast<float>(0xFFFFFFFFu));
}

inline float clamp01(float x) { return x < 0.0f ? 0.0f : (x > 1.0f ? 1.0f : x); }

// hsv_to_rgb, math_color.c:6-21.
void hsv_to_rgb(float h, float s, float v, float rgb[3]) {
  const float nr = clamp01(std::fabs(h * 6.0f - 3.0f) - 1.0f);
  const float ng = clamp01(2.0f - std::fabs(h * 6.0f - 2.0f));
  const float nb = clamp01(2.0f - std::fabs(h * 6.0f - 4.0f));
  rgb[0] = ((nr - 1.0f) * s + 1.0f) * v;
  rgb[1] = ((ng - 1.0f) * s + 1.0f) * v;
  rgb[2] = ((nb - 1.0f) * s + 1.0f) * v;
}

// unit_float_to_uchar_clamp / unit_float_to_ushort_clamp, math_base_inline.c:678-690.
unsigned char unit_to_uchar(float v) {
  const float f = (v <= 0.0f) ? 0.0f : ((v > (1.0f - 0.5f / 255.0f)) ? 255.0f : (255.0f * v) + 0.5f);
  return static_cast<unsigned char>(f);
}
unsigned short unit_to_ushort(float v) {
  const float f = (v >= 1.0f - 0.5f / 65535.0f) ? 65535.0f : ((v <= 0.0f) ? 0.0f : (v * 65535.0f + 0.5f));
  return static_cast<unsigned short>(f);
}

// BLI_color_from_srgb_table (math_color.c:503, filled at 577-581 with
// srgb_to_linearrgb, math_color.c:393-400).
struct SrgbTable {
  float v[256];
  SrgbTable() {
    for (int b = 0; b < 256; b++) {
      const float c = static_cast<float>(b) * (1.0f / 255.0f);
      v[b] = (c < 0.04045f) ? ((c < 0.0f) ? 0.0f : c * (1.0f / 12.92f))
                            : std::pow((c + 0.055f) * (1.0f / 1.055f), 2.4f);
    }
  }
};

inline uint32_t pack_rgb(const unsigned char c[3], bool nondefault) {
  return static_cast<uint32_t>(c[0]) | (static_cast<uint32_t>(c[1]) << 8) |
         (static_cast<uint32_t>(c[2]) << 16) | (nondefault ? (1u << 24) : 0u);
}

// The face-set overlay colour of one face, white for the default face set
// (gpu_buffers.c:249-257 / 601-610).
uint32_t fset_entry(int face_set, const DrawInputs& in) {
  const int fs = std::abs(face_set);
  unsigned char c[3] = {255, 255, 255};
  if (fs != in.color_default) {
    face_set_color(fs, in.seed, c);
    return pack_rgb(c, true);
  }
  return pack_rgb(c, false);
}

}  // namespace

void face_set_color(int face_set, int seed, unsigned char rgb[3]) {
  float hue = 0.618033988749895f * static_cast<float>(std::abs(face_set) + (seed % 10));
  hue = hue - std::floor(hue);
  const float sat = hash_int_01(static_cast<uint32_t>(std::abs(face_set) + seed + 1));
  const float val = hash_int_01(static_cast<uint32_t>(std::abs(face_set) + seed + 2));
  float c[3];
  hsv_to_rgb(hue, 0.6f + (sat * 0.25f), 1.0f - (val * 0.35f), c);
  for (int k = 0; k < 3; k++) rgb[k] = unit_to_uchar(c[k]);
}

bool build_draw_layout(const HostMesh& h, const DrawInputs& in, DrawLayout* out, std::string* err) {
  DrawLayout& L = *out;
  L = DrawLayout{};
  const int totnode = h.totnode;
  const int nleaf = static_cast<int>(h.leaf_nodes.size());
  L.node_vert_off.assign(totnode + 1, 0);
  L.node_tot_tri.assign(totnode, 0);
  L.node_smooth.assign(totnode, 0);
  L.node_material.assign(totnode, 0);
  L.leaf_vert_off.assign(nleaf, 0);
  L.leaf_tri_start.assign(nleaf, 0);
  L.leaf_tri_count.assign(nleaf, 0);
  L.leaf_smooth.assign(nleaf, 0);
  if (h.type == kFaces) {
    if (static_cast<int>(in.vert_flag.size()) != h.totvert || !in.o2n) {
      *err = "vertex flags or numbering missing";
      return false;
    }
    // fset per poly; faces are drawn only with a face-set layer
    // (gpu_pbvh_is_looptri_visible, gpu_buffers.c:166-172)
    L.has_fset = in.face_sets != nullptr;
    if (L.has_fset) {
      L.fset.resize(h.totpoly);
      for (int p = 0; p < h.totpoly; p++) L.fset[p] = fset_entry(in.face_sets[p], in);
    }
    L.show_vcol = (in.loop_colors != nullptr) || (in.vert_colors && in.use_vert_colors);
    const bool use_vtcol = in.vert_colors && in.use_vert_colors;
    static const SrgbTable srgb;
    int64_t off = 0;
    for (int n = 0; n < totnode; n++) {
      L.node_vert_off[n] = off;
      if (!(h.flag[n] & kLeaf)) continue;
      const int p0 = h.prim_off[n], np = h.totprim[n];
      if (np > 0) {
        const int poly = h.lt_poly[h.prim_indices[p0]];
        L.node_smooth[n] = (h.poly_flag[poly] & kMeSmooth) != 0;
        L.node_material[n] = h.poly_mat[poly];
      }
      const int start = static_cast<int>(L.tris.size());
      for (int i = 0; i < np; i++) {
        const int lt = h.prim_indices[p0 + i];
        const int poly = h.lt_poly[lt];
        bool hidden = false;
        for (int j = 0; j < 3; j++) hidden = hidden || (in.vert_flag[h.lt_v[3 * lt + j]] & kMeHide);
        if (hidden || !L.has_fset || in.face_sets[poly] <= 0) continue;
        L.tris.push_back(lt);
        for (int j = 0; j < 3; j++) L.tri_v4.push_back(in.o2n[h.lt_v[3 * lt + j]]);
        L.tri_v4.push_back(poly);
        if (!L.show_vcol) continue;
        for (int j = 0; j < 3; j++) {
          unsigned short s[4];
          if (use_vtcol) {
            const float* c = in.vert_colors + 4 * static_cast<size_t>(h.lt_v[3 * lt + j]);
            for (int k = 0; k < 4; k++) s[k] = unit_to_ushort(c[k]);
          } else {
            const unsigned char* c = in.loop_colors + 4 * static_cast<size_t>(h.lt_loop[3 * lt + j]);
            for (int k = 0; k < 3; k++) s[k] = unit_to_ushort(srgb.v[c[k]]);
            s[3] = unit_to_ushort(c[3] * (1.0f / 255.0f));
          }
          L.col.push_back(s[0] | (static_cast<uint32_t>(s[1]) << 16));
          L.col.push_back(s[2] | (static_cast<uint32_t>(s[3]) << 16));
        }
      }
      const int cnt = static_cast<int>(L.tris.size()) - start;
      L.node_tot_tri[n] = cnt;
      const int leaf = h.node_leaf[n];
      L.leaf_vert_off[leaf] = off;
      L.leaf_tri_start[leaf] = start;
      L.leaf_tri_count[leaf] = cnt;
      L.leaf_smooth[leaf] = L.node_smooth[n];
      int& mu = L.node_smooth[n] ? L.max_units_smooth : L.max_units_flat;
      mu = std::max(mu, cnt);
      off += 3 * static_cast<int64_t>(cnt);
    }
    L.node_vert_off[totnode] = off;
    L.total_verts = off;
    return true;
  }
  // GRIDS: fset per grid through its base face (BKE_subdiv_ccg_grid_to_face_index)
  L.has_fset = in.face_sets != nullptr;
  if (L.has_fset) {
    L.fset.resize(h.num_grids);
    for (int g = 0; g < h.num_grids; g++) L.fset[g] = fset_entry(in.face_sets[h.grid_face[g]], in);
  }
  const int gs = h.grid_size;
  int64_t off = 0;
  for (int n = 0; n < totnode; n++) {
    L.node_vert_off[n] = off;
    if (!(h.flag[n] & kLeaf)) continue;
    const int p0 = h.prim_off[n], ng = h.totprim[n];
    int smooth = 1, mat = 0;
    if (ng > 0 && in.grid_flag_mats) {
      const unsigned char* fm = in.grid_flag_mats + 4 * static_cast<size_t>(h.prim_indices[p0]);
      short mat_nr;
      std::memcpy(&mat_nr, fm, sizeof(short));
      mat = mat_nr;
      smooth = (fm[2] & kMeSmooth) != 0;
    }
    L.node_smooth[n] = smooth;
    L.node_material[n] = mat;
    // GPU_PBVH_Buffers.tot_tri stays 0 for grid buffers
    const int leaf = h.node_leaf[n];
    L.leaf_vert_off[leaf] = off;
    L.leaf_smooth[leaf] = smooth;
    const int units = ng * (smooth ? gs * gs : (gs - 1) * (gs - 1));
    int& mu = smooth ? L.max_units_smooth : L.max_units_flat;
    mu = std::max(mu, units);
    off += static_cast<int64_t>(ng) * (smooth ? gs * gs : (gs - 1) * (gs - 1) * 4);
  }
  L.node_vert_off[totnode] = off;
  L.total_verts = off;
  return true;
}

}  // namespace sgpu
