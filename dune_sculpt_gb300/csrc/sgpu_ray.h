// Ray-cast batch of libsculptgpu (kernels_ray.cu): device arrays of one launch.
#pragma once

#include <cuda_runtime.h>

#include "sgpu_device.cuh"

namespace sgpu {

struct RayBatch {
  const float* rays;      // 6 per ray: start xyz, unit direction xyz
  const float* depth_in;  // per ray: ray length (nullable: FLT_MAX)
  int original;           // boxes from orig_vb instead of vb
  int nearest;            // the nearest-to-ray query (depth_in: starting squared distance)
  const int* n2o;         // device -> caller vertex numbering (nullable: identity)
  // per ray and listed leaf (nleaf slots per ray)
  int* count;
  int* slot_leaf;
  float* slot_tmin;
  int* slot_order;
  unsigned long long* slot_key;
  int* slot_special;  // GRIDS: the leaf has a quad whose second triangle is the closer hit
  // work items (ray * nleaf + slot, chunk) and their count: the first leaves
  // in entry order (round 0), the rest for the rays they did not settle (round 1)
  int2* items;
  int* nitems;
  int2* items2;
  int* nitems2;
  int item_cap;
  int first_leaves;  // leaves tested in round 0 (every leaf: one round)
  // per ray: the traversal state between the rounds (next rank; -1 = done)
  float* st_depth;
  float* st_run;
  int4* st_win;  // winning slot, position, triangle, next rank
  // results per ray
  float* depth_out;
  int* hit;
  int* active_vertex;
  int* active_face;
  float* face_normal;  // 3 per ray
};

size_t ray_leaves_smem(const DevMesh& m);
size_t ray_finish_smem(const DevMesh& m);
int ray_items_per_ray(const DevMesh& m);
cudaError_t configure_ray_kernels(size_t leaves_smem, size_t finish_smem);
cudaError_t launch_raycast(const DevMesh& m, const RayBatch& rb, int nrays, int tris_grid,
                           cudaStream_t s);

}  // namespace sgpu
