// Kernel launchers of libsculptgpu (defined in kernels.cu / kernels_grids.cu).
#pragma once

#include <cuda_runtime.h>

#include "sgpu_device.cuh"

#include "sgpu_draw.h"

namespace sgpu {

cudaError_t launch_cull(const DevMesh& m, const PassParams& pp, cudaStream_t s);
cudaError_t launch_set_list(const DevMesh& m, const int* dev_nodes, int totnode, cudaStream_t s);
// Grab / elastic deform: the union gather of a dab's passes, then the dab.
cudaError_t launch_cull_dab(const DevMesh& m, const DabPasses& dp, float radius_sq, int all,
                            cudaStream_t s);
cudaError_t launch_orig_dab(const DevMesh& m, const DevBrush& b, const DabPasses& dp,
                            cudaStream_t s);
cudaError_t launch_area(const DevMesh& m, const DevBrush& b, const PassParams& pp,
                        cudaStream_t s);
cudaError_t launch_brush(const DevMesh& m, const DevBrush& b, const PassParams& pp,
                         cudaStream_t s);
// One smooth iteration = two launches (compute into scratch, apply).
cudaError_t launch_smooth_compute(const DevMesh& m, const DevBrush& b, const PassParams& pp,
                                  cudaStream_t s);
cudaError_t launch_smooth_apply(const DevMesh& m, cudaStream_t s);
// FACES normals (do_normals) and/or bounds refit + flush (bounds_flag); bounds
// also serve GRIDS meshes.
cudaError_t launch_update_faces(const DevMesh& m, int do_normals, int bounds_flag,
                                cudaStream_t s);
// GRIDS normal update with seam stitching: gather, inner normals, face
// seams and centres, base edges and corners.
cudaError_t launch_grid_gather(const DevMesh& m, cudaStream_t s);
cudaError_t launch_grid_inner(const DevMesh& m, cudaStream_t s);
cudaError_t launch_grid_face_seams(const DevMesh& m, cudaStream_t s);
cudaError_t launch_grid_seams(const DevMesh& m, cudaStream_t s);
// Writes a buffer larger than L2.
cudaError_t launch_l2_flush(void* buf, size_t bytes, cudaStream_t s);
cudaError_t launch_mark_node(const DevMesh& m, int node, cudaStream_t s);
cudaError_t launch_mark_all(const DevMesh& m, int bits, cudaStream_t s);
// Headless draw buffers: fill every leaf flagged PBVH_UpdateDrawBuffers.
cudaError_t launch_draw_fill(const DevMesh& m, const DrawDev& dd, int max_units_smooth,
                             int max_units_flat, cudaStream_t s);
// Refit-chunk boxes of every leaf from the current positions.
cudaError_t launch_chunk_boxes_all(const DevMesh& m, int nchunks, cudaStream_t s);
// out[i] = in[idx[i]]: float4 or float.
cudaError_t launch_gather_f4(float4* out, const float4* in, const int* idx, int n, cudaStream_t s);
cudaError_t launch_gather_f1(float* out, const float* in, const int* idx, int n, cudaStream_t s);
// Packed xyz <-> float4: out[i] = in3[idx[i]] (idx nullable: identity);
// out3[i] = in[idx[i]].xyz.
cudaError_t launch_xyz_to_f4(float4* out, const float* in3, const int* idx, int n, bool keep_w,
                             cudaStream_t s);
cudaError_t launch_f4_to_xyz(float* out3, const float4* in, const int* idx, int n, cudaStream_t s);
// Changed blocks of vertices (caller order through idx, bitwise against in)
// into the mapped host output.
cudaError_t launch_vert_writeback(float4* out, const float4* co, const int* idx, const float4* in, int n,
                                  cudaStream_t s);
// Changed grids' positions (bitwise against in3) into the mapped host output.
cudaError_t launch_grid_writeback(float* out3, const float4* co, const float* in3, int ngrids, int area,
                                  cudaStream_t s);
int cull_smem_limit();
int grid_size_limit();
void configure_kernels();
void configure_grid_kernels();

}  // namespace sgpu
