// Allocation-free smooth dab (sgpu_smooth_dab_noalloc).
//
// For callers that cannot allocate device memory: a host that runs inside a
// memory budget fixed up front (an embedding application's pool, a plug-in
// sandbox, an interactive loop that must not allocate while a stroke runs), so
// it can neither create a
// mesh handle (which allocates) nor call cudaMalloc itself.  They keep the
// mesh arrays in device memory they already own and pass them in; the
// Jacobi scratch of the smooth sweeps lives in a fixed file-scope device array
// of SGPU_NOALLOC_MAX_VERTS entries (1 MiB), so this path allocates nothing.
//
// The arithmetic is the smooth brush's (smooth_vertex in sgpu_device.cuh), so
// the result equals sgpu_do_smooth_brush on the same vertices.
#include <cuda_runtime.h>

#include <cstring>
#include <mutex>
#include <string>

#include "../../include/sculpt_gpu.h"
#include "sgpu_device.cuh"
#include "sgpu_host.h"

namespace sgpu {

// Shared by every call in the process (on every device that loads the
// library), kept until exit; holds the last call's values.
static __device__ __align__(256) float4 g_noalloc_scratch[SGPU_NOALLOC_MAX_VERTS];

// Sets the message sgpu_last_error() returns (api.cu).
void set_error_message(const std::string& msg);

namespace {

constexpr int kNoAllocThreads = 256;
constexpr int kMaxDevices = 64;

std::mutex g_mu;
float4* g_scratch_addr[kMaxDevices] = {};

int noalloc_fail(int code, const std::string& msg) {
  set_error_message(msg);
  return code;
}

// The device address of the scratch array on the current device, looked up
// once per device (host code cannot use the symbol's name as an address).
// A device reset ends the context that held the array, so a cached address
// that the runtime no longer knows as device memory is looked up again.
int scratch_for_device(float4** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return noalloc_fail(SGPU_ERR_CUDA, cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return noalloc_fail(SGPU_ERR_UNSUPPORTED, "device index");
  std::lock_guard<std::mutex> lock(g_mu);
  if (g_scratch_addr[dev]) {
    cudaPointerAttributes attr;
    if (cudaPointerGetAttributes(&attr, g_scratch_addr[dev]) != cudaSuccess ||
        attr.type != cudaMemoryTypeDevice || attr.device != dev) {
      cudaGetLastError();  // a failed query leaves no sticky error
      g_scratch_addr[dev] = nullptr;
    }
  }
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess)
      return noalloc_fail(SGPU_ERR_CUDA, std::string("cudaGetSymbolAddress: ") +
                                             cudaGetErrorString(e));
    g_scratch_addr[dev] = static_cast<float4*>(p);
  }
  *out = g_scratch_addr[dev];
  return SGPU_OK;
}

}  // namespace

// One Jacobi sweep, compute half: every candidate's new position (w = 1 when
// it lies inside the sphere) into the scratch, all of which is overwritten.
__global__ void __launch_bounds__(kNoAllocThreads)
    k_noalloc_compute(DevMesh m, DevBrush b, PassParams pp, const int* verts, int n,
                      float4* scratch) {
  __shared__ float ys[kCurveTable + 1];
  for (int i = threadIdx.x; i <= kCurveTable; i += blockDim.x) ys[i] = b.y[i];
  __syncthreads();
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int v = verts[i];
    float4 out = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    bool moved = false;
    if (smooth_vertex(m, b, ys, pp, v, m.co[v], out, moved)) {
      out.w = 1.0f;
    } else {
      out = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    }
    scratch[i] = out;
  }
}

// Apply half: write the new positions back (keeping each MVert's flag bytes).
__global__ void __launch_bounds__(kNoAllocThreads)
    k_noalloc_apply(DevMesh m, const int* verts, int n, const float4* scratch) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float4 s = scratch[i];
    if (s.w == 0.0f) continue;
    const int v = verts[i];
    float4 co = m.co[v];
    co.x = s.x;
    co.y = s.y;
    co.z = s.z;
    m.co[v] = co;
  }
}

}  // namespace sgpu

using namespace sgpu;

extern "C" int sgpu_smooth_dab_noalloc(float* co, const float* normals, const float* mask,
                                       const float* automask, const int* nb_off,
                                       const int* nb_idx, const int* verts, int nverts,
                                       const SGPU_Brush* brush, const float location[3],
                                       void* stream) {
  if (!co || !nb_off || !nb_idx || !brush || !location || (nverts > 0 && !verts))
    return noalloc_fail(SGPU_ERR_INVALID_ARG, "NULL argument");
  if (nverts < 0 || nverts > SGPU_NOALLOC_MAX_VERTS)
    return noalloc_fail(SGPU_ERR_INVALID_ARG,
                        "nverts " + std::to_string(nverts) + " outside 0.." +
                            std::to_string(SGPU_NOALLOC_MAX_VERTS) +
                            ", the vertices the fixed scratch holds");
  if (!(brush->radius > 0.0f)) return noalloc_fail(SGPU_ERR_INVALID_ARG, "radius must be positive");
  if ((brush->flag & kBrushFrontFace) && !normals)
    return noalloc_fail(SGPU_ERR_INVALID_ARG, "front-face falloff needs normals");
  Curve curve;
  if (!build_curve(brush->curve_preset, &curve))
    return noalloc_fail(SGPU_ERR_INVALID_ARG, "unknown curve preset");
  float4* scratch = nullptr;
  int rc = scratch_for_device(&scratch);
  if (rc) return rc;
  if (nverts == 0) return SGPU_OK;

  DevMesh m;
  std::memset(&m, 0, sizeof(m));
  m.type = kFaces;
  m.co = reinterpret_cast<float4*>(co);
  m.no = reinterpret_cast<float4*>(const_cast<float*>(normals));
  m.mask = const_cast<float*>(mask);
  m.automask = automask;
  m.nb_off = nb_off;
  m.nb_idx = nb_idx;
  DevBrush b;
  std::memset(&b, 0, sizeof(b));
  b.tool = kToolSmooth;
  b.flag = brush->flag;
  b.radius = brush->radius;
  b.strength = brush->strength;
  b.normal_radius_factor = brush->normal_radius_factor;
  b.area_radius_factor = brush->area_radius_factor;
  b.plane_offset = brush->plane_offset;
  b.x_first = curve.x_first;
  b.x_last = curve.x_last;
  b.mintable = curve.mintable;
  b.range = curve.range;
  std::memcpy(b.y, curve.y, sizeof(b.y));
  PassParams pp;
  std::memset(&pp, 0, sizeof(pp));
  for (int k = 0; k < 3; k++) {
    pp.loc[k] = location[k];
    pp.view[k] = brush->view_normal[k];
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int grid = (nverts + kNoAllocThreads - 1) / kNoAllocThreads;
  // The smooth schedule: 4 sub-steps per unit strength, the last fractional.
  float st = brush->strength;
  if (st < 0.0f) st = 0.0f;
  if (st > 1.0f) st = 1.0f;
  const int count = (int)(st * 4.0f);
  const float last = 4.0f * (st - (float)count * 0.25f);
  for (int it = 0; it <= count; it++) {
    pp.iter_strength = (it != count) ? 1.0f : last;
    pp.iteration = it;
    k_noalloc_compute<<<grid, kNoAllocThreads, 0, s>>>(m, b, pp, verts, nverts, scratch);
    k_noalloc_apply<<<grid, kNoAllocThreads, 0, s>>>(m, verts, nverts, scratch);
  }
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return noalloc_fail(SGPU_ERR_CUDA, cudaGetErrorString(e));
  return SGPU_OK;
}
