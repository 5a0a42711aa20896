// Whole-GPU launches of the persistent stroke kernel (team_kernel.cuh): one
// cooperative launch with one CTA per SM, all of them one team, so every dab
// phase of a single stroke is spread over the whole GPU instead of one
// cluster's SMs.  The barriers between phases count arrivals in global memory
// (TeamBarrier<true>); the cooperative launch guarantees that every CTA is
// resident, so every CTA reaches every barrier.
#include <algorithm>
#include <map>
#include <mutex>
#include <utility>
#include <cuda_runtime.h>

#include "team_kernel.cuh"

namespace sgpu {

template <bool kOrig>
static cudaError_t configure_wide(size_t smem) {
  const cudaError_t e = cudaFuncSetAttribute(k_team_stroke<1, kOrig, true>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             static_cast<int>(smem));
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(k_team_stroke<1, kOrig, true, true>,
                              cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
}

int team_wide_ctas(int max_nodes, int max_leaves) {
  static std::mutex mu;
  static std::map<std::pair<int, size_t>, int> cache;
  static std::map<int, size_t> configured;  // per device: largest smem set so far
  const size_t smem = team_smem_bytes(max_nodes, max_leaves);
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  std::lock_guard<std::mutex> lock(mu);
  const auto key = std::make_pair(dev, smem);
  auto it = cache.find(key);
  if (it != cache.end() && configured[dev] >= smem) return it->second;
  int coop = 0, sms = 0;
  if (cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev) != cudaSuccess || !coop)
    return 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
  const size_t want = std::max(smem, configured[dev]);
  if (configure_wide<false>(want) != cudaSuccess || configure_wide<true>(want) != cudaSuccess ||
      configure_wide_sym(want) != cudaSuccess)
    return 0;
  configured[dev] = want;
  int n0 = 0, n1 = 0;
  int n2 = 0, n3 = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n0, k_team_stroke<1, false, true>,
                                                    kTeamThreads, smem) != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n1, k_team_stroke<1, true, true>,
                                                    kTeamThreads, smem) != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n2, k_team_stroke<1, false, true, true>,
                                                    kTeamThreads, smem) != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n3, k_team_stroke<1, true, true, true>,
                                                    kTeamThreads, smem) != cudaSuccess)
    return 0;
  const int n = (std::min(std::min(n0, n1), std::min(n2, n3)) >= 1 && sym_wide_ok(smem))
                    ? std::min(sms, kTeamMaxWideCtas) : 0;
  cache[key] = n;
  return n;
}

cudaError_t launch_team_stroke_wide(const TeamArgs& a, int nctas, cudaStream_t s) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(static_cast<unsigned>(nctas));
  cfg.blockDim = dim3(kTeamThreads);
  cfg.dynamicSmemBytes = team_smem_bytes(a.max_nodes, a.max_leaves);
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  if (a.sym && !a.orig) return launch_team_sym(a, cfg, true);
  if (a.two_level)
    return a.orig ? cudaLaunchKernelEx(&cfg, k_team_stroke<1, true, true, true>, a)
                  : cudaLaunchKernelEx(&cfg, k_team_stroke<1, false, true, true>, a);
  return a.orig ? cudaLaunchKernelEx(&cfg, k_team_stroke<1, true, true>, a)
                : cudaLaunchKernelEx(&cfg, k_team_stroke<1, false, true>, a);
}

}  // namespace sgpu
