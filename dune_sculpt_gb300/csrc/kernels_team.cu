// Cluster-team launches of the persistent stroke kernel (team_kernel.cuh).
#include <algorithm>
#include <map>
#include <mutex>
#include <tuple>
#include <cuda_runtime.h>

#include "team_kernel.cuh"

namespace sgpu {

// Dynamic shared memory: smooth neighbour tables (float4); parents, culled
// list and offsets, leaf vertex counts (int); flush positions, leaf nodes
// (ushort, even counts); node marks (byte; at least the claim bitmap's
// 32-bit words).
size_t team_smem_bytes(int max_nodes, int max_leaves) {
  const size_t n = static_cast<size_t>(max_nodes), l = static_cast<size_t>(max_leaves);
  const size_t even_n = (n + 1) & ~static_cast<size_t>(1), even_l = (l + 1) & ~static_cast<size_t>(1);
  const size_t marks = std::max(n, 4 * ((n + 31) / 32));
  const size_t b = kStageBytes + sizeof(int) * (n + 3 * l + 3) +
                   sizeof(unsigned short) * (even_n + even_l) + marks;
  return (b + 15) & ~static_cast<size_t>(15);
}

int team_max_cluster() { return 16; }

template <int kMinBlocks, bool kOrig, bool kTwoLevel>
cudaError_t configure_team_build(size_t smem) {
  cudaError_t e = cudaFuncSetAttribute(k_team_stroke<kMinBlocks, kOrig, false, kTwoLevel>,
                                       cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(k_team_stroke<kMinBlocks, kOrig, false, kTwoLevel>,
                              cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
}

// The builds of one CTA-per-SM count; the one-CTA-per-SM builds also come
// with the two-level node search (launches with a large tree take them) and
// with paired symmetry passes (kernels_sym.cu).
template <int kMinBlocks>
cudaError_t configure_team_kernel(size_t smem) {
  cudaError_t e = configure_team_build<kMinBlocks, false, false>(smem);
  if (e == cudaSuccess) e = configure_team_build<kMinBlocks, true, false>(smem);
  if constexpr (kMinBlocks == 1) {
    if (e == cudaSuccess) e = configure_team_build<kMinBlocks, false, true>(smem);
    if (e == cudaSuccess) e = configure_team_build<kMinBlocks, true, true>(smem);
    if (e == cudaSuccess) e = configure_team_sym(smem);
  }
  return e;
}

static cudaLaunchConfig_t team_config(int cluster, int nteams, size_t smem, cudaStream_t s,
                                      cudaLaunchAttribute* attr) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(static_cast<unsigned>(cluster * nteams));
  cfg.blockDim = dim3(kTeamThreads);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = static_cast<unsigned>(cluster);
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cfg;
}

// Resident clusters of one build for (cluster size, shared memory), cached
// per device so that a launch makes no occupancy query.
template <int kMinBlocks>
static int active_clusters(int cluster, size_t smem) {
  static std::mutex mu;
  static std::map<std::tuple<int, int, size_t>, int> cache;
  static std::map<int, size_t> configured;  // per device: largest smem set so far
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  std::lock_guard<std::mutex> lock(mu);
  const auto key = std::make_tuple(dev, cluster, smem);
  auto it = cache.find(key);
  if (it != cache.end()) {
    if (configured[dev] < smem) {
      if (configure_team_kernel<kMinBlocks>(smem) != cudaSuccess) return 0;
      configured[dev] = smem;
    }
    return it->second;
  }
  if (configure_team_kernel<kMinBlocks>(std::max(smem, configured[dev])) != cudaSuccess) return 0;
  configured[dev] = std::max(smem, configured[dev]);
  cudaLaunchAttribute attr[1];
  cudaLaunchConfig_t cfg = team_config(cluster, 1, smem, nullptr, attr);
  int n = 0;
  if (cudaOccupancyMaxActiveClusters(&n, k_team_stroke<kMinBlocks, false, false>, &cfg) != cudaSuccess)
    return 0;
  cache[key] = n;
  return n;
}

int team_max_active_clusters(int cluster, int max_nodes, int max_leaves) {
  const size_t smem = team_smem_bytes(max_nodes, max_leaves);
  return std::max(active_clusters<1>(cluster, smem), active_clusters<2>(cluster, smem));
}

cudaError_t launch_team_stroke(const TeamArgs& a, int cluster, cudaStream_t s, int ctas_per_sm) {
  const size_t smem = team_smem_bytes(a.max_nodes, a.max_leaves);
  // auto: the one-CTA-per-SM build when it holds a team for every job
  const int n1 = ctas_per_sm == 2 ? 0 : active_clusters<1>(cluster, smem);
  const int n2 = ctas_per_sm == 1 || (ctas_per_sm == 0 && n1 >= a.njobs)
                     ? 0
                     : active_clusters<2>(cluster, smem);
  const bool two = n2 > n1;
  if ((two ? n2 : n1) <= 0) return cudaErrorInvalidConfiguration;
  const int nteams = std::max(1, std::min(a.njobs, two ? n2 : n1));
  cudaLaunchAttribute attr[1];
  cudaLaunchConfig_t cfg = team_config(cluster, nteams, smem, s, attr);
  if (two)
    return a.orig ? cudaLaunchKernelEx(&cfg, k_team_stroke<2, true, false>, a)
                  : cudaLaunchKernelEx(&cfg, k_team_stroke<2, false, false>, a);
  if (a.sym && !a.orig) return launch_team_sym(a, cfg, false);
  if (a.two_level)
    return a.orig ? cudaLaunchKernelEx(&cfg, k_team_stroke<1, true, false, true>, a)
                  : cudaLaunchKernelEx(&cfg, k_team_stroke<1, false, false, true>, a);
  return a.orig ? cudaLaunchKernelEx(&cfg, k_team_stroke<1, true, false>, a)
                : cudaLaunchKernelEx(&cfg, k_team_stroke<1, false, false>, a);
}

}  // namespace sgpu

