// The persistent stroke kernel's builds that pair the two passes of a
// single-axis symmetry (team_kernel.cuh, kSym): one node search for both
// passes, and one area phase and one sweep for both when their leaf lists
// are disjoint under a tool that reads and writes only the vertex itself.
// One CTA per SM, no stroke-start brushes; cluster teams and the whole-GPU
// team, with the one- and two-level node search.  Kept apart from the other
// builds so that launches without such a stroke run code without the pairing.
#include <cuda_runtime.h>

#include "team_kernel.cuh"

namespace sgpu {

template <bool kTwoLevel>
static cudaError_t configure_cluster_sym(size_t smem) {
  const cudaError_t e = cudaFuncSetAttribute(k_team_stroke<1, false, false, kTwoLevel, true>,
                                             cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(k_team_stroke<1, false, false, kTwoLevel, true>,
                              cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
}

cudaError_t configure_team_sym(size_t smem) {
  const cudaError_t e = configure_cluster_sym<false>(smem);
  return e != cudaSuccess ? e : configure_cluster_sym<true>(smem);
}

cudaError_t configure_wide_sym(size_t smem) {
  const cudaError_t e = cudaFuncSetAttribute(k_team_stroke<1, false, true, false, true>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             static_cast<int>(smem));
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(k_team_stroke<1, false, true, true, true>,
                              cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
}

bool sym_wide_ok(size_t smem) {
  int n0 = 0, n1 = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n0, k_team_stroke<1, false, true, false, true>,
                                                    kTeamThreads, smem) != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n1, k_team_stroke<1, false, true, true, true>,
                                                    kTeamThreads, smem) != cudaSuccess)
    return false;
  return n0 >= 1 && n1 >= 1;
}

cudaError_t launch_team_sym(const TeamArgs& a, const cudaLaunchConfig_t& cfg, bool wide) {
  if (wide)
    return a.two_level ? cudaLaunchKernelEx(&cfg, k_team_stroke<1, false, true, true, true>, a)
                       : cudaLaunchKernelEx(&cfg, k_team_stroke<1, false, true, false, true>, a);
  return a.two_level ? cudaLaunchKernelEx(&cfg, k_team_stroke<1, false, false, true, true>, a)
                     : cudaLaunchKernelEx(&cfg, k_team_stroke<1, false, false, false, true>, a);
}

}  // namespace sgpu
