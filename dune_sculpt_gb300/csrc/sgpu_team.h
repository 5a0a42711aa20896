// Persistent stroke kernel interface (kernels_team.cu).
#pragma once

#include <cuda_runtime.h>

#include "sgpu_device.cuh"

namespace sgpu {

// One mesh's whole stroke.
struct TeamJob {
  int mesh;      // index into TeamArgs::meshes
  int ndabs;
  int symmetry;  // PAINT_SYMM_* bits
  int use_orig;  // cull against orig_vb
  float view[3];
  float pad;
  const float* dabs;  // ndabs * 6 floats (location, grab delta), device memory
  const int* tools;   // per-dab tool or nullptr, device memory
  DevBrush brush;     // brush.tool: the default tool
};

// Per-job state of the lockstep batch launch (k_lock_stroke), in device
// memory, zeroed by the host before the launch.
struct LockJob {
  PassParams pp;       // the job's current symmetry pass (written by its cull CTA)
  BrushFrame frame;    // brush frame of the pass
  int cnt, total;      // culled leaves and their brush-visible vertices
  int go;              // 1: the pass moves vertices (frame valid, leaves marked)
  unsigned int ticket;  // area items of the pass finished (the last one reduces)
  int nh[3];           // smooth hits, by the job's smooth pass number mod 3
  int pad;
};

struct TeamArgs {
  const DevMesh* meshes;
  const TeamJob* jobs;
  int njobs;
  int* next_job;  // job counter, zero at launch
  // whole-GPU team: barrier counter (zero at launch), status word (zero at
  // launch; SGPU_ERR_TIMEOUT when a barrier wait ran out), the wait limit,
  // and extra arrivals the barrier waits for (0; a test hook sets 1)
  unsigned int* bar;
  int* status;
  unsigned long long wait_ns;
  int bar_extra;
  int orig;       // some job has grab, elastic deform or layer dabs
  int two_level;  // some mesh's node search takes two levels (its build runs it)
  int sym;        // some stroke mirrors in one axis (the builds that pair passes run it)
  int max_nodes, max_leaves;  // shared-memory sizing over the meshes
  // profiling (nullable): algorithmic bytes and nanoseconds per phase
  unsigned long long* prof_bytes;  // kTeamPhases entries
  unsigned long long* phase_ns;    // kTeamPhases entries
  // lockstep batch launch only: per-job state and per-job brush (the tool of
  // the current dab is written into it)
  LockJob* lock;
  DevBrush* lbrush;
};

// Phases of a dab in the persistent kernel (profiling).
enum TeamPhase {
  kPhCull = 0,
  kPhArea,
  kPhBrush,
  kPhApply,
  kPhUpdate,
  kPhFlush,
  kPhJob,
  kPhGridFaces,  // GRIDS: inner normals, face seams and centres
  kPhGridSeams,  // GRIDS: base edges and corners
  kTeamPhases
};

size_t team_smem_bytes(int max_nodes, int max_leaves);
int team_max_cluster();
int team_max_active_clusters(int cluster, int max_nodes, int max_leaves);
// Launches min(njobs, resident teams) teams.  ctas_per_sm: 1 or 2 picks the
// build (255 or 128 registers per thread); 0 takes the one-CTA-per-SM build
// when it holds a team for every job, else the one that holds more teams.
cudaError_t launch_team_stroke(const TeamArgs& a, int cluster, cudaStream_t s, int ctas_per_sm);
// The whole-GPU team: CTAs of one cooperative launch (one per SM), or 0 when
// the device or the shared-memory size does not allow it.
int team_wide_ctas(int max_nodes, int max_leaves);
// Upper bound of team_wide_ctas on any device (sizes the smooth slot arrays).
constexpr int kTeamMaxWideCtas = 1024;
cudaError_t launch_team_stroke_wide(const TeamArgs& a, int nctas, cudaStream_t s);
// The builds that pair the passes of a single-axis symmetry (kernels_sym.cu):
// one CTA per SM, no stroke-start brushes; cluster and whole-GPU teams with
// either node search.  configure_* set their shared-memory limit (and the
// cluster builds' non-portable cluster sizes); sym_wide_ok: each whole-GPU
// build holds a CTA on an SM with smem bytes.
cudaError_t configure_team_sym(size_t smem);
cudaError_t configure_wide_sym(size_t smem);
bool sym_wide_ok(size_t smem);
cudaError_t launch_team_sym(const TeamArgs& a, const cudaLaunchConfig_t& cfg, bool wide);

// Lockstep batch launch (kernels_lock.cu): every CTA of one cooperative
// launch (one per SM) runs every stroke of the batch, dab by dab; each phase
// pools the work items of all meshes (leaf blocks, claimed faces, touched
// leaf chunks, tagged vertices) over the whole GPU.  Jobs run no grab,
// elastic deform or layer dabs; GRIDS faces must fit the on-chip stage.
constexpr int kLockMaxJobs = 1024;
size_t lock_smem_bytes(int max_nodes, int max_leaves);
// CTAs of the launch with per_sm (1 or 2) CTAs on every SM, or 0 when the
// device cannot hold it.
int lock_ctas(int max_nodes, int max_leaves, int per_sm);
cudaError_t launch_lock_stroke(const TeamArgs& a, int nctas, int per_sm, cudaStream_t s);
// Whether a claimed face's grids of this size fit the on-chip stage.
bool lock_grids_fit(int grid_size);

}  // namespace sgpu
