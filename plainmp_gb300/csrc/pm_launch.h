// Host-side launchers of the device kernels (implemented in the .cu translation units).
// All pointers are device pointers; every launcher enqueues on `stream` and returns the
// launch status.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "pm_common.h"

namespace pmg {

// ---- opt-in kernel timing (host.cpp): events around a launch on its stream
bool prof_on();
void prof_begin(const char* kernel, cudaStream_t s);
void prof_end(const char* kernel, cudaStream_t s);

// ---- model state (k_plain.cu)
// recs: per joint to set, a PmSlot whose `link` is the child link and mode REV/PRIS.
cudaError_t launch_set_joints(double* state, const PmSlot* recs, const double* q, int n, int accurate, cudaStream_t s);
// base pose from q for PLANAR/FLOATING (q points at the base part), written to row 0.
cudaError_t launch_set_base_from_q(double* state, int base_type, const double* qbase, cudaStream_t s);
// link poses of the current state: parents[n_link] (-1 root), links[n] -> out7[n*7]
cudaError_t launch_link_poses(const double* state, const int32_t* parents, const int32_t* links, int n, double* out7,
                              cudaStream_t s);

// ---- constraint batches (k_plain.cu)
cudaError_t launch_is_valid64(const PmTablesHdr* T, const double* state, const double* q, int64_t B, uint8_t* out,
                              cudaStream_t s);
cudaError_t launch_evaluate64(const PmTablesHdr* T, const double* state, const double* q, int64_t B, int high_accuracy,
                              double* vals, double* jac, cudaStream_t s);
// centres (B x n_spheres x 3) is required: the distances are computed from it
cudaError_t launch_sphere_dist64(const PmTablesHdr* T, const PmTablesHdr& h, const double* state, const double* q, int64_t B,
                                 int high_accuracy, double* dist, double* centres, cudaStream_t s);
// spheres (all: groups=0, group spheres: groups=1) of the current state, out4 n x 4
cudaError_t launch_spheres_of_state(const PmTablesHdr* T, const double* state, int groups, double* out4, cudaStream_t s);
// checkMotion over E edges; seq: 128 x 128 int16 sequence table; width: q_dim (box) or NULL
cudaError_t launch_check_motion64(const PmTablesHdr* T, const double* state, const double* s1, const double* s2, int64_t E,
                                  int type, const double* width, double resolution, const int16_t* seq, uint8_t* out,
                                  unsigned long long* n_checked, cudaStream_t s);

// ---- fast path (k_fast.cu): FP32 decisions + FP64 recheck of uncertain terms.
size_t fast_smem_bytes(const PmTablesHdr& h, int cpb, bool want_dist);
// The fast kernels' queue records hold at most 65,535 spheres and 32,767 primitives.
bool fast_table_sizes_ok(const PmTablesHdr& h);
// SM count of the current device (cached per device); the offset table of the warp searches,
// uploaded to the current device once.
cudaError_t sm_count(int* n);
cudaError_t upload_offsets();
// Tuning of the fast kernels beyond the launch shape (the autotuner's other dimensions).
struct FastTuning {
  int sphere_tile_log2 = 0;  // log2 of the spheres per warp row of sphere tasks (0: the least for the shape)
  int hq_blocks_per_sm = 4;  // k_hard_queries: blocks of 256 threads per SM
};
// bnd: link-position bounds of a composite constraint, decided in the same kernels (none by default).
// hq (hq_cap 32-byte entries) and hq_count (zeroed by the caller): with distances, the hard cloud
// queries are answered by a second kernel over this global queue; null keeps them in the block.
cudaError_t launch_fast_valid(const PmTablesHdr* T, const PmTablesHdr& h, const double* state, const double* q, int64_t B,
                              uint8_t* out, float* dist32, float cutoff, int4* items, unsigned int* count, unsigned int cap,
                              uint8_t* overflow, unsigned long long* stats, int cpb, int nt, cudaStream_t s, void* hq = nullptr,
                              unsigned long long* hq_count = nullptr, unsigned int hq_cap = 0, const FastTuning& tune = FastTuning(),
                              PmLinkBounds bnd = PmLinkBounds{nullptr, 0});

cudaError_t launch_fast_edges(const PmTablesHdr* T, const PmTablesHdr& h, const double* state, const double* s1, const double* s2,
                              int64_t E, int type, const double* width, double resolution, const int16_t* seq, double* sr, int32_t* n,
                              int64_t* off, unsigned long long* next, uint8_t* out, int4* items, unsigned int* count,
                              unsigned int cap, uint8_t* overflow, unsigned long long* stats, int cpb, int nt, int n_sm, cudaStream_t s,
                              PmLinkBounds bnd = PmLinkBounds{nullptr, 0});

// ---- differentiable costs (k_grad.cu): FP32 forward + reverse-mode adjoint
#define PM_GRAD_MAXQ (PM_MAX_CTRL + 8)
struct GradArgs {
  int mode;       // 0: hinge sum (+ pose term); 1: min signed distance over spheres (the ext row)
  int pose_slot;  // FK slot of the pose term, -1: none
  float w_pos, w_rot, w_col, margin, cutoff, w_smooth, lr;
  int steps;      // > 0: gradient descent of that many steps inside the launch
  int clamp;      // descent: clamp q to [lo, hi]
  float lo[PM_GRAD_MAXQ], hi[PM_GRAD_MAXQ], dofw2[PM_GRAD_MAXQ];
};
size_t grad_smem_bytes(const PmTablesHdr& h);
// IK batch: q B x q_dim (updated in place when steps > 0), target B x 7 (x y z qx qy qz qw) or
// NULL; cost B (final cost after a descent), grad B x q_dim or NULL, hist B x steps or NULL.
cudaError_t launch_ik_cost(const PmTablesHdr* T, const PmTablesHdr& h, const double* state, const GradArgs& a, float* q,
                           const float* target, int64_t B, float* cost, float* grad, float* hist, cudaStream_t s);
// Trajectory batch: q n_wp x q_dim, off n_traj + 1 waypoint offsets; wp_cost n_wp scratch.
cudaError_t launch_traj_cost(const PmTablesHdr* T, const PmTablesHdr& h, const double* state, const GradArgs& a, const float* q,
                             const int64_t* off, int64_t n_traj, int64_t n_wp, float* wp_cost, float* cost, float* grad,
                             cudaStream_t s);
// FP64 world pose (x y z qx qy qz qw) of one FK slot for B configurations (sin/cos FK).
cudaError_t launch_link_pose64(const PmTablesHdr* T, const double* state, const double* q, int64_t B, int slot, double* out7,
                               cudaStream_t s);

// ---- pose constraints (k_pose.cu): LinkPoseCst / LinkPositionBoundCst terms
cudaError_t launch_posecst_eval64(const PmTablesHdr* T, const double* state, const PmPoseTerm* terms, int n_terms, int cst_dim,
                                  const double* q, int64_t B, double* vals, double* jac, cudaStream_t s);
cudaError_t launch_posecst_valid64(const PmTablesHdr* T, const double* state, const PmPoseTerm* terms, int n_terms, const double* q,
                                   int64_t B, uint8_t* out, cudaStream_t s);

// ---- SDF utilities (k_plain.cu): prims/clouds describe one SDF (a union is flattened)
cudaError_t launch_sdf_points(const PmPrim* prims, int n_prims, const PmGridDev* clouds, int is_union, const double* pts,
                              const double* radii, int64_t n, double* eval_out, uint8_t* outside_out, cudaStream_t s);
cudaError_t launch_cloud_nearest(const PmGridDev* grid, const double* pts, int64_t n, double* sq, double* near3,
                                 cudaStream_t s);

// ---- FMA throughput microbenchmark (k_peak.cu): blocks x threads threads, 16 flops per iteration
// each; out receives blocks * threads values of the element type (double when fp64).
cudaError_t launch_fma_peak(int fp64, int iters, void* out, int blocks, int threads, cudaStream_t s);

// ---- point-cloud grid build (k_grid.cu)
struct GridBuild {
  // inputs
  const double* pts;  // device, n x 3
  int64_t n;
  double radius;
  double cell;  // fine cell edge
  double field_reach = 0.3;  // nearest-point field: search radius around each cell centre
  double list_reach = 0.25;  // per-cell lists for the cells whose nearest-point bound is below this
  // outputs (owned by the caller after the call; freed with grid_free)
  PmGridDev dev;
  void* allocs[28];
  int n_allocs;
  // sizes of what was built: occupied fine cells, candidate-list entries, device bytes kept
  int64_t n_occupied = 0, n_cand = 0, bytes = 0, n_cell_list = 0;
};
// Builds the grid synchronously on `s` (allocates device memory); returns cudaSuccess or the
// first CUDA error.  host_lb/host_ub receive the CloudSDF AABB.
cudaError_t grid_build(GridBuild& g, cudaStream_t s);
void grid_free(GridBuild& g);

}  // namespace pmg
