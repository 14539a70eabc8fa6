// Shared host/device layout of the flattened constraint tables.
//
// A SphereCollisionCst is flattened once into one contiguous device buffer: a header with
// counts and byte offsets, then FK slots (the links the constraint touches, parents first),
// control-joint records, sphere groups, spheres in structure-of-arrays form, self pairs and
// primitive SDF parameter blocks.  The model's mutable state (per-link local transform and
// base pose) lives in a separate device array so that several constraints share it, like
// the reference's shared KinematicModel (constraints/primitive.hpp:96).
#pragma once
#include <stdint.h>
#include <vector_types.h>

#define PM_MAX_SLOTS 64   // links one constraint can touch (FK slots)
#define PM_MAX_CTRL 64    // control joints (relevance bitmask width)
#define PM_MAX_CLOUDS 8
#define PM_GRID_B 4  // fine cells per block edge of the point-cloud grid
#define PM_GRID_CELLS_PER_BLOCK (PM_GRID_B * PM_GRID_B * PM_GRID_B)
#define PM_CL_UNITS 16  // distance quantum of the cell lists: the fine cell edge / 16
#define PM_GRID_SB 4    // blocks per super-block edge (the coarse level of the unbounded searches)
#define PM_FIELD16_UNIT 2.5e-4f  // metres per unit of the 16-bit field bounds

enum { PM_FK_STATE = 0, PM_FK_REV = 1, PM_FK_PRIS = 2 };
enum { PM_BASE_FIXED = 0, PM_BASE_FLOATING = 1, PM_BASE_PLANAR = 2 };
enum { PM_SDF_UNION = 0, PM_SDF_BOX = 1, PM_SDF_CYLINDER = 2, PM_SDF_SPHERE = 3, PM_SDF_GROUND = 4, PM_SDF_CLOUD = 5 };

// Model state rows of [qx qy qz qw tx ty tz qid] doubles (qid 0/1): row 0 is the base pose,
// row 1 + link is the link's local transform (tf_plink_to_hlink_cache_, kinematics.hpp:91).
#define PM_STATE_STRIDE 8
#define PM_STATE_BASE_ROW 0
#define PM_STATE_LINK_ROW(link) (1 + (link))

struct PmSlot {
  int32_t link;             // model link id (row of the state array)
  int32_t parent;           // parent slot, -1 for the root link (pose = base pose)
  int32_t mode;             // PM_FK_STATE | PM_FK_REV | PM_FK_PRIS
  int32_t qcol;             // q column of the control joint (REV/PRIS)
  int32_t origin_identity;  // joint origin orientation flag |w-1| < 1e-6 (kinematics.cpp:110-113)
  int32_t split;            // two-thread FP32 FK: phase << 1 | thread (phase 0: the trunk; phase 1: each
                            // thread its own subtrees under the trunk's branching slot)
  uint64_t relevant;        // bit i: control joint i moves this link (rptable, kinematics.cpp:340-363)
  double axis[3];
  double oq[4];             // joint origin quaternion x y z w
  double ot[3];             // joint origin translation
};

struct PmJoint {  // one per control joint, for Jacobian columns (algorithm.cpp:359-379)
  int32_t slot;   // slot of the joint's child link, -1 if the constraint never needs it
  int32_t prismatic;
  double axis[3];
};

struct PmGroup {
  int32_t slot;
  int32_t begin;  // first sphere
  int32_t count;
  int32_t only_self;
  double rel[3];  // group sphere centre in the link frame
  double radius;
};

struct PmPrim {
  int32_t kind;
  int32_t axis_aligned;
  int32_t z_axis_aligned;
  int32_t cloud;  // index into the cloud table for PM_SDF_CLOUD
  double lb[3], ub[3];
  double pos[3];
  double rot[9];      // row-major
  double rot_inv[9];  // row-major
  double a, b, c;     // box: half widths; cylinder: r, r^2, h/2; sphere: r, r^2; ground: h; cloud: radius
};

// Device view of one point-cloud grid (exact nearest neighbour).  Points are sorted by
// fine cell; fine cells are numbered block-major (B x B x B cells per block) so the points
// of one block are contiguous.  Only occupied cells carry a record.
struct PmGridDev {
  const double* px;        // sorted points, FP64 SoA
  const double* py;
  const double* pz;
  const float4* p32;       // same points, FP32 (x y z 0)
  const int32_t* blk_occ;  // per block: [first occupied-cell record, end)
  const float* blk_box;    // per block: lo xyz, hi xyz (empty: +inf/-inf)
  const float* cell_box;   // per occupied cell: lo xyz, hi xyz
  const int32_t* cell_pts; // per occupied cell: [first point, end)
  const float4* cell_rec;  // per occupied cell, both in one 32-byte record: (lo xyz, first point as int
                           // bits), (hi xyz, end as int bits)
  const uint8_t* edf;      // per block: Chebyshev distance in blocks to the nearest occupied block (capped at 255)
  const float* cell_lb;    // per fine cell (x fastest): lower bound (m) on the distance from the cell to any point
  const int2* cell_nn;     // per fine cell (x fastest): x = lower bound (m, float bits) on the distance from the
                           // cell centre to any point, y = sorted index of the centre's nearest point (-1: none
                           // within field_reach)
  const float4* cell_np;   // per fine cell: that nearest point itself (x y z as p32, w = its index as int
                           // bits, -1: none), so a query reads point and index in one load
  const uint16_t* cell_lb16;  // per fine cell: cell_nn's bound in units of PM_FIELD16_UNIT, rounded down (capped
                           // at 65535): a 2-byte copy for the checks that need only the bound
  float field_reach;       // cell_nn searched up to this distance from each centre
  int32_t pad_nn;
  const int2* blk_list;    // per block: [first, end) of its candidate list in blk_cand (first = -1: none)
  const int2* blk_cand;    // candidate lists: (occupied block, float bits of its box distance from the listing
                           // block's box), nearest first, within blk_reach
  const float* blk_reach;  // per block: a query in the block whose search bound is below this needs only its list
  const int4* cand4;       // blk_cand widened for the warp searches: (first occupied-cell record, end, block,
                           // float bits of the distance), so one load gives the cell range
  const float4* cand_box;  // per list entry, its block's box: (lo xyz, 0), (hi xyz, 0)
  const int2* cl_rng;      // per fine cell (x fastest): [first, end) of its cell list in cl_ent (first = -1: none)
  const uint32_t* cl_ent;  // cell lists, nearest first: occupied-cell record (low 24 bits) | a lower bound on the
                           // distance between that record's box and the listing cell's box, in units of
                           // cell / PM_CL_UNITS, rounded down and capped at 255 (high 8 bits); a cell's list holds
                           // every occupied cell that can contain the nearest point of a query inside it
  const int2* sb_rng;      // per non-empty super-block (PM_GRID_SB^3 blocks): [first, end) of its occupied blocks in sb_blk
  const int32_t* sb_blk;   // occupied blocks, grouped by super-block
  const float* sb_box;     // per non-empty super-block: box of its points (lo xyz, hi xyz)
  int32_t n_sb;            // non-empty super-blocks
  int32_t pad_sb;
  // FP32 copies for the FP32 queries (no FP64 arithmetic on their path): origin, block edge and
  // its reciprocal, fine cell edge and its reciprocal, and the points' box (rounded outwards)
  float o32[3], blk32, inv_blk32, cell32, inv_cell32;
  float box_lo32[3], box_hi32[3];
  int32_t nbx, nby, nbz;   // blocks per axis
  int32_t n_points;
  double origin[3];        // grid origin (world)
  double block;            // block edge length (PM_GRID_B fine cells)
  double lb[3], ub[3];     // CloudSDF AABB (point bounds -/+ radius)
  double radius;
};

// One term of a pose constraint: LinkPoseCst target of one link (constraints/primitive_link_pose.cpp:
// 31-60; dim 3, 6 or 7) or LinkPositionBoundCst (primitive_link_position_bound.cpp:34-79).
enum { PM_TERM_LINK_POSE = 0, PM_TERM_POSITION_BOUND = 1 };
struct PmPoseTerm {
  int32_t kind;
  int32_t slot;   // FK slot of the link
  int32_t dim;    // rows of this term: 3 / 6 / 7 (pose) or 1 / 2 (bound)
  int32_t axis;   // bound: 0 x, 1 y, 2 z
  int32_t has_lb, has_ub, pad0, pad1;
  double target[7];
  double lb, ub;
};

// Link-position bounds of an IneqCompositeCst (constraints/composite_constraint.hpp:98-105) made of
// a SphereCollisionCst and LinkPositionBoundCst members, checked by the fast kernels on the
// collision constraint's FK: n device terms of kind PM_TERM_POSITION_BOUND whose slots index the
// collision constraint's tables.
struct PmLinkBounds {
  const PmPoseTerm* t;
  int32_t n;
};

struct PmTablesHdr {
  int32_t n_slots, n_ctrl, n_groups, n_spheres;
  int32_t n_pairs, n_prims, q_dim, base_type;
  int32_t root_slot, n_clouds, pad0, pad1;
  int64_t off_slots, off_joints, off_groups, off_sx, off_sy, off_sz, off_sr, off_sgroup, off_pairs, off_prims, off_clouds;
  int64_t total_bytes;
};

#ifdef __CUDACC__
#define PM_HD __host__ __device__ __forceinline__
#else
#define PM_HD inline
#endif

template <class T>
PM_HD const T* pm_at(const PmTablesHdr* h, int64_t off) {
  return reinterpret_cast<const T*>(reinterpret_cast<const char*>(h) + off);
}
