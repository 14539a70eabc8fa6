/*
 * pmgpu.h -- C ABI of the GB300 collision-checking hot path (plainmp_gb300).
 *
 * Drop-in boundary for plainmp's KinematicModel / SphereCollisionCst / primitive SDFs /
 * OMPL motion validator.  Every entry point returns an int status (PMGPU_OK == 0) and never
 * throws; pmgpu_last_error() gives the message of the last failure on the calling thread.
 * Paths cited as file:line are relative to the plainmp project (v0.3.4).
 *
 * Memory: batch entry points take a `mem` argument.  PMGPU_MEM_HOST means all array
 * arguments are host pointers; the call copies them to the device, runs, copies results
 * back and returns after the stream has finished.  PMGPU_MEM_DEVICE means all array
 * arguments are device pointers; the call only enqueues work on `stream` (a cudaStream_t,
 * NULL = legacy default stream) and returns.
 *
 * Threading: objects are thread-compatible, not thread-safe, like the reference (mutable
 * model state, kinematics/kinematics.hpp:89-91).  Use one model/constraint per host thread.
 */
#ifndef PMGPU_H_
#define PMGPU_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PMGPU_OK 0
#define PMGPU_ERR_INVALID 1 /* bad argument: unknown name, size, NaN... (std::invalid_argument) */
#define PMGPU_ERR_RUNTIME 2 /* reference-side runtime_error equivalents (bad URDF, bad pairs) */
#define PMGPU_ERR_CUDA 3    /* CUDA failure or no CUDA device */
#define PMGPU_ERR_TIMEOUT 4 /* a bounded device-side wait gave up */

#define PMGPU_MEM_HOST 0
#define PMGPU_MEM_DEVICE 1

/* BaseType (kinematics/kinematics.hpp:49; bindings/kinematics.cpp:161-164) */
#define PMGPU_BASE_FIXED 0
#define PMGPU_BASE_FLOATING 1
#define PMGPU_BASE_PLANAR 2

/* SDFType (collision/primitive_sdf.hpp:77) */
#define PMGPU_SDF_UNION 0
#define PMGPU_SDF_BOX 1
#define PMGPU_SDF_CYLINDER 2
#define PMGPU_SDF_SPHERE 3
#define PMGPU_SDF_GROUND 4
#define PMGPU_SDF_CLOUD 5

typedef struct pmgpu_model pmgpu_model;
typedef struct pmgpu_sdf pmgpu_sdf;
typedef struct pmgpu_cst pmgpu_cst;

/* Last error message of this thread ("" if none). */
const char* pmgpu_last_error(void);
/* ABI version (major*10000 + minor*100 + patch). */
int pmgpu_version(void);
/* Number of CUDA devices visible (0 on a host without GPU; never fails). */
int pmgpu_device_count(void);

/* ---------------------------------------------------------------- KinematicModel
 * Replaces KinematicModel<double>::KinematicModel(xml) (kinematics/kinematics.cpp:183-223),
 * bound as KinematicModel(urdf_string) (bindings/kinematics.cpp:145-147).  Parsing and the
 * tree numbering are host work; the device state is allocated on first GPU use. */
int pmgpu_model_create(const char* urdf_xml, pmgpu_model** out);
void pmgpu_model_destroy(pmgpu_model* m);
/* counts: links, movable joints (num_dof_), root link id */
int pmgpu_model_counts(const pmgpu_model* m, int* n_links, int* n_joints, int* root_link);
/* get_joint_ids / get_link_ids (kinematics.cpp:236-276): unknown name -> PMGPU_ERR_INVALID */
int pmgpu_model_get_joint_ids(const pmgpu_model* m, const char* const* names, int n, int64_t* ids_out);
int pmgpu_model_get_link_ids(const pmgpu_model* m, const char* const* names, int n, int64_t* ids_out);
/* get_joint_position_limits (kinematics.cpp:251-261) */
int pmgpu_model_get_joint_position_limits(const pmgpu_model* m, const int64_t* ids, int n, double* lower, double* upper);
/* name of a link / joint by id (buffer of size cap; truncated) */
int pmgpu_model_link_name(const pmgpu_model* m, int64_t id, char* buf, int cap);
int pmgpu_model_joint_name(const pmgpu_model* m, int64_t id, char* buf, int cap);
/* Structure dump for tests: per link parent id (-1 root) and initial local transform
 * [x y z qx qy qz qw] + quat-identity flag; per joint child link id, type, axis, origin flag. */
int pmgpu_model_structure(const pmgpu_model* m, int32_t* link_parent, double* link_tf7, int32_t* link_tf_qid,
                          int32_t* joint_child, int32_t* joint_type, double* joint_axis3, int32_t* joint_origin_qid);
/* set_joint_positions(ids, q, accurate) (bindings/kinematics.cpp:150-152 ->
 * algorithm.cpp:88-158): the local transforms are computed on the device. */
int pmgpu_model_set_joint_positions(pmgpu_model* m, const int64_t* ids, int n, const double* q, int accurate);
int pmgpu_model_get_joint_positions(const pmgpu_model* m, const int64_t* ids, int n, double* q);
/* set_base_pose / get_base_pose with [x y z qx qy qz qw] (kinematic_model_wrapper.cpp:208-216) */
int pmgpu_model_set_base_pose(pmgpu_model* m, const double* pose7);
int pmgpu_model_get_base_pose(const pmgpu_model* m, double* pose7);
/* debug_get_link_pose for n links of the current state (kinematic_model_wrapper.cpp:218-222),
 * computed by a device FK pass; out is n x 7. */
int pmgpu_model_link_poses(pmgpu_model* m, const int64_t* link_ids, int n, double* out7);
/* add_new_link(name, parent, xyz, rpy, consider_rotation) (kinematic_model_wrapper.cpp:198-206,
 * kinematics.cpp:278-338).  consider_rotation=0 links keep only the translation. */
int pmgpu_model_add_new_link(pmgpu_model* m, const char* name, const char* parent, const double* xyz, const double* rpy,
                             int consider_rotation, int64_t* id_out);

/* Pose(position, rotation) alignment flags and inverse rotation (primitive_sdf.hpp:30-68):
 * axis_aligned = rotation isApprox identity, z_axis_aligned per the 1e-6 test. */
int pmgpu_pose_flags(const double* rot9, int* axis_aligned, int* z_axis_aligned, double* rot_inv9);

/* ---------------------------------------------------------------- SDFs
 * BoxSDF(width, Pose), CylinderSDF(r, h, Pose), SphereSDF(r, Pose), GroundSDF(h),
 * CloudSDF(points, radius), UnionSDF([...]) (bindings/primitive.cpp:18-111,
 * collision/primitive_sdf.hpp:99-612).  rot is a row-major 3x3 rotation matrix. */
int pmgpu_sdf_box_create(const double* width3, const double* pos3, const double* rot9, pmgpu_sdf** out);
int pmgpu_sdf_cylinder_create(double radius, double height, const double* pos3, const double* rot9, pmgpu_sdf** out);
int pmgpu_sdf_sphere_create(double radius, const double* pos3, const double* rot9, pmgpu_sdf** out);
int pmgpu_sdf_ground_create(double height, pmgpu_sdf** out);
/* CloudSDF: points n x 3 (double; float32 clouds widen exactly).  The device builds a
 * uniform grid that answers exact nearest-neighbour queries in place of the KD-tree
 * (collision/kdtree.cpp:20-96).  cell_size <= 0 picks a size from the point density. */
int pmgpu_sdf_cloud_create(const double* points, int64_t n, double radius, double cell_size, pmgpu_sdf** out);
/* Sizes of a cloud's device grid (built on first call if needed): out6 = {points, occupied fine
 * cells, blocks, fine cells of the nearest-point field, candidate-list entries, device bytes}.
 * No counterpart in the reference (its KD-tree lives in host memory). */
int pmgpu_sdf_cloud_stats(pmgpu_sdf* sdf, int64_t* out6);
/* UnionSDF(members): members are shared, not copied (primitive_sdf.hpp:102) */
int pmgpu_sdf_union_create(pmgpu_sdf* const* members, int n, pmgpu_sdf** out);
/* UnionSDF.add / merge (primitive_sdf.hpp:115-133): clone=1 deep-copies */
int pmgpu_sdf_union_add(pmgpu_sdf* u, pmgpu_sdf* member, int clone);
int pmgpu_sdf_clone(const pmgpu_sdf* s, pmgpu_sdf** out);
/* Release this handle (members of a union stay alive while referenced). */
void pmgpu_sdf_destroy(pmgpu_sdf* s);
/* translate / rotate_z wrt world (primitive_sdf.hpp:135-145, 265-273); Ground and Cloud
 * reject them like the reference (PMGPU_ERR_RUNTIME). */
int pmgpu_sdf_translate(pmgpu_sdf* s, const double* t3);
int pmgpu_sdf_rotate_z(pmgpu_sdf* s, double angle);
/* kind, aabb (lb/ub), pose flags, pose position/rotation (zeros for non-transformable) */
int pmgpu_sdf_info(const pmgpu_sdf* s, int* kind, double* lb3, double* ub3, int* axis_aligned, int* z_axis_aligned,
                   double* pos3, double* rot9);
/* evaluate(p) / evaluate_batch / is_outside(p, r) on the device for n points (n x 3). */
int pmgpu_sdf_evaluate(pmgpu_sdf* s, const double* points, int64_t n, double* out, int mem, void* stream);
int pmgpu_sdf_is_outside(pmgpu_sdf* s, const double* points, const double* radii, int64_t n, uint8_t* out, int mem,
                         void* stream);
/* Cloud grid nearest neighbour (KDTree.sqdist / query, kdtree.cpp:75-87): squared distance and
 * nearest point for n queries. */
int pmgpu_cloud_nearest(pmgpu_sdf* cloud, const double* points, int64_t n, double* sqdist, double* nearest3, int mem,
                        void* stream);

/* ---------------------------------------------------------------- SphereCollisionCst
 * SphereCollisionCst(kin, control_joint_names, base_type, sphere_specs, selcol_pairs,
 * fixed_sdf, reorder_spheres) (bindings/constraint.cpp:73-79;
 * constraints/primitive_sphere_collision.cpp:117-179).  Sphere specs are packed: spec s has
 * counts[s] spheres whose centres are rel_xyz[3*k..3*k+2] and radii[k] (k running over all
 * spheres of all specs in order).  fixed_sdf may be NULL. */
int pmgpu_cst_create(pmgpu_model* kin, const char* const* control_joints, int n_joints, int base_type, int n_specs,
                     const char* const* spec_links, const int32_t* counts, const double* rel_xyz, const double* radii,
                     const uint8_t* only_self, int n_pairs, const char* const* pair_a, const char* const* pair_b,
                     pmgpu_sdf* fixed_sdf, int reorder_spheres, pmgpu_cst** out);
void pmgpu_cst_destroy(pmgpu_cst* c);
/* set_sdf (primitive_sphere_collision.hpp:195-198); NULL clears it. */
int pmgpu_cst_set_sdf(pmgpu_cst* c, pmgpu_sdf* sdf);
/* q_dim (primitive.hpp:68-72), cst_dim (primitive_sphere_collision.hpp:220-223), sphere/group counts */
int pmgpu_cst_dims(const pmgpu_cst* c, int* q_dim, int* cst_dim, int* n_spheres, int* n_groups);
/* Constructed group table (post-reorder sphere order): link id, group radius, group centre
 * (link frame), only-self flag, per-sphere relative centres and radii. */
int pmgpu_cst_groups(const pmgpu_cst* c, int32_t* link, double* radius, double* centre3, int32_t* only_self,
                     double* sphere_rel3, double* sphere_radii);
/* update_kintree(q, high_accuracy) (primitive.hpp:38-62) on the shared model state. */
int pmgpu_cst_update_kintree(pmgpu_cst* c, const double* q, int high_accuracy);
/* get_all_spheres / get_group_spheres (primitive_sphere_collision.cpp:401-424) of the
 * current model state: out is n x 4 [x y z r]. */
int pmgpu_cst_get_all_spheres(pmgpu_cst* c, double* out4);
int pmgpu_cst_get_group_spheres(pmgpu_cst* c, double* out4);

/* is_valid(q) for B configs (IneqConstraintBase::is_valid, primitive.hpp:113-117 ->
 * is_valid_dirty, primitive_sphere_collision.cpp:181-254).  Plain method: FP64, Taylor
 * sin/cos for FIXED bases, the reference's branch structure, one device thread per config.
 * q is B x q_dim row-major; out[b] is 1 (valid) or 0. */
int pmgpu_cst_is_valid(pmgpu_cst* c, const double* q, int64_t B, uint8_t* out, int mem, void* stream);
/* evaluate(q) for B configs (ConstraintBase::evaluate, primitive.hpp:74-79 ->
 * evaluate_dirty, primitive_sphere_collision.cpp:256-399): vals B x cst_dim, jac
 * B x cst_dim x q_dim (row-major), FP64 with libm-accuracy sin/cos. */
int pmgpu_cst_evaluate(pmgpu_cst* c, const double* q, int64_t B, double* vals, double* jac, int mem, void* stream);
/* Per-sphere signed distance min_k(sdf_k.evaluate(c_s) - r_s) over the flattened SDFs and
 * the sphere centres, FP64 (high_accuracy picks the FK sin/cos as in update_kintree).
 * dist is B x n_spheres, centres B x n_spheres x 3; either may be NULL. */
int pmgpu_cst_sphere_distances(pmgpu_cst* c, const double* q, int64_t B, int high_accuracy, double* dist, double* centres,
                               int mem, void* stream);

/* Fast path: FP32 FK/SDF, FP64 recheck of every decision within the derived error bound
 * of its threshold.  Booleans identical to pmgpu_cst_is_valid.  dist32 (optional,
 * B x n_spheres) receives the FP32 per-sphere signed distance; stats (optional, 4 int64:
 * configs, uncertain terms rechecked, configs touched by a recheck, reserved). */
int pmgpu_cst_is_valid_fast(pmgpu_cst* c, const double* q, int64_t B, uint8_t* out, float* dist32, int64_t* stats,
                            int mem, void* stream);

/* Launch shape of the fast kernel: configurations per block and threads per block, one of
 * (16,128) (32,128) (16,256) (32,256) (64,256) (32,512) (64,512) (128,512); chosen per workload by the
 * autotuner (plainmp_gb300/autotune.py).  No counterpart in the reference. */
int pmgpu_cst_set_fast_launch(pmgpu_cst* c, int configs_per_block, int threads_per_block);
int pmgpu_cst_get_fast_launch(const pmgpu_cst* c, int* configs_per_block, int* threads_per_block);
/* The fast kernels' other tuning parameters, chosen per workload by the autotuner.  No counterpart
 * in the reference.  sphere_tile: spheres of one configuration per warp row of sphere tasks (0 or a
 * power of two up to 32; 0 and values below 32 / configurations-per-block give the least);
 * hq_blocks_per_sm: blocks of 256 threads per SM of the hard cloud-query kernel (1..8);
 * edge_configs_per_block, edge_threads: the edge kernel's waypoints and threads per block, one of
 * (16,128) (32,128) (32,256) (64,256).  Defaults: 0, 4, 32, 128. */
int pmgpu_cst_set_fast_tuning(pmgpu_cst* c, int sphere_tile, int hq_blocks_per_sm, int edge_configs_per_block, int edge_threads);
int pmgpu_cst_get_fast_tuning(const pmgpu_cst* c, int* sphere_tile, int* hq_blocks_per_sm, int* edge_configs_per_block,
                              int* edge_threads);

/* Fast path for callers that must not allocate device memory during the call (real-time loops,
 * devices whose memory another allocator owns, code that cannot afford cudaMalloc's implicit
 * synchronisation).  No counterpart in the reference.  Same results as pmgpu_cst_is_valid_fast
 * with PMGPU_MEM_DEVICE: q, out and dist32 (optional) are device pointers and the work is
 * enqueued on `stream`.  Its scratch is a fixed file-scope device array of about 2 MB (held on
 * every device that loads the library until exit); the first call on a device looks up that
 * array's address and uploads a small search table (a synchronous copy, unless an allocating
 * fast call did it before), so make it before any stream capture.  Requirements and limits: B <= 1048576
 * (larger batches return PMGPU_ERR_INVALID); the constraint's tables must already be on the
 * device from an earlier batch call (else PMGPU_ERR_RUNTIME, never an allocation); calls that
 * overlap on the GPU share the scratch array and race.  Error text: pmgpu_last_error(). */
int pmgpu_cst_is_valid_fast_noalloc(pmgpu_cst* c, const double* q, int64_t B, uint8_t* out, float* dist32, void* stream);

/* ---------------------------------------------------------------- motion validator
 * CustomValidatorBase::checkMotion(s1, s2) (ompl/motion_validator.cpp:17-79) for E edges
 * with BoxMotionValidator (type 0, width[q_dim], :89-111) or EuclideanMotionValidator
 * (type 1, resolution, :118-126).  s1/s2 are E x q_dim; out[e] = 1 if the edge is valid.
 * n_checked (optional) receives the number of waypoints the device evaluated. */
#define PMGPU_VALIDATOR_BOX 0
#define PMGPU_VALIDATOR_EUCLIDEAN 1
int pmgpu_check_motion(pmgpu_cst* c, const double* s1, const double* s2, int64_t E, int validator_type, const double* width,
                       double resolution, uint8_t* out, int64_t* n_checked, int mem, void* stream);
/* FP32 + FP64-recheck edge checking through a persistent work-queue kernel. */
int pmgpu_check_motion_fast(pmgpu_cst* c, const double* s1, const double* s2, int64_t E, int validator_type,
                            const double* width, double resolution, uint8_t* out, int64_t* stats, int mem, void* stream);

/* ---------------------------------------------------------------- pose constraints
 * LinkPoseCst(kin, control_joints, base_type, link_names, poses) (constraints/primitive_link_pose.cpp:
 * 16-71; bindings/constraint.cpp:46-53): one target per link, pose_dims[i] = 3 (position), 6
 * (position + RPY) or 7 (position + quaternion x y z w), targets concatenated in `poses`.  Other
 * dimensions give PMGPU_ERR_RUNTIME ("All poses must be 3 or 6 or 7 dimensional").
 * LinkPositionBoundCst(kin, control_joints, base_type, link, axis, lb, ub) (constraints/
 * primitive_link_position_bound.cpp:15-83; bindings/constraint.cpp:98-103): an absent bound has
 * has_lb / has_ub = 0; axis > 2 or no bound give PMGPU_ERR_RUNTIME.
 * Both share one handle type; the model is shared like the reference's KinematicModel. */
typedef struct pmgpu_posecst pmgpu_posecst;
int pmgpu_linkpose_create(pmgpu_model* kin, const char* const* control_joints, int n_joints, int base_type, const char* const* links,
                          int n_links, const double* poses, const int32_t* pose_dims, pmgpu_posecst** out);
int pmgpu_linkbound_create(pmgpu_model* kin, const char* const* control_joints, int n_joints, int base_type, const char* link, int axis,
                           int has_lb, double lb, int has_ub, double ub, pmgpu_posecst** out);
void pmgpu_posecst_destroy(pmgpu_posecst* c);
/* q_dim, cst_dim and whether the constraint is an equality (LinkPoseCst) */
int pmgpu_posecst_dims(const pmgpu_posecst* c, int* q_dim, int* cst_dim, int* is_equality);
/* ConstraintBase::update_kintree(q, high_accuracy) (constraints/primitive.hpp:38-62;
 * bindings/constraint.cpp:31-32) on the shared model state, as pmgpu_cst_update_kintree. */
int pmgpu_posecst_update_kintree(pmgpu_posecst* c, const double* q, int high_accuracy);
/* ConstraintBase::evaluate(q) (constraints/primitive.hpp:74-79) for B configurations, FP64:
 * vals B x cst_dim, jac B x cst_dim x q_dim (row-major), either may be NULL.  The rows follow
 * get_jacobian (kinematics/algorithm.cpp:212-344) with RotationType IGNORE / RPY / XYZW. */
int pmgpu_posecst_evaluate(pmgpu_posecst* c, const double* q, int64_t B, double* vals, double* jac, int mem, void* stream);
/* IneqConstraintBase::is_valid(q) of a LinkPositionBoundCst (update_kintree(q, false) +
 * is_valid_dirty); an equality constraint gives PMGPU_ERR_INVALID. */
int pmgpu_posecst_is_valid(pmgpu_posecst* c, const double* q, int64_t B, uint8_t* out, int mem, void* stream);

/* ---------------------------------------------------------------- composite constraint
 * IneqCompositeCst::is_valid (constraints/composite_constraint.hpp:98-105; bindings/constraint.cpp:
 * 105-112) of the collision constraint c and the LinkPositionBoundCst handles bounds[0..n_bounds)
 * (primitive_link_position_bound.cpp:69-79), in one fast launch: the bounds are decided on the
 * same FP32 FK as c's sphere terms, an undecided one by the FP64 recheck, so the FK runs once per
 * configuration (the reference's one update_kintree(q, false)).  Same booleans as the AND of
 * pmgpu_cst_is_valid and pmgpu_posecst_is_valid.  Every bound must be made on c's kinematic model
 * with c's control joints and base type (else PMGPU_ERR_RUNTIME "All constraints must have the
 * same kinematic chain" or PMGPU_ERR_INVALID); a LinkPoseCst handle gives PMGPU_ERR_INVALID.  A
 * bound's link joins c's FK slots if no sphere chain reaches it.  stats as pmgpu_cst_is_valid_fast.
 * No counterpart entry point in the reference, whose composite is a C++ class. */
int pmgpu_composite_is_valid_fast(pmgpu_cst* c, pmgpu_posecst* const* bounds, int n_bounds, const double* q, int64_t B,
                                  uint8_t* out, int64_t* stats, int mem, void* stream);
/* checkMotion (ompl/motion_validator.cpp:17-79) with the composite's is_valid at every checked
 * waypoint: the constraint CollisionAwareSpaceInformation checks (ompl/ompl_thin_wrap.hpp:114-120)
 * is the problem's global inequality constraint, a composite in general
 * (src/plainmp/ompl_solver.py:250-257; simplify_path takes an IneqCompositeCst, :285-289).
 * Arguments as pmgpu_check_motion_fast and
 * pmgpu_composite_is_valid_fast. */
int pmgpu_composite_check_motion_fast(pmgpu_cst* c, pmgpu_posecst* const* bounds, int n_bounds, const double* s1, const double* s2,
                                      int64_t E, int validator_type, const double* width, double resolution, uint8_t* out,
                                      int64_t* stats, int mem, void* stream);

/* ---------------------------------------------------------------- link poses
 * World pose (x y z qx qy qz qw) of `link` for B configurations, FP64, the FK of
 * ConstraintBase::update_kintree with std::sin/std::cos (constraints/primitive.hpp:38-62)
 * followed by KinematicModel::get_link_pose (kinematics/kinematics.hpp:131-140). */
int pmgpu_cst_link_poses(pmgpu_cst* c, int32_t link, const double* q, int64_t B, double* out7, int mem, void* stream);

/* ---------------------------------------------------------------- differentiable costs
 * FP32 costs with gradients from a hand-written reverse-mode adjoint (FK chain + SDF).  No
 * counterpart in the reference, whose IK (src/plainmp/ik.py:42-156) and smoother
 * (src/plainmp/nlp_solver/sqp_based_solver.py) call the FP64 constraint Jacobians from a CPU solver; the
 * terms reuse its definitions:
 *   d_s       = min over primitives of SDF.evaluate(centre_s) - r_s (the ext row's value,
 *               constraints/primitive_sphere_collision.cpp:256-322), spheres of self-only groups
 *               excluded;
 *   hinge     = w_col * sum_s max(0, margin - d_s)^2;
 *   pose      = w_pos * ||p - p*||^2 + w_rot * ||log(R*^T R)||^2 of pose_link;
 *   smoothing = w_smooth * sum_t sum_d w_d^2 (q[t+1] - 2 q[t] + q[t-1])_d^2, the acceleration
 *               cost of smoothcost_fullmat (nlp_solver/sqp_based_solver.py:74-97).
 * PMGPU_COST_MIN_DISTANCE instead returns min(cutoff, min_s d_s) and its gradient, the value and
 * Jacobian row of SphereCollisionCst's ext row (analytic instead of finite differences). */
#define PMGPU_COST_SUM 0
#define PMGPU_COST_MIN_DISTANCE 1
typedef struct pmgpu_cost_params {
  int32_t mode;              /* PMGPU_COST_SUM | PMGPU_COST_MIN_DISTANCE */
  int32_t pose_link;         /* link id of the pose term, -1: none */
  float w_pos, w_rot;        /* defaults 1, 0.1 */
  float w_col, margin;       /* defaults 1, 0.02 */
  float cutoff;              /* MIN_DISTANCE clamp, default 0.1 */
  float w_smooth;            /* trajectories, default 1 */
  const float* dof_weights;  /* host, q_dim entries (w_d), NULL = ones */
} pmgpu_cost_params;
/* IK batch: q B x q_dim, target B x 7 (x y z qx qy qz qw; NULL when there is no pose term);
 * cost[B]; grad B x q_dim or NULL (cost only). */
int pmgpu_ik_cost(pmgpu_cst* c, const pmgpu_cost_params* p, const float* q, const float* target, int64_t B, float* cost,
                  float* grad, int mem, void* stream);
/* `steps` gradient-descent steps q <- q - lr * grad(q) per problem inside one launch (clamped to
 * the joint limits when clamp_to_limits); q is updated in place, cost[B] (optional) receives the
 * final cost and cost_hist B x steps (optional) the cost before each step. */
int pmgpu_ik_descend(pmgpu_cst* c, const pmgpu_cost_params* p, float* q, const float* target, int64_t B, int32_t steps,
                     float lr, int32_t clamp_to_limits, float* cost, float* cost_hist, int mem, void* stream);
/* Trajectory batch: q n_waypoints x q_dim (trajectories back to back), offsets[n_traj + 1]
 * (int64, offsets[0] = 0, offsets[n_traj] = n_waypoints); cost[n_traj]; grad n_waypoints x q_dim
 * or NULL.  FK is recomputed per waypoint for the gradient; nothing is stored between calls. */
int pmgpu_traj_cost(pmgpu_cst* c, const pmgpu_cost_params* p, const float* q, const int64_t* offsets, int64_t n_traj,
                    int64_t n_waypoints, float* cost, float* grad, int mem, void* stream);

/* ---------------------------------------------------------------- instrumentation
 * Opt-in timing of the library's own kernels: when enabled, CUDA events are recorded around
 * every kernel launch on the stream it is launched on.  pmgpu_profile_read synchronises,
 * returns the summed device time (ms) and launch count of the named kernel since the last
 * read ("*" = all kernels) and clears them.  No counterpart in the reference. */
int pmgpu_profile_enable(int on);
/* Measured FMA throughput of this GPU (TFLOP/s, 2 flops per FMA): fp64 = 0 for FP32, 1 for FP64.
 * Runs a short microbenchmark kernel on the stream and synchronises.  The denominator of the
 * rooflines of arithmetic-bound kernels.  No counterpart in the reference. */
int pmgpu_measure_fma_peak(int fp64, double* tflops, void* stream);
int pmgpu_profile_read(const char* kernel, double* total_ms, int64_t* launches);

#ifdef __cplusplus
}
#endif
#endif /* PMGPU_H_ */
