// Device view of the flattened constraint tables and the plain FP64 validity logic
// (exact replica of is_valid_dirty, constraints/primitive_sphere_collision.cpp:181-254),
// shared by the plain kernels and the FP64 recheck of the fast path.
#pragma once
#include "pm_sdf.cuh"

namespace pmd {

struct TView {
  const PmTablesHdr* T;
  const PmSlot* S;
  const PmJoint* J;
  const PmGroup* G;
  const double *sx, *sy, *sz, *sr;
  const int32_t* pairs;
  const int32_t* sgroup;
  const PmPrim* P;
  const PmGridDev* C;
  __device__ explicit TView(const PmTablesHdr* t)
      : T(t),
        S(pm_at<PmSlot>(t, t->off_slots)),
        J(pm_at<PmJoint>(t, t->off_joints)),
        G(pm_at<PmGroup>(t, t->off_groups)),
        sx(pm_at<double>(t, t->off_sx)),
        sy(pm_at<double>(t, t->off_sy)),
        sz(pm_at<double>(t, t->off_sz)),
        sr(pm_at<double>(t, t->off_sr)),
        pairs(pm_at<int32_t>(t, t->off_pairs)),
        sgroup(pm_at<int32_t>(t, t->off_sgroup)),
        P(pm_at<PmPrim>(t, t->off_prims)),
        C(pm_at<PmGridDev>(t, t->off_clouds)) {}
  __device__ D3 rel(int k) const { return D3{sx[k], sy[k], sz[k]}; }
};

// SphereGroup::create_group_sphere_position_cache (primitive_sphere_collision.cpp:26-36)
__device__ __forceinline__ D3 group_centre(const TView& v, const PmGroup& g, const DPose& lp, DM3& R) {
  R = qmat(lp.q);
  return add(mv(R, D3{g.rel[0], g.rel[1], g.rel[2]}), lp.t);
}

// check_ext_collision (primitive_sphere_collision.cpp:191-220)
__device__ inline bool ext_ok(const TView& v, const DPose* pose) {
  for (int gi = 0; gi < v.T->n_groups; gi++) {
    const PmGroup& g = v.G[gi];
    if (g.only_self) continue;
    const DPose& lp = pose[g.slot];
    DM3 R;
    D3 gc = group_centre(v, g, lp, R);
    for (int pi = 0; pi < v.T->n_prims; pi++) {
      const PmPrim& P = v.P[pi];
      if (!outside_aabb(P, gc, g.radius)) {
        if (!prim_outside(P, v.C, gc, g.radius)) {
          for (int k = g.begin; k < g.begin + g.count; k++) {
            D3 c = add(mv(R, v.rel(k)), lp.t);
            if (!outside_aabb(P, c, v.sr[k])) {
              if (!prim_outside(P, v.C, c, v.sr[k])) return false;
            }
          }
        }
      }
    }
  }
  return true;
}

// check_self_collision (primitive_sphere_collision.cpp:222-254)
__device__ inline bool self_ok(const TView& v, const DPose* pose) {
  for (int pr = 0; pr < v.T->n_pairs; pr++) {
    const PmGroup& g1 = v.G[v.pairs[2 * pr]];
    const PmGroup& g2 = v.G[v.pairs[2 * pr + 1]];
    DM3 R1, R2;
    D3 c1 = group_centre(v, g1, pose[g1.slot], R1);
    D3 c2 = group_centre(v, g2, pose[g2.slot], R2);
    double osq = sqn(sub(c1, c2));
    double ors = g1.radius + g2.radius;
    if (osq > ors * ors) continue;
    const D3 t1 = pose[g1.slot].t, t2 = pose[g2.slot].t;
    for (int i = g1.begin; i < g1.begin + g1.count; i++) {
      D3 a = add(mv(R1, v.rel(i)), t1);
      for (int j = g2.begin; j < g2.begin + g2.count; j++) {
        D3 b = add(mv(R2, v.rel(j)), t2);
        double sq = sqn(sub(a, b));
        double rs = v.sr[i] + v.sr[j];
        if (sq < rs * rs) return false;
      }
    }
  }
  return true;
}

// LinkPositionBoundCst::is_valid_dirty (primitive_link_position_bound.cpp:69-79) of every bound
// term, on the poses of one configuration.
__device__ inline bool bounds_ok(const PmLinkBounds& b, const DPose* pose) {
  for (int k = 0; k < b.n; k++) {
    const PmPoseTerm& t = b.t[k];
    const D3& p = pose[t.slot].t;
    const double x = t.axis == 0 ? p.x : (t.axis == 1 ? p.y : p.z);
    if (t.has_lb && x < t.lb) return false;
    if (t.has_ub && x > t.ub) return false;
  }
  return true;
}

// IneqConstraintBase::is_valid for one q (primitive.hpp:113-117, :181-189); with link-position
// bounds, IneqCompositeCst::is_valid of the collision constraint and those bounds
// (composite_constraint.hpp:98-105): one update_kintree(q, false), then every member.
__device__ inline bool is_valid_cfg(const TView& v, const double* state, const double* q, PmLinkBounds bnd = PmLinkBounds{nullptr, 0}) {
  DPose pose[PM_MAX_SLOTS];
  fk64(v.T, state, q, v.T->base_type == PM_BASE_FIXED, pose);
  if (v.T->n_prims > 0 && !ext_ok(v, pose)) return false;
  if (v.T->n_pairs > 0 && !self_ok(v, pose)) return false;
  return bnd.n == 0 || bounds_ok(bnd, pose);
}

}  // namespace pmd
