// Plain FP64 method: one device thread per configuration (or edge), replicating the
// reference's branch structure and early exits (constraints/primitive_sphere_collision.cpp,
// ompl/motion_validator.cpp) with bit-identical FP64 arithmetic (compiled --fmad=false).
#include "pm_launch.h"
#include "pm_view.cuh"

using namespace pmd;

namespace {

__global__ void k_is_valid64(const PmTablesHdr* __restrict__ T, const double* __restrict__ state, const double* __restrict__ q,
                             int64_t B, uint8_t* __restrict__ out) {
  int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (b >= B) return;
  TView v(T);
  out[b] = is_valid_cfg(v, state, q + b * T->q_dim) ? 1 : 0;
}

// get_attached_point_jacobian (algorithm.cpp:346-433); column c of the 3 x dof jacobian is
// written to jac[3*c .. 3*c+2]
__device__ void attached_jacobian(const TView& v, const DPose* pose, int plink_slot, const D3& p, double* jac) {
  const int nc = v.T->n_ctrl;
  const uint64_t rel = v.S[plink_slot].relevant;
  for (int i = 0; i < nc; i++) {
    double* c = jac + 3 * i;
    const PmJoint& J = v.J[i];
    if (J.slot < 0 || !((rel >> i) & 1ull)) {
      c[0] = c[1] = c[2] = 0.0;
      continue;
    }
    const DPose& tc = pose[J.slot];
    D3 wa = qrot(tc.q, D3{J.axis[0], J.axis[1], J.axis[2]});
    D3 d = J.prismatic ? wa : cross(wa, sub(p, tc.t));
    c[0] = d.x;
    c[1] = d.y;
    c[2] = d.z;
  }
  if (v.T->base_type == PM_BASE_FIXED) return;
  DPose te;
  te.q = DQ{0, 0, 0, 1};
  te.t = p;
  const DPose tb = pose[v.T->root_slot];
  DPose tbinv = pose_inverse(tb);
  D3 rpy = get_rpy(tb.q);
  DPose tbe = pose_mul(tbinv, te);
  const double eps = 1e-7;
  double rpya[3] = {rpy.x, rpy.y, rpy.z};
  if (v.T->base_type == PM_BASE_FLOATING) {
    for (int k = 0; k < 9; k++) jac[3 * nc + k] = 0.0;
    jac[3 * (nc + 0) + 0] = 1.0;
    jac[3 * (nc + 1) + 1] = 1.0;
    jac[3 * (nc + 2) + 2] = 1.0;
    for (int k = 0; k < 3; k++) {
      double r2[3] = {rpya[0], rpya[1], rpya[2]};
      r2[k] += eps;
      DPose tw = tb;
      tw.q = quat_from_rpy(r2[0], r2[1], r2[2]);
      DPose o = pose_mul(tw, tbe);
      D3 dp = sub(o.t, te.t);
      jac[3 * (nc + 3 + k) + 0] = dp.x / eps;
      jac[3 * (nc + 3 + k) + 1] = dp.y / eps;
      jac[3 * (nc + 3 + k) + 2] = dp.z / eps;
    }
  } else {
    for (int k = 0; k < 9; k++) jac[3 * nc + k] = 0.0;
    jac[3 * (nc + 0) + 0] = 1.0;
    jac[3 * (nc + 1) + 1] = 1.0;
    double r2[3] = {rpya[0], rpya[1], rpya[2] + eps};
    DPose tw = tb;
    tw.q = quat_from_rpy(r2[0], r2[1], r2[2]);
    DPose o = pose_mul(tw, tbe);
    D3 dp = sub(o.t, te.t);
    jac[3 * (nc + 2) + 0] = dp.x / eps;
    jac[3 * (nc + 2) + 1] = dp.y / eps;
    jac[3 * (nc + 2) + 2] = dp.z / eps;
  }
}

#define PM_CUTOFF 0.1

// evaluate_ext_collision (primitive_sphere_collision.cpp:256-322)
__device__ double eval_ext(const TView& v, const DPose* pose, double* grad, double* jtmp) {
  const int dof = v.T->q_dim;
  double minv = PM_CUTOFF;
  int mg = -1, mp = -1, mk = -1;
  for (int gi = 0; gi < v.T->n_groups; gi++) {
    const PmGroup& g = v.G[gi];
    if (g.only_self) continue;
    const DPose& lp = pose[g.slot];
    DM3 R;
    D3 gc = group_centre(v, g, lp, R);
    for (int pi = 0; pi < v.T->n_prims; pi++) {
      const PmPrim& P = v.P[pi];
      if (!outside_aabb(P, gc, g.radius + PM_CUTOFF)) {
        if (!prim_outside(P, v.C, gc, g.radius + PM_CUTOFF)) {
          for (int k = g.begin; k < g.begin + g.count; k++) {
            D3 c = add(mv(R, v.rel(k)), lp.t);
            if (outside_aabb(P, c, v.sr[k] + PM_CUTOFF)) continue;
            double val = prim_eval(P, v.C, c) - v.sr[k];
            if (val < minv) {
              minv = val;
              mg = gi;
              mp = pi;
              mk = k;
            }
          }
        }
      }
    }
  }
  if (mg < 0) {
    for (int d = 0; d < dof; d++) grad[d] = 0.0;
    return minv;
  }
  const PmGroup& g = v.G[mg];
  DM3 R = qmat(pose[g.slot].q);
  D3 sc = add(mv(R, v.rel(mk)), pose[g.slot].t);
  double r = v.sr[mk];
  double g3[3];
  for (int i = 0; i < 3; i++) {
    D3 pc = sc;
    if (i == 0) pc.x += 1e-6;
    if (i == 1) pc.y += 1e-6;
    if (i == 2) pc.z += 1e-6;
    double val = prim_eval(v.P[mp], v.C, pc) - r;
    g3[i] = (val - minv) / 1e-6;
  }
  attached_jacobian(v, pose, g.slot, sc, jtmp);
  for (int d = 0; d < dof; d++) grad[d] = jtmp[3 * d + 0] * g3[0] + jtmp[3 * d + 1] * g3[1] + jtmp[3 * d + 2] * g3[2];
  return minv;
}

// evaluate_self_collision (primitive_sphere_collision.cpp:324-383)
__device__ double eval_self(const TView& v, const DPose* pose, double* grad, double* jtmp, double* jtmp2) {
  const int dof = v.T->q_dim;
  double dmin = PM_CUTOFF;
  int a = -1, ai = -1, b = -1, bj = -1;
  for (int pr = 0; pr < v.T->n_pairs; pr++) {
    const int ga = v.pairs[2 * pr], gb = v.pairs[2 * pr + 1];
    const PmGroup& g1 = v.G[ga];
    const PmGroup& g2 = v.G[gb];
    DM3 R1, R2;
    D3 c1 = group_centre(v, g1, pose[g1.slot], R1);
    D3 c2 = group_centre(v, g2, pose[g2.slot], R2);
    double osq = sqn(sub(c1, c2));
    double orm = g1.radius + g2.radius + PM_CUTOFF;
    if (osq > orm * orm) continue;
    const D3 t1 = pose[g1.slot].t, t2 = pose[g2.slot].t;
    for (int i = g1.begin; i < g1.begin + g1.count; i++) {
      D3 s1 = add(mv(R1, v.rel(i)), t1);
      for (int j = g2.begin; j < g2.begin + g2.count; j++) {
        D3 s2 = add(mv(R2, v.rel(j)), t2);
        double d = nrm(sub(s1, s2)) - (v.sr[i] + v.sr[j]);
        if (d < dmin) {
          dmin = d;
          a = ga;
          ai = i;
          b = gb;
          bj = j;
        }
      }
    }
  }
  if (a < 0) {
    for (int d = 0; d < dof; d++) grad[d] = 0.0;
    return dmin;
  }
  const PmGroup& g1 = v.G[a];
  const PmGroup& g2 = v.G[b];
  D3 c1 = add(mv(qmat(pose[g1.slot].q), v.rel(ai)), pose[g1.slot].t);
  D3 c2 = add(mv(qmat(pose[g2.slot].q), v.rel(bj)), pose[g2.slot].t);
  D3 cd = sub(c1, c2);
  attached_jacobian(v, pose, g1.slot, c1, jtmp);
  attached_jacobian(v, pose, g2.slot, c2, jtmp2);
  double ni = 1.0 / nrm(cd);
  for (int d = 0; d < dof; d++) {
    grad[d] = cd.x * ni * (jtmp[3 * d + 0] - jtmp2[3 * d + 0]) + cd.y * ni * (jtmp[3 * d + 1] - jtmp2[3 * d + 1]) +
              cd.z * ni * (jtmp[3 * d + 2] - jtmp2[3 * d + 2]);
  }
  return dmin;
}

#define PM_MAX_DOF (PM_MAX_CTRL + 6)

__global__ void k_evaluate64(const PmTablesHdr* __restrict__ T, const double* __restrict__ state, const double* __restrict__ q,
                             int64_t B, int high_accuracy, double* __restrict__ vals, double* __restrict__ jac) {
  int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (b >= B) return;
  TView v(T);
  const int dof = T->q_dim;
  const int m = (T->n_prims > 0 ? 1 : 0) + (T->n_pairs > 0 ? 1 : 0);
  DPose pose[PM_MAX_SLOTS];
  double jtmp[3 * PM_MAX_DOF], jtmp2[3 * PM_MAX_DOF];
  const double* qb = q + b * dof;
  fk64(T, state, qb, !high_accuracy, pose);
  double* vb = vals + b * m;
  double* jb = jac + b * (int64_t)m * dof;
  int head = 0;
  if (T->n_prims > 0) {
    vb[head] = eval_ext(v, pose, jb + head * dof, jtmp);
    head++;
  }
  if (T->n_pairs > 0) vb[head] = eval_self(v, pose, jb + head * dof, jtmp, jtmp2);
}

// Per-sphere signed distances in two launches: the FP64 sphere centres (one thread per configuration:
// the FK), then the SDF of every (configuration, sphere) in its own thread, so the nearest-point
// searches of a batch run side by side instead of one configuration's 120 in a row.
__global__ void k_sphere_centres64(const PmTablesHdr* __restrict__ T, const double* __restrict__ state, const double* __restrict__ q,
                                   int64_t B, int high_accuracy, double* __restrict__ centres) {
  int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (b >= B) return;
  TView v(T);
  DPose pose[PM_MAX_SLOTS];
  fk64(T, state, q + b * T->q_dim, !high_accuracy, pose);
  const int ns = T->n_spheres;
  for (int gi = 0; gi < T->n_groups; gi++) {
    const PmGroup& g = v.G[gi];
    DM3 R = qmat(pose[g.slot].q);
    for (int k = g.begin; k < g.begin + g.count; k++) {
      D3 c = add(mv(R, v.rel(k)), pose[g.slot].t);
      centres[(b * ns + k) * 3 + 0] = c.x;
      centres[(b * ns + k) * 3 + 1] = c.y;
      centres[(b * ns + k) * 3 + 2] = c.z;
    }
  }
}
__global__ void k_sphere_sdf64(const PmTablesHdr* __restrict__ T, const double* __restrict__ centres, int64_t n,
                               double* __restrict__ dist) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  TView v(T);
  const int k = (int)(i % T->n_spheres);
  const D3 c{centres[3 * i], centres[3 * i + 1], centres[3 * i + 2]};
  double d = INFINITY;
  for (int pi = 0; pi < T->n_prims; pi++) d = fmin(d, prim_eval(v.P[pi], v.C, c) - v.sr[k]);
  dist[i] = d;
}

__global__ void k_spheres_of_state(const PmTablesHdr* __restrict__ T, const double* __restrict__ state, int groups,
                                   double* __restrict__ out4) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  TView v(T);
  DPose pose[PM_MAX_SLOTS];
  // the state already holds the local transforms of every joint
  const PmSlot* S = v.S;
  bool dummy;
  DPose base = state_pose(state, PM_STATE_BASE_ROW, dummy);
  for (int i = 0; i < T->n_slots; i++) {
    if (S[i].parent < 0) {
      pose[i] = base;
      continue;
    }
    bool lid;
    DPose l = state_pose(state, PM_STATE_LINK_ROW(S[i].link), lid);
    pose[i] = compose(pose[S[i].parent], l.q, l.t, lid);
  }
  int k = 0;
  for (int gi = 0; gi < T->n_groups; gi++) {
    const PmGroup& g = v.G[gi];
    DM3 R;
    D3 gc = group_centre(v, g, pose[g.slot], R);
    if (groups) {
      out4[4 * gi + 0] = gc.x;
      out4[4 * gi + 1] = gc.y;
      out4[4 * gi + 2] = gc.z;
      out4[4 * gi + 3] = g.radius;
      continue;
    }
    for (int s = g.begin; s < g.begin + g.count; s++, k++) {
      D3 c = add(mv(R, v.rel(s)), pose[g.slot].t);
      out4[4 * k + 0] = c.x;
      out4[4 * k + 1] = c.y;
      out4[4 * k + 2] = c.z;
      out4[4 * k + 3] = v.sr[s];
    }
  }
}

// ------------------------------------------------------------------ motion validator
// CustomValidatorBase::checkMotion (motion_validator.cpp:17-79), one thread per edge
__global__ void k_check_motion64(const PmTablesHdr* __restrict__ T, const double* __restrict__ state, const double* __restrict__ s1,
                                 const double* __restrict__ s2, int64_t E, int type, const double* __restrict__ width,
                                 double resolution, const int16_t* __restrict__ seq, uint8_t* __restrict__ out,
                                 unsigned long long* n_checked) {
  int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= E) return;
  TView v(T);
  const int dim = T->q_dim;
  const double* a = s1 + e * dim;
  const double* b = s2 + e * dim;
  double sr;
  if (type == 0) {  // BoxMotionValidator::determine_step_ratio (:89-111)
    double diff_long = 0.0, max_diff = -INFINITY;
    int li = 0;
    for (int i = 0; i < dim; i++) {
      double diff = b[i] - a[i];
      double asd = fabs(diff) * (1.0 / width[i]);
      if (asd > max_diff) {
        max_diff = asd;
        li = i;
        diff_long = diff;
      }
    }
    sr = fabs(diff_long) < 1e-6 ? INFINITY : width[li] / fabs(diff_long);
  } else {  // EuclideanMotionValidator (:118-126)
    double dist = 0.0;
    for (int i = 0; i < dim; i++) {
      double d = a[i] - b[i];
      dist += d * d;
    }
    sr = resolution / sqrt(dist);
  }
  if (sr == INFINITY) {
    out[e] = 1;
    return;
  }
  // NaN / non-positive step ratios, and edges needing more than 2^26 waypoints, are reported
  // invalid instead of looping (the reference has no bound here)
  if (!(sr > 0.0) || 1.0 / sr > 67108864.0) {
    out[e] = 0;
    return;
  }
  unsigned long long n_test = (unsigned long long)(floor(1 / sr) + 2);
  double qt[PM_MAX_DOF];
  unsigned long long cnt = 1;
  bool ok = is_valid_cfg(v, state, b);
  if (ok) {
    if (n_test < 129) {
      const int16_t* sq = seq + (n_test - 1) * 128;
      for (unsigned long long i = 2; i < n_test && ok; i++) {
        double t = (double)sq[i] * sr;
        for (int k = 0; k < dim; k++) qt[k] = a[k] + (b[k] - a[k]) * t;
        cnt++;
        ok = is_valid_cfg(v, state, qt);
      }
    } else {
      for (unsigned long long i = 1; i < n_test - 1 && ok; i++) {
        double t = (double)i * sr;
        for (int k = 0; k < dim; k++) qt[k] = a[k] + (b[k] - a[k]) * t;
        cnt++;
        ok = is_valid_cfg(v, state, qt);
      }
    }
  }
  out[e] = ok ? 1 : 0;
  if (n_checked) atomicAdd(n_checked, cnt);
}

// ------------------------------------------------------------------ model state
__global__ void k_set_joints(double* state, const PmSlot* recs, const double* q, int n, int accurate) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  for (int i = 0; i < n; i++) {  // in order: a repeated joint keeps its last value
    DQ lq;
    D3 lt;
    bool lid;
    joint_local(recs[i], q[i], accurate == 0, lq, lt, lid);
    double* r = state + (int64_t)PM_STATE_LINK_ROW(recs[i].link) * PM_STATE_STRIDE;
    r[0] = lq.x;
    r[1] = lq.y;
    r[2] = lq.z;
    r[3] = lq.w;
    r[4] = lt.x;
    r[5] = lt.y;
    r[6] = lt.z;
    r[7] = lid ? 1.0 : 0.0;
  }
}

__global__ void k_set_base_from_q(double* state, int base_type, const double* qb) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  DQ q;
  D3 t;
  if (base_type == PM_BASE_FLOATING) {
    t = D3{qb[0], qb[1], qb[2]};
    q = quat_from_rpy(qb[3], qb[4], qb[5]);
  } else {
    t = D3{qb[0], qb[1], 0.0};
    q = quat_from_rpy(0, 0, qb[2]);
  }
  double* r = state + PM_STATE_BASE_ROW * PM_STATE_STRIDE;
  r[0] = q.x;
  r[1] = q.y;
  r[2] = q.z;
  r[3] = q.w;
  r[4] = t.x;
  r[5] = t.y;
  r[6] = t.z;
  r[7] = 0.0;
}

// build_cache_until for selected links (algorithm.cpp:160-210)
__global__ void k_link_poses(const double* __restrict__ state, const int32_t* __restrict__ parents, const int32_t* __restrict__ links,
                             int n, double* __restrict__ out7) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int chain[256];
  int depth = 0;
  int h = links[i];
  while (h >= 0 && parents[h] >= 0 && depth < 256) {
    chain[depth++] = h;
    h = parents[h];
  }
  bool dummy;
  DPose p = state_pose(state, PM_STATE_BASE_ROW, dummy);
  while (depth > 0) {
    int l = chain[--depth];
    bool lid;
    DPose loc = state_pose(state, PM_STATE_LINK_ROW(l), lid);
    p = compose(p, loc.q, loc.t, lid);
  }
  double* o = out7 + 7 * i;
  o[0] = p.t.x;
  o[1] = p.t.y;
  o[2] = p.t.z;
  o[3] = p.q.x;
  o[4] = p.q.y;
  o[5] = p.q.z;
  o[6] = p.q.w;
}

// ------------------------------------------------------------------ SDF utilities
__global__ void k_sdf_points(const PmPrim* __restrict__ prims, int n_prims, const PmGridDev* __restrict__ clouds, int is_union,
                             const double* __restrict__ pts, const double* __restrict__ radii, int64_t n, double* eval_out,
                             uint8_t* outside_out) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  D3 p{pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]};
  if (eval_out) {
    double v = is_union ? 1.7976931348623157e308 : 0.0;
    if (is_union) {
      for (int k = 0; k < n_prims; k++) v = fmin(v, prim_eval(prims[k], clouds, p));
    } else if (n_prims > 0) {
      v = prim_eval(prims[0], clouds, p);
    }
    eval_out[i] = v;
  }
  if (outside_out) {
    bool o = true;
    for (int k = 0; k < n_prims && o; k++) o = prim_outside(prims[k], clouds, p, radii[i]);
    outside_out[i] = o ? 1 : 0;
  }
}

__global__ void k_cloud_nearest(const PmGridDev* __restrict__ grid, const double* __restrict__ pts, int64_t n, double* sq,
                                double* near3) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  D3 p{pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]};
  NNResult64 r = grid_nearest64(*grid, p);
  if (sq) sq[i] = r.d2;
  if (near3) {
    double x = NAN, y = NAN, z = NAN;
    if (r.idx >= 0) {
      x = grid->px[r.idx];
      y = grid->py[r.idx];
      z = grid->pz[r.idx];
    }
    near3[3 * i] = x;
    near3[3 * i + 1] = y;
    near3[3 * i + 2] = z;
  }
}

inline unsigned grid_for(int64_t n, int bs) { return (unsigned)((n + bs - 1) / bs); }

}  // namespace

namespace pmg {

cudaError_t launch_set_joints(double* state, const PmSlot* recs, const double* q, int n, int accurate, cudaStream_t s) {
  k_set_joints<<<1, 1, 0, s>>>(state, recs, q, n, accurate);
  return cudaGetLastError();
}
cudaError_t launch_set_base_from_q(double* state, int base_type, const double* qbase, cudaStream_t s) {
  k_set_base_from_q<<<1, 1, 0, s>>>(state, base_type, qbase);
  return cudaGetLastError();
}
cudaError_t launch_link_poses(const double* state, const int32_t* parents, const int32_t* links, int n, double* out7,
                              cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_link_poses<<<grid_for(n, 64), 64, 0, s>>>(state, parents, links, n, out7);
  return cudaGetLastError();
}
cudaError_t launch_is_valid64(const PmTablesHdr* T, const double* state, const double* q, int64_t B, uint8_t* out,
                              cudaStream_t s) {
  if (B <= 0) return cudaSuccess;
  prof_begin("k_is_valid64", s);
  k_is_valid64<<<grid_for(B, 128), 128, 0, s>>>(T, state, q, B, out);
  prof_end("k_is_valid64", s);
  return cudaGetLastError();
}
cudaError_t launch_evaluate64(const PmTablesHdr* T, const double* state, const double* q, int64_t B, int high_accuracy,
                              double* vals, double* jac, cudaStream_t s) {
  if (B <= 0) return cudaSuccess;
  k_evaluate64<<<grid_for(B, 64), 64, 0, s>>>(T, state, q, B, high_accuracy, vals, jac);
  return cudaGetLastError();
}
cudaError_t launch_sphere_dist64(const PmTablesHdr* T, const PmTablesHdr& h, const double* state, const double* q, int64_t B,
                                 int high_accuracy, double* dist, double* centres, cudaStream_t s) {
  if (B <= 0 || h.n_spheres <= 0) return cudaSuccess;
  k_sphere_centres64<<<grid_for(B, 128), 128, 0, s>>>(T, state, q, B, high_accuracy, centres);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess || !dist) return e;
  const int64_t n = B * h.n_spheres;
  k_sphere_sdf64<<<grid_for(n, 128), 128, 0, s>>>(T, centres, n, dist);
  return cudaGetLastError();
}
cudaError_t launch_spheres_of_state(const PmTablesHdr* T, const double* state, int groups, double* out4, cudaStream_t s) {
  k_spheres_of_state<<<1, 1, 0, s>>>(T, state, groups, out4);
  return cudaGetLastError();
}
cudaError_t launch_check_motion64(const PmTablesHdr* T, const double* state, const double* s1, const double* s2, int64_t E,
                                  int type, const double* width, double resolution, const int16_t* seq, uint8_t* out,
                                  unsigned long long* n_checked, cudaStream_t s) {
  if (E <= 0) return cudaSuccess;
  k_check_motion64<<<grid_for(E, 64), 64, 0, s>>>(T, state, s1, s2, E, type, width, resolution, seq, out, n_checked);
  return cudaGetLastError();
}
cudaError_t launch_sdf_points(const PmPrim* prims, int n_prims, const PmGridDev* clouds, int is_union, const double* pts,
                              const double* radii, int64_t n, double* eval_out, uint8_t* outside_out, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_sdf_points<<<grid_for(n, 128), 128, 0, s>>>(prims, n_prims, clouds, is_union, pts, radii, n, eval_out, outside_out);
  return cudaGetLastError();
}
cudaError_t launch_cloud_nearest(const PmGridDev* grid, const double* pts, int64_t n, double* sq, double* near3,
                                 cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_cloud_nearest<<<grid_for(n, 128), 128, 0, s>>>(grid, pts, n, sq, near3);
  return cudaGetLastError();
}

}  // namespace pmg
