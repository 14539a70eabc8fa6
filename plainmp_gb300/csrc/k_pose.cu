// Pose constraints in FP64: LinkPoseCst and LinkPositionBoundCst, batched over configurations.
//
// One thread per configuration: the FK of ConstraintBase::update_kintree (constraints/
// primitive.hpp:38-62) over the constraint's slots, then per term the value and the rows of
// KinematicModel::get_jacobian (kinematics/algorithm.cpp:212-344): joint columns from the child
// link's world axis (revolute: axis x (p_e - p_c), plus the RPY or quaternion-rate rows of
// rpy_derivative / q_derivative, algorithm.cpp:20-47), base columns by the reference's forward
// differences (eps 1e-7).
#include "pm_launch.h"
#include "pm_view.cuh"

using namespace pmd;

namespace {

// rpy_derivative (algorithm.cpp:20-32)
__device__ __forceinline__ D3 rpy_derivative(const D3& rpy, const D3& axis) {
  const double a2 = -rpy.y, a3 = -rpy.z;
  D3 o;
  o.x = cos(a3) / cos(a2) * axis.x - sin(a3) / cos(a2) * axis.y;
  o.y = sin(a3) * axis.x + cos(a3) * axis.y;
  o.z = -cos(a3) * sin(a2) / cos(a2) * axis.x + sin(a3) * sin(a2) / cos(a2) * axis.y + axis.z;
  return o;
}
// q_derivative (algorithm.cpp:34-47): returned as Quaternion(-dw, dx, dy, dz)
__device__ __forceinline__ DQ q_derivative(const DQ& q, const D3& w) {
  const double dx = 0.5 * (w.z * q.y - w.y * q.z + w.x * q.w);
  const double dy = 0.5 * (-w.z * q.x + 0 * q.y + w.x * q.z + w.y * q.w);
  const double dz = 0.5 * (w.y * q.x - w.x * q.y + 0 * q.z + w.z * q.w);
  const double dw = 0.5 * (-w.x * q.x - w.y * q.y - w.z * q.z + 0 * q.w);
  return DQ{dx, dy, dz, -dw};
}

// get_jacobian(elink, control joints, rot_type, base_type) of slot es into J (rows x dof,
// row-major with leading dimension ld): rot 0 IGNORE (3 rows), 1 RPY (6), 2 XYZW (7).
__device__ void link_jacobian(const TView& v, const DPose* pose, int es, int rot, double* J, int ld) {
  const int nc = v.T->n_ctrl, dof = v.T->q_dim;
  const int rows = 3 + (rot == 1) * 3 + (rot == 2) * 4;
  for (int r = 0; r < rows; r++)
    for (int c = 0; c < dof; c++) J[r * ld + c] = 0.0;
  const DPose& te = pose[es];
  D3 erpy{0, 0, 0};
  DQ einv{0, 0, 0, 1};
  if (rot == 1) erpy = get_rpy(te.q);
  if (rot == 2) einv = pose_inverse(te).q;
  const uint64_t rel = v.S[es].relevant;
  for (int i = 0; i < nc; i++) {
    const PmJoint& Jt = v.J[i];
    if (Jt.slot < 0 || !((rel >> i) & 1ull)) continue;  // rptable_.isRelevant
    const DPose& tc = pose[Jt.slot];
    const D3 wa = qrot(tc.q, D3{Jt.axis[0], Jt.axis[1], Jt.axis[2]});
    const D3 d = Jt.prismatic ? wa : cross(wa, sub(te.t, tc.t));
    J[0 * ld + i] = d.x;
    J[1 * ld + i] = d.y;
    J[2 * ld + i] = d.z;
    if (Jt.prismatic) continue;
    if (rot == 1) {
      const D3 dr = rpy_derivative(erpy, wa);
      J[3 * ld + i] = dr.x;
      J[4 * ld + i] = dr.y;
      J[5 * ld + i] = dr.z;
    } else if (rot == 2) {
      const DQ dq = q_derivative(einv, wa);
      J[3 * ld + i] = dq.x;
      J[4 * ld + i] = dq.y;
      J[5 * ld + i] = dq.z;
      J[6 * ld + i] = dq.w;
    }
  }
  const int bt = v.T->base_type;
  if (bt == PM_BASE_FIXED) return;
  const DPose tb = pose[v.T->root_slot];
  const DPose tbe = pose_mul(pose_inverse(tb), te);
  const D3 rpyb = get_rpy(tb.q);
  const double eps = 1e-7;
  auto fill = [&](int col, int k) {
    double r2[3] = {rpyb.x, rpyb.y, rpyb.z};
    r2[k] += eps;
    DPose tw = tb;
    tw.q = quat_from_rpy(r2[0], r2[1], r2[2]);
    const DPose po = pose_mul(tw, tbe);
    const D3 dp = sub(po.t, te.t);
    J[0 * ld + col] = dp.x / eps;
    J[1 * ld + col] = dp.y / eps;
    J[2 * ld + col] = dp.z / eps;
    if (rot == 1) {
      const D3 e2 = get_rpy(po.q);
      J[3 * ld + col] = (e2.x - erpy.x) / eps;
      J[4 * ld + col] = (e2.y - erpy.y) / eps;
      J[5 * ld + col] = (e2.z - erpy.z) / eps;
    } else if (rot == 2) {
      J[3 * ld + col] = (po.q.x - te.q.x) / eps;
      J[4 * ld + col] = (po.q.y - te.q.y) / eps;
      J[5 * ld + col] = (po.q.z - te.q.z) / eps;
      J[6 * ld + col] = (po.q.w - te.q.w) / eps;
    }
  };
  if (bt == PM_BASE_FLOATING) {
    J[0 * ld + nc + 0] = 1.0;
    J[1 * ld + nc + 1] = 1.0;
    J[2 * ld + nc + 2] = 1.0;
    for (int k = 0; k < 3; k++) fill(nc + 3 + k, k);
  } else {
    J[0 * ld + nc + 0] = 1.0;
    J[1 * ld + nc + 1] = 1.0;
    fill(nc + 2, 2);
  }
}

struct Poses {
  DPose p[PM_MAX_SLOTS];
  __device__ DPose& operator[](int k) { return p[k]; }
};

// evaluate(q) of the constraint = update_kintree(q, high accuracy) + evaluate_dirty: vals
// B x cst_dim, jac B x cst_dim x q_dim (either may be null).
__global__ void k_posecst_eval64(const PmTablesHdr* __restrict__ T, const double* __restrict__ state, const PmPoseTerm* __restrict__ terms,
                                 int n_terms, int cst_dim, const double* __restrict__ q, int64_t B, double* __restrict__ vals,
                                 double* __restrict__ jac) {
  const int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= B) return;
  TView v(T);
  const int dof = T->q_dim;
  Poses pose;
  fk64(T, state, q + b * dof, false, pose);
  double* vb = vals ? vals + b * cst_dim : nullptr;
  double* jb = jac ? jac + b * (int64_t)cst_dim * dof : nullptr;
  int row = 0;
  for (int k = 0; k < n_terms; k++) {
    const PmPoseTerm& t = terms[k];
    const DPose& te = pose[t.slot];
    if (t.kind == PM_TERM_LINK_POSE) {
      if (vb) {
        vb[row + 0] = te.t.x - t.target[0];
        vb[row + 1] = te.t.y - t.target[1];
        vb[row + 2] = te.t.z - t.target[2];
        if (t.dim == 6) {
          const D3 rpy = get_rpy(te.q);
          vb[row + 3] = rpy.x - t.target[3];
          vb[row + 4] = rpy.y - t.target[4];
          vb[row + 5] = rpy.z - t.target[5];
        } else if (t.dim == 7) {  // quat().coeffs() = x y z w
          vb[row + 3] = te.q.x - t.target[3];
          vb[row + 4] = te.q.y - t.target[4];
          vb[row + 5] = te.q.z - t.target[5];
          vb[row + 6] = te.q.w - t.target[6];
        }
      }
      if (jb) link_jacobian(v, &pose.p[0], t.slot, t.dim == 3 ? 0 : (t.dim == 6 ? 1 : 2), jb + (int64_t)row * dof, dof);
      row += t.dim;
    } else {
      const double pos = t.axis == 0 ? te.t.x : (t.axis == 1 ? te.t.y : te.t.z);
      double Jp[3 * (PM_MAX_CTRL + 6)];
      if (jb) link_jacobian(v, &pose.p[0], t.slot, 0, Jp, dof);
      if (t.has_lb) {
        if (vb) vb[row] = pos - t.lb;
        if (jb)
          for (int c = 0; c < dof; c++) jb[(int64_t)row * dof + c] = Jp[t.axis * dof + c];
        row++;
      }
      if (t.has_ub) {
        if (vb) vb[row] = t.ub - pos;
        if (jb)
          for (int c = 0; c < dof; c++) jb[(int64_t)row * dof + c] = -Jp[t.axis * dof + c];
        row++;
      }
    }
  }
}

// is_valid(q) = update_kintree(q, false) + is_valid_dirty of the bound terms
// (primitive_link_position_bound.cpp:62-73).
__global__ void k_posecst_valid64(const PmTablesHdr* __restrict__ T, const double* __restrict__ state, const PmPoseTerm* __restrict__ terms,
                                  int n_terms, const double* __restrict__ q, int64_t B, uint8_t* __restrict__ out) {
  const int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= B) return;
  Poses pose;
  fk64(T, state, q + b * T->q_dim, T->base_type == PM_BASE_FIXED, pose);
  bool ok = true;
  for (int k = 0; k < n_terms && ok; k++) {
    const PmPoseTerm& t = terms[k];
    if (t.kind != PM_TERM_POSITION_BOUND) continue;
    const DPose& te = pose[t.slot];
    const double pos = t.axis == 0 ? te.t.x : (t.axis == 1 ? te.t.y : te.t.z);
    if (t.has_lb && pos < t.lb) ok = false;
    if (t.has_ub && pos > t.ub) ok = false;
  }
  out[b] = ok ? 1 : 0;
}

}  // namespace

namespace pmg {

cudaError_t launch_posecst_eval64(const PmTablesHdr* T, const double* state, const PmPoseTerm* terms, int n_terms, int cst_dim,
                                  const double* q, int64_t B, double* vals, double* jac, cudaStream_t s) {
  if (B <= 0) return cudaSuccess;
  k_posecst_eval64<<<(unsigned)((B + 127) / 128), 128, 0, s>>>(T, state, terms, n_terms, cst_dim, q, B, vals, jac);
  return cudaGetLastError();
}

cudaError_t launch_posecst_valid64(const PmTablesHdr* T, const double* state, const PmPoseTerm* terms, int n_terms, const double* q,
                                   int64_t B, uint8_t* out, cudaStream_t s) {
  if (B <= 0) return cudaSuccess;
  k_posecst_valid64<<<(unsigned)((B + 127) / 128), 128, 0, s>>>(T, state, terms, n_terms, q, B, out);
  return cudaGetLastError();
}

}  // namespace pmg
