// Device arithmetic of the hot path.
//
// FP64 functions reproduce the reference's operation order (quaternion product and
// rotation as in transform.hpp:56-86, rotation matrix as in
// primitive_sphere_collision.cpp:32, three-term sums as a0 + (a1 + a2)).  Translation units
// including this header are compiled with --fmad=false, so no multiply-add is contracted
// and every FP64 result is bit-identical to the same expression evaluated on the host with
// -ffp-contract=off.  FP32 helpers use explicit fmaf where they want a fused operation.
#pragma once
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "pm_common.h"

namespace pmd {

struct D3 {
  double x, y, z;
};
struct DQ {
  double x, y, z, w;
};
struct DPose {
  DQ q;
  D3 t;
};
struct DM3 {
  double m[9];  // row-major
};

__device__ __forceinline__ D3 add(const D3& a, const D3& b) { return D3{a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ D3 sub(const D3& a, const D3& b) { return D3{a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ double dot(const D3& a, const D3& b) { return a.x * b.x + (a.y * b.y + a.z * b.z); }
__device__ __forceinline__ double sqn(const D3& a) { return a.x * a.x + (a.y * a.y + a.z * a.z); }
__device__ __forceinline__ double nrm(const D3& a) { return sqrt(sqn(a)); }
__device__ __forceinline__ D3 cross(const D3& a, const D3& b) {
  return D3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}

// quaternion product a*b (transform.hpp:60, algorithm.cpp:147)
__device__ __forceinline__ DQ qmul(const DQ& a, const DQ& b) {
  DQ r;
  r.w = a.w * b.w - a.x * b.x - a.y * b.y - a.z * b.z;
  r.x = a.w * b.x + a.x * b.w + a.y * b.z - a.z * b.y;
  r.y = a.w * b.y + a.y * b.w + a.z * b.x - a.x * b.z;
  r.z = a.w * b.z + a.z * b.w + a.x * b.y - a.y * b.x;
  return r;
}
// quaternion * vector (transform.hpp:58)
__device__ __forceinline__ D3 qrot(const DQ& q, const D3& v) {
  D3 qv{q.x, q.y, q.z};
  D3 uv = cross(qv, v);
  uv = add(uv, uv);
  D3 c = cross(qv, uv);
  return D3{(v.x + q.w * uv.x) + c.x, (v.y + q.w * uv.y) + c.y, (v.z + q.w * uv.z) + c.z};
}
// toRotationMatrix (primitive_sphere_collision.cpp:32)
__device__ __forceinline__ DM3 qmat(const DQ& q) {
  double tx = 2.0 * q.x, ty = 2.0 * q.y, tz = 2.0 * q.z;
  double twx = tx * q.w, twy = ty * q.w, twz = tz * q.w;
  double txx = tx * q.x, txy = ty * q.x, txz = tz * q.x;
  double tyy = ty * q.y, tyz = tz * q.y, tzz = tz * q.z;
  DM3 r;
  r.m[0] = 1.0 - (tyy + tzz);
  r.m[1] = txy - twz;
  r.m[2] = txz + twy;
  r.m[3] = txy + twz;
  r.m[4] = 1.0 - (txx + tzz);
  r.m[5] = tyz - twx;
  r.m[6] = txz - twy;
  r.m[7] = tyz + twx;
  r.m[8] = 1.0 - (txx + tyy);
  return r;
}
__device__ __forceinline__ D3 mv(const DM3& R, const D3& v) {
  return D3{R.m[0] * v.x + (R.m[1] * v.y + R.m[2] * v.z), R.m[3] * v.x + (R.m[4] * v.y + R.m[5] * v.z),
            R.m[6] * v.x + (R.m[7] * v.y + R.m[8] * v.z)};
}
__device__ __forceinline__ D3 mv9(const double* R, const D3& v) {
  return D3{R[0] * v.x + (R[1] * v.y + R[2] * v.z), R[3] * v.x + (R[4] * v.y + R[5] * v.z), R[6] * v.x + (R[7] * v.y + R[8] * v.z)};
}
__device__ __forceinline__ D3 col9(const double* R, int j) { return D3{R[j], R[3 + j], R[6 + j]}; }

// quat_identity_sensitive_mult_and_assign (transform.hpp:64-74)
__device__ __forceinline__ DPose compose(const DPose& parent, const DQ& lq, const D3& lt, bool local_identity) {
  DPose o;
  o.q = local_identity ? parent.q : qmul(parent.q, lq);
  o.t = add(parent.t, qrot(parent.q, lt));
  return o;
}

// compute_approx_sin_cos (algorithm.cpp:50-86)
__device__ __forceinline__ void approx_sin_cos(double x, double& s, double& c) {
  const double coeff2 = 1.0 / (1.0 * 2.0);
  const double coeff3 = 1.0 / (1.0 * 2.0 * 3.0);
  const double coeff4 = 1.0 / (1.0 * 2.0 * 3.0 * 4.0);
  const double coeff5 = 1.0 / (1.0 * 2.0 * 3.0 * 4.0 * 5.0);
  const double coeff6 = 1.0 / (1.0 * 2.0 * 3.0 * 4.0 * 5.0 * 6.0);
  const double coeff7 = 1.0 / (1.0 * 2.0 * 3.0 * 4.0 * 5.0 * 6.0 * 7.0);
  const double coeff8 = 1.0 / (1.0 * 2.0 * 3.0 * 4.0 * 5.0 * 6.0 * 7.0 * 8.0);
  const double coeff9 = 1.0 / (1.0 * 2.0 * 3.0 * 4.0 * 5.0 * 6.0 * 7.0 * 8.0 * 9.0);
  const double pi = 3.14159265358979323846;
  const double half_pi = pi * 0.5;
  const double one_dev_2pi = 1.0 / (2 * pi);
  double cos_sign = 1.0;
  if (x > half_pi || x < -half_pi) {
    if (x > pi || x < -pi) x = x - 2 * pi * floor(x * one_dev_2pi + 0.5);
    if (x < -half_pi) {
      x = -x - pi;
      cos_sign = -1.0;
    } else if (x > half_pi) {
      x = -x + pi;
      cos_sign = -1.0;
    }
  }
  double xx = x * x;
  double xxxx = xx * xx;
  double xxxxxx = xxxx * xx;
  double xxxxxxxx = xxxx * xxxx;
  s = x * (1 - xx * coeff3 + xxxx * coeff5 - xxxxxx * coeff7 + xxxxxxxx * coeff9);
  c = cos_sign * (1 - xx * coeff2 + xxxx * coeff4 - xxxxxx * coeff6 + xxxxxxxx * coeff8);
}

// setQuaternionFromRPY (transform.hpp:122-130)
__device__ __forceinline__ DQ quat_from_rpy(double r, double p, double y) {
  double phi = r / 2.0, the = p / 2.0, psi = y / 2.0;
  double sphi, cphi, sthe, cthe, spsi, cpsi;
  sincos(phi, &sphi, &cphi);
  sincos(the, &sthe, &cthe);
  sincos(psi, &spsi, &cpsi);
  DQ q;
  q.x = sphi * cthe * cpsi - cphi * sthe * spsi;
  q.y = cphi * sthe * cpsi + sphi * cthe * spsi;
  q.z = cphi * cthe * spsi - sphi * sthe * cpsi;
  q.w = cphi * cthe * cpsi + sphi * sthe * spsi;
  return q;
}

// Local transform of a revolute / prismatic joint at angle theta (algorithm.cpp:116-157).
__device__ __forceinline__ void joint_local(const PmSlot& s, double theta, bool taylor, DQ& lq, D3& lt, bool& lid) {
  if (s.mode == PM_FK_PRIS) {
    D3 tr{s.axis[0] * theta, s.axis[1] * theta, s.axis[2] * theta};
    lt = add(D3{s.ot[0], s.ot[1], s.ot[2]}, tr);
    lq = DQ{0.0, 0.0, 0.0, 1.0};
    lid = true;
    return;
  }
  double x = theta * 0.5;
  double sn, cs;
  if (taylor) {
    approx_sin_cos(x, sn, cs);
  } else {
    sincos(x, &sn, &cs);
  }
  DQ jq{sn * s.axis[0], sn * s.axis[1], sn * s.axis[2], cs};
  if (s.origin_identity) {
    lq = jq;
  } else {
    DQ oq{s.oq[0], s.oq[1], s.oq[2], s.oq[3]};
    lq = qmul(oq, jq);
  }
  lt = D3{s.ot[0], s.ot[1], s.ot[2]};
  lid = false;
}

__device__ __forceinline__ DPose state_pose(const double* st, int row, bool& qid) {
  const double* r = st + (int64_t)row * PM_STATE_STRIDE;
  qid = r[7] != 0.0;
  return DPose{DQ{r[0], r[1], r[2], r[3]}, D3{r[4], r[5], r[6]}};
}

// Base pose of update_kintree (constraints/primitive.hpp:38-62)
__device__ __forceinline__ DPose base_pose(const PmTablesHdr* T, const double* state, const double* q, int n_ctrl) {
  if (T->base_type == PM_BASE_FIXED) {
    bool dummy;
    return state_pose(state, PM_STATE_BASE_ROW, dummy);
  }
  DPose b;
  if (T->base_type == PM_BASE_FLOATING) {
    b.t = D3{q[n_ctrl], q[n_ctrl + 1], q[n_ctrl + 2]};
    b.q = quat_from_rpy(q[n_ctrl + 3], q[n_ctrl + 4], q[n_ctrl + 5]);
  } else {
    b.t = D3{q[n_ctrl], q[n_ctrl + 1], 0.0};
    b.q = quat_from_rpy(0, 0, q[n_ctrl + 2]);
  }
  return b;
}

// Full FK of the constraint's slots for one config.  taylor selects compute_approx_sin_cos
// (is_valid on a FIXED base); otherwise sin/cos.  pose[] receives every slot's world pose.
template <class PoseArr>
__device__ __forceinline__ void fk64(const PmTablesHdr* T, const double* state, const double* q, bool taylor, PoseArr& pose) {
  const PmSlot* S = pm_at<PmSlot>(T, T->off_slots);
  DPose base = base_pose(T, state, q, T->n_ctrl);
  for (int i = 0; i < T->n_slots; i++) {
    const PmSlot& s = S[i];
    if (s.parent < 0) {
      pose[i] = base;
      continue;
    }
    DQ lq;
    D3 lt;
    bool lid;
    if (s.mode == PM_FK_STATE) {
      DPose l = state_pose(state, PM_STATE_LINK_ROW(s.link), lid);
      lq = l.q;
      lt = l.t;
    } else {
      joint_local(s, q[s.qcol], taylor, lq, lt, lid);
    }
    pose[i] = compose(pose[s.parent], lq, lt, lid);
  }
}

// The same FK restricted to the slots whose bit is set in `need` (a set closed under parents,
// e.g. from slot_chain); the values of those slots are the full FK's, bit for bit.
__device__ __forceinline__ uint64_t slot_chain(const PmTablesHdr* T, int slot) {
  const PmSlot* S = pm_at<PmSlot>(T, T->off_slots);
  uint64_t m = 0;
  for (int i = slot; i >= 0; i = S[i].parent) m |= 1ull << i;
  return m;
}
template <class PoseArr>
__device__ __forceinline__ void fk64_need(const PmTablesHdr* T, const double* state, const double* q, bool taylor, uint64_t need,
                                          PoseArr& pose) {
  const PmSlot* S = pm_at<PmSlot>(T, T->off_slots);
  for (int i = 0; i < T->n_slots; i++) {
    if (!((need >> i) & 1ull)) continue;
    const PmSlot& s = S[i];
    if (s.parent < 0) {
      pose[i] = base_pose(T, state, q, T->n_ctrl);
      continue;
    }
    DQ lq;
    D3 lt;
    bool lid;
    if (s.mode == PM_FK_STATE) {
      DPose l = state_pose(state, PM_STATE_LINK_ROW(s.link), lid);
      lq = l.q;
      lt = l.t;
    } else {
      joint_local(s, q[s.qcol], taylor, lq, lt, lid);
    }
    pose[i] = compose(pose[s.parent], lq, lt, lid);
  }
}

// Warp-cooperative fk64_need for latency-bound single configurations (all 32 lanes, identical
// arguments; every lane ends with the poses).  Each lane computes the local transform of one slot;
// then, slot by slot, lanes 0-3 compute the four components of the quaternion product and lanes
// 0-2 the three components of the rotated translation.  Every component is evaluated with the
// expression (operand pairs, signs, summation order) of qmul / qrot / add, so the poses are bit for
// bit those of fk64_need; lanes differ only in which operands they select, so the warp does not
// diverge.  GB300 issues an FP64 warp instruction at a cost that does not shrink with inactive
// lanes, so spreading the components cuts the dependent FP64 chain per slot from 61 to 18.
__device__ __forceinline__ double sel4(int k, double a0, double a1, double a2, double a3) {
  return k == 0 ? a0 : (k == 1 ? a1 : (k == 2 ? a2 : a3));
}
__device__ __forceinline__ double neg_if(bool n, double v) {
  return __longlong_as_double(__double_as_longlong(v) ^ (n ? (long long)0x8000000000000000ull : 0ll));
}
template <class PoseArr>
__device__ void fk64_need_warp(const PmTablesHdr* T, const double* state, const double* q, bool taylor, uint64_t need, PoseArr& pose) {
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const PmSlot* S = pm_at<PmSlot>(T, T->off_slots);
  const int n = T->n_slots;
  // component index of this lane (lanes 4-31 repeat lanes 0-3; their results are not used)
  const int k4 = lane & 3, k3 = lane % 3;
  for (int base = 0; base < n; base += 32) {
    const int i = base + lane;
    DQ lq{0, 0, 0, 1};
    D3 lt{0, 0, 0};
    bool lid = true;
    if (i < n && ((need >> i) & 1ull) && S[i].parent >= 0) {
      const PmSlot& s = S[i];
      if (s.mode == PM_FK_STATE) {
        const DPose l = state_pose(state, PM_STATE_LINK_ROW(s.link), lid);
        lq = l.q;
        lt = l.t;
      } else {
        joint_local(s, q[s.qcol], taylor, lq, lt, lid);
      }
    }
    for (int k = 0; k < 32 && base + k < n; k++) {
      const int si = base + k;
      if (!((need >> si) & 1ull)) continue;
      const PmSlot& s = S[si];
      if (s.parent < 0) {
        pose[si] = base_pose(T, state, q, T->n_ctrl);
        continue;
      }
      const DQ b{__shfl_sync(FULL, lq.x, k), __shfl_sync(FULL, lq.y, k), __shfl_sync(FULL, lq.z, k), __shfl_sync(FULL, lq.w, k)};
      const D3 v{__shfl_sync(FULL, lt.x, k), __shfl_sync(FULL, lt.y, k), __shfl_sync(FULL, lt.z, k)};
      const bool id = __shfl_sync(FULL, lid ? 1 : 0, k) != 0;
      const DPose P = pose[s.parent];
      const DQ& a = P.q;
      DPose o;
      if (id) {
        o.q = a;
      } else {
        // qmul(a, b): w: aw*bw - ax*bx - ay*by - az*bz;  x: aw*bx + ax*bw + ay*bz - az*by;
        //             y: aw*by + ay*bw + az*bx - ax*bz;   z: aw*bz + az*bw + ax*by - ay*bx
        const double p0 = a.w * sel4(k4, b.w, b.x, b.y, b.z);
        const double p1 = sel4(k4, a.x, a.x, a.y, a.z) * sel4(k4, b.x, b.w, b.w, b.w);
        const double p2 = sel4(k4, a.y, a.y, a.z, a.x) * sel4(k4, b.y, b.z, b.x, b.y);
        const double p3 = sel4(k4, a.z, a.z, a.x, a.y) * sel4(k4, b.z, b.y, b.z, b.x);
        const double r = ((p0 + neg_if(k4 == 0, p1)) + neg_if(k4 == 0, p2)) - p3;
        o.q = DQ{__shfl_sync(FULL, r, 1), __shfl_sync(FULL, r, 2), __shfl_sync(FULL, r, 3), __shfl_sync(FULL, r, 0)};
      }
      // qrot(a, v): uv = cross(a.vec, v); uv += uv; c = cross(a.vec, uv); (v + a.w * uv) + c; then add(P.t, .)
      const D3 av{a.x, a.y, a.z};
      const double u1 = sel4(k3, av.y, av.z, av.x, 0.0) * sel4(k3, v.z, v.x, v.y, 0.0);
      const double u2 = sel4(k3, av.z, av.x, av.y, 0.0) * sel4(k3, v.y, v.z, v.x, 0.0);
      double uvk = u1 - u2;
      uvk = uvk + uvk;
      const D3 uv{__shfl_sync(FULL, uvk, 0), __shfl_sync(FULL, uvk, 1), __shfl_sync(FULL, uvk, 2)};
      const double c1 = sel4(k3, av.y, av.z, av.x, 0.0) * sel4(k3, uv.z, uv.x, uv.y, 0.0);
      const double c2 = sel4(k3, av.z, av.x, av.y, 0.0) * sel4(k3, uv.y, uv.z, uv.x, 0.0);
      const double ck = c1 - c2;
      const double rk = (sel4(k3, v.x, v.y, v.z, 0.0) + a.w * sel4(k3, uv.x, uv.y, uv.z, 0.0)) + ck;
      const double tk = sel4(k3, P.t.x, P.t.y, P.t.z, 0.0) + rk;
      o.t = D3{__shfl_sync(FULL, tk, 0), __shfl_sync(FULL, tk, 1), __shfl_sync(FULL, tk, 2)};
      pose[si] = o;
    }
  }
}

// ------------------------------------------------------------------------- transforms for jacobians
__device__ __forceinline__ DPose pose_inverse(const DPose& a) {  // transform.hpp:88-91
  double n2 = (a.q.x * a.q.x + a.q.y * a.q.y) + (a.q.z * a.q.z + a.q.w * a.q.w);
  DQ qi;
  if (n2 > 0) {
    qi = DQ{-a.q.x / n2, -a.q.y / n2, -a.q.z / n2, a.q.w / n2};
  } else {
    qi = DQ{0, 0, 0, 0};
  }
  DPose r;
  r.q = qi;
  r.t = qrot(qi, D3{-a.t.x, -a.t.y, -a.t.z});
  return r;
}
__device__ __forceinline__ DPose pose_mul(const DPose& a, const DPose& b) {  // transform.hpp:56-62 (b not identity-flagged)
  DPose r;
  r.q = qmul(a.q, b.q);
  r.t = add(a.t, qrot(a.q, b.t));
  return r;
}
__device__ __forceinline__ D3 get_rpy(const DQ& q) {  // transform.hpp:93-120
  double sqx = q.x * q.x, sqy = q.y * q.y, sqz = q.z * q.z, sqw = q.w * q.w;
  double sarg = -2 * (q.x * q.z - q.w * q.y);
  const double pi_2 = 1.57079632679489661923;
  double roll, pitch, yaw;
  if (sarg <= -0.99999) {
    pitch = -pi_2;
    roll = 0;
    yaw = -2 * atan2(q.x, q.y);
  } else if (sarg >= 0.99999) {
    pitch = pi_2;
    roll = 0;
    yaw = 2 * atan2(q.x, q.y);
  } else {
    pitch = asin(sarg);
    roll = atan2(2 * (q.y * q.z + q.w * q.x), sqw - sqx - sqy + sqz);
    yaw = atan2(2 * (q.x * q.y + q.w * q.z), sqw + sqx - sqy - sqz);
  }
  return D3{roll, pitch, yaw};
}

// ------------------------------------------------------------------------- primitive SDFs
// collision/primitive_sdf.hpp:180-184
__device__ __forceinline__ bool outside_aabb(const PmPrim& P, const D3& p, double r) {
  return p.x < P.lb[0] - r || p.x > P.ub[0] + r || p.y < P.lb[1] - r || p.y > P.ub[1] + r || p.z < P.lb[2] - r ||
         p.z > P.ub[2] + r;
}

// BoxSDF::is_outside (primitive_sdf.hpp:313-398)
__device__ __forceinline__ bool box_outside(const PmPrim& P, const D3& p, double radius) {
  double xs, ys, zs;
  if (P.axis_aligned) {
    xs = fabs(p.x - P.pos[0]) - P.a;
    if (xs > radius) return true;
    ys = fabs(p.y - P.pos[1]) - P.b;
    if (ys > radius) return true;
    zs = fabs(p.z - P.pos[2]) - P.c;
    if (zs > radius) return true;
  } else if (P.z_axis_aligned) {
    zs = fabs(p.z - P.pos[2]) - P.c;
    if (zs > radius) return true;
    D3 d = sub(p, D3{P.pos[0], P.pos[1], P.pos[2]});
    xs = fabs(dot(d, col9(P.rot, 0))) - P.a;
    if (xs > radius) return true;
    ys = fabs(dot(d, col9(P.rot, 1))) - P.b;
    if (ys > radius) return true;
  } else {
    D3 d = sub(p, D3{P.pos[0], P.pos[1], P.pos[2]});
    xs = fabs(dot(d, col9(P.rot, 0))) - P.a;
    if (xs > radius) return true;
    ys = fabs(dot(d, col9(P.rot, 1))) - P.b;
    if (ys > radius) return true;
    zs = fabs(dot(d, col9(P.rot, 2))) - P.c;
    if (zs > radius) return true;
  }
  if (radius < 1e-6) return false;
  bool xo = xs > 0, yo = ys > 0, zo = zs > 0;
  int cnt = (int)xo + (int)yo + (int)zo;
  if (cnt < 2) return false;
  if (cnt == 3) return xs * xs + ys * ys + zs * zs > radius * radius;
  if (!xo) return ys * ys + zs * zs > radius * radius;
  if (!yo) return xs * xs + zs * zs > radius * radius;
  return xs * xs + ys * ys > radius * radius;
}
// BoxSDF::evaluate (primitive_sdf.hpp:299-311)
__device__ __forceinline__ double box_eval(const PmPrim& P, const D3& p) {
  D3 d = sub(p, D3{P.pos[0], P.pos[1], P.pos[2]});
  D3 l = P.axis_aligned ? d : mv9(P.rot_inv, d);
  D3 sd{fabs(l.x) - P.a, fabs(l.y) - P.b, fabs(l.z) - P.c};
  D3 mp{fmax(sd.x, 0.0), fmax(sd.y, 0.0), fmax(sd.z, 0.0)};
  double out = nrm(mp);
  double in = fmax(fmin(sd.x, 0.0), fmax(fmin(sd.y, 0.0), fmin(sd.z, 0.0)));
  return out + in;
}
// CylinderSDF (primitive_sdf.hpp:444-498)
__device__ __forceinline__ void cyl_parts(const PmPrim& P, const D3& p, double& zs, double& xa, double& ya) {
  if (P.z_axis_aligned) {
    zs = fabs(p.z - P.pos[2]) - P.c;
    xa = fabs(p.x - P.pos[0]);
    ya = fabs(p.y - P.pos[1]);
  } else {
    D3 d = sub(p, D3{P.pos[0], P.pos[1], P.pos[2]});
    zs = fabs(dot(d, col9(P.rot, 2))) - P.c;
    xa = fabs(dot(d, col9(P.rot, 0)));
    ya = fabs(dot(d, col9(P.rot, 1)));
  }
}
__device__ __forceinline__ bool cyl_outside(const PmPrim& P, const D3& p, double radius) {
  double zs, xa, ya;
  if (P.z_axis_aligned) {
    zs = fabs(p.z - P.pos[2]) - P.c;
    if (zs > radius) return true;
    xa = fabs(p.x - P.pos[0]);
    ya = fabs(p.y - P.pos[1]);
  } else {
    D3 d = sub(p, D3{P.pos[0], P.pos[1], P.pos[2]});
    zs = fabs(dot(d, col9(P.rot, 2))) - P.c;
    if (zs > radius) return true;
    xa = fabs(dot(d, col9(P.rot, 0)));
    ya = fabs(dot(d, col9(P.rot, 1)));
  }
  double dsq = xa * xa + ya * ya;
  if (radius < 1e-6) return dsq > P.b;
  if (dsq > (P.a + radius) * (P.a + radius)) return true;
  bool ho = zs > 0, ro = dsq > P.b;
  if (ho && ro) {
    double rs = sqrt(dsq) - P.a;
    return zs * zs + rs * rs > radius * radius;
  }
  return false;
}
__device__ __forceinline__ double cyl_eval(const PmPrim& P, const D3& p) {
  double zs, xa, ya;
  cyl_parts(P, p, zs, xa, ya);
  double rs = sqrt(xa * xa + ya * ya) - P.a;
  double a = fmax(rs, 0.0), b = fmax(zs, 0.0);
  double out = sqrt(a * a + b * b);
  double in = fmax(fmin(rs, 0.0), fmin(zs, 0.0));
  return out + in;
}
// SphereSDF (primitive_sdf.hpp:540-552)
__device__ __forceinline__ bool sph_outside(const PmPrim& P, const D3& p, double radius) {
  double d2 = sqn(sub(p, D3{P.pos[0], P.pos[1], P.pos[2]}));
  if (radius < 1e-6) return d2 > P.b;
  return d2 > (P.a + radius) * (P.a + radius);
}
__device__ __forceinline__ double sph_eval(const PmPrim& P, const D3& p) { return nrm(sub(p, D3{P.pos[0], P.pos[1], P.pos[2]})) - P.a; }

}  // namespace pmd
