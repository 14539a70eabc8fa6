// FP32 quaternion helpers of the differentiable costs (collision-aware IK, trajectory
// smoothing): Hamilton product, rotation of a vector, rotation matrix and the rotation-vector
// error of a pose target.
#pragma once
#include <cuda_runtime.h>

namespace pmd {

struct FQ {
  float x, y, z, w;
};

__device__ __forceinline__ FQ fqmul(const FQ& a, const FQ& b) {
  return FQ{fmaf(a.w, b.x, fmaf(a.x, b.w, fmaf(a.y, b.z, -a.z * b.y))), fmaf(a.w, b.y, fmaf(a.y, b.w, fmaf(a.z, b.x, -a.x * b.z))),
            fmaf(a.w, b.z, fmaf(a.z, b.w, fmaf(a.x, b.y, -a.y * b.x))), fmaf(a.w, b.w, -fmaf(a.x, b.x, fmaf(a.y, b.y, a.z * b.z)))};
}
__device__ __forceinline__ void fqrot(const FQ& q, const float v[3], float o[3]) {
  const float ux = fmaf(q.y, v[2], -q.z * v[1]) * 2.f, uy = fmaf(q.z, v[0], -q.x * v[2]) * 2.f, uz = fmaf(q.x, v[1], -q.y * v[0]) * 2.f;
  o[0] = v[0] + fmaf(q.w, ux, fmaf(q.y, uz, -q.z * uy));
  o[1] = v[1] + fmaf(q.w, uy, fmaf(q.z, ux, -q.x * uz));
  o[2] = v[2] + fmaf(q.w, uz, fmaf(q.x, uy, -q.y * ux));
}
__device__ __forceinline__ void fqmat(const FQ& q, float R[9]) {
  const float tx = 2.f * q.x, ty = 2.f * q.y, tz = 2.f * q.z;
  const float twx = tx * q.w, twy = ty * q.w, twz = tz * q.w, txx = tx * q.x, txy = ty * q.x, txz = tz * q.x, tyy = ty * q.y,
              tyz = tz * q.y, tzz = tz * q.z;
  R[0] = 1.f - (tyy + tzz);
  R[1] = txy - twz;
  R[2] = txz + twy;
  R[3] = txy + twz;
  R[4] = 1.f - (txx + tzz);
  R[5] = tyz - twx;
  R[6] = txz - twy;
  R[7] = tyz + twx;
  R[8] = 1.f - (txx + tyy);
}

// Rotation-vector error phi = log(q_t^-1 * q) (shortest arc) of a unit quaternion pair.
__device__ __forceinline__ void rotvec_error(const FQ& q, const FQ& qt, float phi[3]) {
  FQ e = fqmul(FQ{-qt.x, -qt.y, -qt.z, qt.w}, q);
  if (e.w < 0.f) e = FQ{-e.x, -e.y, -e.z, -e.w};
  const float s = sqrtf(fmaf(e.x, e.x, fmaf(e.y, e.y, e.z * e.z)));
  const float k = s > 1e-7f ? 2.f * atan2f(s, e.w) / s : 2.f / fmaxf(e.w, 1e-30f);
  phi[0] = k * e.x;
  phi[1] = k * e.y;
  phi[2] = k * e.z;
}

}  // namespace pmd
