// Primitive SDF dispatch (FP64, exact replicas of collision/primitive_sdf.hpp) shared by the
// plain kernels, the evaluate kernel and the FP64 recheck of the fast path.
#pragma once
#include "pm_grid.cuh"
#include "pm_math.cuh"

namespace pmd {

// PrimitiveSDFBase::is_outside (virtual) for one primitive
__device__ __forceinline__ bool prim_outside(const PmPrim& P, const PmGridDev* clouds, const D3& p, double r) {
  switch (P.kind) {
    case PM_SDF_BOX:
      return box_outside(P, p, r);
    case PM_SDF_CYLINDER:
      return cyl_outside(P, p, r);
    case PM_SDF_SPHERE:
      return sph_outside(P, p, r);
    case PM_SDF_GROUND:  // primitive_sdf.hpp:246-248
      return p.z + P.a > r;
    case PM_SDF_CLOUD: {  // primitive_sdf.hpp:597-603
      // Only whether some point lies within r + radius matters: search below a reach slightly
      // beyond it.  A point found there gives the exact KD-tree distance; none found means
      // sqrt(d2) - radius > r holds with a 1e-12 relative slack, far above rounding.
      const double reach = (r + P.a) * (1.0 + 1e-12) + 1e-12;
      NNResult64 nn = grid_nearest64(clouds[P.cloud], p, reach * reach);
      if (nn.idx < 0) return true;
      return sqrt(nn.d2) - P.a > r;
    }
  }
  return true;
}

// PrimitiveSDFBase::evaluate (virtual) for one primitive
__device__ __forceinline__ double prim_eval(const PmPrim& P, const PmGridDev* clouds, const D3& p) {
  switch (P.kind) {
    case PM_SDF_BOX:
      return box_eval(P, p);
    case PM_SDF_CYLINDER:
      return cyl_eval(P, p);
    case PM_SDF_SPHERE:
      return sph_eval(P, p);
    case PM_SDF_GROUND:
      return p.z + P.a;
    case PM_SDF_CLOUD: {
      NNResult64 nn = grid_nearest64(clouds[P.cloud], p);
      return sqrt(nn.d2) - P.a;
    }
  }
  return 0.0;
}

}  // namespace pmd
