// FP32 fast path with FP64 recheck (filled in by the fast-path kernels).
#include "pm_launch.h"
#include "pmgpu.h"

extern "C" {
int pmgpu_cst_is_valid_fast(pmgpu_cst*, const double*, int64_t, uint8_t*, float*, int64_t*, int, void*) { return PMGPU_ERR_RUNTIME; }
int pmgpu_check_motion_fast(pmgpu_cst*, const double*, const double*, int64_t, int, const double*, double, uint8_t*, int64_t*, int,
                            void*) {
  return PMGPU_ERR_RUNTIME;
}
}
