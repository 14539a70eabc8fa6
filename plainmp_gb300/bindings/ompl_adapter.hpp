// OMPL adapter of the C ABI: the state-validity callback and the box motion validator that
// CollisionAwareSpaceInformation installs (ompl/ompl_thin_wrap.hpp:114-120, 181-182;
// ompl/motion_validator.hpp:29-34), each call a batch of one through include/pmgpu.h's fast entry
// points (FP32 with the FP64 recheck: the reference's booleans, at a fraction of the plain FP64
// method's per-call latency).
// Header-only: it includes the two OMPL headers it needs and the C ABI's header.
#pragma once
#include <stdexcept>
#include <utility>
#include <vector>

#include <ompl/base/MotionValidator.h>
#include <ompl/base/spaces/RealVectorStateSpace.h>

#include "pmgpu.h"
// bounds: the LinkPositionBoundCst members when the planner's constraint is an IneqCompositeCst of
// the collision constraint and link-position bounds (checked in the same fused launch); empty for
// the collision constraint alone.
struct GpuValidity {
  pmgpu_cst* cst; int dim;
  std::vector<pmgpu_posecst*> bounds;
  bool operator()(const ompl::base::State* s) const {
    const double* q = s->as<ompl::base::RealVectorStateSpace::StateType>()->values;
    uint8_t ok = 0;
    const int rc = bounds.empty()
                       ? pmgpu_cst_is_valid_fast(cst, q, 1, &ok, nullptr, nullptr, PMGPU_MEM_HOST, nullptr)
                       : pmgpu_composite_is_valid_fast(cst, bounds.data(), (int)bounds.size(), q, 1, &ok, nullptr, PMGPU_MEM_HOST, nullptr);
    if (rc != PMGPU_OK) throw std::runtime_error(pmgpu_last_error());
    return ok != 0;
  }
};
class GpuBoxMotionValidator : public ompl::base::MotionValidator {
 public:
  GpuBoxMotionValidator(const ompl::base::SpaceInformationPtr& si, pmgpu_cst* c, std::vector<double> w,
                        std::vector<pmgpu_posecst*> bounds = {})
      : MotionValidator(si), cst_(c), w_(std::move(w)), bounds_(std::move(bounds)) {}
  bool checkMotion(const ompl::base::State* a, const ompl::base::State* b) const override {
    using RV = ompl::base::RealVectorStateSpace::StateType;
    const double* s1 = a->as<RV>()->values;
    const double* s2 = b->as<RV>()->values;
    uint8_t ok = 0;
    const int rc = bounds_.empty()
                       ? pmgpu_check_motion_fast(cst_, s1, s2, 1, PMGPU_VALIDATOR_BOX, w_.data(), 0.0, &ok, nullptr, PMGPU_MEM_HOST, nullptr)
                       : pmgpu_composite_check_motion_fast(cst_, bounds_.data(), (int)bounds_.size(), s1, s2, 1, PMGPU_VALIDATOR_BOX,
                                                           w_.data(), 0.0, &ok, nullptr, PMGPU_MEM_HOST, nullptr);
    if (rc != PMGPU_OK) throw std::runtime_error(pmgpu_last_error());
    return ok != 0;
  }
  bool checkMotion(const ompl::base::State* a, const ompl::base::State* b, std::pair<ompl::base::State*, double>&) const override {
    return checkMotion(a, b);
  }
 private:
  pmgpu_cst* cst_; std::vector<double> w_; std::vector<pmgpu_posecst*> bounds_;
};
