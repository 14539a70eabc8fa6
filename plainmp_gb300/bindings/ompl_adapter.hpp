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
struct GpuValidity {
  pmgpu_cst* cst; int dim;
  bool operator()(const ompl::base::State* s) const {
    const double* q = s->as<ompl::base::RealVectorStateSpace::StateType>()->values;
    uint8_t ok = 0;
    if (pmgpu_cst_is_valid_fast(cst, q, 1, &ok, nullptr, nullptr, PMGPU_MEM_HOST, nullptr) != PMGPU_OK)
      throw std::runtime_error(pmgpu_last_error());
    return ok != 0;
  }
};
class GpuBoxMotionValidator : public ompl::base::MotionValidator {
 public:
  GpuBoxMotionValidator(const ompl::base::SpaceInformationPtr& si, pmgpu_cst* c, std::vector<double> w)
      : MotionValidator(si), cst_(c), w_(std::move(w)) {}
  bool checkMotion(const ompl::base::State* a, const ompl::base::State* b) const override {
    using RV = ompl::base::RealVectorStateSpace::StateType;
    uint8_t ok = 0;
    if (pmgpu_check_motion_fast(cst_, a->as<RV>()->values, b->as<RV>()->values, 1, PMGPU_VALIDATOR_BOX, w_.data(), 0.0,
                                &ok, nullptr, PMGPU_MEM_HOST, nullptr) != PMGPU_OK)
      throw std::runtime_error(pmgpu_last_error());
    return ok != 0;
  }
  bool checkMotion(const ompl::base::State* a, const ompl::base::State* b, std::pair<ompl::base::State*, double>&) const override {
    return checkMotion(a, b);
  }
 private:
  pmgpu_cst* cst_; std::vector<double> w_;
};
