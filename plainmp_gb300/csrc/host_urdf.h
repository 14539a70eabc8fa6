// Minimal URDF reader for the kinematic part of a robot description.
//
// Follows the semantics plainmp inherits from its vendored urdfdom parser:
//   * numbers parse with the classic locale, whole token (third/urdf_parser/include/urdf_model/utils.h:73-88);
//   * vectors are 3 space-separated numbers (urdf_model/pose.h:69-92);
//   * an origin rotation is built from rpy and normalised (pose.h:202-216, 231-254);
//   * a joint without <axis> gets (1, 0, 0) unless fixed/floating (src/joint.cpp:424-445);
//   * revolute and prismatic joints must carry <limit>; missing lower/upper read as 0;
//   * the tree attaches children in joint-name order (std::map, urdf_model/model.h:113-150)
//     and the root is the one link without a parent (model.h:152-177).
#pragma once
#include <map>
#include <string>
#include <vector>

namespace pmg {

enum UrdfJointType { UJ_UNKNOWN = 0, UJ_REVOLUTE = 1, UJ_CONTINUOUS = 2, UJ_PRISMATIC = 3, UJ_FLOATING = 4, UJ_PLANAR = 5, UJ_FIXED = 6 };

struct UrdfJoint {
  std::string name;
  int type = UJ_UNKNOWN;
  std::string parent, child;
  double xyz[3] = {0, 0, 0};
  double quat[4] = {0, 0, 0, 1};  // x y z w
  double axis[3] = {1, 0, 0};
  bool has_limits = false;
  double lower = 0, upper = 0;
};

struct UrdfRobot {
  std::vector<std::string> links;                   // document order
  std::map<std::string, UrdfJoint> joints;          // by name
  std::map<std::string, std::vector<std::string>> child_joints;  // parent link -> joint names (name order)
  std::map<std::string, std::string> parent_joint;  // child link -> joint name
  std::string root;
};

// Throws std::runtime_error on malformed input.
UrdfRobot parse_urdf(const std::string& xml);

}  // namespace pmg
