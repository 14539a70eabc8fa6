// Test infrastructure only: dumps what the reference's vendored urdfdom parser
// (third/urdf_parser) reads from a URDF file, as JSON: the root, per link its parent and its
// children in attachment order, per joint type / parent / child / origin (position and the
// normalised quaternion) / axis / limits.  Built by oracle/ref/build_ref.sh into oracle/_ref/.
#include <cstdio>
#include <fstream>
#include <sstream>
#include <string>

#include "urdf_parser/urdf_parser.h"

static void num(double v) { std::printf("%.17g", v); }

int main(int argc, char** argv) {
  if (argc != 2) {
    std::fprintf(stderr, "usage: urdf_dump file.urdf\n");
    return 2;
  }
  std::ifstream f(argv[1]);
  std::stringstream ss;
  ss << f.rdbuf();
  urdf::ModelInterfaceSharedPtr m;
  try {
    m = urdf::parseURDF(ss.str());
  } catch (std::exception& e) {
    std::printf("{\"error\": \"%s\"}\n", e.what());
    return 0;
  }
  if (!m) {
    std::printf("{\"error\": \"parse failed\"}\n");
    return 0;
  }
  std::printf("{\"root\": \"%s\", \"links\": {", m->root_link_->name.c_str());
  bool first = true;
  for (auto& kv : m->links_) {
    auto& l = kv.second;
    std::printf("%s\"%s\": {\"parent\": ", first ? "" : ", ", kv.first.c_str());
    first = false;
    if (l->getParent())
      std::printf("\"%s\"", l->getParent()->name.c_str());
    else
      std::printf("null");
    std::printf(", \"children\": [");
    for (size_t i = 0; i < l->child_links.size(); i++) std::printf("%s\"%s\"", i ? ", " : "", l->child_links[i]->name.c_str());
    std::printf("], \"child_joints\": [");
    for (size_t i = 0; i < l->child_joints.size(); i++) std::printf("%s\"%s\"", i ? ", " : "", l->child_joints[i]->name.c_str());
    std::printf("]}");
  }
  std::printf("}, \"joints\": {");
  first = true;
  for (auto& kv : m->joints_) {
    auto& j = kv.second;
    std::printf("%s\"%s\": {\"type\": %d, \"parent\": \"%s\", \"child\": \"%s\", \"xyz\": [", first ? "" : ", ", kv.first.c_str(),
                (int)j->type, j->parent_link_name.c_str(), j->child_link_name.c_str());
    first = false;
    auto& o = j->parent_to_joint_origin_transform;
    num(o.position.x); std::printf(", "); num(o.position.y); std::printf(", "); num(o.position.z);
    std::printf("], \"quat\": [");
    num(o.rotation.x); std::printf(", "); num(o.rotation.y); std::printf(", "); num(o.rotation.z); std::printf(", "); num(o.rotation.w);
    std::printf("], \"axis\": [");
    num(j->axis.x); std::printf(", "); num(j->axis.y); std::printf(", "); num(j->axis.z);
    std::printf("], \"limits\": ");
    if (j->limits) {
      std::printf("["); num(j->limits->lower); std::printf(", "); num(j->limits->upper); std::printf("]");
    } else {
      std::printf("null");
    }
    std::printf("}");
  }
  std::printf("}}\n");
  return 0;
}
