// Host side of the drop-in boundary: KinematicModel, primitive SDFs and SphereCollisionCst
// objects, their flattening into device tables, and the extern "C" entry points of
// include/pmgpu.h.  Construction-time bookkeeping (URDF tree numbering, pose flags, AABBs,
// sphere-group statistics) runs here as it does in the reference's constructors; every
// per-configuration computation runs on the device.
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <atomic>
#include <cmath>
#include <cstring>
#include <limits>
#include <map>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include "host_urdf.h"
#include "pm_common.h"
#include "pm_launch.h"
#include "pmgpu.h"

namespace pmg {

// ---------------------------------------------------------------------------- errors
static thread_local std::string g_last_error;

struct PmError : std::runtime_error {
  int code;
  PmError(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};
[[noreturn]] static void fail(int code, const std::string& msg) { throw PmError(code, msg); }
static void cuda_check(cudaError_t e, const char* what) {
  if (e != cudaSuccess) {
    cudaGetLastError();
    fail(PMGPU_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
  }
}

template <class F>
static int guarded(F&& f) {
  try {
    f();
    g_last_error.clear();
    return PMGPU_OK;
  } catch (const PmError& e) {
    g_last_error = e.what();
    return e.code;
  } catch (const std::invalid_argument& e) {
    g_last_error = e.what();
    return PMGPU_ERR_INVALID;
  } catch (const std::bad_alloc&) {
    g_last_error = "host allocation failed";
    return PMGPU_ERR_RUNTIME;
  } catch (const std::exception& e) {
    g_last_error = e.what();
    return PMGPU_ERR_RUNTIME;
  }
}

static void require_device() {
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0) {
    cudaGetLastError();
    fail(PMGPU_ERR_CUDA, "no CUDA device available: the GB300 kernels cannot run on this host");
  }
}

// The CUDA device current on the calling thread.
static int current_device() {
  int d = -1;
  cuda_check(cudaGetDevice(&d), "cudaGetDevice");
  return d;
}
// Device data (model state, constraint tables, cloud grids, SDF images) stay on the device that was
// current at their first batch call.  A call made while another device is current would hand that
// device's kernels foreign pointers, so it is refused.
static void check_device(int owner, const char* what) {
  const int cur = current_device();
  if (cur != owner)
    fail(PMGPU_ERR_INVALID, std::string(what) + " was placed on CUDA device " + std::to_string(owner) +
                                " by its first batch call, but the calling thread's current device is " + std::to_string(cur));
}

// ---------------------------------------------------------------------------- kernel timing
namespace {
struct ProfRec {
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> pending;
  double total_ms = 0;
  int64_t launches = 0;
};
std::mutex g_prof_mu;
std::map<std::string, ProfRec> g_prof;
std::map<std::string, cudaEvent_t> g_prof_open;
std::atomic<bool> g_prof_enabled{false};
}  // namespace

bool prof_on() { return g_prof_enabled.load(); }
void prof_begin(const char* kernel, cudaStream_t s) {
  if (!prof_on()) return;
  cudaEvent_t e;
  if (cudaEventCreate(&e) != cudaSuccess) return;
  cudaEventRecord(e, s);
  std::lock_guard<std::mutex> lk(g_prof_mu);
  g_prof_open[kernel] = e;
}
void prof_end(const char* kernel, cudaStream_t s) {
  if (!prof_on()) return;
  std::lock_guard<std::mutex> lk(g_prof_mu);
  auto it = g_prof_open.find(kernel);
  if (it == g_prof_open.end()) return;
  cudaEvent_t e;
  if (cudaEventCreate(&e) != cudaSuccess) return;
  cudaEventRecord(e, s);
  g_prof[kernel].pending.push_back({it->second, e});
  g_prof[kernel].launches++;
  g_prof_open.erase(it);
}

// ---------------------------------------------------------------------------- device buffers
struct DevBuf {
  void* p = nullptr;
  size_t n = 0;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  ~DevBuf() { release(); }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  void* ensure(size_t bytes) {
    if (bytes <= n && p) return p;
    release();
    size_t b = std::max<size_t>(bytes, 256);
    cuda_check(cudaMalloc(&p, b), "cudaMalloc");
    n = b;
    return p;
  }
  template <class T>
  T* as() const {
    return reinterpret_cast<T*>(p);
  }
};

// Page-locked host buffer (grows, never shrinks): staging of small host-memory calls, so their
// copies are plain DMA transfers on the stream instead of the driver's pageable-memory path.
struct PinBuf {
  void* p = nullptr;
  size_t n = 0;
  PinBuf() = default;
  PinBuf(const PinBuf&) = delete;
  PinBuf& operator=(const PinBuf&) = delete;
  ~PinBuf() {
    if (p) cudaFreeHost(p);
  }
  char* ensure(size_t bytes) {
    if (bytes <= n && p) return static_cast<char*>(p);
    if (p) cudaFreeHost(p);
    p = nullptr;
    n = 0;
    const size_t b = std::max<size_t>(bytes, 4096);
    cuda_check(cudaHostAlloc(&p, b, cudaHostAllocDefault), "cudaHostAlloc");
    n = b;
    return static_cast<char*>(p);
  }
};
static size_t up16(size_t x) { return (x + 15) & ~(size_t)15; }

// ---------------------------------------------------------------------------- host quaternion
// construction-time helpers (setQuaternionFromRPY, transform.hpp:122-130)
static void quat_from_rpy(double r, double p, double y, double q[4]) {
  double phi = r / 2.0, the = p / 2.0, psi = y / 2.0;
  q[0] = std::sin(phi) * std::cos(the) * std::cos(psi) - std::cos(phi) * std::sin(the) * std::sin(psi);
  q[1] = std::cos(phi) * std::sin(the) * std::cos(psi) + std::sin(phi) * std::cos(the) * std::sin(psi);
  q[2] = std::cos(phi) * std::cos(the) * std::sin(psi) - std::sin(phi) * std::sin(the) * std::cos(psi);
  q[3] = std::cos(phi) * std::cos(the) * std::cos(psi) + std::sin(phi) * std::sin(the) * std::sin(psi);
}

// ---------------------------------------------------------------------------- KinematicModel
struct HostJoint {
  std::string name;
  int type;  // UrdfJointType
  int child;
  double axis[3], pos[3], quat[4];
  bool qid;
  double lower, upper;
};

struct HostModel {
  std::vector<std::string> link_name;
  std::map<std::string, int> link_id;
  std::vector<int> parent;
  std::vector<std::vector<int>> children;
  std::vector<char> consider_rotation;
  std::vector<HostJoint> joints;
  std::map<std::string, int> joint_id;
  std::vector<int> link_parent_joint;  // movable joint id owning the link, -1 otherwise
  int root = 0;
  std::vector<double> state_init;  // rows of PM_STATE_STRIDE doubles (row 0 = base)
  std::vector<double> angles;
  double base7[7] = {0, 0, 0, 0, 0, 0, 1};
  uint64_t version = 1;  // bumped when the link set changes
  // device
  DevBuf d_state;
  DevBuf d_parents;
  DevBuf d_scratch;
  int dev_rows = 0;
  bool dev_ready = false;
  int device = -1;  // the CUDA device holding d_state, d_parents and every constraint's tables

  int n_link() const { return (int)link_name.size(); }

  void ensure_device() {
    if (dev_ready) check_device(device, "the kinematic model");
    if (dev_ready && dev_rows == n_link() + 1) return;
    require_device();
    if (!dev_ready) device = current_device();
    size_t rows = n_link() + 1;
    std::vector<double> host(state_init);
    if (dev_ready && dev_rows > 0) {  // keep the current state when links were appended
      std::vector<double> old((size_t)dev_rows * PM_STATE_STRIDE);
      cuda_check(cudaMemcpy(old.data(), d_state.p, old.size() * 8, cudaMemcpyDeviceToHost), "state readback");
      std::copy(old.begin(), old.end(), host.begin());
      d_state.release();
    }
    d_state.ensure(rows * PM_STATE_STRIDE * 8);
    cuda_check(cudaMemcpy(d_state.p, host.data(), rows * PM_STATE_STRIDE * 8, cudaMemcpyHostToDevice), "state upload");
    std::vector<int32_t> par(parent.begin(), parent.end());
    d_parents.release();
    d_parents.ensure(par.size() * 4);
    cuda_check(cudaMemcpy(d_parents.p, par.data(), par.size() * 4, cudaMemcpyHostToDevice), "parents upload");
    dev_rows = (int)rows;
    dev_ready = true;
  }
};

static void set_row(std::vector<double>& st, int row, const double q[4], const double t[3], bool qid) {
  double* r = st.data() + (size_t)row * PM_STATE_STRIDE;
  r[0] = q[0];
  r[1] = q[1];
  r[2] = q[2];
  r[3] = q[3];
  r[4] = t[0];
  r[5] = t[1];
  r[6] = t[2];
  r[7] = qid ? 1.0 : 0.0;
}

// KinematicModel ctor (kinematics.cpp:183-223): stack-DFS link numbering, stack-DFS numbering
// of movable joints, local transforms from joint origins, identity flags.
static std::shared_ptr<HostModel> build_model(const std::string& xml) {
  UrdfRobot r = parse_urdf(xml);
  auto m = std::make_shared<HostModel>();
  std::map<std::string, std::vector<std::string>> child_links;
  for (auto& kv : r.child_joints)
    for (auto& jn : kv.second) child_links[kv.first].push_back(r.joints.at(jn).child);
  std::vector<std::string> order;
  std::vector<std::string> st{r.root};
  while (!st.empty()) {
    std::string l = st.back();
    st.pop_back();
    m->link_id[l] = (int)order.size();
    order.push_back(l);
    for (auto& c : child_links[l]) st.push_back(c);
  }
  int nl = (int)order.size();
  if (nl != (int)r.links.size()) fail(PMGPU_ERR_RUNTIME, "URDF: the links do not form one tree");
  m->link_name = order;
  m->parent.assign(nl, -1);
  m->children.resize(nl);
  m->consider_rotation.assign(nl, 1);
  m->link_parent_joint.assign(nl, -1);
  for (int i = 0; i < nl; i++) {
    auto pj = r.parent_joint.find(order[i]);
    if (pj != r.parent_joint.end()) m->parent[i] = m->link_id[r.joints.at(pj->second).parent];
    for (auto& c : child_links[order[i]]) m->children[i].push_back(m->link_id[c]);
  }
  m->root = 0;
  // joints (kinematics.cpp:66-145)
  std::vector<std::string> jst;
  for (auto& jn : r.child_joints[r.root]) jst.push_back(jn);
  while (!jst.empty()) {
    const UrdfJoint& j = r.joints.at(jst.back());
    jst.pop_back();
    if (j.type == UJ_REVOLUTE || j.type == UJ_CONTINUOUS || j.type == UJ_PRISMATIC) {
      HostJoint h;
      h.name = j.name;
      h.type = j.type;
      h.child = m->link_id[j.child];
      std::memcpy(h.axis, j.axis, sizeof(h.axis));
      std::memcpy(h.pos, j.xyz, sizeof(h.pos));
      std::memcpy(h.quat, j.quat, sizeof(h.quat));
      h.qid = std::abs(h.quat[3] - 1.0) < 1e-6;
      if (j.type == UJ_CONTINUOUS) {
        h.lower = -std::numeric_limits<double>::infinity();
        h.upper = std::numeric_limits<double>::infinity();
      } else {
        h.lower = j.lower;
        h.upper = j.upper;
      }
      m->joint_id[h.name] = (int)m->joints.size();
      m->link_parent_joint[h.child] = (int)m->joints.size();
      m->joints.push_back(h);
    }
    auto cj = r.child_joints.find(j.child);
    if (cj != r.child_joints.end())
      for (auto& jn : cj->second) jst.push_back(jn);
  }
  m->angles.assign(m->joints.size(), 0.0);
  // state rows: base = Transform::Identity(); links = joint origin transforms (kinematics.cpp:147-181)
  m->state_init.assign((size_t)(nl + 1) * PM_STATE_STRIDE, 0.0);
  const double qi[4] = {0, 0, 0, 1}, z3[3] = {0, 0, 0};
  set_row(m->state_init, PM_STATE_BASE_ROW, qi, z3, false);
  for (int i = 0; i < nl; i++) {
    auto pj = r.parent_joint.find(order[i]);
    if (pj == r.parent_joint.end()) {  // the root's local transform is never composed
      set_row(m->state_init, PM_STATE_LINK_ROW(i), qi, z3, false);
      continue;
    }
    const UrdfJoint& j = r.joints.at(pj->second);
    set_row(m->state_init, PM_STATE_LINK_ROW(i), j.quat, j.xyz, std::abs(j.quat[3] - 1.0) < 1e-6);
  }
  return m;
}

// ---------------------------------------------------------------------------- SDFs
static std::atomic<uint64_t> g_sdf_version{1};

struct CloudData {
  GridBuild g{};
  DevBuf d_grid;  // one PmGridDev on the device
  std::vector<double> pts;
  double radius = 0;
  double cell = 0;
  double lb[3], ub[3];
  bool built = false;
  int device = -1;  // the CUDA device holding the grid
  ~CloudData() {
    if (built) grid_free(g);
  }
};

struct HostSdf {
  int kind = PM_SDF_BOX;
  uint64_t version = 0;
  double lb[3] = {0, 0, 0}, ub[3] = {0, 0, 0};
  double pos[3] = {0, 0, 0};
  double rot[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
  double rot_inv[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
  bool axis_aligned = true, z_axis_aligned = true;
  double w[3] = {0, 0, 0};  // box width
  double r = 0, h = 0;      // cylinder / sphere radius, cylinder height, ground height
  std::vector<std::shared_ptr<HostSdf>> members;
  std::shared_ptr<CloudData> cloud;

  void touch() { version = g_sdf_version++; }
  bool transformable() const { return kind == PM_SDF_BOX || kind == PM_SDF_CYLINDER || kind == PM_SDF_SPHERE; }
  // Pose::update_alignment_flags_ and rot_.inverse() (primitive_sdf.hpp:30-68)
  void update_pose() {
    const double* R = rot;
    double cof[9];
    cof[0] = R[4] * R[8] - R[5] * R[7];
    cof[1] = R[5] * R[6] - R[3] * R[8];
    cof[2] = R[3] * R[7] - R[4] * R[6];
    cof[3] = R[2] * R[7] - R[1] * R[8];
    cof[4] = R[0] * R[8] - R[2] * R[6];
    cof[5] = R[1] * R[6] - R[0] * R[7];
    cof[6] = R[1] * R[5] - R[2] * R[4];
    cof[7] = R[2] * R[3] - R[0] * R[5];
    cof[8] = R[0] * R[4] - R[1] * R[3];
    double det = R[0] * cof[0] + R[1] * cof[1] + R[2] * cof[2];
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) rot_inv[3 * i + j] = cof[3 * j + i] / det;
    double d2 = 0, n2 = 0;
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) {
        double e = R[3 * i + j] - (i == j ? 1.0 : 0.0);
        d2 += e * e;
        n2 += R[3 * i + j] * R[3 * i + j];
      }
    axis_aligned = d2 <= 1e-12 * 1e-12 * std::min(n2, 3.0);  // Eigen isApprox with dummy_precision 1e-12
    if (axis_aligned) {
      z_axis_aligned = true;
    } else {
      const double tol = 1e-6;
      z_axis_aligned = (std::abs(R[8] - 1.0) < tol) && (std::abs(R[2]) < tol) && (std::abs(R[5]) < tol) && (std::abs(R[6]) < tol) &&
                       (std::abs(R[7]) < tol);
    }
  }
  // update_aabb (primitive_sdf.hpp:250-255, 400-421, 500-521, 558-561)
  void update_aabb() {
    if (kind == PM_SDF_BOX || kind == PM_SDF_CYLINDER) {
      double ex = kind == PM_SDF_BOX ? w[0] * 0.5 : r, ey = kind == PM_SDF_BOX ? w[1] * 0.5 : r,
             ez = kind == PM_SDF_BOX ? w[2] * 0.5 : 0.5 * h;
      const double sx[8] = {-ex, ex, -ex, ex, -ex, ex, -ex, ex};
      const double sy[8] = {-ey, -ey, ey, ey, -ey, -ey, ey, ey};
      const double sz[8] = {-ez, -ez, -ez, -ez, ez, ez, ez, ez};
      for (int k = 0; k < 8; k++) {
        double v[3];
        for (int a = 0; a < 3; a++) v[a] = (rot[3 * a] * sx[k] + (rot[3 * a + 1] * sy[k] + rot[3 * a + 2] * sz[k])) + pos[a];
        for (int a = 0; a < 3; a++) {
          if (k == 0 || v[a] < lb[a]) lb[a] = v[a];
          if (k == 0 || v[a] > ub[a]) ub[a] = v[a];
        }
      }
    } else if (kind == PM_SDF_SPHERE) {
      for (int a = 0; a < 3; a++) {
        lb[a] = pos[a] - r;
        ub[a] = pos[a] + r;
      }
    } else if (kind == PM_SDF_GROUND) {
      const double inf = std::numeric_limits<double>::infinity();
      lb[0] = lb[1] = -inf;
      ub[0] = ub[1] = inf;
      lb[2] = ub[2] = 0.0;
    }
  }
  void translate(const double* t) {
    if (kind == PM_SDF_UNION) {
      for (auto& m : members) m->translate(t);
      return;
    }
    if (kind == PM_SDF_GROUND) fail(PMGPU_ERR_RUNTIME, "GroundSDF does not support translation");
    // the reference's CloudSDF raises this very message (collision/primitive_sdf.hpp:584-607)
    if (kind == PM_SDF_CLOUD) fail(PMGPU_ERR_RUNTIME, "TODO: Not implemented yet");
    for (int a = 0; a < 3; a++) pos[a] += t[a];
    update_aabb();
    touch();
  }
  void rotate_z(double ang) {  // Pose::rotate_z (primitive_sdf.hpp:45-53)
    if (kind == PM_SDF_UNION) {
      for (auto& m : members) m->rotate_z(ang);
      return;
    }
    if (kind == PM_SDF_GROUND) fail(PMGPU_ERR_RUNTIME, "GroundSDF does not support rotation");
    if (kind == PM_SDF_CLOUD) fail(PMGPU_ERR_RUNTIME, "TODO: Not implemented yet");
    double c = std::cos(ang), s = std::sin(ang);
    const double rz[9] = {c, -s, 0, s, c, 0, 0, 0, 1};
    double nr[9];
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) nr[3 * i + j] = rz[3 * i] * rot[j] + (rz[3 * i + 1] * rot[3 + j] + rz[3 * i + 2] * rot[6 + j]);
    std::memcpy(rot, nr, sizeof(rot));
    update_pose();
    update_aabb();
    touch();
  }
  std::shared_ptr<HostSdf> clone() const {
    if (kind == PM_SDF_CLOUD) fail(PMGPU_ERR_RUNTIME, "TODO: Not implemented yet");
    auto c = std::make_shared<HostSdf>(*this);
    if (kind == PM_SDF_UNION) {
      c->members.clear();
      for (auto& m : members) c->members.push_back(m->clone());
    }
    c->touch();
    return c;
  }
  // PmPrim block of a leaf
  PmPrim to_prim(int cloud_index) const {
    PmPrim p;
    std::memset(&p, 0, sizeof(p));
    p.kind = kind;
    p.axis_aligned = axis_aligned;
    p.z_axis_aligned = z_axis_aligned;
    p.cloud = cloud_index;
    for (int a = 0; a < 3; a++) {
      p.lb[a] = lb[a];
      p.ub[a] = ub[a];
      p.pos[a] = pos[a];
    }
    std::memcpy(p.rot, rot, sizeof(p.rot));
    std::memcpy(p.rot_inv, rot_inv, sizeof(p.rot_inv));
    switch (kind) {
      case PM_SDF_BOX:
        p.a = 0.5 * w[0];
        p.b = 0.5 * w[1];
        p.c = 0.5 * w[2];
        break;
      case PM_SDF_CYLINDER:
        p.a = r;
        p.b = r * r;
        p.c = 0.5 * h;
        break;
      case PM_SDF_SPHERE:
        p.a = r;
        p.b = r * r;
        break;
      case PM_SDF_GROUND:
        p.a = h;
        break;
      case PM_SDF_CLOUD:
        p.a = cloud->radius;
        break;
    }
    return p;
  }
};

// set_all_sdfs_inner (primitive_sphere_collision.cpp:436-448)
static void flatten(const std::shared_ptr<HostSdf>& s, std::vector<std::shared_ptr<HostSdf>>& out) {
  if (s->kind == PM_SDF_UNION) {
    for (auto& m : s->members) flatten(m, out);
  } else {
    out.push_back(s);
  }
}

static void check_rotation(const double* rot) {
  for (int i = 0; i < 9; i++)
    if (!std::isfinite(rot[i])) throw std::invalid_argument("rotation matrix has non-finite entries");
}

// Device image of one SDF tree (for SDF-level evaluate / is_outside calls).
struct SdfDeviceImage {
  DevBuf prims, clouds;
  int n_prims = 0;
  int device = -1;
  std::vector<std::pair<const HostSdf*, uint64_t>> sig;
};

static void build_cloud(CloudData& cd) {
  require_device();
  cd.device = current_device();
  int64_t n = (int64_t)(cd.pts.size() / 3);
  DevBuf dpts;
  dpts.ensure(std::max<size_t>(cd.pts.size() * 8, 8));
  if (n > 0) cuda_check(cudaMemcpy(dpts.p, cd.pts.data(), cd.pts.size() * 8, cudaMemcpyHostToDevice), "cloud upload");
  double lo[3], hi[3];
  for (int a = 0; a < 3; a++) {
    lo[a] = std::numeric_limits<double>::infinity();
    hi[a] = -std::numeric_limits<double>::infinity();
  }
  for (int64_t i = 0; i < n; i++)
    for (int a = 0; a < 3; a++) {
      lo[a] = std::min(lo[a], cd.pts[3 * i + a]);
      hi[a] = std::max(hi[a], cd.pts[3 * i + a]);
    }
  double cell = cd.cell > 0 ? cd.cell : 0.012;
  double blk = cell * PM_GRID_B;
  // the grid extends the points' box by the nearest-point field's reach, so queries near the
  // cloud but outside its box still get the field's bounds
  const double pad = n > 0 ? cd.g.field_reach : 0.0;
  int nb[3];
  for (;;) {
    int64_t tot = 1;
    for (int a = 0; a < 3; a++) {
      double ext = n > 0 ? (hi[a] - lo[a]) + 2.0 * pad : 0.0;
      nb[a] = (int)std::floor(ext / blk) + 1;
      tot *= nb[a];
    }
    if (tot * PM_GRID_CELLS_PER_BLOCK <= (int64_t)64 << 20) break;  // at most 64M fine cells
    cell *= 1.25;
    blk = cell * PM_GRID_B;
  }
  GridBuild& g = cd.g;
  g.pts = dpts.as<double>();
  g.n = n;
  g.radius = cd.radius;
  g.cell = cell;
  g.dev.nbx = nb[0];
  g.dev.nby = nb[1];
  g.dev.nbz = nb[2];
  for (int a = 0; a < 3; a++) g.dev.origin[a] = n > 0 ? lo[a] - pad : 0.0;
  g.dev.block = blk;
  g.dev.radius = cd.radius;
  for (int a = 0; a < 3; a++) {
    g.dev.lb[a] = cd.lb[a];
    g.dev.ub[a] = cd.ub[a];
  }
  cuda_check(grid_build(g, 0), "cloud grid build");
  cd.built = true;
  cd.cell = cell;
  cd.d_grid.ensure(sizeof(PmGridDev));
  cuda_check(cudaMemcpy(cd.d_grid.p, &g.dev, sizeof(PmGridDev), cudaMemcpyHostToDevice), "grid descriptor upload");
}
// The grid of a cloud, built on first use; later uses must come from the same device.
static void use_cloud(CloudData& cd) {
  if (!cd.built)
    build_cloud(cd);
  else
    check_device(cd.device, "a CloudSDF's grid");
}

// ---------------------------------------------------------------------------- SphereCollisionCst
struct HostGroup {
  std::string link_name;
  int link = 0;
  std::vector<std::array<double, 3>> rel;
  std::vector<double> radii;
  double radius = 0;
  std::array<double, 3> centre{0, 0, 0};
  bool only_self = false;
};

// reorder_spheres_for_informative_collision_check (primitive_sphere_collision.cpp:53-96); the
// unvisited set is walked in libstdc++ unordered_set order, i.e. descending index.
static std::vector<size_t> farthest_order(const std::vector<std::array<double, 3>>& pos) {
  size_t n = pos.size();
  std::vector<size_t> visited;
  if (n == 0) return visited;
  std::vector<size_t> unvisited;
  for (size_t i = n; i-- > 0;) unvisited.push_back(i);
  visited.push_back(unvisited.front());
  unvisited.erase(unvisited.begin());
  auto nrm = [](const std::array<double, 3>& a, const std::array<double, 3>& b) {
    double d0 = a[0] - b[0], d1 = a[1] - b[1], d2 = a[2] - b[2];
    return std::sqrt(d0 * d0 + (d1 * d1 + d2 * d2));
  };
  for (size_t it = 0; it + 1 < n; it++) {
    double max_dist = 0.0;
    size_t best = 0;
    for (size_t k = 0; k < unvisited.size(); k++) {
      double md = std::numeric_limits<double>::max();
      for (size_t vv : visited) {
        double d = nrm(pos[unvisited[k]], pos[vv]);
        if (d < md) md = d;
      }
      if (md > max_dist) {
        max_dist = md;
        best = k;
      }
    }
    visited.push_back(unvisited[best]);
    unvisited.erase(unvisited.begin() + best);
  }
  return visited;
}

// Two-stream pipeline of a host-memory fast call: chunk i runs on stream i % 2 (the caller's stream,
// or an internal non-blocking one) with buffer set i % 2, so each chunk's copies overlap the
// neighbouring chunks' kernels.  Chunks on the same stream run in order, so a buffer set is reused
// only after the chunk before it on that stream has finished.
struct FastPipe {
  cudaStream_t aux = nullptr;
  cudaEvent_t ev_in = nullptr, ev_out = nullptr;
  DevBuf in[2], out[2], dist[2], items[2], hq[2];
  DevBuf ctl, ovf;  // per chunk counters (64 B each) and per-config overflow flags, for the whole call
  FastPipe() = default;
  FastPipe(const FastPipe&) = delete;
  FastPipe& operator=(const FastPipe&) = delete;
  ~FastPipe() {
    if (ev_in) cudaEventDestroy(ev_in);
    if (ev_out) cudaEventDestroy(ev_out);
    if (aux) cudaStreamDestroy(aux);
  }
  void init() {
    if (aux) return;
    cuda_check(cudaStreamCreateWithFlags(&aux, cudaStreamNonBlocking), "stream");
    cuda_check(cudaEventCreateWithFlags(&ev_in, cudaEventDisableTiming), "event");
    cuda_check(cudaEventCreateWithFlags(&ev_out, cudaEventDisableTiming), "event");
  }
};

struct HostCst {
  std::shared_ptr<HostModel> kin;
  std::vector<int> ids;
  int base_type = PM_BASE_FIXED;
  std::vector<HostGroup> groups;
  std::vector<std::pair<int, int>> pairs;
  std::shared_ptr<HostSdf> fixed_sdf, sdf;
  // device tables and their signature
  DevBuf d_tables;
  std::vector<std::pair<const HostSdf*, uint64_t>> sig;
  uint64_t sig_model_version = 0;
  std::vector<std::shared_ptr<HostSdf>> flat;
  PmTablesHdr hdr{};  // host copy of the device table header
  int fast_cpb = 32;  // configurations per block of the fast kernel
  int fast_nt = 256;  // threads per block of the fast kernel
  FastTuning tune;    // the fast kernels' other autotuned parameters
  int edge_cpb = 32, edge_nt = 128;  // waypoints and threads per block of the edge kernel
  std::vector<int> slot_of_link;
  std::vector<PmSlot> ctrl_recs;  // per control joint (child link, REV/PRIS) for state updates
  DevBuf d_ctrl_recs;
  // workspaces for host-memory calls
  DevBuf w_in, w_in2, w_out, w_out2, w_aux, w_seq, w_width;
  DevBuf f_items, f_ctl, f_overflow;  // fast-path recheck queue, counters, per-config overflow flags
  DevBuf f_hq;                        // fast-path hard cloud queries (distances mode)
  PinBuf h_pin;                       // pinned staging of small host-memory calls
  DevBuf w_cen;                       // sphere centres of a device-memory distances call without centres
  FastPipe pipe;                      // host-memory fast calls of large batches
  DevBuf e_sr, e_n, e_off;            // fast edge path: step ratios, waypoint counts and offsets
  DevBuf g_wp;                        // trajectory costs: per-waypoint partial costs
  std::vector<int16_t> seq_host;
  std::vector<int> extra_links;  // links a pose term needs that no sphere chain reaches
  DevBuf d_bnd;                       // a composite call's link-position bounds, as last uploaded
  std::vector<PmPoseTerm> bnd_up;     // their host copy (re-uploaded when they change)

  // FK slot of `link`; the link (and its ancestors) joins the tables if it is not there yet.
  int slot_for_link(int link) {
    if (link < 0 || link >= kin->n_link()) fail(PMGPU_ERR_INVALID, "link id out of range");
    tables();
    if (slot_of_link[link] < 0) {
      extra_links.push_back(link);
      d_tables.release();
      tables();
    }
    return slot_of_link[link];
  }

  int q_dim() const { return (int)ids.size() + (base_type == PM_BASE_FLOATING) * 6 + (base_type == PM_BASE_PLANAR) * 3; }
  int n_spheres() const {
    int n = 0;
    for (auto& g : groups) n += (int)g.radii.size();
    return n;
  }
  int cst_dim() {
    std::vector<std::shared_ptr<HostSdf>> f;
    if (fixed_sdf) flatten(fixed_sdf, f);
    if (sdf) flatten(sdf, f);
    return (f.empty() ? 0 : 1) + (pairs.empty() ? 0 : 1);
  }

  const PmTablesHdr* tables() {
    kin->ensure_device();
    std::vector<std::shared_ptr<HostSdf>> f;
    if (fixed_sdf) flatten(fixed_sdf, f);
    if (sdf) flatten(sdf, f);
    std::vector<std::pair<const HostSdf*, uint64_t>> s;
    for (auto& x : f) s.push_back({x.get(), x->version});
    if (d_tables.p && s == sig && sig_model_version == kin->version) return d_tables.as<PmTablesHdr>();
    flat = f;
    build_tables();
    sig = s;
    sig_model_version = kin->version;
    return d_tables.as<PmTablesHdr>();
  }

  // The fast kernels' two-thread FK: the trunk (the slots up to the first one with two children,
  // and every slot outside the subtrees below it) in phase 0 by thread 0; then the subtrees of the
  // branching slot's children in phase 1, spread over the two threads by size (largest first onto
  // the lighter thread).  A slot's parent is then computed earlier by the same thread or in phase 0.
  // Without a branching slot everything is phase 0, thread 0.
  static void split_slots(std::vector<PmSlot>& slots) {
    const int n = (int)slots.size();
    std::vector<std::vector<int>> kids(n);
    for (int i = 0; i < n; i++)
      if (slots[i].parent >= 0) kids[slots[i].parent].push_back(i);
    int br = -1;
    for (int i = 0; i < n && br < 0; i++)
      if (kids[i].size() >= 2) br = i;
    for (auto& s : slots) s.split = 0;
    if (br < 0) return;
    std::vector<int> size(n, 1);
    for (int i = n - 1; i >= 0; i--)  // parents come first: children's sizes are final here
      if (slots[i].parent >= 0) size[slots[i].parent] += size[i];
    std::vector<int> order = kids[br];
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return size[a] > size[b]; });
    int load[2] = {0, 0};
    std::vector<int> owner(n, -1);
    for (int c : order) {
      const int t = load[1] < load[0] ? 1 : 0;
      load[t] += size[c];
      owner[c] = t;
    }
    for (int i = 0; i < n; i++) {  // a slot inherits its subtree root's thread
      const int p = slots[i].parent;
      if (owner[i] < 0 && p >= 0 && owner[p] >= 0) owner[i] = owner[p];
      slots[i].split = owner[i] < 0 ? 0 : (2 | owner[i]);
    }
  }

  void build_tables() {
    HostModel& m = *kin;
    const int nl = m.n_link();
    // links the constraint touches: sphere links and all their ancestors (+ root)
    std::vector<char> need(nl, 0);
    need[m.root] = 1;
    for (auto& g : groups)
      for (int l = g.link; l >= 0; l = m.parent[l]) need[l] = 1;
    for (int e : extra_links)
      for (int l = e; l >= 0; l = m.parent[l]) need[l] = 1;
    std::vector<int> links;
    for (int l = 0; l < nl; l++)
      if (need[l]) links.push_back(l);  // DFS numbering puts parents before children
    if ((int)links.size() > PM_MAX_SLOTS)
      fail(PMGPU_ERR_INVALID, "constraint touches " + std::to_string(links.size()) + " links; the device limit is " +
                                  std::to_string(PM_MAX_SLOTS));
    if ((int)ids.size() > PM_MAX_CTRL) fail(PMGPU_ERR_INVALID, "more than 64 control joints");
    slot_of_link.assign(nl, -1);
    for (size_t i = 0; i < links.size(); i++) slot_of_link[links[i]] = (int)i;
    // which control column drives each link (the last occurrence wins, as in set_joint_angles)
    std::vector<int> ctrl_col(nl, -1);
    for (size_t i = 0; i < ids.size(); i++) ctrl_col[m.joints[ids[i]].child] = (int)i;
    // subtree membership for the relevance table (kinematics.cpp:340-363)
    auto in_subtree = [&](int link, int top) {
      for (int l = link; l >= 0; l = m.parent[l])
        if (l == top) return true;
      return false;
    };
    std::vector<PmSlot> slots(links.size());
    for (size_t i = 0; i < links.size(); i++) {
      PmSlot& s = slots[i];
      std::memset(&s, 0, sizeof(s));
      int l = links[i];
      s.link = l;
      s.parent = m.parent[l] < 0 ? -1 : slot_of_link[m.parent[l]];
      s.mode = PM_FK_STATE;
      s.qcol = -1;
      if (ctrl_col[l] >= 0) {
        const HostJoint& j = m.joints[ids[ctrl_col[l]]];
        s.mode = j.type == UJ_PRISMATIC ? PM_FK_PRIS : PM_FK_REV;
        s.qcol = ctrl_col[l];
        s.origin_identity = j.qid;
        std::memcpy(s.axis, j.axis, sizeof(s.axis));
        std::memcpy(s.oq, j.quat, sizeof(s.oq));
        std::memcpy(s.ot, j.pos, sizeof(s.ot));
      }
      uint64_t rel = 0;
      for (size_t c = 0; c < ids.size(); c++)
        if (in_subtree(l, m.joints[ids[c]].child)) rel |= (1ull << c);
      s.relevant = rel;
    }
    split_slots(slots);
    std::vector<PmJoint> jrec(ids.size());
    for (size_t c = 0; c < ids.size(); c++) {
      const HostJoint& j = m.joints[ids[c]];
      jrec[c].slot = slot_of_link[j.child];
      jrec[c].prismatic = j.type == UJ_PRISMATIC;
      std::memcpy(jrec[c].axis, j.axis, sizeof(jrec[c].axis));
    }
    std::vector<PmGroup> grec(groups.size());
    std::vector<double> sx, sy, sz, sr;
    std::vector<int32_t> sgroup;
    for (size_t g = 0; g < groups.size(); g++) {
      const HostGroup& G = groups[g];
      grec[g].slot = slot_of_link[G.link];
      grec[g].begin = (int)sx.size();
      grec[g].count = (int)G.radii.size();
      grec[g].only_self = G.only_self;
      for (int a = 0; a < 3; a++) grec[g].rel[a] = G.centre[a];
      grec[g].radius = G.radius;
      for (size_t k = 0; k < G.radii.size(); k++) {
        sx.push_back(G.rel[k][0]);
        sy.push_back(G.rel[k][1]);
        sz.push_back(G.rel[k][2]);
        sr.push_back(G.radii[k]);
        sgroup.push_back((int)g);
      }
    }
    std::vector<int32_t> prs;
    for (auto& p : pairs) {
      prs.push_back(p.first);
      prs.push_back(p.second);
    }
    std::vector<PmPrim> prims;
    std::vector<PmGridDev> clouds;
    for (auto& x : flat) {
      int ci = -1;
      if (x->kind == PM_SDF_CLOUD) {
        use_cloud(*x->cloud);
        ci = (int)clouds.size();
        clouds.push_back(x->cloud->g.dev);
      }
      prims.push_back(x->to_prim(ci));
    }
    // pack
    PmTablesHdr h;
    std::memset(&h, 0, sizeof(h));
    h.n_slots = (int)slots.size();
    h.n_ctrl = (int)ids.size();
    h.n_groups = (int)grec.size();
    h.n_spheres = (int)sr.size();
    h.n_pairs = (int)pairs.size();
    h.n_prims = (int)prims.size();
    h.q_dim = q_dim();
    h.base_type = base_type;
    h.root_slot = slot_of_link[m.root];
    h.n_clouds = (int)clouds.size();
    std::vector<char> buf;
    auto align = [&]() {
      while (buf.size() % 16) buf.push_back(0);
    };
    auto put = [&](const void* p, size_t bytes) -> int64_t {
      align();
      int64_t off = (int64_t)buf.size();
      buf.insert(buf.end(), (const char*)p, (const char*)p + bytes);
      return off;
    };
    buf.resize(sizeof(PmTablesHdr));
    h.off_slots = put(slots.data(), slots.size() * sizeof(PmSlot));
    h.off_joints = put(jrec.data(), jrec.size() * sizeof(PmJoint));
    h.off_groups = put(grec.data(), grec.size() * sizeof(PmGroup));
    h.off_sx = put(sx.data(), sx.size() * 8);
    h.off_sy = put(sy.data(), sy.size() * 8);
    h.off_sz = put(sz.data(), sz.size() * 8);
    h.off_sr = put(sr.data(), sr.size() * 8);
    h.off_sgroup = put(sgroup.data(), sgroup.size() * 4);
    h.off_pairs = put(prs.data(), prs.size() * 4);
    h.off_prims = put(prims.data(), prims.size() * sizeof(PmPrim));
    h.off_clouds = put(clouds.data(), clouds.size() * sizeof(PmGridDev));
    align();
    h.total_bytes = (int64_t)buf.size();
    std::memcpy(buf.data(), &h, sizeof(h));
    hdr = h;
    d_tables.release();
    d_tables.ensure(buf.size());
    cuda_check(cudaMemcpy(d_tables.p, buf.data(), buf.size(), cudaMemcpyHostToDevice), "tables upload");
    // control joint records for update_kintree
    ctrl_recs.resize(ids.size());
    for (size_t c = 0; c < ids.size(); c++) {
      const HostJoint& j = m.joints[ids[c]];
      PmSlot& s = ctrl_recs[c];
      std::memset(&s, 0, sizeof(s));
      s.link = j.child;
      s.mode = j.type == UJ_PRISMATIC ? PM_FK_PRIS : PM_FK_REV;
      s.origin_identity = j.qid;
      std::memcpy(s.axis, j.axis, sizeof(s.axis));
      std::memcpy(s.oq, j.quat, sizeof(s.oq));
      std::memcpy(s.ot, j.pos, sizeof(s.ot));
    }
    d_ctrl_recs.release();
    d_ctrl_recs.ensure(std::max<size_t>(ctrl_recs.size(), 1) * sizeof(PmSlot));
    if (!ctrl_recs.empty())
      cuda_check(cudaMemcpy(d_ctrl_recs.p, ctrl_recs.data(), ctrl_recs.size() * sizeof(PmSlot), cudaMemcpyHostToDevice),
                 "control records upload");
  }

  const int16_t* seq_table() {
    if (!w_seq.p) {
      // find_farthest_sequence_fast (ompl/generate_sequence.py:11-63), 128 x 128
      seq_host.assign(128 * 128, 0);
      for (int n = 1; n <= 128; n++) {
        std::vector<int> res(n, 0);
        std::vector<char> used(n, 0);
        used[0] = 1;
        for (int i = 1; i < n; i++) {
          int best_md = -1, best = -1;
          for (int num = 0; num < n; num++) {
            if (used[num]) continue;
            int md = std::numeric_limits<int>::max();
            for (int j = 0; j < i; j++) md = std::min(md, std::abs(num - res[j]));
            if (md > best_md || (md == best_md && num > best)) {
              best_md = md;
              best = num;
            }
          }
          res[i] = best;
          used[best] = 1;
        }
        for (int j = 0; j < n; j++) seq_host[(n - 1) * 128 + j] = (int16_t)res[j];
      }
      w_seq.ensure(seq_host.size() * 2);
      cuda_check(cudaMemcpy(w_seq.p, seq_host.data(), seq_host.size() * 2, cudaMemcpyHostToDevice), "sequence upload");
    }
    return w_seq.as<int16_t>();
  }
};

// Device view of a constraint whose tables and model state already live on the device
// (built by an earlier batch call); false instead of building them.  Allocates nothing.
bool cst_device_view(pmgpu_cst* c, const PmTablesHdr** T, PmTablesHdr* hdr, const double** state, int* cpb, int* nt);

}  // namespace pmg

// ============================================================================ C ABI
using namespace pmg;

struct pmgpu_model {
  std::shared_ptr<HostModel> m;
};
struct pmgpu_sdf {
  std::shared_ptr<HostSdf> s;
  SdfDeviceImage img;
};
struct pmgpu_cst {
  HostCst c;
};

namespace {

cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

void check_mem(int mem) {
  if (mem != PMGPU_MEM_HOST && mem != PMGPU_MEM_DEVICE) throw std::invalid_argument("mem must be PMGPU_MEM_HOST or PMGPU_MEM_DEVICE");
}
void check_ptr(const void* p, const char* what) {
  if (!p) throw std::invalid_argument(std::string(what) + " is NULL");
}
// A required array of a batch call: NULL is refused unless the batch is empty (in device memory a
// NULL array would fault the kernel that reads it; in host memory, the copy).
void check_arr(const void* p, int64_t n, const char* what) {
  if (n > 0 && !p) throw std::invalid_argument(std::string(what) + " is NULL");
}

// Device image of an SDF tree for SDF-level calls
const PmPrim* sdf_image(pmgpu_sdf* h, int* n_prims, const PmGridDev** clouds) {
  std::vector<std::shared_ptr<HostSdf>> f;
  flatten(h->s, f);
  std::vector<std::pair<const HostSdf*, uint64_t>> sig;
  for (auto& x : f) sig.push_back({x.get(), x->version});
  if (h->img.prims.p) check_device(h->img.device, "this SDF");
  if (!h->img.prims.p || sig != h->img.sig) {
    require_device();
    h->img.device = current_device();
    std::vector<PmPrim> prims;
    std::vector<PmGridDev> cl;
    for (auto& x : f) {
      int ci = -1;
      if (x->kind == PM_SDF_CLOUD) {
        use_cloud(*x->cloud);
        ci = (int)cl.size();
        cl.push_back(x->cloud->g.dev);
      }
      prims.push_back(x->to_prim(ci));
    }
    h->img.prims.release();
    h->img.prims.ensure(std::max<size_t>(prims.size(), 1) * sizeof(PmPrim));
    if (!prims.empty()) cuda_check(cudaMemcpy(h->img.prims.p, prims.data(), prims.size() * sizeof(PmPrim), cudaMemcpyHostToDevice), "sdf upload");
    h->img.clouds.release();
    h->img.clouds.ensure(std::max<size_t>(cl.size(), 1) * sizeof(PmGridDev));
    if (!cl.empty()) cuda_check(cudaMemcpy(h->img.clouds.p, cl.data(), cl.size() * sizeof(PmGridDev), cudaMemcpyHostToDevice), "sdf upload");
    h->img.n_prims = (int)prims.size();
    h->img.sig = sig;
  }
  *n_prims = h->img.n_prims;
  *clouds = h->img.clouds.as<PmGridDev>();
  return h->img.prims.as<PmPrim>();
}

// Host-memory staging: copies `bytes` from host to a workspace buffer, returns device ptr
template <class T>
T* stage_in(DevBuf& buf, const T* host, size_t count, cudaStream_t s) {
  T* d = reinterpret_cast<T*>(buf.ensure(std::max<size_t>(count * sizeof(T), 16)));
  if (count) cuda_check(cudaMemcpyAsync(d, host, count * sizeof(T), cudaMemcpyHostToDevice, s), "H2D copy");
  return d;
}
template <class T>
void stage_out(T* host, const T* dev, size_t count, cudaStream_t s) {
  if (count) cuda_check(cudaMemcpyAsync(host, dev, count * sizeof(T), cudaMemcpyDeviceToHost, s), "D2H copy");
}

GradArgs grad_args(HostCst& C, const pmgpu_cost_params* p, bool want_pose) {
  GradArgs a;
  std::memset(&a, 0, sizeof(a));
  a.mode = p ? p->mode : PMGPU_COST_SUM;
  if (a.mode != PMGPU_COST_SUM && a.mode != PMGPU_COST_MIN_DISTANCE) fail(PMGPU_ERR_INVALID, "unknown cost mode");
  a.w_pos = p ? p->w_pos : 1.0f;
  a.w_rot = p ? p->w_rot : 0.1f;
  a.w_col = p ? p->w_col : 1.0f;
  a.margin = p ? p->margin : 0.02f;
  a.cutoff = p ? p->cutoff : 0.1f;
  a.w_smooth = p ? p->w_smooth : 1.0f;
  for (float v : {a.w_pos, a.w_rot, a.w_col, a.margin, a.cutoff, a.w_smooth})
    if (!std::isfinite(v)) fail(PMGPU_ERR_INVALID, "cost parameters must be finite");
  const int d = C.q_dim();
  if (d > PM_GRAD_MAXQ) fail(PMGPU_ERR_INVALID, "q_dim above the cost kernels' limit");
  for (int j = 0; j < PM_GRAD_MAXQ; j++) {
    const float w = (p && p->dof_weights && j < d) ? p->dof_weights[j] : 1.0f;
    a.dofw2[j] = w * w;
    a.lo[j] = -INFINITY;
    a.hi[j] = INFINITY;
  }
  for (size_t c = 0; c < C.ids.size(); c++) {
    a.lo[c] = (float)C.kin->joints[C.ids[c]].lower;
    a.hi[c] = (float)C.kin->joints[C.ids[c]].upper;
  }
  a.pose_slot = -1;
  if (want_pose && p && p->pose_link >= 0 && a.mode == PMGPU_COST_SUM) a.pose_slot = C.slot_for_link(p->pose_link);
  return a;
}

void check_joint_ids(const HostModel& m, const int64_t* ids, int n) {
  for (int i = 0; i < n; i++)
    if (ids[i] < 0 || ids[i] >= (int64_t)m.joints.size()) throw std::invalid_argument("joint id out of range");
}

}  // namespace

extern "C" {

const char* pmgpu_last_error(void) { return g_last_error.c_str(); }
int pmgpu_version(void) { return 100; }
int pmgpu_device_count(void) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return n;
}

// ---------------------------------------------------------------- model
int pmgpu_model_create(const char* urdf_xml, pmgpu_model** out) {
  return guarded([&] {
    check_ptr(urdf_xml, "urdf_xml");
    check_ptr(out, "out");
    auto* h = new pmgpu_model();
    try {
      h->m = build_model(urdf_xml);
    } catch (...) {
      delete h;
      throw;
    }
    *out = h;
  });
}
void pmgpu_model_destroy(pmgpu_model* m) { delete m; }
int pmgpu_model_counts(const pmgpu_model* m, int* n_links, int* n_joints, int* root_link) {
  return guarded([&] {
    check_ptr(m, "model");
    if (n_links) *n_links = m->m->n_link();
    if (n_joints) *n_joints = (int)m->m->joints.size();
    if (root_link) *root_link = m->m->root;
  });
}
int pmgpu_model_get_joint_ids(const pmgpu_model* m, const char* const* names, int n, int64_t* ids_out) {
  return guarded([&] {
    check_ptr(m, "model");
    for (int i = 0; i < n; i++) {
      auto it = m->m->joint_id.find(names[i]);
      if (it == m->m->joint_id.end()) throw std::invalid_argument(std::string("no joint named ") + names[i]);
      ids_out[i] = it->second;
    }
  });
}
int pmgpu_model_get_link_ids(const pmgpu_model* m, const char* const* names, int n, int64_t* ids_out) {
  return guarded([&] {
    check_ptr(m, "model");
    for (int i = 0; i < n; i++) {
      auto it = m->m->link_id.find(names[i]);
      if (it == m->m->link_id.end()) throw std::invalid_argument(std::string("no link named ") + names[i]);
      ids_out[i] = it->second;
    }
  });
}
int pmgpu_model_get_joint_position_limits(const pmgpu_model* m, const int64_t* ids, int n, double* lower, double* upper) {
  return guarded([&] {
    check_ptr(m, "model");
    check_joint_ids(*m->m, ids, n);
    for (int i = 0; i < n; i++) {
      lower[i] = m->m->joints[ids[i]].lower;
      upper[i] = m->m->joints[ids[i]].upper;
    }
  });
}
int pmgpu_model_link_name(const pmgpu_model* m, int64_t id, char* buf, int cap) {
  return guarded([&] {
    check_ptr(m, "model");
    if (id < 0 || id >= m->m->n_link()) throw std::invalid_argument("link id out of range");
    std::snprintf(buf, (size_t)cap, "%s", m->m->link_name[id].c_str());
  });
}
int pmgpu_model_joint_name(const pmgpu_model* m, int64_t id, char* buf, int cap) {
  return guarded([&] {
    check_ptr(m, "model");
    if (id < 0 || id >= (int64_t)m->m->joints.size()) throw std::invalid_argument("joint id out of range");
    std::snprintf(buf, (size_t)cap, "%s", m->m->joints[id].name.c_str());
  });
}
int pmgpu_model_structure(const pmgpu_model* m, int32_t* link_parent, double* link_tf7, int32_t* link_tf_qid, int32_t* joint_child,
                          int32_t* joint_type, double* joint_axis3, int32_t* joint_origin_qid) {
  return guarded([&] {
    check_ptr(m, "model");
    const HostModel& M = *m->m;
    for (int l = 0; l < M.n_link(); l++) {
      if (link_parent) link_parent[l] = M.parent[l];
      const double* r = M.state_init.data() + (size_t)PM_STATE_LINK_ROW(l) * PM_STATE_STRIDE;
      if (link_tf7) {
        double v[7] = {r[4], r[5], r[6], r[0], r[1], r[2], r[3]};
        std::memcpy(link_tf7 + 7 * l, v, sizeof(v));
      }
      if (link_tf_qid) link_tf_qid[l] = r[7] != 0.0;
    }
    for (size_t j = 0; j < M.joints.size(); j++) {
      if (joint_child) joint_child[j] = M.joints[j].child;
      if (joint_type) joint_type[j] = M.joints[j].type;
      if (joint_axis3) std::memcpy(joint_axis3 + 3 * j, M.joints[j].axis, 24);
      if (joint_origin_qid) joint_origin_qid[j] = M.joints[j].qid;
    }
  });
}
int pmgpu_model_set_joint_positions(pmgpu_model* m, const int64_t* ids, int n, const double* q, int accurate) {
  return guarded([&] {
    check_ptr(m, "model");
    HostModel& M = *m->m;
    check_joint_ids(M, ids, n);
    M.ensure_device();
    std::vector<PmSlot> recs(n);
    for (int i = 0; i < n; i++) {
      const HostJoint& j = M.joints[ids[i]];
      PmSlot& s = recs[i];
      std::memset(&s, 0, sizeof(s));
      s.link = j.child;
      s.mode = j.type == UJ_PRISMATIC ? PM_FK_PRIS : PM_FK_REV;
      s.origin_identity = j.qid;
      std::memcpy(s.axis, j.axis, 24);
      std::memcpy(s.oq, j.quat, 32);
      std::memcpy(s.ot, j.pos, 24);
      M.angles[ids[i]] = q[i];
    }
    if (n == 0) return;
    size_t rb = recs.size() * sizeof(PmSlot);
    char* d = (char*)M.d_scratch.ensure(rb + (size_t)n * 8 + 64);
    cuda_check(cudaMemcpy(d, recs.data(), rb, cudaMemcpyHostToDevice), "H2D");
    double* dq = (double*)(d + ((rb + 15) / 16) * 16);
    cuda_check(cudaMemcpy(dq, q, (size_t)n * 8, cudaMemcpyHostToDevice), "H2D");
    cuda_check(launch_set_joints(M.d_state.as<double>(), (const PmSlot*)d, dq, n, accurate, 0), "set joints");
    cuda_check(cudaDeviceSynchronize(), "set joints");
  });
}
int pmgpu_model_get_joint_positions(const pmgpu_model* m, const int64_t* ids, int n, double* q) {
  return guarded([&] {
    check_ptr(m, "model");
    check_joint_ids(*m->m, ids, n);
    for (int i = 0; i < n; i++) q[i] = m->m->angles[ids[i]];
  });
}
int pmgpu_model_set_base_pose(pmgpu_model* m, const double* pose7) {
  return guarded([&] {
    check_ptr(m, "model");
    HostModel& M = *m->m;
    std::memcpy(M.base7, pose7, sizeof(M.base7));
    const double q[4] = {pose7[3], pose7[4], pose7[5], pose7[6]}, t[3] = {pose7[0], pose7[1], pose7[2]};
    set_row(M.state_init, PM_STATE_BASE_ROW, q, t, false);
    if (M.dev_ready) {
      double row[PM_STATE_STRIDE] = {q[0], q[1], q[2], q[3], t[0], t[1], t[2], 0.0};
      cuda_check(cudaMemcpy(M.d_state.p, row, sizeof(row), cudaMemcpyHostToDevice), "base pose upload");
    }
  });
}
int pmgpu_model_get_base_pose(const pmgpu_model* m, double* pose7) {
  return guarded([&] {
    check_ptr(m, "model");
    const HostModel& M = *m->m;
    if (M.dev_ready) {
      double row[PM_STATE_STRIDE];
      cuda_check(cudaMemcpy(row, M.d_state.p, sizeof(row), cudaMemcpyDeviceToHost), "base pose readback");
      double v[7] = {row[4], row[5], row[6], row[0], row[1], row[2], row[3]};
      std::memcpy(pose7, v, sizeof(v));
    } else {
      std::memcpy(pose7, M.base7, sizeof(M.base7));
    }
  });
}
int pmgpu_model_link_poses(pmgpu_model* m, const int64_t* link_ids, int n, double* out7) {
  return guarded([&] {
    check_ptr(m, "model");
    HostModel& M = *m->m;
    for (int i = 0; i < n; i++)
      if (link_ids[i] < 0 || link_ids[i] >= M.n_link()) throw std::invalid_argument("link id out of range");
    M.ensure_device();
    if (n == 0) return;
    std::vector<int32_t> l32(link_ids, link_ids + n);
    char* d = (char*)M.d_scratch.ensure((size_t)n * 4 + (size_t)n * 56 + 64);
    double* dout = (double*)(d + (((size_t)n * 4 + 15) / 16) * 16);
    cuda_check(cudaMemcpy(d, l32.data(), (size_t)n * 4, cudaMemcpyHostToDevice), "H2D");
    cuda_check(launch_link_poses(M.d_state.as<double>(), M.d_parents.as<int32_t>(), (const int32_t*)d, n, dout, 0), "link poses");
    cuda_check(cudaMemcpy(out7, dout, (size_t)n * 56, cudaMemcpyDeviceToHost), "D2H");
  });
}
int pmgpu_model_add_new_link(pmgpu_model* m, const char* name, const char* parent, const double* xyz, const double* rpy,
                             int consider_rotation, int64_t* id_out) {
  return guarded([&] {
    check_ptr(m, "model");
    HostModel& M = *m->m;
    auto pit = M.link_id.find(parent);
    if (pit == M.link_id.end()) throw std::invalid_argument(std::string("no link named ") + parent);
    if (M.link_id.count(name)) fail(PMGPU_ERR_RUNTIME, std::string("link name : ") + name + " already exists");
    int id = M.n_link();
    M.link_id[name] = id;
    M.link_name.push_back(name);
    M.parent.push_back(pit->second);
    M.children.push_back({});
    M.children[pit->second].push_back(id);
    M.consider_rotation.push_back(consider_rotation ? 1 : 0);
    M.link_parent_joint.push_back(-1);
    double q[4];
    quat_from_rpy(rpy[0], rpy[1], rpy[2], q);
    const double qi[4] = {0, 0, 0, 1};
    M.state_init.resize((size_t)(id + 2) * PM_STATE_STRIDE, 0.0);
    // consider_rotation=false keeps only the translation (algorithm.cpp:164-178)
    if (consider_rotation)
      set_row(M.state_init, PM_STATE_LINK_ROW(id), q, xyz, false);
    else
      set_row(M.state_init, PM_STATE_LINK_ROW(id), qi, xyz, true);
    M.version++;
    // a model already on the device grows there: ensure_device() sees the new row count, keeps the
    // current state of the existing rows and uploads the appended row from state_init
    if (M.dev_ready) M.ensure_device();
    if (id_out) *id_out = id;
  });
}

// ---------------------------------------------------------------- SDFs
int pmgpu_pose_flags(const double* rot9, int* axis_aligned, int* z_axis_aligned, double* rot_inv9) {
  return guarded([&] {
    check_ptr(rot9, "rotation");
    check_rotation(rot9);
    HostSdf tmp;
    std::memcpy(tmp.rot, rot9, 72);
    tmp.update_pose();
    if (axis_aligned) *axis_aligned = tmp.axis_aligned;
    if (z_axis_aligned) *z_axis_aligned = tmp.z_axis_aligned;
    if (rot_inv9) std::memcpy(rot_inv9, tmp.rot_inv, 72);
  });
}
static pmgpu_sdf* wrap(std::shared_ptr<HostSdf> s) {
  auto* h = new pmgpu_sdf();
  h->s = std::move(s);
  return h;
}
int pmgpu_sdf_box_create(const double* width3, const double* pos3, const double* rot9, pmgpu_sdf** out) {
  return guarded([&] {
    check_rotation(rot9);
    auto s = std::make_shared<HostSdf>();
    s->kind = PM_SDF_BOX;
    std::memcpy(s->w, width3, 24);
    std::memcpy(s->pos, pos3, 24);
    std::memcpy(s->rot, rot9, 72);
    s->update_pose();
    s->update_aabb();
    s->touch();
    *out = wrap(s);
  });
}
int pmgpu_sdf_cylinder_create(double radius, double height, const double* pos3, const double* rot9, pmgpu_sdf** out) {
  return guarded([&] {
    check_rotation(rot9);
    auto s = std::make_shared<HostSdf>();
    s->kind = PM_SDF_CYLINDER;
    s->r = radius;
    s->h = height;
    std::memcpy(s->pos, pos3, 24);
    std::memcpy(s->rot, rot9, 72);
    s->update_pose();
    s->update_aabb();
    s->touch();
    *out = wrap(s);
  });
}
int pmgpu_sdf_sphere_create(double radius, const double* pos3, const double* rot9, pmgpu_sdf** out) {
  return guarded([&] {
    check_rotation(rot9);
    auto s = std::make_shared<HostSdf>();
    s->kind = PM_SDF_SPHERE;
    s->r = radius;
    std::memcpy(s->pos, pos3, 24);
    std::memcpy(s->rot, rot9, 72);
    s->update_pose();
    s->update_aabb();
    s->touch();
    *out = wrap(s);
  });
}
int pmgpu_sdf_ground_create(double height, pmgpu_sdf** out) {
  return guarded([&] {
    auto s = std::make_shared<HostSdf>();
    s->kind = PM_SDF_GROUND;
    s->h = height;
    s->update_aabb();
    s->touch();
    *out = wrap(s);
  });
}
int pmgpu_sdf_cloud_stats(pmgpu_sdf* sdf, int64_t* out6) {
  return guarded([&] {
    check_ptr(sdf, "sdf");
    check_ptr(out6, "out");
    if (!sdf->s || !sdf->s->cloud) throw std::invalid_argument("not a CloudSDF");
    CloudData& cd = *sdf->s->cloud;
    if (!cd.built) build_cloud(cd);
    const PmGridDev& d = cd.g.dev;
    const int64_t nblocks = (int64_t)d.nbx * d.nby * d.nbz;
    out6[0] = (int64_t)(cd.pts.size() / 3);
    out6[1] = cd.g.n_occupied;
    out6[2] = nblocks;
    out6[3] = nblocks * PM_GRID_CELLS_PER_BLOCK;
    out6[4] = cd.g.n_cand;
    out6[5] = cd.g.bytes;
  });
}

int pmgpu_sdf_cloud_create(const double* points, int64_t n, double radius, double cell_size, pmgpu_sdf** out) {
  return guarded([&] {
    if (n < 0) throw std::invalid_argument("negative point count");
    if (n > 0) check_ptr(points, "points");
    if (n > (int64_t)1 << 30) throw std::invalid_argument("cloud too large");
    auto s = std::make_shared<HostSdf>();
    s->kind = PM_SDF_CLOUD;
    auto cd = std::make_shared<CloudData>();
    cd->pts.assign(points, points + 3 * n);
    for (int64_t i = 0; i < 3 * n; i++)
      if (!std::isfinite(cd->pts[i])) throw std::invalid_argument("cloud point with a non-finite coordinate");
    cd->radius = radius;
    cd->cell = cell_size;
    // CloudSDF ctor (primitive_sdf.hpp:571-583)
    for (int a = 0; a < 3; a++) {
      cd->lb[a] = std::numeric_limits<double>::infinity();
      cd->ub[a] = -std::numeric_limits<double>::infinity();
    }
    for (int64_t i = 0; i < n; i++)
      for (int a = 0; a < 3; a++) {
        cd->lb[a] = std::min(cd->lb[a], cd->pts[3 * i + a]);
        cd->ub[a] = std::max(cd->ub[a], cd->pts[3 * i + a]);
      }
    for (int a = 0; a < 3; a++) {
      cd->lb[a] -= radius;
      cd->ub[a] += radius;
      s->lb[a] = cd->lb[a];
      s->ub[a] = cd->ub[a];
    }
    s->cloud = cd;
    s->touch();
    *out = wrap(s);
  });
}
int pmgpu_sdf_union_create(pmgpu_sdf* const* members, int n, pmgpu_sdf** out) {
  return guarded([&] {
    auto s = std::make_shared<HostSdf>();
    s->kind = PM_SDF_UNION;
    for (int i = 0; i < n; i++) {
      check_ptr(members[i], "member");
      s->members.push_back(members[i]->s);
    }
    s->touch();
    *out = wrap(s);
  });
}
int pmgpu_sdf_union_add(pmgpu_sdf* u, pmgpu_sdf* member, int clone) {
  return guarded([&] {
    check_ptr(u, "union");
    check_ptr(member, "member");
    if (u->s->kind != PM_SDF_UNION) throw std::invalid_argument("not a UnionSDF");
    u->s->members.push_back(clone ? member->s->clone() : member->s);
    u->s->touch();
  });
}
int pmgpu_sdf_clone(const pmgpu_sdf* s, pmgpu_sdf** out) {
  return guarded([&] {
    check_ptr(s, "sdf");
    *out = wrap(s->s->clone());
  });
}
void pmgpu_sdf_destroy(pmgpu_sdf* s) { delete s; }
int pmgpu_sdf_translate(pmgpu_sdf* s, const double* t3) {
  return guarded([&] {
    check_ptr(s, "sdf");
    s->s->translate(t3);
  });
}
int pmgpu_sdf_rotate_z(pmgpu_sdf* s, double angle) {
  return guarded([&] {
    check_ptr(s, "sdf");
    s->s->rotate_z(angle);
  });
}
int pmgpu_sdf_info(const pmgpu_sdf* s, int* kind, double* lb3, double* ub3, int* axis_aligned, int* z_axis_aligned, double* pos3,
                   double* rot9) {
  return guarded([&] {
    check_ptr(s, "sdf");
    const HostSdf& x = *s->s;
    if (kind) *kind = x.kind;
    if (lb3) std::memcpy(lb3, x.lb, 24);
    if (ub3) std::memcpy(ub3, x.ub, 24);
    if (axis_aligned) *axis_aligned = x.axis_aligned;
    if (z_axis_aligned) *z_axis_aligned = x.z_axis_aligned;
    if (pos3) std::memcpy(pos3, x.pos, 24);
    if (rot9) std::memcpy(rot9, x.rot, 72);
  });
}
int pmgpu_sdf_evaluate(pmgpu_sdf* s, const double* points, int64_t n, double* out, int mem, void* stream) {
  return guarded([&] {
    check_ptr(s, "sdf");
    check_mem(mem);
    if (n < 0) throw std::invalid_argument("negative count");
    check_arr(points, n, "points");
    check_arr(out, n, "out");
    int np;
    const PmGridDev* cl;
    const PmPrim* pr = sdf_image(s, &np, &cl);
    cudaStream_t st = as_stream(stream);
    if (mem == PMGPU_MEM_DEVICE) {
      cuda_check(launch_sdf_points(pr, np, cl, s->s->kind == PM_SDF_UNION, points, nullptr, n, out, nullptr, st), "sdf evaluate");
      return;
    }
    DevBuf a, b;
    const double* dp = stage_in(a, points, (size_t)n * 3, st);
    double* dout = (double*)b.ensure(std::max<size_t>((size_t)n * 8, 16));
    cuda_check(launch_sdf_points(pr, np, cl, s->s->kind == PM_SDF_UNION, dp, nullptr, n, dout, nullptr, st), "sdf evaluate");
    stage_out(out, dout, (size_t)n, st);
    cuda_check(cudaStreamSynchronize(st), "sdf evaluate");
  });
}
int pmgpu_sdf_is_outside(pmgpu_sdf* s, const double* points, const double* radii, int64_t n, uint8_t* out, int mem, void* stream) {
  return guarded([&] {
    check_ptr(s, "sdf");
    check_mem(mem);
    if (n < 0) throw std::invalid_argument("negative count");
    check_arr(points, n, "points");
    check_arr(radii, n, "radii");
    check_arr(out, n, "out");
    int np;
    const PmGridDev* cl;
    const PmPrim* pr = sdf_image(s, &np, &cl);
    cudaStream_t st = as_stream(stream);
    if (mem == PMGPU_MEM_DEVICE) {
      cuda_check(launch_sdf_points(pr, np, cl, 1, points, radii, n, nullptr, out, st), "sdf is_outside");
      return;
    }
    DevBuf a, b, c;
    const double* dp = stage_in(a, points, (size_t)n * 3, st);
    const double* dr = stage_in(b, radii, (size_t)n, st);
    uint8_t* dout = (uint8_t*)c.ensure(std::max<size_t>((size_t)n, 16));
    cuda_check(launch_sdf_points(pr, np, cl, 1, dp, dr, n, nullptr, dout, st), "sdf is_outside");
    stage_out(out, dout, (size_t)n, st);
    cuda_check(cudaStreamSynchronize(st), "sdf is_outside");
  });
}
int pmgpu_cloud_nearest(pmgpu_sdf* cloud, const double* points, int64_t n, double* sqdist, double* nearest3, int mem, void* stream) {
  return guarded([&] {
    check_ptr(cloud, "cloud");
    check_mem(mem);
    if (cloud->s->kind != PM_SDF_CLOUD) throw std::invalid_argument("not a CloudSDF");
    if (n < 0) throw std::invalid_argument("negative count");
    check_arr(points, n, "points");
    int np;
    const PmGridDev* cl;
    sdf_image(cloud, &np, &cl);
    cudaStream_t st = as_stream(stream);
    if (mem == PMGPU_MEM_DEVICE) {
      cuda_check(launch_cloud_nearest(cl, points, n, sqdist, nearest3, st), "cloud nearest");
      return;
    }
    DevBuf a, b, c;
    const double* dp = stage_in(a, points, (size_t)n * 3, st);
    double* dsq = sqdist ? (double*)b.ensure(std::max<size_t>((size_t)n * 8, 16)) : nullptr;
    double* dnr = nearest3 ? (double*)c.ensure(std::max<size_t>((size_t)n * 24, 16)) : nullptr;
    cuda_check(launch_cloud_nearest(cl, dp, n, dsq, dnr, st), "cloud nearest");
    if (sqdist) stage_out(sqdist, dsq, (size_t)n, st);
    if (nearest3) stage_out(nearest3, dnr, (size_t)n * 3, st);
    cuda_check(cudaStreamSynchronize(st), "cloud nearest");
  });
}

// ---------------------------------------------------------------- SphereCollisionCst
int pmgpu_cst_create(pmgpu_model* kin, const char* const* control_joints, int n_joints, int base_type, int n_specs,
                     const char* const* spec_links, const int32_t* counts, const double* rel_xyz, const double* radii,
                     const uint8_t* only_self, int n_pairs, const char* const* pair_a, const char* const* pair_b, pmgpu_sdf* fixed_sdf,
                     int reorder_spheres, pmgpu_cst** out) {
  return guarded([&] {
    check_ptr(kin, "kin");
    if (base_type < 0 || base_type > 2) throw std::invalid_argument("unknown base type");
    auto* h = new pmgpu_cst();
    try {
      HostCst& c = h->c;
      c.kin = kin->m;
      HostModel& M = *c.kin;
      for (int i = 0; i < n_joints; i++) {  // ConstraintBase ctor -> get_joint_ids (primitive.hpp:30-36)
        auto it = M.joint_id.find(control_joints[i]);
        if (it == M.joint_id.end()) throw std::invalid_argument(std::string("no joint named ") + control_joints[i]);
        c.ids.push_back(it->second);
      }
      c.base_type = base_type;
      size_t off = 0;
      for (int s = 0; s < n_specs; s++) {  // primitive_sphere_collision.cpp:127-160
        HostGroup g;
        g.link_name = spec_links[s];
        auto it = M.link_id.find(g.link_name);
        if (it == M.link_id.end()) throw std::invalid_argument("no link named " + g.link_name);
        g.link = it->second;
        int n = counts[s];
        if (n <= 0) throw std::invalid_argument("sphere spec with no spheres");
        double ctr[3] = {0, 0, 0};
        for (int j = 0; j < n; j++) {
          std::array<double, 3> v{rel_xyz[3 * (off + j)], rel_xyz[3 * (off + j) + 1], rel_xyz[3 * (off + j) + 2]};
          g.rel.push_back(v);
          g.radii.push_back(radii[off + j]);
          for (int a = 0; a < 3; a++) ctr[a] = ctr[a] + v[a];
        }
        for (int a = 0; a < 3; a++) g.centre[a] = ctr[a] / n;
        double md = 0.0;
        for (int j = 0; j < n; j++) {
          double d0 = g.rel[j][0] - g.centre[0], d1 = g.rel[j][1] - g.centre[1], d2 = g.rel[j][2] - g.centre[2];
          double d = std::sqrt(d0 * d0 + (d1 * d1 + d2 * d2)) + g.radii[j];
          if (d > md) md = d;
        }
        g.radius = md;
        g.only_self = only_self ? only_self[s] != 0 : false;
        off += n;
        c.groups.push_back(g);
        if (reorder_spheres) {  // re-applied to every group so far, as the constructor loop does
          for (auto& gg : c.groups) {
            auto ord = farthest_order(gg.rel);
            std::vector<std::array<double, 3>> r2(gg.rel.size());
            std::vector<double> rad2(gg.rel.size());
            for (size_t i = 0; i < ord.size(); i++) {
              r2[i] = gg.rel[ord[i]];
              rad2[i] = gg.radii[ord[i]];
            }
            gg.rel = r2;
            gg.radii = rad2;
          }
        }
      }
      for (int p = 0; p < n_pairs; p++) {  // :162-177
        int a = -1, b = -1;
        for (size_t k = 0; k < c.groups.size(); k++) {
          if (a < 0 && c.groups[k].link_name == pair_a[p]) a = (int)k;
          if (b < 0 && c.groups[k].link_name == pair_b[p]) b = (int)k;
        }
        if (a < 0 || b < 0) fail(PMGPU_ERR_RUNTIME, "(cpp) Invalid pair of link names for self collision");
        c.pairs.push_back({a, b});
      }
      if (fixed_sdf) c.fixed_sdf = fixed_sdf->s;
    } catch (...) {
      delete h;
      throw;
    }
    *out = h;
  });
}
void pmgpu_cst_destroy(pmgpu_cst* c) { delete c; }
int pmgpu_cst_set_sdf(pmgpu_cst* c, pmgpu_sdf* sdf) {
  return guarded([&] {
    check_ptr(c, "cst");
    c->c.sdf = sdf ? sdf->s : nullptr;
  });
}
int pmgpu_cst_dims(const pmgpu_cst* c, int* q_dim, int* cst_dim, int* n_spheres, int* n_groups) {
  return guarded([&] {
    check_ptr(c, "cst");
    HostCst& C = const_cast<pmgpu_cst*>(c)->c;
    if (q_dim) *q_dim = C.q_dim();
    if (cst_dim) *cst_dim = C.cst_dim();
    if (n_spheres) *n_spheres = C.n_spheres();
    if (n_groups) *n_groups = (int)C.groups.size();
  });
}
int pmgpu_cst_groups(const pmgpu_cst* c, int32_t* link, double* radius, double* centre3, int32_t* only_self, double* sphere_rel3,
                     double* sphere_radii) {
  return guarded([&] {
    check_ptr(c, "cst");
    size_t k = 0;
    for (size_t g = 0; g < c->c.groups.size(); g++) {
      const HostGroup& G = c->c.groups[g];
      if (link) link[g] = G.link;
      if (radius) radius[g] = G.radius;
      if (centre3) std::memcpy(centre3 + 3 * g, G.centre.data(), 24);
      if (only_self) only_self[g] = G.only_self;
      for (size_t i = 0; i < G.radii.size(); i++, k++) {
        if (sphere_rel3) std::memcpy(sphere_rel3 + 3 * k, G.rel[i].data(), 24);
        if (sphere_radii) sphere_radii[k] = G.radii[i];
      }
    }
  });
}
}  // extern "C"

// ConstraintBase::update_kintree(q, high_accuracy) (primitive.hpp:38-62) on the shared model state:
// the control joints, then the base for PLANAR / FLOATING bases, whose joints always use exact
// sin/cos.
static void update_kintree_of(HostCst& C, const double* q, int high_accuracy) {
  check_arr(q, C.q_dim(), "q");
  C.tables();
  HostModel& M = *C.kin;
  int nq = C.q_dim(), nc = (int)C.ids.size();
  for (int i = 0; i < nc; i++) M.angles[C.ids[i]] = q[i];
  double* dq = (double*)C.w_aux.ensure((size_t)nq * 8 + 16);
  cuda_check(cudaMemcpy(dq, q, (size_t)nq * 8, cudaMemcpyHostToDevice), "H2D");
  int accurate = (C.base_type != PM_BASE_FIXED) ? 1 : (high_accuracy ? 1 : 0);
  if (nc > 0) cuda_check(launch_set_joints(M.d_state.as<double>(), C.d_ctrl_recs.as<PmSlot>(), dq, nc, accurate, 0), "update_kintree");
  if (C.base_type != PM_BASE_FIXED) cuda_check(launch_set_base_from_q(M.d_state.as<double>(), C.base_type, dq + nc, 0), "update_kintree");
  cuda_check(cudaDeviceSynchronize(), "update_kintree");
}

extern "C" {

int pmgpu_cst_update_kintree(pmgpu_cst* c, const double* q, int high_accuracy) {
  return guarded([&] {
    check_ptr(c, "cst");
    update_kintree_of(c->c, q, high_accuracy);
  });
}
static int spheres_of_state(pmgpu_cst* c, double* out4, int groups) {
  return guarded([&] {
    check_ptr(c, "cst");
    HostCst& C = c->c;
    const PmTablesHdr* T = C.tables();
    size_t n = groups ? C.groups.size() : (size_t)C.n_spheres();
    double* d = (double*)C.w_aux.ensure(std::max<size_t>(n * 32, 16));
    cuda_check(launch_spheres_of_state(T, C.kin->d_state.as<double>(), groups, d, 0), "spheres");
    cuda_check(cudaMemcpy(out4, d, n * 32, cudaMemcpyDeviceToHost), "D2H");
  });
}
int pmgpu_cst_get_all_spheres(pmgpu_cst* c, double* out4) { return spheres_of_state(c, out4, 0); }
int pmgpu_cst_get_group_spheres(pmgpu_cst* c, double* out4) { return spheres_of_state(c, out4, 1); }

int pmgpu_cst_is_valid(pmgpu_cst* c, const double* q, int64_t B, uint8_t* out, int mem, void* stream) {
  return guarded([&] {
    check_ptr(c, "cst");
    check_mem(mem);
    if (B < 0) throw std::invalid_argument("negative batch");
    HostCst& C = c->c;
    check_arr(q, B * C.q_dim(), "q");
    check_arr(out, B, "out");
    const PmTablesHdr* T = C.tables();
    const double* st = C.kin->d_state.as<double>();
    cudaStream_t s = as_stream(stream);
    if (mem == PMGPU_MEM_DEVICE) {
      cuda_check(launch_is_valid64(T, st, q, B, out, s), "is_valid");
      return;
    }
    const double* dq = stage_in(C.w_in, q, (size_t)B * C.q_dim(), s);
    uint8_t* dout = (uint8_t*)C.w_out.ensure(std::max<size_t>((size_t)B, 16));
    cuda_check(launch_is_valid64(T, st, dq, B, dout, s), "is_valid");
    stage_out(out, dout, (size_t)B, s);
    cuda_check(cudaStreamSynchronize(s), "is_valid");
  });
}
int pmgpu_cst_evaluate(pmgpu_cst* c, const double* q, int64_t B, double* vals, double* jac, int mem, void* stream) {
  return guarded([&] {
    check_ptr(c, "cst");
    check_mem(mem);
    if (B < 0) throw std::invalid_argument("negative batch");
    HostCst& C = c->c;
    check_arr(q, B * C.q_dim(), "q");
    check_arr(vals, B * C.cst_dim(), "vals");
    check_arr(jac, B * C.cst_dim() * C.q_dim(), "jac");
    const PmTablesHdr* T = C.tables();
    const double* st = C.kin->d_state.as<double>();
    cudaStream_t s = as_stream(stream);
    int m = C.cst_dim(), d = C.q_dim();
    if (mem == PMGPU_MEM_DEVICE) {
      cuda_check(launch_evaluate64(T, st, q, B, 1, vals, jac, s), "evaluate");
      return;
    }
    const double* dq = stage_in(C.w_in, q, (size_t)B * d, s);
    double* dv = (double*)C.w_out.ensure(std::max<size_t>((size_t)B * m * 8, 16));
    double* dj = (double*)C.w_out2.ensure(std::max<size_t>((size_t)B * m * d * 8, 16));
    cuda_check(launch_evaluate64(T, st, dq, B, 1, dv, dj, s), "evaluate");
    stage_out(vals, dv, (size_t)B * m, s);
    stage_out(jac, dj, (size_t)B * m * d, s);
    cuda_check(cudaStreamSynchronize(s), "evaluate");
  });
}
int pmgpu_cst_sphere_distances(pmgpu_cst* c, const double* q, int64_t B, int high_accuracy, double* dist, double* centres, int mem,
                               void* stream) {
  return guarded([&] {
    check_ptr(c, "cst");
    check_mem(mem);
    if (B < 0) throw std::invalid_argument("negative batch");
    HostCst& C = c->c;
    check_arr(q, B * C.q_dim(), "q");
    const PmTablesHdr* T = C.tables();
    const double* st = C.kin->d_state.as<double>();
    cudaStream_t s = as_stream(stream);
    int ns = C.n_spheres();
    if (mem == PMGPU_MEM_DEVICE) {
      // the centres go to the caller's array, or to a workspace when only distances are wanted
      double* dc = centres ? centres : (double*)C.w_cen.ensure(std::max<size_t>((size_t)B * ns * 24, 16));
      cuda_check(launch_sphere_dist64(T, C.hdr, st, q, B, high_accuracy, dist, dc, s), "sphere distances");
      return;
    }
    const double* dq = stage_in(C.w_in, q, (size_t)B * C.q_dim(), s);
    double* dd = dist ? (double*)C.w_out.ensure(std::max<size_t>((size_t)B * ns * 8, 16)) : nullptr;
    double* dc = (double*)C.w_out2.ensure(std::max<size_t>((size_t)B * ns * 24, 16));
    cuda_check(launch_sphere_dist64(T, C.hdr, st, dq, B, high_accuracy, dd, dc, s), "sphere distances");
    if (dist) stage_out(dist, dd, (size_t)B * ns, s);
    if (centres) stage_out(centres, dc, (size_t)B * ns * 3, s);
    cuda_check(cudaStreamSynchronize(s), "sphere distances");
  });
}
}  // extern "C"
namespace pmg {
void set_last_error(const char* msg) { g_last_error = msg; }
bool cst_device_view(pmgpu_cst* c, const PmTablesHdr** T, PmTablesHdr* hdr, const double** state, int* cpb, int* nt) {
  HostCst& C = c->c;
  if (!C.d_tables.p || !C.kin->dev_ready || C.sig_model_version != C.kin->version) return false;
  int cur = -1;
  if (cudaGetDevice(&cur) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  if (cur != C.kin->device) return false;  // the tables live on another device
  std::vector<std::shared_ptr<HostSdf>> f;
  if (C.fixed_sdf) flatten(C.fixed_sdf, f);
  if (C.sdf) flatten(C.sdf, f);
  std::vector<std::pair<const HostSdf*, uint64_t>> s;
  for (auto& x : f) s.push_back({x.get(), x->version});
  if (s != C.sig) return false;  // the scene changed since the tables were built
  *T = C.d_tables.as<PmTablesHdr>();
  *hdr = C.hdr;
  *state = C.kin->d_state.as<double>();
  *cpb = C.fast_cpb;
  *nt = C.fast_nt;
  return true;
}
}  // namespace pmg
extern "C" {

int pmgpu_cst_set_fast_launch(pmgpu_cst* c, int configs_per_block, int threads_per_block) {
  return guarded([&] {
    check_ptr(c, "cst");
    static const int ok[][2] = {{16, 128}, {32, 128}, {16, 256}, {32, 256}, {64, 256}, {32, 512}, {64, 512}, {128, 512}};
    bool found = false;
    for (auto& p : ok) found = found || (p[0] == configs_per_block && p[1] == threads_per_block);
    if (!found) throw std::invalid_argument("unsupported (configs_per_block, threads_per_block) pair");
    c->c.fast_cpb = configs_per_block;
    c->c.fast_nt = threads_per_block;
  });
}
int pmgpu_cst_set_fast_tuning(pmgpu_cst* c, int sphere_tile, int hq_blocks_per_sm, int edge_configs_per_block, int edge_threads) {
  return guarded([&] {
    check_ptr(c, "cst");
    int l = -1;
    for (int k = 0; k <= 5; k++)
      if (sphere_tile == (1 << k)) l = k;
    if (sphere_tile != 0 && l < 0) throw std::invalid_argument("sphere_tile must be 0 or a power of two up to 32");
    if (hq_blocks_per_sm < 1 || hq_blocks_per_sm > 8) throw std::invalid_argument("hq_blocks_per_sm must be in [1, 8]");
    static const int ok[][2] = {{16, 128}, {32, 128}, {32, 256}, {64, 256}};
    bool found = false;
    for (auto& p : ok) found = found || (p[0] == edge_configs_per_block && p[1] == edge_threads);
    if (!found) throw std::invalid_argument("unsupported edge (configs_per_block, threads_per_block) pair");
    c->c.tune.sphere_tile_log2 = sphere_tile == 0 ? 0 : l;
    c->c.tune.hq_blocks_per_sm = hq_blocks_per_sm;
    c->c.edge_cpb = edge_configs_per_block;
    c->c.edge_nt = edge_threads;
  });
}
int pmgpu_cst_get_fast_tuning(const pmgpu_cst* c, int* sphere_tile, int* hq_blocks_per_sm, int* edge_configs_per_block,
                              int* edge_threads) {
  return guarded([&] {
    check_ptr(c, "cst");
    if (sphere_tile) *sphere_tile = c->c.tune.sphere_tile_log2 == 0 ? 0 : (1 << c->c.tune.sphere_tile_log2);
    if (hq_blocks_per_sm) *hq_blocks_per_sm = c->c.tune.hq_blocks_per_sm;
    if (edge_configs_per_block) *edge_configs_per_block = c->c.edge_cpb;
    if (edge_threads) *edge_threads = c->c.edge_nt;
  });
}
int pmgpu_cst_get_fast_launch(const pmgpu_cst* c, int* configs_per_block, int* threads_per_block) {
  return guarded([&] {
    check_ptr(c, "cst");
    *configs_per_block = c->c.fast_cpb;
    *threads_per_block = c->c.fast_nt;
  });
}
// Capacity of the global hard-query queue of a fast call with distances: 16 per configuration (the
// dual-arm cloud batch needs about 8), at most one per sphere; a block whose queries do not fit
// answers them itself.
static unsigned hard_query_cap(int64_t B, int64_t ns) {
  return (unsigned)std::min<int64_t>(std::min<int64_t>(B * ns, std::max<int64_t>(B * 16, 1 << 16)), (int64_t)1 << 26);
}

// Host-memory fast call of a large batch, in 2 to 4 chunks on two
// streams (FastPipe).  Every configuration is independent, so the outcome is the same as one launch.
static void fast_host_pipelined(HostCst& C, const PmTablesHdr* T, const double* st, const double* q, int64_t B, uint8_t* out,
                                float* dist32, int64_t* stats, cudaStream_t s, PmLinkBounds bnd) {
  FastPipe& P = C.pipe;
  P.init();
  const int64_t d = C.q_dim(), ns = C.n_spheres();
  // 2 to 4 chunks of at least 32,768 configurations: on GB300 (190 GB/s pinned copies each way) 2
  // chunks of the 65,536-configuration batch measured 0.80 ms end to end, 4 chunks 0.81, 8 chunks 0.87
  const int64_t n_chunks = std::max<int64_t>(2, std::min<int64_t>(4, B / 32768));
  const int64_t chunk = ((B + n_chunks - 1) / n_chunks + 127) / 128 * 128;
  const unsigned cap = (unsigned)std::min<int64_t>(std::max<int64_t>(4 * chunk, 1 << 16), (int64_t)1 << 28);
  char* ctl = (char*)P.ctl.ensure((size_t)n_chunks * 64);
  uint8_t* ovf = (uint8_t*)P.ovf.ensure(std::max<size_t>((size_t)B, 16));
  double* din[2];
  uint8_t* dout[2];
  float* ddist[2];
  int4* items[2];
  void* hqb[2];
  const unsigned hq_cap = hard_query_cap(chunk, ns);
  for (int k = 0; k < 2; k++) {  // sized once per call, before any chunk is in flight
    hqb[k] = dist32 ? P.hq[k].ensure((size_t)hq_cap * 32) : nullptr;
    din[k] = (double*)P.in[k].ensure((size_t)chunk * d * 8);
    dout[k] = (uint8_t*)P.out[k].ensure(std::max<size_t>((size_t)chunk, 16));
    ddist[k] = dist32 ? (float*)P.dist[k].ensure((size_t)chunk * ns * 4) : nullptr;
    items[k] = (int4*)P.items[k].ensure((size_t)cap * sizeof(int4));
  }
  cuda_check(cudaMemsetAsync(ctl, 0, (size_t)n_chunks * 64, s), "memset");
  cuda_check(cudaMemsetAsync(ovf, 0, std::max<size_t>((size_t)B, 16), s), "memset");
  cuda_check(cudaEventRecord(P.ev_in, s), "event");  // the second stream starts after the caller's prior work
  cuda_check(cudaStreamWaitEvent(P.aux, P.ev_in, 0), "event");
  for (int64_t i = 0; i < n_chunks; i++) {
    const int64_t c0 = i * chunk;
    if (c0 >= B) break;
    const int64_t n = std::min<int64_t>(chunk, B - c0);
    const int k = (int)(i & 1);
    cudaStream_t cs = k ? P.aux : s;
    cuda_check(cudaMemcpyAsync(din[k], q + c0 * d, (size_t)(n * d) * 8, cudaMemcpyHostToDevice, cs), "H2D copy");
    char* cc = ctl + i * 64;
    cuda_check(launch_fast_valid(T, C.hdr, st, din[k], n, dout[k], ddist[k], 0.1f, items[k], (unsigned int*)cc, cap, ovf + c0,
                                 (unsigned long long*)(cc + 16), C.fast_cpb, C.fast_nt, cs, hqb[k], (unsigned long long*)(cc + 48), hq_cap,
                                 C.tune, bnd),
               "is_valid_fast");
    cuda_check(cudaMemcpyAsync(out + c0, dout[k], (size_t)n, cudaMemcpyDeviceToHost, cs), "D2H copy");
    if (dist32) cuda_check(cudaMemcpyAsync(dist32 + c0 * ns, ddist[k], (size_t)(n * ns) * 4, cudaMemcpyDeviceToHost, cs), "D2H copy");
  }
  cuda_check(cudaEventRecord(P.ev_out, P.aux), "event");
  cuda_check(cudaStreamWaitEvent(s, P.ev_out, 0), "event");
  cuda_check(cudaStreamSynchronize(s), "is_valid_fast");
  if (stats) {
    std::vector<unsigned long long> h((size_t)n_chunks * 8, 0);
    cuda_check(cudaMemcpy(h.data(), ctl, (size_t)n_chunks * 64, cudaMemcpyDeviceToHost), "D2H");
    stats[0] = B;
    stats[1] = stats[2] = stats[3] = 0;
    for (int64_t i = 0; i < n_chunks; i++) {
      stats[1] += (int64_t)(unsigned)h[8 * i];
      stats[2] += (int64_t)h[8 * i + 4];
    }
  }
}

// pmgpu_cst_is_valid_fast, and with link-position bounds the fused composite check
static int fast_valid_entry(pmgpu_cst* c, const double* q, int64_t B, uint8_t* out, float* dist32, int64_t* stats, int mem,
                            void* stream, PmLinkBounds bnd) {
  return guarded([&] {
    check_ptr(c, "cst");
    check_mem(mem);
    if (B < 0) throw std::invalid_argument("negative batch");
    HostCst& C = c->c;
    check_arr(q, B * C.q_dim(), "q");
    check_arr(out, B, "out");
    const PmTablesHdr* T = C.tables();
    if (!fast_table_sizes_ok(C.hdr))
      fail(PMGPU_ERR_INVALID, "is_valid_fast: at most 65535 spheres and 32767 primitives (use is_valid_batch)");
    const double* st = C.kin->d_state.as<double>();
    cudaStream_t s = as_stream(stream);
    if (mem == PMGPU_MEM_HOST && B >= 16384) {
      fast_host_pipelined(C, T, st, q, B, out, dist32, stats, s, bnd);
      return;
    }
    const unsigned cap = (unsigned)std::min<int64_t>(std::max<int64_t>(4 * B, 1 << 16), (int64_t)1 << 28);
    int4* items = (int4*)C.f_items.ensure((size_t)cap * sizeof(int4));
    char* ctl = (char*)C.f_ctl.ensure(64);
    unsigned int* count = (unsigned int*)ctl;
    unsigned long long* dstats = (unsigned long long*)(ctl + 16);
    uint8_t* ovf = (uint8_t*)C.f_overflow.ensure(std::max<size_t>((size_t)B, 16));
    cuda_check(cudaMemsetAsync(ctl, 0, 64, s), "memset");
    cuda_check(cudaMemsetAsync(ovf, 0, std::max<size_t>((size_t)B, 16), s), "memset");
    const double* dq = q;
    uint8_t* dout = out;
    float* dd = dist32;
    // host memory: one pinned staging buffer [q | out | dist | counters]
    const size_t nq = (size_t)B * C.q_dim() * 8, nd = dist32 ? (size_t)B * C.n_spheres() * 4 : 0;
    char* pin = nullptr;
    if (mem == PMGPU_MEM_HOST) {
      pin = C.h_pin.ensure(up16(nq) + up16((size_t)B) + up16(nd) + 64);
      std::memcpy(pin, q, nq);
      double* dqw = (double*)C.w_in.ensure(std::max<size_t>(nq, 16));
      if (nq) cuda_check(cudaMemcpyAsync(dqw, pin, nq, cudaMemcpyHostToDevice, s), "H2D copy");
      dq = dqw;
      dout = (uint8_t*)C.w_out.ensure(std::max<size_t>((size_t)B, 16));
      dd = dist32 ? (float*)C.w_out2.ensure(std::max<size_t>(nd, 16)) : nullptr;
    }
    const unsigned hq_cap = hard_query_cap(B, C.n_spheres());
    void* hq = dd ? C.f_hq.ensure((size_t)hq_cap * 32) : nullptr;
    cuda_check(launch_fast_valid(T, C.hdr, st, dq, B, dout, dd, 0.1f, items, count, cap, ovf, dstats, C.fast_cpb, C.fast_nt, s, hq,
                                 (unsigned long long*)(ctl + 48), hq_cap, C.tune, bnd),
               "is_valid_fast");
    char* pin_out = pin ? pin + up16(nq) : nullptr;
    char* pin_dist = pin ? pin_out + up16((size_t)B) : nullptr;
    unsigned long long local_ctl[6] = {0, 0, 0, 0, 0, 0};
    unsigned long long* h = pin ? reinterpret_cast<unsigned long long*>(pin_dist + up16(nd)) : local_ctl;
    if (mem == PMGPU_MEM_HOST) {
      if (B) cuda_check(cudaMemcpyAsync(pin_out, dout, (size_t)B, cudaMemcpyDeviceToHost, s), "D2H copy");
      if (nd) cuda_check(cudaMemcpyAsync(pin_dist, dd, nd, cudaMemcpyDeviceToHost, s), "D2H copy");
    }
    if (stats || mem == PMGPU_MEM_HOST) {
      cuda_check(cudaMemcpyAsync(h, ctl, 48, cudaMemcpyDeviceToHost, s), "D2H");
      cuda_check(cudaStreamSynchronize(s), "is_valid_fast");
      if (mem == PMGPU_MEM_HOST) {
        std::memcpy(out, pin_out, (size_t)B);
        if (nd) std::memcpy(dist32, pin_dist, nd);
      }
      if (stats) {
        stats[0] = B;
        stats[1] = (int64_t)(unsigned)h[0];
        stats[2] = (int64_t)h[2 + 2];
        stats[3] = 0;
      }
    }
  });
}
int pmgpu_cst_is_valid_fast(pmgpu_cst* c, const double* q, int64_t B, uint8_t* out, float* dist32, int64_t* stats, int mem,
                            void* stream) {
  return fast_valid_entry(c, q, B, out, dist32, stats, mem, stream, PmLinkBounds{nullptr, 0});
}
int pmgpu_check_motion(pmgpu_cst* c, const double* s1, const double* s2, int64_t E, int validator_type, const double* width,
                       double resolution, uint8_t* out, int64_t* n_checked, int mem, void* stream) {
  return guarded([&] {
    check_ptr(c, "cst");
    check_mem(mem);
    if (validator_type != PMGPU_VALIDATOR_BOX && validator_type != PMGPU_VALIDATOR_EUCLIDEAN)
      fail(PMGPU_ERR_RUNTIME, "unknown validator type");
    if (E < 0) throw std::invalid_argument("negative edge count");
    HostCst& C = c->c;
    check_arr(s1, E * C.q_dim(), "s1");
    check_arr(s2, E * C.q_dim(), "s2");
    check_arr(out, E, "out");
    const PmTablesHdr* T = C.tables();
    const double* st = C.kin->d_state.as<double>();
    cudaStream_t s = as_stream(stream);
    const int16_t* seq = C.seq_table();
    int d = C.q_dim();
    const double* dw = nullptr;
    if (validator_type == PMGPU_VALIDATOR_BOX) {
      check_ptr(width, "width");
      dw = (const double*)C.w_width.ensure((size_t)d * 8 + 16);
      if (mem == PMGPU_MEM_DEVICE)
        cuda_check(cudaMemcpyAsync((void*)dw, width, (size_t)d * 8, cudaMemcpyDeviceToDevice, s), "width");
      else
        cuda_check(cudaMemcpyAsync((void*)dw, width, (size_t)d * 8, cudaMemcpyHostToDevice, s), "width");
    }
    unsigned long long* cnt = (unsigned long long*)C.w_aux.ensure(64);
    cuda_check(cudaMemsetAsync(cnt, 0, 8, s), "memset");
    if (mem == PMGPU_MEM_DEVICE) {
      cuda_check(launch_check_motion64(T, st, s1, s2, E, validator_type, dw, resolution, seq, out, cnt, s), "check_motion");
      if (n_checked) {
        unsigned long long h = 0;
        cuda_check(cudaMemcpyAsync(&h, cnt, 8, cudaMemcpyDeviceToHost, s), "D2H");
        cuda_check(cudaStreamSynchronize(s), "check_motion");
        *n_checked = (int64_t)h;
      }
      return;
    }
    const double* d1 = stage_in(C.w_in, s1, (size_t)E * d, s);
    const double* d2 = stage_in(C.w_in2, s2, (size_t)E * d, s);
    uint8_t* dout = (uint8_t*)C.w_out.ensure(std::max<size_t>((size_t)E, 16));
    cuda_check(launch_check_motion64(T, st, d1, d2, E, validator_type, dw, resolution, seq, dout, cnt, s), "check_motion");
    stage_out(out, dout, (size_t)E, s);
    unsigned long long h = 0;
    cuda_check(cudaMemcpyAsync(&h, cnt, 8, cudaMemcpyDeviceToHost, s), "D2H");
    cuda_check(cudaStreamSynchronize(s), "check_motion");
    if (n_checked) *n_checked = (int64_t)h;
  });
}

// pmgpu_check_motion_fast, and with link-position bounds the fused composite check
static int fast_edges_entry(pmgpu_cst* c, const double* s1, const double* s2, int64_t E, int validator_type, const double* width,
                            double resolution, uint8_t* out, int64_t* stats, int mem, void* stream, PmLinkBounds bnd) {
  return guarded([&] {
    check_ptr(c, "cst");
    check_mem(mem);
    if (validator_type != PMGPU_VALIDATOR_BOX && validator_type != PMGPU_VALIDATOR_EUCLIDEAN)
      fail(PMGPU_ERR_RUNTIME, "unknown validator type");
    if (E < 0) throw std::invalid_argument("negative edge count");
    HostCst& C = c->c;
    check_arr(s1, E * C.q_dim(), "s1");
    check_arr(s2, E * C.q_dim(), "s2");
    check_arr(out, E, "out");
    const PmTablesHdr* T = C.tables();
    if (!fast_table_sizes_ok(C.hdr))
      fail(PMGPU_ERR_INVALID, "check_motion_fast: at most 65535 spheres and 32767 primitives (use check_motion_batch)");
    const double* st = C.kin->d_state.as<double>();
    cudaStream_t s = as_stream(stream);
    const int16_t* seq = C.seq_table();
    const int d = C.q_dim();
    const bool box = validator_type == PMGPU_VALIDATOR_BOX;
    if (box) check_ptr(width, "width");
    // host memory: one pinned staging buffer [s1 | s2 | width | out | counters]
    const size_t ns_ = (size_t)E * d * 8, nw = box ? (size_t)d * 8 : 0;
    char* pin = nullptr;
    if (mem == PMGPU_MEM_HOST) {
      pin = C.h_pin.ensure(2 * up16(ns_) + up16(nw) + up16((size_t)E) + 80);
      std::memcpy(pin, s1, ns_);
      std::memcpy(pin + up16(ns_), s2, ns_);
      if (box) std::memcpy(pin + 2 * up16(ns_), width, nw);
    }
    const double* dw = nullptr;
    if (box) {
      dw = (const double*)C.w_width.ensure((size_t)d * 8 + 16);
      if (mem == PMGPU_MEM_DEVICE)
        cuda_check(cudaMemcpyAsync((void*)dw, width, nw, cudaMemcpyDeviceToDevice, s), "width");
      else
        cuda_check(cudaMemcpyAsync((void*)dw, pin + 2 * up16(ns_), nw, cudaMemcpyHostToDevice, s), "width");
    }
    const size_t En = (size_t)std::max<int64_t>(E, 1);
    double* sr = (double*)C.e_sr.ensure(En * 8);
    int32_t* n = (int32_t*)C.e_n.ensure(En * 4);
    int64_t* off = (int64_t*)C.e_off.ensure(En * 8);
    const unsigned cap = 1u << 18;
    int4* items = (int4*)C.f_items.ensure((size_t)cap * sizeof(int4));
    char* ctl = (char*)C.f_ctl.ensure(64);
    unsigned int* count = (unsigned int*)ctl;
    unsigned long long* next = (unsigned long long*)(ctl + 8);
    unsigned long long* dstats = (unsigned long long*)(ctl + 16);
    uint8_t* ovf = (uint8_t*)C.f_overflow.ensure(std::max<size_t>(En, 16));
    cuda_check(cudaMemsetAsync(ctl, 0, 64, s), "memset");
    cuda_check(cudaMemsetAsync(ovf, 0, std::max<size_t>(En, 16), s), "memset");
    const double* d1 = s1;
    const double* d2 = s2;
    uint8_t* dout = out;
    if (mem == PMGPU_MEM_HOST) {
      double* w1 = (double*)C.w_in.ensure(std::max<size_t>(ns_, 16));
      double* w2 = (double*)C.w_in2.ensure(std::max<size_t>(ns_, 16));
      if (ns_) {
        cuda_check(cudaMemcpyAsync(w1, pin, ns_, cudaMemcpyHostToDevice, s), "H2D copy");
        cuda_check(cudaMemcpyAsync(w2, pin + up16(ns_), ns_, cudaMemcpyHostToDevice, s), "H2D copy");
      }
      d1 = w1;
      d2 = w2;
      dout = (uint8_t*)C.w_out.ensure(std::max<size_t>((size_t)E, 16));
    }
    int n_sm = 0;
    cuda_check(sm_count(&n_sm), "device attribute");
    cuda_check(launch_fast_edges(T, C.hdr, st, d1, d2, E, validator_type, dw, resolution, seq, sr, n, off, next, dout, items, count, cap,
                                 ovf, dstats, C.edge_cpb, C.edge_nt, n_sm, s, bnd),
               "check_motion_fast");
    char* pin_out = pin ? pin + 2 * up16(ns_) + up16(nw) : nullptr;
    if (mem == PMGPU_MEM_HOST && E) cuda_check(cudaMemcpyAsync(pin_out, dout, (size_t)E, cudaMemcpyDeviceToHost, s), "D2H copy");
    if (stats || mem == PMGPU_MEM_HOST) {
      unsigned long long local_ctl[8] = {0, 0, 0, 0, 0, 0, 0, 0};
      unsigned long long* h = pin ? reinterpret_cast<unsigned long long*>(pin_out + up16((size_t)E)) : local_ctl;
      int64_t* last_off = reinterpret_cast<int64_t*>(h + 6);
      int32_t* last_n = reinterpret_cast<int32_t*>(h + 7);
      *last_off = 0;
      *last_n = 0;
      cuda_check(cudaMemcpyAsync(h, ctl, 48, cudaMemcpyDeviceToHost, s), "D2H");
      if (E > 0 && stats) {
        cuda_check(cudaMemcpyAsync(last_off, off + E - 1, 8, cudaMemcpyDeviceToHost, s), "D2H");
        cuda_check(cudaMemcpyAsync(last_n, n + E - 1, 4, cudaMemcpyDeviceToHost, s), "D2H");
      }
      cuda_check(cudaStreamSynchronize(s), "check_motion_fast");
      if (mem == PMGPU_MEM_HOST) std::memcpy(out, pin_out, (size_t)E);
      if (stats) {
        stats[0] = E > 0 ? *last_off + *last_n : 0;
        stats[1] = (int64_t)(unsigned)h[0];
        stats[2] = (int64_t)h[4];
        stats[3] = 0;
      }
    }
  });
}

int pmgpu_check_motion_fast(pmgpu_cst* c, const double* s1, const double* s2, int64_t E, int validator_type, const double* width,
                            double resolution, uint8_t* out, int64_t* stats, int mem, void* stream) {
  return fast_edges_entry(c, s1, s2, E, validator_type, width, resolution, out, stats, mem, stream, PmLinkBounds{nullptr, 0});
}

// ------------------------------------------------------------------ link poses, differentiable costs

int pmgpu_cst_link_poses(pmgpu_cst* c, int32_t link, const double* q, int64_t B, double* out7, int mem, void* stream) {
  return guarded([&] {
    check_ptr(c, "cst");
    check_mem(mem);
    if (B < 0) throw std::invalid_argument("negative batch");
    HostCst& C = c->c;
    check_arr(q, B * C.q_dim(), "q");
    check_arr(out7, B, "out7");
    const int slot = C.slot_for_link(link);
    const PmTablesHdr* T = C.tables();
    const double* st = C.kin->d_state.as<double>();
    cudaStream_t s = as_stream(stream);
    const double* dq = q;
    double* dout = out7;
    if (mem == PMGPU_MEM_HOST) {
      dq = stage_in(C.w_in, q, (size_t)B * C.q_dim(), s);
      dout = (double*)C.w_out.ensure(std::max<size_t>((size_t)B * 7 * 8, 16));
    }
    cuda_check(launch_link_pose64(T, st, dq, B, slot, dout, s), "link_poses");
    if (mem == PMGPU_MEM_HOST) {
      stage_out(out7, dout, (size_t)B * 7, s);
      cuda_check(cudaStreamSynchronize(s), "link_poses");
    }
  });
}

int pmgpu_ik_cost(pmgpu_cst* c, const pmgpu_cost_params* p, const float* q, const float* target, int64_t B, float* cost,
                  float* grad, int mem, void* stream) {
  return guarded([&] {
    check_ptr(c, "cst");
    check_mem(mem);
    if (B < 0) throw std::invalid_argument("negative batch");
    HostCst& C = c->c;
    check_arr(q, B * C.q_dim(), "q");
    check_arr(cost, B, "cost");
    GradArgs a = grad_args(C, p, target != nullptr);
    a.steps = 0;
    const PmTablesHdr* T = C.tables();
    const double* st = C.kin->d_state.as<double>();
    cudaStream_t s = as_stream(stream);
    const int d = C.q_dim();
    const float* dq = q;
    const float* dt = target;
    float* dc = cost;
    float* dg = grad;
    if (mem == PMGPU_MEM_HOST) {
      dq = stage_in(C.w_in, q, (size_t)B * d, s);
      if (target) dt = stage_in(C.w_in2, target, (size_t)B * 7, s);
      dc = (float*)C.w_out.ensure(std::max<size_t>((size_t)B * 4, 16));
      if (grad) dg = (float*)C.w_out2.ensure(std::max<size_t>((size_t)B * d * 4, 16));
    }
    cuda_check(launch_ik_cost(T, C.hdr, st, a, const_cast<float*>(dq), dt, B, dc, dg, nullptr, s), "ik_cost");
    if (mem == PMGPU_MEM_HOST) {
      stage_out(cost, dc, (size_t)B, s);
      if (grad) stage_out(grad, dg, (size_t)B * d, s);
      cuda_check(cudaStreamSynchronize(s), "ik_cost");
    }
  });
}

int pmgpu_ik_descend(pmgpu_cst* c, const pmgpu_cost_params* p, float* q, const float* target, int64_t B, int32_t steps,
                     float lr, int32_t clamp_to_limits, float* cost, float* cost_hist, int mem, void* stream) {
  return guarded([&] {
    check_ptr(c, "cst");
    check_mem(mem);
    if (B < 0) throw std::invalid_argument("negative batch");
    if (steps < 1) throw std::invalid_argument("steps must be positive");
    if (!std::isfinite(lr)) throw std::invalid_argument("lr must be finite");
    HostCst& C = c->c;
    check_arr(q, B * C.q_dim(), "q");
    GradArgs a = grad_args(C, p, target != nullptr);
    if (a.mode != PMGPU_COST_SUM) fail(PMGPU_ERR_INVALID, "descent minimises the PMGPU_COST_SUM cost");
    a.steps = steps;
    a.lr = lr;
    a.clamp = clamp_to_limits != 0;
    const PmTablesHdr* T = C.tables();
    const double* st = C.kin->d_state.as<double>();
    cudaStream_t s = as_stream(stream);
    const int d = C.q_dim();
    float* dq = q;
    const float* dt = target;
    float* dc = cost;
    float* dh = cost_hist;
    if (mem == PMGPU_MEM_HOST) {
      dq = stage_in(C.w_in, (const float*)q, (size_t)B * d, s);
      if (target) dt = stage_in(C.w_in2, target, (size_t)B * 7, s);
      if (cost) dc = (float*)C.w_out.ensure(std::max<size_t>((size_t)B * 4, 16));
      if (cost_hist) dh = (float*)C.w_out2.ensure(std::max<size_t>((size_t)B * steps * 4, 16));
    }
    cuda_check(launch_ik_cost(T, C.hdr, st, a, dq, dt, B, dc, nullptr, dh, s), "ik_descend");
    if (mem == PMGPU_MEM_HOST) {
      stage_out(q, (const float*)dq, (size_t)B * d, s);
      if (cost) stage_out(cost, dc, (size_t)B, s);
      if (cost_hist) stage_out(cost_hist, dh, (size_t)B * steps, s);
      cuda_check(cudaStreamSynchronize(s), "ik_descend");
    }
  });
}

int pmgpu_traj_cost(pmgpu_cst* c, const pmgpu_cost_params* p, const float* q, const int64_t* offsets, int64_t n_traj,
                    int64_t n_waypoints, float* cost, float* grad, int mem, void* stream) {
  return guarded([&] {
    check_ptr(c, "cst");
    check_mem(mem);
    if (n_traj < 0 || n_waypoints < 0) throw std::invalid_argument("negative count");
    check_ptr(offsets, "offsets");
    check_arr(cost, n_traj, "cost");
    check_arr(q, n_waypoints * c->c.q_dim(), "q");
    if (mem == PMGPU_MEM_HOST) {  // the device clamps offsets into range; host input is checked
      if (offsets[0] != 0 || offsets[n_traj] != n_waypoints)
        throw std::invalid_argument("offsets must start at 0 and end at n_waypoints");
      for (int64_t i = 0; i < n_traj; i++)
        if (offsets[i + 1] < offsets[i]) throw std::invalid_argument("offsets must be non-decreasing");
    }
    HostCst& C = c->c;
    GradArgs a = grad_args(C, p, false);
    if (a.mode != PMGPU_COST_SUM) fail(PMGPU_ERR_INVALID, "trajectory costs use PMGPU_COST_SUM");
    a.steps = 0;
    const PmTablesHdr* T = C.tables();
    const double* st = C.kin->d_state.as<double>();
    cudaStream_t s = as_stream(stream);
    const int d = C.q_dim();
    float* wp = (float*)C.g_wp.ensure(std::max<size_t>((size_t)n_waypoints * 4, 16));
    const float* dq = q;
    const int64_t* doff = offsets;
    float* dc = cost;
    float* dg = grad;
    if (mem == PMGPU_MEM_HOST) {
      dq = stage_in(C.w_in, q, (size_t)n_waypoints * d, s);
      doff = stage_in(C.w_in2, offsets, (size_t)n_traj + 1, s);
      dc = (float*)C.w_out.ensure(std::max<size_t>((size_t)n_traj * 4, 16));
      if (grad) dg = (float*)C.w_out2.ensure(std::max<size_t>((size_t)n_waypoints * d * 4, 16));
    }
    cuda_check(launch_traj_cost(T, C.hdr, st, a, dq, doff, n_traj, n_waypoints, wp, dc, dg, s), "traj_cost");
    if (mem == PMGPU_MEM_HOST) {
      stage_out(cost, dc, (size_t)n_traj, s);
      if (grad) stage_out(grad, dg, (size_t)n_waypoints * d, s);
      cuda_check(cudaStreamSynchronize(s), "traj_cost");
    }
  });
}

// ------------------------------------------------------------------ pose constraints
}  // extern "C"
struct pmgpu_posecst {
  HostCst c;  // kinematic slots of the constrained links (no spheres)
  std::vector<PmPoseTerm> terms;
  std::vector<int> links;
  DevBuf d_terms;
  uint64_t terms_sig = ~0ull;  // slot numbering the device terms were written with
  int cst_dim = 0;
  bool equality = true;
  const PmPoseTerm* device_terms() {
    c.tables();
    uint64_t sig = 0;
    for (size_t i = 0; i < terms.size(); i++) {
      terms[i].slot = c.slot_for_link(links[i]);
      sig = sig * 1315423911ull + (uint64_t)terms[i].slot + 1;
    }
    if (!d_terms.p || sig != terms_sig) {
      d_terms.release();
      d_terms.ensure(std::max<size_t>(terms.size(), 1) * sizeof(PmPoseTerm));
      if (!terms.empty())
        cuda_check(cudaMemcpy(d_terms.p, terms.data(), terms.size() * sizeof(PmPoseTerm), cudaMemcpyHostToDevice), "terms upload");
      terms_sig = sig;
    }
    return d_terms.as<PmPoseTerm>();
  }
};
namespace {
void posecst_init(pmgpu_posecst* h, pmgpu_model* kin, const char* const* control_joints, int n_joints, int base_type) {
  check_ptr(kin, "kin");
  if (base_type < 0 || base_type > 2) throw std::invalid_argument("unknown base type");
  HostCst& c = h->c;
  c.kin = kin->m;
  for (int i = 0; i < n_joints; i++) {  // ConstraintBase ctor -> get_joint_ids (primitive.hpp:30-36)
    auto it = c.kin->joint_id.find(control_joints[i]);
    if (it == c.kin->joint_id.end()) throw std::invalid_argument(std::string("no joint named ") + control_joints[i]);
    c.ids.push_back(it->second);
  }
  c.base_type = base_type;
}
int link_of(const HostModel& M, const char* name) {
  auto it = M.link_id.find(name);
  if (it == M.link_id.end()) throw std::invalid_argument(std::string("no link named ") + name);
  return it->second;
}
}  // namespace
extern "C" {

int pmgpu_linkpose_create(pmgpu_model* kin, const char* const* control_joints, int n_joints, int base_type, const char* const* links,
                          int n_links, const double* poses, const int32_t* pose_dims, pmgpu_posecst** out) {
  return guarded([&] {
    auto* h = new pmgpu_posecst();
    try {
      posecst_init(h, kin, control_joints, n_joints, base_type);
      size_t off = 0;
      for (int i = 0; i < n_links; i++) {  // primitive_link_pose.cpp:16-29
        const int d = pose_dims[i];
        if (d != 3 && d != 6 && d != 7) fail(PMGPU_ERR_RUNTIME, "All poses must be 3 or 6 or 7 dimensional");
        PmPoseTerm t;
        std::memset(&t, 0, sizeof(t));
        t.kind = PM_TERM_LINK_POSE;
        t.dim = d;
        for (int k = 0; k < d; k++) t.target[k] = poses[off + k];
        off += d;
        h->links.push_back(link_of(*h->c.kin, links[i]));
        h->terms.push_back(t);
        h->cst_dim += d;
      }
      h->equality = true;
      *out = h;
    } catch (...) {
      delete h;
      throw;
    }
  });
}

int pmgpu_linkbound_create(pmgpu_model* kin, const char* const* control_joints, int n_joints, int base_type, const char* link, int axis,
                           int has_lb, double lb, int has_ub, double ub, pmgpu_posecst** out) {
  return guarded([&] {
    auto* h = new pmgpu_posecst();
    try {
      posecst_init(h, kin, control_joints, n_joints, base_type);
      // primitive_link_position_bound.cpp:15-32
      if (axis < 0 || axis > 2) fail(PMGPU_ERR_RUNTIME, "Axis index must be 0 (x), 1 (y), or 2 (z).");
      if (!has_lb && !has_ub) fail(PMGPU_ERR_RUNTIME, "At least one of lower or upper bound must be provided.");
      PmPoseTerm t;
      std::memset(&t, 0, sizeof(t));
      t.kind = PM_TERM_POSITION_BOUND;
      t.axis = axis;
      t.has_lb = has_lb != 0;
      t.has_ub = has_ub != 0;
      t.lb = lb;
      t.ub = ub;
      t.dim = t.has_lb + t.has_ub;
      h->links.push_back(link_of(*h->c.kin, link));
      h->terms.push_back(t);
      h->cst_dim = t.dim;
      h->equality = false;
      *out = h;
    } catch (...) {
      delete h;
      throw;
    }
  });
}

void pmgpu_posecst_destroy(pmgpu_posecst* c) { delete c; }

// ------------------------------------------------------------------ composite (IneqCompositeCst)
}  // extern "C"
namespace {
// The link-position bounds of `bounds` as device terms on c's tables: every handle must be a
// LinkPositionBoundCst on c's kinematic model with c's control joints and base type (the
// composite's members share one update_kintree, composite_constraint.hpp:27-37, 98-105).  A
// bound's link joins c's FK slots if no sphere chain reaches it.
PmLinkBounds composite_bounds(HostCst& C, pmgpu_posecst* const* bounds, int n_bounds, cudaStream_t s) {
  if (n_bounds < 0) throw std::invalid_argument("negative bound count");
  if (n_bounds > 0) check_ptr(bounds, "bounds");
  std::vector<std::pair<int, PmPoseTerm>> terms;
  for (int i = 0; i < n_bounds; i++) {
    const pmgpu_posecst* b = bounds[i];
    check_ptr(b, "bound");
    if (b->equality) fail(PMGPU_ERR_INVALID, "composite is_valid: members must be inequality constraints (LinkPositionBoundCst)");
    if (b->c.kin.get() != C.kin.get()) fail(PMGPU_ERR_RUNTIME, "All constraints must have the same kinematic chain");
    if (b->c.ids != C.ids || b->c.base_type != C.base_type)
      fail(PMGPU_ERR_INVALID, "composite is_valid: members need the same control joints and base type");
    for (size_t j = 0; j < b->terms.size(); j++) {
      if (b->terms[j].kind != PM_TERM_POSITION_BOUND) fail(PMGPU_ERR_INVALID, "composite is_valid: not a link-position bound");
      terms.push_back({b->links[j], b->terms[j]});
    }
  }
  if (terms.empty()) return PmLinkBounds{nullptr, 0};
  if (terms.size() > 4096) fail(PMGPU_ERR_INVALID, "composite is_valid: at most 4096 link-position bounds");
  for (auto& t : terms) C.slot_for_link(t.first);  // first every link joins the tables, then the slots are final
  C.tables();
  std::vector<PmPoseTerm> up;
  for (auto& t : terms) {
    PmPoseTerm x = t.second;
    x.slot = C.slot_of_link[t.first];
    up.push_back(x);
  }
  const size_t bytes = up.size() * sizeof(PmPoseTerm);
  if (!C.d_bnd.p || up.size() != C.bnd_up.size() || std::memcmp(up.data(), C.bnd_up.data(), bytes) != 0) {
    C.bnd_up = up;  // the copy's source stays alive until the next change
    cuda_check(cudaMemcpyAsync(C.d_bnd.ensure(bytes), C.bnd_up.data(), bytes, cudaMemcpyHostToDevice, s), "bounds upload");
  }
  return PmLinkBounds{C.d_bnd.as<PmPoseTerm>(), (int32_t)up.size()};
}
}  // namespace
extern "C" {

int pmgpu_composite_is_valid_fast(pmgpu_cst* c, pmgpu_posecst* const* bounds, int n_bounds, const double* q, int64_t B,
                                  uint8_t* out, int64_t* stats, int mem, void* stream) {
  PmLinkBounds bnd{nullptr, 0};
  const int rc = guarded([&] {
    check_ptr(c, "cst");
    bnd = composite_bounds(c->c, bounds, n_bounds, as_stream(stream));
  });
  if (rc != PMGPU_OK) return rc;
  return fast_valid_entry(c, q, B, out, nullptr, stats, mem, stream, bnd);
}
int pmgpu_composite_check_motion_fast(pmgpu_cst* c, pmgpu_posecst* const* bounds, int n_bounds, const double* s1, const double* s2,
                                      int64_t E, int validator_type, const double* width, double resolution, uint8_t* out,
                                      int64_t* stats, int mem, void* stream) {
  PmLinkBounds bnd{nullptr, 0};
  const int rc = guarded([&] {
    check_ptr(c, "cst");
    bnd = composite_bounds(c->c, bounds, n_bounds, as_stream(stream));
  });
  if (rc != PMGPU_OK) return rc;
  return fast_edges_entry(c, s1, s2, E, validator_type, width, resolution, out, stats, mem, stream, bnd);
}

int pmgpu_posecst_dims(const pmgpu_posecst* c, int* q_dim, int* cst_dim, int* is_equality) {
  return guarded([&] {
    check_ptr(c, "constraint");
    if (q_dim) *q_dim = c->c.q_dim();
    if (cst_dim) *cst_dim = c->cst_dim;
    if (is_equality) *is_equality = c->equality ? 1 : 0;
  });
}

int pmgpu_posecst_update_kintree(pmgpu_posecst* c, const double* q, int high_accuracy) {
  return guarded([&] {
    check_ptr(c, "constraint");
    update_kintree_of(c->c, q, high_accuracy);
  });
}

int pmgpu_posecst_evaluate(pmgpu_posecst* c, const double* q, int64_t B, double* vals, double* jac, int mem, void* stream) {
  return guarded([&] {
    check_ptr(c, "constraint");
    check_mem(mem);
    if (B < 0) throw std::invalid_argument("negative batch");
    check_arr(q, B * c->c.q_dim(), "q");
    const PmPoseTerm* dt = c->device_terms();
    const PmTablesHdr* T = c->c.tables();
    const double* st = c->c.kin->d_state.as<double>();
    cudaStream_t s = as_stream(stream);
    const int d = c->c.q_dim(), m = c->cst_dim;
    const double* dq = q;
    double* dv = vals;
    double* dj = jac;
    if (mem == PMGPU_MEM_HOST) {
      dq = stage_in(c->c.w_in, q, (size_t)B * d, s);
      if (vals) dv = (double*)c->c.w_out.ensure(std::max<size_t>((size_t)B * m * 8, 16));
      if (jac) dj = (double*)c->c.w_out2.ensure(std::max<size_t>((size_t)B * m * d * 8, 16));
    }
    cuda_check(launch_posecst_eval64(T, st, dt, (int)c->terms.size(), m, dq, B, dv, dj, s), "pose constraint evaluate");
    if (mem == PMGPU_MEM_HOST) {
      if (vals) stage_out(vals, dv, (size_t)B * m, s);
      if (jac) stage_out(jac, dj, (size_t)B * m * d, s);
      cuda_check(cudaStreamSynchronize(s), "pose constraint evaluate");
    }
  });
}

int pmgpu_posecst_is_valid(pmgpu_posecst* c, const double* q, int64_t B, uint8_t* out, int mem, void* stream) {
  return guarded([&] {
    check_ptr(c, "constraint");
    check_mem(mem);
    if (B < 0) throw std::invalid_argument("negative batch");
    if (c->equality) fail(PMGPU_ERR_INVALID, "an equality constraint has no is_valid");
    check_arr(q, B * c->c.q_dim(), "q");
    check_arr(out, B, "out");
    const PmPoseTerm* dt = c->device_terms();
    const PmTablesHdr* T = c->c.tables();
    const double* st = c->c.kin->d_state.as<double>();
    cudaStream_t s = as_stream(stream);
    const double* dq = q;
    uint8_t* dout = out;
    if (mem == PMGPU_MEM_HOST) {
      dq = stage_in(c->c.w_in, q, (size_t)B * c->c.q_dim(), s);
      dout = (uint8_t*)c->c.w_out.ensure(std::max<size_t>((size_t)B, 16));
    }
    cuda_check(launch_posecst_valid64(T, st, dt, (int)c->terms.size(), dq, B, dout, s), "pose constraint is_valid");
    if (mem == PMGPU_MEM_HOST) {
      stage_out(out, dout, (size_t)B, s);
      cuda_check(cudaStreamSynchronize(s), "pose constraint is_valid");
    }
  });
}

int pmgpu_measure_fma_peak(int fp64, double* tflops, void* stream) {
  return guarded([&] {
    check_ptr(tflops, "tflops");
    cudaStream_t s = as_stream(stream);
    int dev = 0, n_sm = 0;
    cuda_check(cudaGetDevice(&dev), "device");
    cuda_check(cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev), "device");
    const int threads = 256, blocks = n_sm * 8;  // 64 warps per SM: every scheduler has work
    const int iters = fp64 ? 512 : 8192;
    DevBuf out;
    out.ensure((size_t)blocks * threads * 8);
    cudaEvent_t e0, e1;
    cuda_check(cudaEventCreate(&e0), "event");
    cuda_check(cudaEventCreate(&e1), "event");
    float best = 0.f;
    for (int r = 0; r < 6; r++) {  // the first launch warms up; the best of the rest counts
      cuda_check(cudaEventRecord(e0, s), "event");
      cuda_check(launch_fma_peak(fp64, iters, out.p, blocks, threads, s), "fma_peak");
      cuda_check(cudaEventRecord(e1, s), "event");
      cuda_check(cudaEventSynchronize(e1), "event");
      float ms = 0.f;
      cuda_check(cudaEventElapsedTime(&ms, e0, e1), "event");
      if (r > 0 && (best == 0.f || ms < best)) best = ms;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    *tflops = 16.0 * iters * (double)blocks * threads / (best * 1e-3) / 1e12;
  });
}

int pmgpu_profile_enable(int on) {
  return guarded([&] { g_prof_enabled = on != 0; });
}
int pmgpu_profile_read(const char* kernel, double* total_ms, int64_t* launches) {
  return guarded([&] {
    std::lock_guard<std::mutex> lk(g_prof_mu);
    double tot = 0;
    int64_t n = 0;
    for (auto& kv : g_prof) {
      if (kernel && std::strcmp(kernel, "*") != 0 && kv.first != kernel) continue;
      for (auto& pr : kv.second.pending) {
        cuda_check(cudaEventSynchronize(pr.second), "profile");
        float ms = 0;
        cuda_check(cudaEventElapsedTime(&ms, pr.first, pr.second), "profile");
        kv.second.total_ms += ms;
        cudaEventDestroy(pr.first);
        cudaEventDestroy(pr.second);
      }
      kv.second.pending.clear();
      tot += kv.second.total_ms;
      n += kv.second.launches;
      kv.second.total_ms = 0;
      kv.second.launches = 0;
    }
    if (total_ms) *total_ms = tot;
    if (launches) *launches = n;
  });
}

}  // extern "C"
