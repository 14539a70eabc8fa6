// Test infrastructure only -- NOT part of the product.
//
// CPU FP64 restatement of plainmp's collision-checking hot path, against which tests/,
// __graft_entry__.smoke() and bench.py's CPU-baseline leg compare the device path.  It is
// written from the reference's behaviour (cited file:line per function, paths relative to
// the plainmp project) and compiled with -ffp-contract=off; oracle/ORDER.md fixes the
// arithmetic order.  Nothing in the product links or calls this file.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

namespace orc {

// ---------------------------------------------------------------- small algebra
struct V3 {
  double x = 0, y = 0, z = 0;
  double operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
  double& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
};
struct Q4 {
  double x = 0, y = 0, z = 0, w = 1;
};
struct M3 {
  double m[3][3];
};

static inline V3 add(const V3& a, const V3& b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
static inline V3 sub(const V3& a, const V3& b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
static inline double dot(const V3& a, const V3& b) { return a.x * b.x + (a.y * b.y + a.z * b.z); }
static inline double sqn(const V3& a) { return a.x * a.x + (a.y * a.y + a.z * a.z); }
static inline double nrm(const V3& a) { return std::sqrt(sqn(a)); }
static inline V3 cross(const V3& a, const V3& b) {
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
// transform.hpp:56-86 (Eigen quaternion product)
static inline Q4 qmul(const Q4& a, const Q4& b) {
  Q4 r;
  r.w = a.w * b.w - a.x * b.x - a.y * b.y - a.z * b.z;
  r.x = a.w * b.x + a.x * b.w + a.y * b.z - a.z * b.y;
  r.y = a.w * b.y + a.y * b.w + a.z * b.x - a.x * b.z;
  r.z = a.w * b.z + a.z * b.w + a.x * b.y - a.y * b.x;
  return r;
}
// transform.hpp:58 (Eigen quaternion * vector)
static inline V3 qrot(const Q4& q, const V3& v) {
  V3 qv{q.x, q.y, q.z};
  V3 uv = cross(qv, v);
  uv = add(uv, uv);
  V3 c = cross(qv, uv);
  return {(v.x + q.w * uv.x) + c.x, (v.y + q.w * uv.y) + c.y, (v.z + q.w * uv.z) + c.z};
}
// primitive_sphere_collision.cpp:32 (Eigen toRotationMatrix)
static inline M3 qmat(const Q4& q) {
  double tx = 2.0 * q.x, ty = 2.0 * q.y, tz = 2.0 * q.z;
  double twx = tx * q.w, twy = ty * q.w, twz = tz * q.w;
  double txx = tx * q.x, txy = ty * q.x, txz = tz * q.x;
  double tyy = ty * q.y, tyz = tz * q.y, tzz = tz * q.z;
  M3 r;
  r.m[0][0] = 1.0 - (tyy + tzz);
  r.m[0][1] = txy - twz;
  r.m[0][2] = txz + twy;
  r.m[1][0] = txy + twz;
  r.m[1][1] = 1.0 - (txx + tzz);
  r.m[1][2] = tyz - twx;
  r.m[2][0] = txz - twy;
  r.m[2][1] = tyz + twx;
  r.m[2][2] = 1.0 - (txx + tyy);
  return r;
}
static inline V3 mv(const M3& R, const V3& v) {
  V3 r;
  for (int i = 0; i < 3; i++) r[i] = R.m[i][0] * v.x + (R.m[i][1] * v.y + R.m[i][2] * v.z);
  return r;
}
static inline V3 col(const M3& R, int j) { return {R.m[0][j], R.m[1][j], R.m[2][j]}; }

// transform.hpp:16-162
struct QT {
  Q4 q;
  V3 t;
  bool qid = false;
};
// transform.hpp:64-74
static inline void mult_assign(const QT& a, const QT& b, QT& out) {
  if (b.qid) {
    out.q = a.q;
  } else {
    out.q = qmul(a.q, b.q);
  }
  out.t = add(a.t, qrot(a.q, b.t));
}
// transform.hpp:56-62
static inline QT mul(const QT& a, const QT& b) {
  QT r;
  r.q = b.qid ? a.q : qmul(a.q, b.q);
  r.t = add(a.t, qrot(a.q, b.t));
  return r;
}
// transform.hpp:88-91 (Eigen quaternion inverse = conjugate / squaredNorm)
static inline QT inverse(const QT& a) {
  double n2 = (a.q.x * a.q.x + a.q.y * a.q.y) + (a.q.z * a.q.z + a.q.w * a.q.w);
  Q4 qi;
  if (n2 > 0) {
    qi.x = -a.q.x / n2;
    qi.y = -a.q.y / n2;
    qi.z = -a.q.z / n2;
    qi.w = a.q.w / n2;
  } else {
    qi.x = qi.y = qi.z = qi.w = 0.0;
  }
  QT r;
  r.q = qi;
  V3 mt{-a.t.x, -a.t.y, -a.t.z};
  r.t = qrot(qi, mt);
  return r;
}
// transform.hpp:93-120
static inline V3 get_rpy(const Q4& q) {
  double sqx = q.x * q.x, sqy = q.y * q.y, sqz = q.z * q.z, sqw = q.w * q.w;
  double sarg = -2 * (q.x * q.z - q.w * q.y);
  const double pi_2 = 1.57079632679489661923;
  double roll, pitch, yaw;
  if (sarg <= -0.99999) {
    pitch = -pi_2;
    roll = 0;
    yaw = -2 * std::atan2(q.x, q.y);
  } else if (sarg >= 0.99999) {
    pitch = pi_2;
    roll = 0;
    yaw = 2 * std::atan2(q.x, q.y);
  } else {
    pitch = std::asin(sarg);
    roll = std::atan2(2 * (q.y * q.z + q.w * q.x), sqw - sqx - sqy + sqz);
    yaw = std::atan2(2 * (q.x * q.y + q.w * q.z), sqw + sqx - sqy - sqz);
  }
  return {roll, pitch, yaw};
}
// transform.hpp:122-130
static inline Q4 quat_from_rpy(double r, double p, double y) {
  double phi = r / 2.0, the = p / 2.0, psi = y / 2.0;
  Q4 q;
  q.x = std::sin(phi) * std::cos(the) * std::cos(psi) - std::cos(phi) * std::sin(the) * std::sin(psi);
  q.y = std::cos(phi) * std::sin(the) * std::cos(psi) + std::sin(phi) * std::cos(the) * std::sin(psi);
  q.z = std::cos(phi) * std::cos(the) * std::sin(psi) - std::sin(phi) * std::sin(the) * std::cos(psi);
  q.w = std::cos(phi) * std::cos(the) * std::cos(psi) + std::sin(phi) * std::sin(the) * std::sin(psi);
  return q;
}

// algorithm.cpp:50-86
static inline void approx_sin_cos(double x, double& s, double& c) {
  constexpr double coeff2 = 1.0 / (1.0 * 2.0);
  constexpr double coeff3 = 1.0 / (1.0 * 2.0 * 3.0);
  constexpr double coeff4 = 1.0 / (1.0 * 2.0 * 3.0 * 4.0);
  constexpr double coeff5 = 1.0 / (1.0 * 2.0 * 3.0 * 4.0 * 5.0);
  constexpr double coeff6 = 1.0 / (1.0 * 2.0 * 3.0 * 4.0 * 5.0 * 6.0);
  constexpr double coeff7 = 1.0 / (1.0 * 2.0 * 3.0 * 4.0 * 5.0 * 6.0 * 7.0);
  constexpr double coeff8 = 1.0 / (1.0 * 2.0 * 3.0 * 4.0 * 5.0 * 6.0 * 7.0 * 8.0);
  constexpr double coeff9 = 1.0 / (1.0 * 2.0 * 3.0 * 4.0 * 5.0 * 6.0 * 7.0 * 8.0 * 9.0);
  constexpr double pi = 3.14159265358979323846;
  constexpr double half_pi = pi * 0.5;
  constexpr double one_dev_2pi = 1.0 / (2 * pi);
  double cos_sign = 1.0;
  if (x > half_pi || x < -half_pi) {
    if (x > pi || x < -pi) x = x - 2 * pi * std::floor(x * one_dev_2pi + 0.5);
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

// ---------------------------------------------------------------- kinematic model
enum JType { J_UNKNOWN = 0, J_REVOLUTE = 1, J_CONTINUOUS = 2, J_PRISMATIC = 3, J_FLOATING = 4, J_PLANAR = 5, J_FIXED = 6 };
enum BaseType { B_FIXED = 0, B_FLOATING = 1, B_PLANAR = 2 };

struct UrdfJoint {
  std::string name;
  int type;
  int parent, child;  // link indices in the caller's link list
  double xyz[3];
  double rpy[3];
  bool has_rpy;
  double axis[3];
  double lower, upper;
};

// Immutable structure of kinematics.hpp:51-169 / kinematics.cpp:29-223.
struct Model {
  int n_link = 0, root = 0;
  std::map<std::string, int> link_id;
  std::vector<std::string> link_name;  // by id
  std::vector<int> parent;             // by id; -1 for root
  std::vector<std::vector<int>> children;
  std::vector<int> jtype;
  std::vector<V3> jaxis, jpos;
  std::vector<Q4> jquat;
  std::vector<bool> jqid;
  bool all_qid = true;
  std::vector<int> jchild;
  std::vector<double> jlower, jupper;
  std::map<std::string, int> joint_id;
  std::vector<QT> tf_init;                   // tf_plink_to_hlink_cache_ at construction
  std::vector<std::vector<char>> rptable;    // [link][joint]
};

// Mutable per-thread state: joint angles, local transforms and the lazy link-pose cache.
struct KinState {
  std::vector<double> angles;
  std::vector<QT> tf_local;  // tf_plink_to_hlink_cache_
  std::vector<QT> cache;
  std::vector<char> cached;
  QT base;
  void clear_cache(const Model& m) {  // kinematics.hpp:116-119
    std::fill(cached.begin(), cached.end(), 0);
    cache[m.root] = base;
    cached[m.root] = 1;
  }
};

static Model build_model(const std::vector<std::string>& names, const std::vector<UrdfJoint>& joints_in) {
  // urdfdom initTree / initRoot: children are attached in joint-name order.
  std::map<std::string, const UrdfJoint*> jmap;
  for (auto& j : joints_in) {
    if (jmap.count(j.name)) throw std::runtime_error("duplicate joint name " + j.name);
    jmap[j.name] = &j;
  }
  size_t nl = names.size();
  std::vector<int> par(nl, -1);
  std::vector<const UrdfJoint*> pjoint(nl, nullptr);
  std::vector<std::vector<int>> child_links(nl);
  std::vector<std::vector<const UrdfJoint*>> child_joints(nl);
  for (auto& kv : jmap) {
    const UrdfJoint* j = kv.second;
    par[j->child] = j->parent;
    pjoint[j->child] = j;
    child_joints[j->parent].push_back(j);
    child_links[j->parent].push_back(j->child);
  }
  std::map<std::string, int> by_name;
  for (size_t i = 0; i < nl; i++) by_name[names[i]] = (int)i;
  int root_in = -1;
  for (auto& kv : by_name) {
    if (par[kv.second] == -1) {
      if (root_in != -1) throw std::runtime_error("two root links");
      root_in = kv.second;
    }
  }
  if (root_in < 0) throw std::runtime_error("no root link");

  Model m;
  // kinematics.cpp:192-206 (stack DFS link numbering)
  std::vector<int> order;
  std::vector<int> new_id(nl, -1);
  std::vector<int> stack{root_in};
  while (!stack.empty()) {
    int l = stack.back();
    stack.pop_back();
    new_id[l] = (int)order.size();
    order.push_back(l);
    for (int c : child_links[l]) stack.push_back(c);
  }
  m.n_link = (int)order.size();
  m.root = 0;
  m.link_name.resize(m.n_link);
  m.parent.assign(m.n_link, -1);
  m.children.resize(m.n_link);
  for (int id = 0; id < m.n_link; id++) {
    int l = order[id];
    m.link_name[id] = names[l];
    m.link_id[names[l]] = id;
    m.parent[id] = par[l] < 0 ? -1 : new_id[par[l]];
    for (int c : child_links[l]) m.children[id].push_back(new_id[c]);
  }
  // kinematics.cpp:66-145 (stack DFS joint numbering)
  std::vector<const UrdfJoint*> jstack;
  for (auto* j : child_joints[root_in]) jstack.push_back(j);
  int counter = 0;
  while (!jstack.empty()) {
    const UrdfJoint* j = jstack.back();
    jstack.pop_back();
    int t = j->type;
    if (t == J_REVOLUTE || t == J_CONTINUOUS || t == J_PRISMATIC) {
      m.jtype.push_back(t);
      m.jaxis.push_back({j->axis[0], j->axis[1], j->axis[2]});
      m.jpos.push_back({j->xyz[0], j->xyz[1], j->xyz[2]});
      Q4 q;  // urdfdom Rotation: identity unless rpy given; RPY -> quaternion -> normalise
      if (j->has_rpy) {
        q = quat_from_rpy(j->rpy[0], j->rpy[1], j->rpy[2]);
        double s = std::sqrt(q.x * q.x + q.y * q.y + q.z * q.z + q.w * q.w);
        if (s == 0.0) {
          q = Q4{};
        } else {
          q.x /= s;
          q.y /= s;
          q.z /= s;
          q.w /= s;
        }
      }
      m.jquat.push_back(q);
      bool qid = std::abs(q.w - 1.0) < 1e-6;
      m.jqid.push_back(qid);
      m.jchild.push_back(new_id[j->child]);
      m.joint_id[j->name] = counter;
      if (t == J_CONTINUOUS) {
        m.jlower.push_back(-std::numeric_limits<double>::infinity());
        m.jupper.push_back(std::numeric_limits<double>::infinity());
      } else {
        m.jlower.push_back(j->lower);
        m.jupper.push_back(j->upper);
      }
      counter++;
    }
    for (auto* cj : child_joints[j->child]) jstack.push_back(cj);
  }
  m.all_qid = true;
  for (bool f : m.jqid) m.all_qid = m.all_qid && f;
  // kinematics.cpp:147-181
  m.tf_init.resize(m.n_link);
  for (int id = 0; id < m.n_link; id++) {
    const UrdfJoint* j = pjoint[order[id]];
    if (!j) continue;
    QT tf;
    tf.t = {j->xyz[0], j->xyz[1], j->xyz[2]};
    Q4 q;
    if (j->has_rpy) {
      q = quat_from_rpy(j->rpy[0], j->rpy[1], j->rpy[2]);
      double s = std::sqrt(q.x * q.x + q.y * q.y + q.z * q.z + q.w * q.w);
      if (s == 0.0) {
        q = Q4{};
      } else {
        q.x /= s;
        q.y /= s;
        q.z /= s;
        q.w /= s;
      }
    }
    tf.q = q;
    tf.qid = std::abs(q.w - 1.0) < 1e-6;
    m.tf_init[id] = tf;
  }
  // kinematics.cpp:340-363
  int nd = (int)m.jtype.size();
  m.rptable.assign(m.n_link, std::vector<char>(nd, 0));
  for (int jid = 0; jid < nd; jid++) {
    std::vector<int> st{m.jchild[jid]};
    while (!st.empty()) {
      int h = st.back();
      st.pop_back();
      m.rptable[h][jid] = 1;
      for (int c : m.children[h]) st.push_back(c);
    }
  }
  return m;
}

static KinState new_state(const Model& m) {
  KinState s;
  s.angles.assign(m.jtype.size(), 0.0);
  s.tf_local = m.tf_init;
  s.cache.resize(m.n_link);
  s.cached.assign(m.n_link, 0);
  s.base = QT{};  // Transform::Identity()
  s.clear_cache(m);
  return s;
}

// algorithm.cpp:88-158
static void set_joint_angles(const Model& m, KinState& s, const std::vector<int>& ids, const double* q, bool high_accuracy) {
  for (size_t i = 0; i < ids.size(); i++) {
    int jid = ids[i];
    s.angles[jid] = q[i];
    QT& tf = s.tf_local[m.jchild[jid]];
    const V3& pos = m.jpos[jid];
    if (m.jtype[jid] != J_PRISMATIC) {
      double x = q[i] * 0.5;
      double sn, cs;
      if (high_accuracy) {
        sn = std::sin(x);
        cs = std::cos(x);
      } else {
        approx_sin_cos(x, sn, cs);
      }
      Q4 jq{sn * m.jaxis[jid].x, sn * m.jaxis[jid].y, sn * m.jaxis[jid].z, cs};
      if (m.all_qid) {
        tf.q = jq;
      } else {
        tf.q = m.jqid[jid] ? jq : qmul(m.jquat[jid], jq);
      }
      tf.t = pos;
      tf.qid = false;
    } else {
      V3 tr{m.jaxis[jid].x * q[i], m.jaxis[jid].y * q[i], m.jaxis[jid].z * q[i]};
      tf.t = add(pos, tr);
      tf.q = Q4{};
      tf.qid = true;
    }
  }
  s.clear_cache(m);
}

// algorithm.cpp:160-210 (links are always "consider rotation" here)
static const QT& link_pose(const Model& m, KinState& s, int link) {
  if (s.cached[link]) return s.cache[link];
  int stack[256];
  int idx = 0;
  int h = link;
  while (!s.cached[h]) {
    stack[idx++] = h;
    h = m.parent[h];
  }
  int hid = h;
  while (idx > 0) {
    int prev = hid;
    hid = stack[--idx];
    mult_assign(s.cache[prev], s.tf_local[hid], s.cache[hid]);
    s.cached[hid] = 1;
  }
  return s.cache[link];
}

static void set_base_pose(const Model& m, KinState& s, const QT& p) {
  s.base = p;
  s.clear_cache(m);
}

// constraints/primitive.hpp:38-62
static void update_kintree(const Model& m, KinState& s, const std::vector<int>& ids, int base_type, const double* q, bool high_accuracy) {
  if (base_type != B_FIXED) {
    size_t n = ids.size();
    set_joint_angles(m, s, ids, q, true);
    QT pose;
    if (base_type == B_FLOATING) {
      pose.t = {q[n], q[n + 1], q[n + 2]};
      pose.q = quat_from_rpy(q[n + 3], q[n + 4], q[n + 5]);
    } else {
      pose.t = {q[n], q[n + 1], 0.0};
      pose.q = quat_from_rpy(0, 0, q[n + 2]);
    }
    set_base_pose(m, s, pose);
  } else {
    set_joint_angles(m, s, ids, q, high_accuracy);
  }
}

// algorithm.cpp:346-433: 3 x dof, column-major storage jac[c*3 + r]
static void attached_point_jacobian(const Model& m, KinState& s, int plink, const V3& p, const std::vector<int>& ids, int base_type,
                                    std::vector<double>& jac) {
  size_t nj = ids.size();
  size_t dof = nj + (base_type == B_FLOATING) * 6 + (base_type == B_PLANAR) * 3;
  jac.assign(3 * dof, 0.0);
  for (size_t i = 0; i < nj; i++) {
    int jid = ids[i];
    if (!m.rptable[plink][jid]) continue;
    const QT& tc = link_pose(m, s, m.jchild[jid]);
    V3 wa = qrot(tc.q, m.jaxis[jid]);
    V3 d;
    if (m.jtype[jid] == J_PRISMATIC) {
      d = wa;
    } else {
      d = cross(wa, sub(p, tc.t));
    }
    jac[i * 3 + 0] = d.x;
    jac[i * 3 + 1] = d.y;
    jac[i * 3 + 2] = d.z;
  }
  if (base_type == B_FIXED) return;
  QT te;  // Transform::Identity() with the point as translation (flag stays false)
  te.t = p;
  QT tb = link_pose(m, s, m.root);
  QT tbinv = inverse(tb);
  V3 rpy = get_rpy(tb.q);
  QT tbe = mul(tbinv, te);
  const double eps = 1e-7;
  if (base_type == B_FLOATING) {
    jac[(nj + 0) * 3 + 0] = 1.0;
    jac[(nj + 1) * 3 + 1] = 1.0;
    jac[(nj + 2) * 3 + 2] = 1.0;
    for (int k = 0; k < 3; k++) {
      V3 r2 = rpy;
      r2[k] += eps;
      QT tw = tb;
      tw.q = quat_from_rpy(r2.x, r2.y, r2.z);
      QT out = mul(tw, tbe);
      V3 dp = sub(out.t, te.t);
      for (int r = 0; r < 3; r++) jac[(nj + 3 + k) * 3 + r] = dp[r] / eps;
    }
  } else {
    jac[(nj + 0) * 3 + 0] = 1.0;
    jac[(nj + 1) * 3 + 1] = 1.0;
    V3 r2 = rpy;
    r2.z += eps;
    QT tw = tb;
    tw.q = quat_from_rpy(r2.x, r2.y, r2.z);
    QT out = mul(tw, tbe);
    V3 dp = sub(out.t, te.t);
    for (int r = 0; r < 3; r++) jac[(nj + 2) * 3 + r] = dp[r] / eps;
  }
}

// ---------------------------------------------------------------- SDFs (primitive_sdf.hpp)
struct Pose {  // :30-75
  V3 pos;
  M3 rot, rot_inv;
  bool axis_aligned = false, z_axis_aligned = false;
  void set(const V3& p, const M3& r) {
    pos = p;
    rot = r;
    update();
  }
  void update() {
    const M3& R = rot;
    double cof[3][3];
    cof[0][0] = R.m[1][1] * R.m[2][2] - R.m[1][2] * R.m[2][1];
    cof[0][1] = R.m[1][2] * R.m[2][0] - R.m[1][0] * R.m[2][2];
    cof[0][2] = R.m[1][0] * R.m[2][1] - R.m[1][1] * R.m[2][0];
    cof[1][0] = R.m[0][2] * R.m[2][1] - R.m[0][1] * R.m[2][2];
    cof[1][1] = R.m[0][0] * R.m[2][2] - R.m[0][2] * R.m[2][0];
    cof[1][2] = R.m[0][1] * R.m[2][0] - R.m[0][0] * R.m[2][1];
    cof[2][0] = R.m[0][1] * R.m[1][2] - R.m[0][2] * R.m[1][1];
    cof[2][1] = R.m[0][2] * R.m[1][0] - R.m[0][0] * R.m[1][2];
    cof[2][2] = R.m[0][0] * R.m[1][1] - R.m[0][1] * R.m[1][0];
    double det = R.m[0][0] * cof[0][0] + R.m[0][1] * cof[0][1] + R.m[0][2] * cof[0][2];
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) rot_inv.m[i][j] = cof[j][i] / det;
    double d2 = 0, n2 = 0;
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) {
        double e = R.m[i][j] - (i == j ? 1.0 : 0.0);
        d2 += e * e;
        n2 += R.m[i][j] * R.m[i][j];
      }
    axis_aligned = d2 <= 1e-12 * 1e-12 * std::min(n2, 3.0);  // Eigen isApprox, dummy_precision 1e-12
    if (axis_aligned) {
      z_axis_aligned = true;
    } else {
      double tol = 1e-6;
      z_axis_aligned = (std::abs(R.m[2][2] - 1.0) < tol) && (std::abs(R.m[0][2]) < tol) && (std::abs(R.m[1][2]) < tol) &&
                       (std::abs(R.m[2][0]) < tol) && (std::abs(R.m[2][1]) < tol);
    }
  }
  void translate(const V3& t) { pos = add(pos, t); }
  void rotate_z(double a) {  // :45-53
    double c = std::cos(a), s = std::sin(a);
    M3 rz{{{c, -s, 0}, {s, c, 0}, {0, 0, 1}}};
    M3 r;
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) r.m[i][j] = rz.m[i][0] * rot.m[0][j] + (rz.m[i][1] * rot.m[1][j] + rz.m[i][2] * rot.m[2][j]);
    rot = r;
    update();
  }
};

struct KD;

enum SdfKind { S_UNION = 0, S_BOX = 1, S_CYLINDER = 2, S_SPHERE = 3, S_GROUND = 4, S_CLOUD = 5 };

struct Sdf {
  int kind;
  V3 lb, ub;
  Pose pose;
  double w[3] = {0, 0, 0}, hw[3] = {0, 0, 0};  // box
  double r = 0, rsq = 0, h = 0, hh = 0;        // cylinder / sphere / ground height / cloud radius
  std::shared_ptr<KD> kd;
  std::vector<std::shared_ptr<Sdf>> members;  // union
  void update_aabb();
  double evaluate(const V3& p) const;
  bool is_outside(const V3& p, double radius) const;
  bool is_outside_aabb(const V3& p, double radius) const {  // :180-184
    return p.x < lb.x - radius || p.x > ub.x + radius || p.y < lb.y - radius || p.y > ub.y + radius || p.z < lb.z - radius ||
           p.z > ub.z + radius;
  }
};

// collision/kdtree.cpp:20-96
struct KD {
  struct Node {
    V3 p;
    int axis, left, right;
  };
  std::vector<Node> nodes;
  int root = -1;
  explicit KD(std::vector<V3> pts) {
    nodes.reserve(pts.size());
    root = build(pts.begin(), pts.end(), 0);
  }
  int build(std::vector<V3>::iterator b, std::vector<V3>::iterator e, int depth) {
    if (b >= e) return -1;
    int axis = depth % 3;
    auto n = std::distance(b, e);
    auto mid = b + n / 2;
    std::nth_element(b, mid, e, [axis](const V3& a, const V3& c) { return a[axis] < c[axis]; });
    nodes.push_back({*mid, axis, -1, -1});
    int idx = (int)nodes.size() - 1;
    int l = build(b, mid, depth + 1);
    nodes[idx].left = l;
    int r = build(mid + 1, e, depth + 1);
    nodes[idx].right = r;
    return idx;
  }
  void nearest(int ni, const V3& t, double& best, V3& bp) const {
    if (ni == -1) return;
    const Node& nd = nodes[ni];
    double d = sqn(sub(nd.p, t));
    if (d < best) {
      best = d;
      bp = nd.p;
    }
    double diff = t[nd.axis] - nd.p[nd.axis];
    int first = diff < 0 ? nd.left : nd.right;
    int second = diff < 0 ? nd.right : nd.left;
    nearest(first, t, best, bp);
    if (diff * diff < best) nearest(second, t, best, bp);
  }
  double sqdist(const V3& t, V3* bp_out = nullptr) const {
    double best = std::numeric_limits<double>::max();
    V3 bp;
    nearest(root, t, best, bp);
    if (bp_out) *bp_out = bp;
    return best;
  }
};

void Sdf::update_aabb() {
  if (kind == S_BOX || kind == S_CYLINDER) {  // :400-421, :500-521
    double ex = kind == S_BOX ? w[0] * 0.5 : r, ey = kind == S_BOX ? w[1] * 0.5 : r, ez = kind == S_BOX ? w[2] * 0.5 : hh;
    double sx[8] = {-ex, ex, -ex, ex, -ex, ex, -ex, ex};
    double sy[8] = {-ey, -ey, ey, ey, -ey, -ey, ey, ey};
    double sz[8] = {-ez, -ez, -ez, -ez, ez, ez, ez, ez};
    for (int k = 0; k < 8; k++) {
      V3 v = add(mv(pose.rot, V3{sx[k], sy[k], sz[k]}), pose.pos);
      for (int a = 0; a < 3; a++) {
        if (k == 0 || v[a] < lb[a]) lb[a] = v[a];
        if (k == 0 || v[a] > ub[a]) ub[a] = v[a];
      }
    }
  } else if (kind == S_SPHERE) {  // :558-561
    lb = sub(pose.pos, V3{r, r, r});
    ub = add(pose.pos, V3{r, r, r});
  } else if (kind == S_GROUND) {  // :250-255
    double inf = std::numeric_limits<double>::infinity();
    lb = {-inf, -inf, 0.0};
    ub = {inf, inf, 0.0};
  }
}

double Sdf::evaluate(const V3& p) const {
  switch (kind) {
    case S_UNION: {  // :155-161
      double v = std::numeric_limits<double>::max();
      for (auto& s : members) v = std::min(v, s->evaluate(p));
      return v;
    }
    case S_BOX: {  // :299-311
      V3 d = sub(p, pose.pos);
      V3 loc = pose.axis_aligned ? d : mv(pose.rot_inv, d);
      V3 sd{std::abs(loc.x) - hw[0], std::abs(loc.y) - hw[1], std::abs(loc.z) - hw[2]};
      V3 mpos{std::max(sd.x, 0.0), std::max(sd.y, 0.0), std::max(sd.z, 0.0)};
      double out = nrm(mpos);
      double in = std::max(std::min(sd.x, 0.0), std::max(std::min(sd.y, 0.0), std::min(sd.z, 0.0)));
      return out + in;
    }
    case S_CYLINDER: {  // :444-462
      double zs, xa, ya;
      if (pose.z_axis_aligned) {
        zs = std::abs(p.z - pose.pos.z) - hh;
        xa = std::abs(p.x - pose.pos.x);
        ya = std::abs(p.y - pose.pos.y);
      } else {
        V3 d = sub(p, pose.pos);
        zs = std::abs(dot(d, col(pose.rot, 2))) - hh;
        xa = std::abs(dot(d, col(pose.rot, 0)));
        ya = std::abs(dot(d, col(pose.rot, 1)));
      }
      double rs = std::sqrt(xa * xa + ya * ya) - r;
      double a = std::max(rs, 0.0), b = std::max(zs, 0.0);
      double out = std::sqrt(a * a + b * b);
      double in = std::max(std::min(rs, 0.0), std::min(zs, 0.0));
      return out + in;
    }
    case S_SPHERE:  // :540-544
      return nrm(sub(p, pose.pos)) - r;
    case S_GROUND:  // :245
      return p.z + h;
    case S_CLOUD:  // :597-599
      return std::sqrt(kd->sqdist(p)) - r;
  }
  return 0;
}

bool Sdf::is_outside(const V3& p, double radius) const {
  switch (kind) {
    case S_UNION:  // :163-170
      for (auto& s : members)
        if (!s->is_outside(p, radius)) return false;
      return true;
    case S_BOX: {  // :313-398
      double xs, ys, zs;
      if (pose.axis_aligned) {
        xs = std::abs(p.x - pose.pos.x) - hw[0];
        if (xs > radius) return true;
        ys = std::abs(p.y - pose.pos.y) - hw[1];
        if (ys > radius) return true;
        zs = std::abs(p.z - pose.pos.z) - hw[2];
        if (zs > radius) return true;
      } else if (pose.z_axis_aligned) {
        zs = std::abs(p.z - pose.pos.z) - hw[2];
        if (zs > radius) return true;
        V3 d = sub(p, pose.pos);
        xs = std::abs(dot(d, col(pose.rot, 0))) - hw[0];
        if (xs > radius) return true;
        ys = std::abs(dot(d, col(pose.rot, 1))) - hw[1];
        if (ys > radius) return true;
      } else {
        V3 d = sub(p, pose.pos);
        xs = std::abs(dot(d, col(pose.rot, 0))) - hw[0];
        if (xs > radius) return true;
        ys = std::abs(dot(d, col(pose.rot, 1))) - hw[1];
        if (ys > radius) return true;
        zs = std::abs(dot(d, col(pose.rot, 2))) - hw[2];
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
    case S_CYLINDER: {  // :464-498
      double zs, xa, ya;
      if (pose.z_axis_aligned) {
        zs = std::abs(p.z - pose.pos.z) - hh;
        if (zs > radius) return true;
        xa = std::abs(p.x - pose.pos.x);
        ya = std::abs(p.y - pose.pos.y);
      } else {
        V3 d = sub(p, pose.pos);
        zs = std::abs(dot(d, col(pose.rot, 2))) - hh;
        if (zs > radius) return true;
        xa = std::abs(dot(d, col(pose.rot, 0)));
        ya = std::abs(dot(d, col(pose.rot, 1)));
      }
      double dsq = xa * xa + ya * ya;
      if (radius < 1e-6) return dsq > rsq;
      if (dsq > (r + radius) * (r + radius)) return true;
      bool ho = zs > 0, ro = dsq > rsq;
      if (ho && ro) {
        double rs = std::sqrt(dsq) - r;
        return zs * zs + rs * rs > radius * radius;
      }
      return false;
    }
    case S_SPHERE:  // :546-552
      if (radius < 1e-6) return sqn(sub(p, pose.pos)) > rsq;
      return sqn(sub(p, pose.pos)) > (r + radius) * (r + radius);
    case S_GROUND:  // :246-248
      return p.z + h > radius;
    case S_CLOUD:  // :601-603
      return evaluate(p) > radius;
  }
  return true;
}

// ---------------------------------------------------------------- sphere collision constraint
struct Group {  // primitive_sphere_collision.hpp:23-53
  std::string link_name;
  int link = 0;
  std::vector<V3> rel;
  std::vector<double> radii;
  double group_radius = 0;
  bool only_self = false;
  V3 group_rel;
};

struct Cst {
  const Model* m = nullptr;
  std::vector<int> ids;
  int base_type = B_FIXED;
  std::vector<Group> groups;
  std::vector<std::pair<int, int>> pairs;
  std::shared_ptr<Sdf> fixed_sdf, sdf;
  std::vector<const Sdf*> all;  // flattened primitives (set_all_sdfs, :426-448)
  double cutoff = 0.1;
  size_t q_dim() const { return ids.size() + (base_type == B_FLOATING) * 6 + (base_type == B_PLANAR) * 3; }
  size_t cst_dim() const { return (all.empty() ? 0 : 1) + (pairs.empty() ? 0 : 1); }
  void flatten(const std::shared_ptr<Sdf>& s) {
    if (s->kind == S_UNION) {
      for (auto& c : s->members) flatten(c);
    } else {
      all.push_back(s.get());
    }
  }
  void set_all() {
    all.clear();
    if (fixed_sdf) flatten(fixed_sdf);
    if (sdf) flatten(sdf);
  }
};

// :53-96 (visit order = libstdc++ unordered_set order: descending index)
static std::vector<size_t> farthest_order(const std::vector<V3>& pos) {
  size_t n = pos.size();
  std::vector<size_t> visited;
  std::vector<size_t> unvisited;  // kept in iteration order (descending)
  for (size_t i = n; i-- > 0;) unvisited.push_back(i);
  if (n == 0) return visited;
  visited.push_back(unvisited.front());
  unvisited.erase(unvisited.begin());
  for (size_t it = 0; it + 1 < n; it++) {
    double max_dist = 0.0;
    size_t best = 0;
    for (size_t k = 0; k < unvisited.size(); k++) {
      double md = std::numeric_limits<double>::max();
      for (size_t v : visited) {
        double d = nrm(sub(pos[unvisited[k]], pos[v]));
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

static void reorder(Group& g) {  // :98-115
  auto ord = farthest_order(g.rel);
  std::vector<V3> r2(g.rel.size());
  std::vector<double> rad2(g.rel.size());
  for (size_t i = 0; i < ord.size(); i++) {
    r2[i] = g.rel[ord[i]];
    rad2[i] = g.radii[ord[i]];
  }
  g.rel = r2;
  g.radii = rad2;
}

// Per-thread caches of SphereGroup (:23-51) plus the kinematic state.
struct CstState {
  KinState kin;
  std::vector<M3> rot;
  std::vector<V3> gpos;
  std::vector<char> gdirty, sdirty;
  std::vector<std::vector<V3>> spos;
  std::vector<double> jtmp, jtmp2;
};

static CstState new_cst_state(const Cst& c) {
  CstState st;
  st.kin = new_state(*c.m);
  size_t ng = c.groups.size();
  st.rot.resize(ng);
  st.gpos.resize(ng);
  st.gdirty.assign(ng, 1);
  st.sdirty.assign(ng, 1);
  st.spos.resize(ng);
  for (size_t i = 0; i < ng; i++) st.spos[i].resize(c.groups[i].rel.size());
  return st;
}

static inline void group_cache(const Cst& c, CstState& st, size_t gi) {  // :26-36
  if (!st.gdirty[gi]) return;
  const Group& g = c.groups[gi];
  QT pose = link_pose(*c.m, st.kin, g.link);
  st.rot[gi] = qmat(pose.q);
  st.gpos[gi] = add(mv(st.rot[gi], g.group_rel), pose.t);
  st.gdirty[gi] = 0;
}
static inline void sphere_cache(const Cst& c, CstState& st, size_t gi) {  // :38-51
  if (!st.sdirty[gi]) return;
  const Group& g = c.groups[gi];
  const V3& t = st.kin.cache[g.link].t;
  for (size_t i = 0; i < g.rel.size(); i++) st.spos[gi][i] = add(mv(st.rot[gi], g.rel[i]), t);
  st.sdirty[gi] = 0;
}
static inline void post_update(CstState& st) {
  std::fill(st.gdirty.begin(), st.gdirty.end(), 1);
  std::fill(st.sdirty.begin(), st.sdirty.end(), 1);
}

static bool check_ext(const Cst& c, CstState& st) {  // :191-220
  for (size_t gi = 0; gi < c.groups.size(); gi++) {
    const Group& g = c.groups[gi];
    if (g.only_self) continue;
    group_cache(c, st, gi);
    for (const Sdf* s : c.all) {
      if (!s->is_outside_aabb(st.gpos[gi], g.group_radius)) {
        if (!s->is_outside(st.gpos[gi], g.group_radius)) {
          sphere_cache(c, st, gi);
          for (size_t i = 0; i < g.radii.size(); i++) {
            if (!s->is_outside_aabb(st.spos[gi][i], g.radii[i])) {
              if (!s->is_outside(st.spos[gi][i], g.radii[i])) return false;
            }
          }
        }
      }
    }
  }
  return true;
}

static bool check_self(const Cst& c, CstState& st) {  // :222-254
  for (auto& pr : c.pairs) {
    const Group& g1 = c.groups[pr.first];
    const Group& g2 = c.groups[pr.second];
    group_cache(c, st, pr.first);
    group_cache(c, st, pr.second);
    double osq = sqn(sub(st.gpos[pr.first], st.gpos[pr.second]));
    double ors = g1.group_radius + g2.group_radius;
    if (osq > ors * ors) continue;
    sphere_cache(c, st, pr.first);
    sphere_cache(c, st, pr.second);
    for (size_t i = 0; i < g1.radii.size(); i++) {
      for (size_t j = 0; j < g2.radii.size(); j++) {
        double sq = sqn(sub(st.spos[pr.first][i], st.spos[pr.second][j]));
        double rs = g1.radii[i] + g2.radii[j];
        if (sq < rs * rs) return false;
      }
    }
  }
  return true;
}

static bool is_valid(const Cst& c, CstState& st, const double* q) {  // primitive.hpp:113-117, :181-189
  update_kintree(*c.m, st.kin, c.ids, c.base_type, q, false);
  post_update(st);
  if (!c.all.empty() && !check_ext(c, st)) return false;
  if (!c.pairs.empty()) return check_self(c, st);
  return true;
}

// :256-322
static double eval_ext(const Cst& c, CstState& st, double* grad) {
  size_t dof = c.q_dim();
  double minv = c.cutoff;
  int mg = -1, ms = -1, mk = -1;
  for (size_t i = 0; i < c.groups.size(); i++) {
    const Group& g = c.groups[i];
    if (g.only_self) continue;
    group_cache(c, st, i);
    for (size_t j = 0; j < c.all.size(); j++) {
      const Sdf* s = c.all[j];
      if (!s->is_outside_aabb(st.gpos[i], g.group_radius + c.cutoff)) {
        if (!s->is_outside(st.gpos[i], g.group_radius + c.cutoff)) {
          sphere_cache(c, st, i);
          for (size_t k = 0; k < g.radii.size(); k++) {
            const V3& sc = st.spos[i][k];
            if (s->is_outside_aabb(sc, g.radii[k] + c.cutoff)) continue;
            double v = s->evaluate(sc) - g.radii[k];
            if (v < minv) {
              minv = v;
              mg = (int)i;
              ms = (int)j;
              mk = (int)k;
            }
          }
        }
      }
    }
  }
  if (mg < 0) {
    for (size_t d = 0; d < dof; d++) grad[d] = 0.0;
    return minv;
  }
  const V3 sc = st.spos[mg][mk];
  double r = c.groups[mg].radii[mk];
  double g3[3];
  for (int i = 0; i < 3; i++) {
    V3 pc = sc;
    pc[i] += 1e-6;
    double v = c.all[ms]->evaluate(pc) - r;
    g3[i] = (v - minv) / 1e-6;
  }
  attached_point_jacobian(*c.m, st.kin, c.groups[mg].link, sc, c.ids, c.base_type, st.jtmp);
  for (size_t d = 0; d < dof; d++) grad[d] = st.jtmp[d * 3 + 0] * g3[0] + st.jtmp[d * 3 + 1] * g3[1] + st.jtmp[d * 3 + 2] * g3[2];
  return minv;
}

// :324-383
static double eval_self(const Cst& c, CstState& st, double* grad) {
  size_t dof = c.q_dim();
  double dmin = c.cutoff;
  int a = -1, ai = -1, b = -1, bj = -1;
  for (auto& pr : c.pairs) {
    const Group& g1 = c.groups[pr.first];
    const Group& g2 = c.groups[pr.second];
    group_cache(c, st, pr.first);
    group_cache(c, st, pr.second);
    double osq = sqn(sub(st.gpos[pr.first], st.gpos[pr.second]));
    double orm = g1.group_radius + g2.group_radius + c.cutoff;
    if (osq > orm * orm) continue;
    sphere_cache(c, st, pr.first);
    sphere_cache(c, st, pr.second);
    for (size_t i = 0; i < g1.radii.size(); i++) {
      for (size_t j = 0; j < g2.radii.size(); j++) {
        double d = nrm(sub(st.spos[pr.first][i], st.spos[pr.second][j])) - (g1.radii[i] + g2.radii[j]);
        if (d < dmin) {
          dmin = d;
          a = pr.first;
          ai = (int)i;
          b = pr.second;
          bj = (int)j;
        }
      }
    }
  }
  if (a < 0) {
    for (size_t d = 0; d < dof; d++) grad[d] = 0.0;
    return dmin;
  }
  V3 c1 = st.spos[a][ai], c2 = st.spos[b][bj];
  V3 cd = sub(c1, c2);
  attached_point_jacobian(*c.m, st.kin, c.groups[a].link, c1, c.ids, c.base_type, st.jtmp);
  attached_point_jacobian(*c.m, st.kin, c.groups[b].link, c2, c.ids, c.base_type, st.jtmp2);
  double ni = 1.0 / nrm(cd);
  for (size_t d = 0; d < dof; d++) {
    double s = cd.x * ni * (st.jtmp[d * 3 + 0] - st.jtmp2[d * 3 + 0]) + cd.y * ni * (st.jtmp[d * 3 + 1] - st.jtmp2[d * 3 + 1]) +
               cd.z * ni * (st.jtmp[d * 3 + 2] - st.jtmp2[d * 3 + 2]);
    grad[d] = s;
  }
  return dmin;
}

// primitive.hpp:74-79, :385-399; vals[cst_dim], jac[cst_dim * dof] row-major
static void evaluate(const Cst& c, CstState& st, const double* q, double* vals, double* jac) {
  update_kintree(*c.m, st.kin, c.ids, c.base_type, q, true);
  post_update(st);
  size_t head = 0, dof = c.q_dim();
  if (!c.all.empty()) {
    vals[head] = eval_ext(c, st, jac + head * dof);
    head++;
  }
  if (!c.pairs.empty()) vals[head] = eval_self(c, st, jac + head * dof);
}

// ---------------------------------------------------------------- motion validator
// ompl/generate_sequence.py:11-63
static std::vector<std::vector<int64_t>> make_sequence_table(int n_max) {
  std::vector<std::vector<int64_t>> tab;
  for (int n = 1; n <= n_max; n++) {
    std::vector<int64_t> res(n, 0);
    std::vector<char> used(n, 0);
    used[0] = 1;
    int cur = 1;
    for (int i = 1; i < n; i++) {
      long long best_md = -1, best = -1;
      for (int num = 0; num < n; num++) {
        if (used[num]) continue;
        long long md = std::numeric_limits<long long>::max();
        for (int j = 0; j < cur; j++) {
          long long d = std::llabs((long long)num - (long long)res[j]);
          if (d < md) md = d;
        }
        if (md > best_md || (md == best_md && num > best)) {
          best_md = md;
          best = num;
        }
      }
      res[i] = best;
      used[best] = 1;
      cur++;
    }
    tab.push_back(res);
  }
  return tab;
}

static const std::vector<std::vector<int64_t>>& seq_table() {
  static const auto tab = make_sequence_table(128);
  return tab;
}

struct Validator {
  int type = 0;  // 0 box, 1 euclidean
  std::vector<double> width, inv_width;
  double resolution = 0.05;
  double step_ratio(const double* s1, const double* s2, size_t dim) const {
    if (type == 0) {  // motion_validator.cpp:89-111
      double diff_long = 0.0, max_diff = -std::numeric_limits<double>::infinity();
      size_t li = 0;
      for (size_t i = 0; i < dim; i++) {
        double diff = s2[i] - s1[i];
        double asd = std::abs(diff) * inv_width[i];
        if (asd > max_diff) {
          max_diff = asd;
          li = i;
          diff_long = diff;
        }
      }
      if (std::abs(diff_long) < 1e-6) return std::numeric_limits<double>::infinity();
      return width[li] / std::abs(diff_long);
    }
    double dist = 0.0;  // motion_validator.cpp:118-126 with OMPL's Euclidean distance
    for (size_t i = 0; i < dim; i++) {
      double d = s1[i] - s2[i];
      dist += d * d;
    }
    return resolution / std::sqrt(dist);
  }
};

// motion_validator.cpp:17-79; waypoints_out counts isValid calls
static bool check_motion(const Cst& c, CstState& st, const Validator& v, const double* s1, const double* s2, std::vector<double>& tmp,
                         long long* n_checked) {
  size_t dim = c.q_dim();
  double sr = v.step_ratio(s1, s2, dim);
  if (sr == std::numeric_limits<double>::infinity()) return true;
  size_t n_test = (size_t)(std::floor(1 / sr) + 2);
  tmp.resize(dim);
  auto interp = [&](double t) {
    for (size_t i = 0; i < dim; i++) tmp[i] = s1[i] + (s2[i] - s1[i]) * t;
  };
  const auto& tab = seq_table();
  if (n_checked) (*n_checked)++;
  if (!is_valid(c, st, s2)) return false;
  if (n_test < tab.size() + 1) {
    const auto& seq = tab[n_test - 1];
    for (size_t i = 2; i < n_test; i++) {
      interp((double)seq[i] * sr);
      if (n_checked) (*n_checked)++;
      if (!is_valid(c, st, tmp.data())) return false;
    }
    return true;
  }
  for (size_t i = 1; i < n_test - 1; i++) {
    interp((double)i * sr);
    if (n_checked) (*n_checked)++;
    if (!is_valid(c, st, tmp.data())) return false;
  }
  return true;
}

// ---------------------------------------------------------------- link pose jacobian (algorithm.cpp:212-344), RotationType
static void rpy_derivative(const V3& rpy, const V3& axis, V3& out) {  // algorithm.cpp:20-32
  double a2 = -rpy.y, a3 = -rpy.z;
  out.x = std::cos(a3) / std::cos(a2) * axis.x - std::sin(a3) / std::cos(a2) * axis.y;
  out.y = std::sin(a3) * axis.x + std::cos(a3) * axis.y;
  out.z = -std::cos(a3) * std::sin(a2) / std::cos(a2) * axis.x + std::sin(a3) * std::sin(a2) / std::cos(a2) * axis.y + axis.z;
}
static Q4 q_derivative(const Q4& q, const V3& w) {  // algorithm.cpp:34-47
  const double dx = 0.5 * (w.z * q.y - w.y * q.z + w.x * q.w);
  const double dy = 0.5 * (-w.z * q.x + 0 * q.y + w.x * q.z + w.y * q.w);
  const double dz = 0.5 * (w.y * q.x - w.x * q.y + 0 * q.z + w.z * q.w);
  const double dw = 0.5 * (-w.x * q.x - w.y * q.y - w.z * q.z + 0 * q.w);
  Q4 r;
  r.w = -dw;
  r.x = dx;
  r.y = dy;
  r.z = dz;
  return r;
}

}  // namespace orc

// ================================================================ C ABI (ctypes)
using namespace orc;

static thread_local std::string g_err;

struct OrcModel {
  Model m;
  KinState s;
};
struct OrcSdf {
  std::shared_ptr<Sdf> p;
};
struct OrcCst {
  Cst c;
  OrcModel* om = nullptr;  // the shared KinematicModel (state included)
  CstState fresh() const {
    CstState st = new_cst_state(c);
    st.kin = om->s;
    return st;
  }
};

#define ORC_TRY(...)             \
  try {                          \
    __VA_ARGS__;                 \
    return 0;                    \
  } catch (std::exception & e) { \
    g_err = e.what();            \
    return 1;                    \
  }

extern "C" {

const char* orc_last_error() { return g_err.c_str(); }

// URDF is given pre-parsed (xml.etree on the Python side): link names, and per joint
// name/type/parent/child/xyz/rpy(+flag)/axis/limits.
int orc_model_create(int n_links, const char** link_names, int n_joints, const char** jnames, const int* jtypes, const int* jparent,
                     const int* jchild, const double* xyz, const double* rpy, const int* has_rpy, const double* axis, const double* lower,
                     const double* upper, void** out) {
  ORC_TRY({
    std::vector<std::string> names(link_names, link_names + n_links);
    std::vector<UrdfJoint> js(n_joints);
    for (int i = 0; i < n_joints; i++) {
      js[i].name = jnames[i];
      js[i].type = jtypes[i];
      js[i].parent = jparent[i];
      js[i].child = jchild[i];
      for (int k = 0; k < 3; k++) {
        js[i].xyz[k] = xyz[3 * i + k];
        js[i].rpy[k] = rpy[3 * i + k];
        js[i].axis[k] = axis[3 * i + k];
      }
      js[i].has_rpy = has_rpy[i] != 0;
      js[i].lower = lower[i];
      js[i].upper = upper[i];
    }
    auto* om = new OrcModel();
    om->m = build_model(names, js);
    om->s = new_state(om->m);
    *out = om;
  })
}
void orc_model_destroy(void* p) { delete (OrcModel*)p; }
int orc_model_counts(void* p, int* n_link, int* n_dof) {
  auto* om = (OrcModel*)p;
  *n_link = om->m.n_link;
  *n_dof = (int)om->m.jtype.size();
  return 0;
}
int orc_model_link_id(void* p, const char* name, int* out) {
  auto* om = (OrcModel*)p;
  auto it = om->m.link_id.find(name);
  if (it == om->m.link_id.end()) {
    g_err = std::string("no link named ") + name;
    return 1;
  }
  *out = it->second;
  return 0;
}
int orc_model_joint_id(void* p, const char* name, int* out) {
  auto* om = (OrcModel*)p;
  auto it = om->m.joint_id.find(name);
  if (it == om->m.joint_id.end()) {
    g_err = std::string("no joint named ") + name;
    return 1;
  }
  *out = it->second;
  return 0;
}
// structure dump: parent ids, joint child link ids, identity flags, local transforms
int orc_model_structure(void* p, int* parent, int* jchild, int* jqid, double* tf_local /*n_link*7*/, int* tf_qid) {
  auto* om = (OrcModel*)p;
  for (int i = 0; i < om->m.n_link; i++) {
    parent[i] = om->m.parent[i];
    const QT& t = om->m.tf_init[i];
    double v[7] = {t.t.x, t.t.y, t.t.z, t.q.x, t.q.y, t.q.z, t.q.w};
    std::memcpy(tf_local + 7 * i, v, sizeof(v));
    tf_qid[i] = t.qid;
  }
  for (size_t j = 0; j < om->m.jtype.size(); j++) {
    jchild[j] = om->m.jchild[j];
    jqid[j] = om->m.jqid[j];
  }
  return 0;
}
int orc_model_set_joint_positions(void* p, const int* ids, int n, const double* q, int accurate) {
  auto* om = (OrcModel*)p;
  std::vector<int> v(ids, ids + n);
  set_joint_angles(om->m, om->s, v, q, accurate != 0);
  return 0;
}
int orc_model_set_base_pose(void* p, const double* pose7) {
  auto* om = (OrcModel*)p;
  QT t;
  t.t = {pose7[0], pose7[1], pose7[2]};
  t.q = {pose7[3], pose7[4], pose7[5], pose7[6]};
  set_base_pose(om->m, om->s, t);
  return 0;
}
int orc_model_link_pose(void* p, int link, double* out7) {
  auto* om = (OrcModel*)p;
  const QT& t = link_pose(om->m, om->s, link);
  double v[7] = {t.t.x, t.t.y, t.t.z, t.q.x, t.q.y, t.q.z, t.q.w};
  std::memcpy(out7, v, sizeof(v));
  return 0;
}

int orc_sdf_box(const double* width, const double* pos, const double* rot, void** out) {
  ORC_TRY({
    auto* s = new OrcSdf{std::make_shared<Sdf>()};
    s->p->kind = S_BOX;
    M3 r;
    std::memcpy(r.m, rot, sizeof(r.m));
    s->p->pose.set({pos[0], pos[1], pos[2]}, r);
    for (int k = 0; k < 3; k++) {
      s->p->w[k] = width[k];
      s->p->hw[k] = 0.5 * width[k];
    }
    s->p->update_aabb();
    *out = s;
  })
}
int orc_sdf_cylinder(double radius, double height, const double* pos, const double* rot, void** out) {
  ORC_TRY({
    auto* s = new OrcSdf{std::make_shared<Sdf>()};
    s->p->kind = S_CYLINDER;
    M3 r;
    std::memcpy(r.m, rot, sizeof(r.m));
    s->p->pose.set({pos[0], pos[1], pos[2]}, r);
    s->p->r = radius;
    s->p->rsq = radius * radius;
    s->p->h = height;
    s->p->hh = 0.5 * height;
    s->p->update_aabb();
    *out = s;
  })
}
int orc_sdf_sphere(double radius, const double* pos, const double* rot, void** out) {
  ORC_TRY({
    auto* s = new OrcSdf{std::make_shared<Sdf>()};
    s->p->kind = S_SPHERE;
    M3 r;
    std::memcpy(r.m, rot, sizeof(r.m));
    s->p->pose.set({pos[0], pos[1], pos[2]}, r);
    s->p->r = radius;
    s->p->rsq = radius * radius;
    s->p->update_aabb();
    *out = s;
  })
}
int orc_sdf_ground(double height, void** out) {
  ORC_TRY({
    auto* s = new OrcSdf{std::make_shared<Sdf>()};
    s->p->kind = S_GROUND;
    s->p->h = height;
    s->p->update_aabb();
    *out = s;
  })
}
// points: n x 3 doubles (callers widen float32 clouds exactly)
int orc_sdf_cloud(const double* pts, long long n, double radius, void** out) {
  ORC_TRY({
    auto* s = new OrcSdf{std::make_shared<Sdf>()};
    s->p->kind = S_CLOUD;
    std::vector<V3> v(n);
    double inf = std::numeric_limits<double>::infinity();
    s->p->lb = {inf, inf, inf};
    s->p->ub = {-inf, -inf, -inf};
    for (long long i = 0; i < n; i++) {
      v[i] = {pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]};
      for (int k = 0; k < 3; k++) {
        s->p->lb[k] = std::min(s->p->lb[k], v[i][k]);
        s->p->ub[k] = std::max(s->p->ub[k], v[i][k]);
      }
    }
    for (int k = 0; k < 3; k++) {
      s->p->lb[k] -= radius;
      s->p->ub[k] += radius;
    }
    s->p->kd = std::make_shared<KD>(v);
    s->p->r = radius;
    *out = s;
  })
}
int orc_sdf_union(void** members, int n, void** out) {
  ORC_TRY({
    auto* s = new OrcSdf{std::make_shared<Sdf>()};
    s->p->kind = S_UNION;
    for (int i = 0; i < n; i++) s->p->members.push_back(((OrcSdf*)members[i])->p);
    *out = s;
  })
}
void orc_sdf_destroy(void* p) { delete (OrcSdf*)p; }
int orc_sdf_translate(void* p, const double* t) {
  auto* s = (OrcSdf*)p;
  std::vector<Sdf*> st{s->p.get()};
  while (!st.empty()) {
    Sdf* x = st.back();
    st.pop_back();
    if (x->kind == S_UNION) {
      for (auto& m : x->members) st.push_back(m.get());
    } else if (x->kind == S_BOX || x->kind == S_CYLINDER || x->kind == S_SPHERE) {
      x->pose.translate({t[0], t[1], t[2]});
      x->update_aabb();
    } else {
      g_err = "translate not supported";
      return 1;
    }
  }
  return 0;
}
int orc_sdf_rotate_z(void* p, double a) {
  auto* s = (OrcSdf*)p;
  std::vector<Sdf*> st{s->p.get()};
  while (!st.empty()) {
    Sdf* x = st.back();
    st.pop_back();
    if (x->kind == S_UNION) {
      for (auto& m : x->members) st.push_back(m.get());
    } else if (x->kind == S_BOX || x->kind == S_CYLINDER || x->kind == S_SPHERE) {
      x->pose.rotate_z(a);
      x->update_aabb();
    } else {
      g_err = "rotate_z not supported";
      return 1;
    }
  }
  return 0;
}
int orc_sdf_info(void* p, double* lb, double* ub, int* flags) {
  auto* s = (OrcSdf*)p;
  for (int k = 0; k < 3; k++) {
    lb[k] = s->p->lb[k];
    ub[k] = s->p->ub[k];
  }
  flags[0] = s->p->pose.axis_aligned;
  flags[1] = s->p->pose.z_axis_aligned;
  return 0;
}
int orc_sdf_evaluate(void* p, const double* pts, long long n, double* out) {
  auto* s = (OrcSdf*)p;
  for (long long i = 0; i < n; i++) out[i] = s->p->evaluate({pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]});
  return 0;
}
int orc_sdf_is_outside(void* p, const double* pts, long long n, const double* radii, unsigned char* out) {
  auto* s = (OrcSdf*)p;
  for (long long i = 0; i < n; i++) out[i] = s->p->is_outside({pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]}, radii[i]);
  return 0;
}
int orc_sdf_is_outside_aabb(void* p, const double* pts, long long n, const double* radii, unsigned char* out) {
  auto* s = (OrcSdf*)p;
  for (long long i = 0; i < n; i++) out[i] = s->p->is_outside_aabb({pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]}, radii[i]);
  return 0;
}
// KD-tree on its own: nearest squared distance and point
int orc_cloud_nearest(void* p, const double* pts, long long n, double* sq, double* near) {
  auto* s = (OrcSdf*)p;
  if (s->p->kind != S_CLOUD) {
    g_err = "not a cloud";
    return 1;
  }
  for (long long i = 0; i < n; i++) {
    V3 bp;
    sq[i] = s->p->kd->sqdist({pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]}, &bp);
    if (near) {
      near[3 * i] = bp.x;
      near[3 * i + 1] = bp.y;
      near[3 * i + 2] = bp.z;
    }
  }
  return 0;
}

// SphereCollisionCst(kin, joints, base, specs, pairs, fixed_sdf, reorder) -- :117-179
int orc_cst_create(void* model, const char** joints, int n_joints, int base_type, int n_specs, const char** spec_links, const int* counts,
                   const double* rel /*3 x total, column per sphere*/, const double* radii, const int* only_self, int n_pairs,
                   const char** pair_a, const char** pair_b, void* fixed_sdf, int reorder_spheres, void** out) {
  ORC_TRY({
    auto* om = (OrcModel*)model;
    auto* oc = new OrcCst();
    oc->c.m = &om->m;
    oc->om = om;
    for (int i = 0; i < n_joints; i++) {
      auto it = om->m.joint_id.find(joints[i]);
      if (it == om->m.joint_id.end()) {
        delete oc;
        throw std::invalid_argument(std::string("no joint named ") + joints[i]);
      }
      oc->c.ids.push_back(it->second);
    }
    oc->c.base_type = base_type;
    size_t off = 0;
    for (int s = 0; s < n_specs; s++) {
      Group g;
      g.link_name = spec_links[s];
      auto it = om->m.link_id.find(g.link_name);
      if (it == om->m.link_id.end()) {
        delete oc;
        throw std::invalid_argument("no link named " + g.link_name);
      }
      g.link = it->second;
      int n = counts[s];
      V3 ctr{0, 0, 0};
      for (int j = 0; j < n; j++) {
        V3 v{rel[3 * (off + j)], rel[3 * (off + j) + 1], rel[3 * (off + j) + 2]};
        g.rel.push_back(v);
        g.radii.push_back(radii[off + j]);
        ctr = add(ctr, v);
      }
      ctr = {ctr.x / n, ctr.y / n, ctr.z / n};
      double md = 0.0;
      for (int j = 0; j < n; j++) {
        double d = nrm(sub(g.rel[j], ctr)) + g.radii[j];
        if (d > md) md = d;
      }
      g.group_radius = md;
      g.group_rel = ctr;
      g.only_self = only_self[s] != 0;
      off += n;
      oc->c.groups.push_back(g);
      if (reorder_spheres)
        for (auto& gg : oc->c.groups) reorder(gg);
    }
    for (int p = 0; p < n_pairs; p++) {
      int a = -1, b = -1;
      for (size_t k = 0; k < oc->c.groups.size(); k++) {
        if (a < 0 && oc->c.groups[k].link_name == pair_a[p]) a = (int)k;
        if (b < 0 && oc->c.groups[k].link_name == pair_b[p]) b = (int)k;
      }
      if (a < 0 || b < 0) {
        delete oc;
        throw std::runtime_error("(cpp) Invalid pair of link names for self collision");
      }
      oc->c.pairs.push_back({a, b});
    }
    if (fixed_sdf) oc->c.fixed_sdf = ((OrcSdf*)fixed_sdf)->p;
    oc->c.set_all();
    *out = oc;
  })
}
void orc_cst_destroy(void* p) { delete (OrcCst*)p; }
int orc_cst_set_sdf(void* p, void* sdf) {
  auto* oc = (OrcCst*)p;
  oc->c.sdf = sdf ? ((OrcSdf*)sdf)->p : nullptr;
  oc->c.set_all();
  return 0;
}
int orc_cst_dims(void* p, int* q_dim, int* cst_dim, int* n_spheres) {
  auto* oc = (OrcCst*)p;
  *q_dim = (int)oc->c.q_dim();
  *cst_dim = (int)oc->c.cst_dim();
  int n = 0;
  for (auto& g : oc->c.groups) n += (int)g.radii.size();
  *n_spheres = n;
  return 0;
}
// group table after construction: link id, group radius, group centre, only_self, sphere rel/radii (post-reorder)
int orc_cst_groups(void* p, int* link, double* gr, double* grel, int* only_self, double* rel, double* radii) {
  auto* oc = (OrcCst*)p;
  size_t off = 0;
  for (size_t g = 0; g < oc->c.groups.size(); g++) {
    auto& G = oc->c.groups[g];
    link[g] = G.link;
    gr[g] = G.group_radius;
    grel[3 * g] = G.group_rel.x;
    grel[3 * g + 1] = G.group_rel.y;
    grel[3 * g + 2] = G.group_rel.z;
    only_self[g] = G.only_self;
    for (size_t i = 0; i < G.rel.size(); i++, off++) {
      rel[3 * off] = G.rel[i].x;
      rel[3 * off + 1] = G.rel[i].y;
      rel[3 * off + 2] = G.rel[i].z;
      radii[off] = G.radii[i];
    }
  }
  return 0;
}

}  // extern "C"
template <class F>
static void parallel_for(long long n, int nthreads, F f) {
  if (nthreads <= 1 || n < 2) {
    f(0, 0, n);
    return;
  }
  std::vector<std::thread> th;
  long long chunk = (n + nthreads - 1) / nthreads;
  for (int t = 0; t < nthreads; t++) {
    long long b = t * chunk, e = std::min(n, b + chunk);
    if (b >= e) break;
    th.emplace_back([=]() { f(t, b, e); });
  }
  for (auto& x : th) x.join();
}
extern "C" {

int orc_cst_is_valid(void* p, const double* q, long long B, unsigned char* out, int nthreads) {
  auto* oc = (OrcCst*)p;
  size_t d = oc->c.q_dim();
  ORC_TRY(parallel_for(B, nthreads, [&](int, long long b, long long e) {
    CstState st = oc->fresh();  // start from the shared model's current state
    for (long long i = b; i < e; i++) out[i] = is_valid(oc->c, st, q + i * d);
  }))
}
int orc_cst_evaluate(void* p, const double* q, long long B, double* vals, double* jac, int nthreads) {
  auto* oc = (OrcCst*)p;
  size_t d = oc->c.q_dim(), m = oc->c.cst_dim();
  ORC_TRY(parallel_for(B, nthreads, [&](int, long long b, long long e) {
    CstState st = oc->fresh();
    for (long long i = b; i < e; i++) evaluate(oc->c, st, q + i * d, vals + i * m, jac + i * m * d);
  }))
}
// per-sphere signed distance min_k (sdf_k.evaluate(c) - r) over all flattened SDFs (no cutoff,
// no gates); plus the sphere centres (high_accuracy selects the FK sin/cos)
// World pose [x y z qx qy qz qw] of `link` after update_kintree(q, high_accuracy=true)
// (constraints/primitive.hpp:38-62, kinematics/kinematics.hpp:131-136), for B configurations.
int orc_cst_link_poses(void* p, const double* q, long long B, int link, double* out7, int nthreads) {
  auto* oc = (OrcCst*)p;
  size_t d = oc->c.q_dim();
  ORC_TRY(parallel_for(B, nthreads, [&](int, long long b, long long e) {
    CstState st = oc->fresh();
    for (long long i = b; i < e; i++) {
      update_kintree(*oc->c.m, st.kin, oc->c.ids, oc->c.base_type, q + i * d, true);
      const QT& t = link_pose(*oc->c.m, st.kin, link);
      double* o = out7 + i * 7;
      o[0] = t.t.x;
      o[1] = t.t.y;
      o[2] = t.t.z;
      o[3] = t.q.x;
      o[4] = t.q.y;
      o[5] = t.q.z;
      o[6] = t.q.w;
    }
  }))
}

int orc_cst_sphere_distances(void* p, const double* q, long long B, int high_accuracy, double* dist, double* centres, int nthreads) {
  auto* oc = (OrcCst*)p;
  size_t d = oc->c.q_dim();
  int ns = 0;
  for (auto& g : oc->c.groups) ns += (int)g.radii.size();
  ORC_TRY(parallel_for(B, nthreads, [&](int, long long b, long long e) {
    CstState st = oc->fresh();
    for (long long i = b; i < e; i++) {
      update_kintree(*oc->c.m, st.kin, oc->c.ids, oc->c.base_type, q + i * d, high_accuracy != 0);
      post_update(st);
      int k = 0;
      for (size_t g = 0; g < oc->c.groups.size(); g++) {
        group_cache(oc->c, st, g);
        sphere_cache(oc->c, st, g);
        for (size_t s = 0; s < oc->c.groups[g].radii.size(); s++, k++) {
          const V3& c = st.spos[g][s];
          if (centres) {
            centres[(i * ns + k) * 3 + 0] = c.x;
            centres[(i * ns + k) * 3 + 1] = c.y;
            centres[(i * ns + k) * 3 + 2] = c.z;
          }
          if (dist) {
            double v = std::numeric_limits<double>::infinity();
            for (const Sdf* sd : oc->c.all) v = std::min(v, sd->evaluate(c) - oc->c.groups[g].radii[s]);
            dist[i * ns + k] = v;
          }
        }
      }
    }
  }))
}
int orc_check_motion(void* p, const double* s1, const double* s2, long long E, int type, const double* width, double resolution,
                     unsigned char* out, long long* n_checked, int nthreads) {
  auto* oc = (OrcCst*)p;
  size_t d = oc->c.q_dim();
  Validator v;
  v.type = type;
  if (type == 0) {
    for (size_t i = 0; i < d; i++) {
      v.width.push_back(width[i]);
      v.inv_width.push_back(1.0 / width[i]);
    }
  }
  v.resolution = resolution;
  std::atomic<long long> total{0};
  ORC_TRY({
    parallel_for(E, nthreads, [&](int, long long b, long long e) {
      CstState st = oc->fresh();
      std::vector<double> tmp;
      long long cnt = 0;
      for (long long i = b; i < e; i++) out[i] = check_motion(oc->c, st, v, s1 + i * d, s2 + i * d, tmp, &cnt);
      total += cnt;
    });
    if (n_checked) *n_checked = total.load();
  })
}
int orc_sequence_table(int n_max, long long* out /* n_max x n_max, zero padded */) {
  auto tab = make_sequence_table(n_max);
  for (int i = 0; i < n_max; i++)
    for (int j = 0; j < n_max; j++) out[i * n_max + j] = j < (int)tab[i].size() ? tab[i][j] : 0;
  return 0;
}
// Taylor sin/cos restatement exposed for the known-answer checks
void orc_approx_sin_cos(const double* x, long long n, double* s, double* c) {
  for (long long i = 0; i < n; i++) approx_sin_cos(x[i], s[i], c[i]);
}
// link-pose jacobian of get_jacobian (algorithm.cpp:212-344) for the model's current state;
// rot_type 0 IGNORE, 1 RPY, 2 XYZW; out (3|6|7) x dof column-major
int orc_model_link_jacobian(void* p, int elink, const int* ids, int n, int rot_type, int base_type, double* out) {
  auto* om = (OrcModel*)p;
  Model& m = om->m;
  KinState& s = om->s;
  size_t dimj = 3 + (rot_type == 1) * 3 + (rot_type == 2) * 4;
  size_t dof = n + (base_type == B_FLOATING) * 6 + (base_type == B_PLANAR) * 3;
  std::fill(out, out + dimj * dof, 0.0);
  QT te = link_pose(m, s, elink);
  V3 erpy;
  Q4 einv;
  if (rot_type == 1) erpy = get_rpy(te.q);
  if (rot_type == 2) einv = inverse(te).q;
  for (int i = 0; i < n; i++) {
    int jid = ids[i];
    if (!m.rptable[elink][jid]) continue;
    const QT& tc = link_pose(m, s, m.jchild[jid]);
    V3 wa = qrot(tc.q, m.jaxis[jid]);
    V3 d = m.jtype[jid] == J_PRISMATIC ? wa : cross(wa, sub(te.t, tc.t));
    out[i * dimj + 0] = d.x;
    out[i * dimj + 1] = d.y;
    out[i * dimj + 2] = d.z;
    if (m.jtype[jid] != J_PRISMATIC) {
      if (rot_type == 1) {
        V3 dr;
        rpy_derivative(erpy, wa, dr);
        out[i * dimj + 3] = dr.x;
        out[i * dimj + 4] = dr.y;
        out[i * dimj + 5] = dr.z;
      }
      if (rot_type == 2) {
        Q4 dq = q_derivative(einv, wa);
        out[i * dimj + 3] = dq.x;
        out[i * dimj + 4] = dq.y;
        out[i * dimj + 5] = dq.z;
        out[i * dimj + 6] = dq.w;
      }
    }
  }
  if (base_type == B_FIXED) return 0;
  QT tb = link_pose(m, s, m.root);
  QT tbinv = inverse(tb);
  V3 rpyb = get_rpy(tb.q);
  QT tbe = mul(tbinv, te);
  const double eps = 1e-7;
  auto fill_col = [&](size_t colidx, int k) {
    V3 r2 = rpyb;
    r2[k] += eps;
    QT tw = tb;
    tw.q = quat_from_rpy(r2.x, r2.y, r2.z);
    QT po = mul(tw, tbe);
    V3 dp = sub(po.t, te.t);
    for (int r = 0; r < 3; r++) out[colidx * dimj + r] = dp[r] / eps;
    if (rot_type == 1) {
      V3 e2 = get_rpy(po.q);
      out[colidx * dimj + 3] = (e2.x - erpy.x) / eps;
      out[colidx * dimj + 4] = (e2.y - erpy.y) / eps;
      out[colidx * dimj + 5] = (e2.z - erpy.z) / eps;
    }
    if (rot_type == 2) {
      out[colidx * dimj + 3] = (po.q.x - te.q.x) / eps;
      out[colidx * dimj + 4] = (po.q.y - te.q.y) / eps;
      out[colidx * dimj + 5] = (po.q.z - te.q.z) / eps;
      out[colidx * dimj + 6] = (po.q.w - te.q.w) / eps;
    }
  };
  if (base_type == B_FLOATING) {
    out[(n + 0) * dimj + 0] = 1.0;
    out[(n + 1) * dimj + 1] = 1.0;
    out[(n + 2) * dimj + 2] = 1.0;
    for (int k = 0; k < 3; k++) fill_col(n + 3 + k, k);
  } else {
    out[(n + 0) * dimj + 0] = 1.0;
    out[(n + 1) * dimj + 1] = 1.0;
    fill_col(n + 2, 2);
  }
  return 0;
}
// update_kintree on the shared model (for link-pose / jacobian queries after a config)
int orc_cst_update_kintree(void* p, const double* q, int high_accuracy) {
  auto* oc = (OrcCst*)p;
  update_kintree(*oc->c.m, oc->om->s, oc->c.ids, oc->c.base_type, q, high_accuracy != 0);
  return 0;
}

}  // extern "C"
