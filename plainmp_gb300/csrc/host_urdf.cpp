// URDF reader (see host_urdf.h for the semantics it keeps).
#include "host_urdf.h"

#include <cmath>
#include <cstdlib>
#include <cstring>
#include <locale>
#include <sstream>
#include <stdexcept>

namespace pmg {
namespace {

struct XmlNode {
  std::string tag;
  std::vector<std::pair<std::string, std::string>> attrs;
  std::vector<XmlNode> children;
  const std::string* attr(const char* k) const {
    for (auto& a : attrs)
      if (a.first == k) return &a.second;
    return nullptr;
  }
  const XmlNode* child(const char* t) const {
    for (auto& c : children)
      if (c.tag == t) return &c;
    return nullptr;
  }
};

class XmlReader {
 public:
  explicit XmlReader(const std::string& s) : s_(s) {}
  XmlNode parse_document() {
    skip_misc();
    if (pos_ >= s_.size() || s_[pos_] != '<') fail("expected root element");
    XmlNode root = parse_element();
    skip_misc();
    return root;
  }

 private:
  const std::string& s_;
  size_t pos_ = 0;

  [[noreturn]] void fail(const std::string& m) {
    throw std::runtime_error("URDF/XML parse error at offset " + std::to_string(pos_) + ": " + m);
  }
  void skip_ws() {
    while (pos_ < s_.size() && std::isspace(static_cast<unsigned char>(s_[pos_]))) pos_++;
  }
  bool starts(const char* p) const { return s_.compare(pos_, std::strlen(p), p) == 0; }
  void skip_until(const char* end) {
    size_t e = s_.find(end, pos_);
    if (e == std::string::npos) fail(std::string("unterminated construct, expected ") + end);
    pos_ = e + std::strlen(end);
  }
  // whitespace, comments, processing instructions, doctype
  void skip_misc() {
    for (;;) {
      skip_ws();
      if (starts("<?")) {
        skip_until("?>");
      } else if (starts("<!--")) {
        skip_until("-->");
      } else if (starts("<!")) {
        skip_until(">");
      } else {
        return;
      }
    }
  }
  std::string name() {
    size_t b = pos_;
    while (pos_ < s_.size()) {
      char c = s_[pos_];
      if (std::isalnum(static_cast<unsigned char>(c)) || c == '_' || c == '-' || c == ':' || c == '.')
        pos_++;
      else
        break;
    }
    if (b == pos_) fail("expected a name");
    return s_.substr(b, pos_ - b);
  }
  static std::string decode(const std::string& v) {
    std::string o;
    for (size_t i = 0; i < v.size(); i++) {
      if (v[i] == '&') {
        size_t e = v.find(';', i);
        if (e != std::string::npos) {
          std::string ent = v.substr(i + 1, e - i - 1);
          if (ent == "lt") o += '<';
          else if (ent == "gt") o += '>';
          else if (ent == "amp") o += '&';
          else if (ent == "quot") o += '"';
          else if (ent == "apos") o += '\'';
          else o += v.substr(i, e - i + 1);
          i = e;
          continue;
        }
      }
      o += v[i];
    }
    return o;
  }
  XmlNode parse_element() {
    XmlNode n;
    pos_++;  // '<'
    n.tag = name();
    for (;;) {
      skip_ws();
      if (pos_ >= s_.size()) fail("unterminated tag <" + n.tag + ">");
      if (starts("/>")) {
        pos_ += 2;
        return n;
      }
      if (s_[pos_] == '>') {
        pos_++;
        break;
      }
      std::string k = name();
      skip_ws();
      if (pos_ >= s_.size() || s_[pos_] != '=') fail("expected '=' after attribute " + k);
      pos_++;
      skip_ws();
      if (pos_ >= s_.size() || (s_[pos_] != '"' && s_[pos_] != '\'')) fail("expected quoted value for " + k);
      char q = s_[pos_++];
      size_t e = s_.find(q, pos_);
      if (e == std::string::npos) fail("unterminated attribute value");
      n.attrs.emplace_back(k, decode(s_.substr(pos_, e - pos_)));
      pos_ = e + 1;
    }
    // content
    for (;;) {
      size_t lt = s_.find('<', pos_);
      if (lt == std::string::npos) fail("unterminated element <" + n.tag + ">");
      pos_ = lt;
      if (starts("<!--")) {
        skip_until("-->");
      } else if (starts("<![CDATA[")) {
        skip_until("]]>");
      } else if (starts("<?")) {
        skip_until("?>");
      } else if (starts("</")) {
        pos_ += 2;
        std::string t = name();
        if (t != n.tag) fail("mismatched </" + t + "> for <" + n.tag + ">");
        skip_ws();
        if (pos_ >= s_.size() || s_[pos_] != '>') fail("expected '>'");
        pos_++;
        return n;
      } else {
        n.children.push_back(parse_element());
      }
    }
  }
};

double to_double(const std::string& tok) {
  std::istringstream ss(tok);
  ss.imbue(std::locale::classic());
  double v;
  ss >> v;
  if (ss.fail() || !ss.eof()) throw std::runtime_error("URDF: cannot convert '" + tok + "' to a number");
  return v;
}

void vec3(const std::string& str, double out[3]) {
  std::vector<double> v;
  size_t i = 0;
  while (i <= str.size()) {
    size_t e = str.find(' ', i);
    if (e == std::string::npos) e = str.size();
    if (e > i) v.push_back(to_double(str.substr(i, e - i)));
    i = e + 1;
  }
  if (v.size() != 3) throw std::runtime_error("URDF: expected 3 numbers in '" + str + "'");
  out[0] = v[0];
  out[1] = v[1];
  out[2] = v[2];
}

// urdf_model/pose.h:202-216 (setFromRPY followed by normalize)
void rpy_to_quat(const double rpy[3], double q[4]) {
  double phi = rpy[0] / 2.0, the = rpy[1] / 2.0, psi = rpy[2] / 2.0;
  double x = std::sin(phi) * std::cos(the) * std::cos(psi) - std::cos(phi) * std::sin(the) * std::sin(psi);
  double y = std::cos(phi) * std::sin(the) * std::cos(psi) + std::sin(phi) * std::cos(the) * std::sin(psi);
  double z = std::cos(phi) * std::cos(the) * std::sin(psi) - std::sin(phi) * std::sin(the) * std::cos(psi);
  double w = std::cos(phi) * std::cos(the) * std::cos(psi) + std::sin(phi) * std::sin(the) * std::sin(psi);
  double s = std::sqrt(x * x + y * y + z * z + w * w);
  if (s == 0.0) {
    q[0] = q[1] = q[2] = 0.0;
    q[3] = 1.0;
  } else {
    q[0] = x / s;
    q[1] = y / s;
    q[2] = z / s;
    q[3] = w / s;
  }
}

}  // namespace

UrdfRobot parse_urdf(const std::string& xml) {
  if (xml.empty()) throw std::runtime_error("xml string is empty");
  XmlReader rd(xml);
  XmlNode root = rd.parse_document();
  if (root.tag != "robot") throw std::runtime_error("URDF: root element is <" + root.tag + ">, expected <robot>");
  UrdfRobot r;
  std::map<std::string, int> seen;
  for (auto& c : root.children) {
    if (c.tag != "link") continue;
    const std::string* nm = c.attr("name");
    if (!nm) throw std::runtime_error("URDF: link without a name");
    if (seen.count(*nm)) throw std::runtime_error("URDF: link '" + *nm + "' is not unique");
    seen[*nm] = 1;
    r.links.push_back(*nm);
  }
  if (r.links.empty()) throw std::runtime_error("URDF: no link elements");
  for (auto& c : root.children) {
    if (c.tag != "joint") continue;
    UrdfJoint j;
    const std::string* nm = c.attr("name");
    if (!nm) throw std::runtime_error("URDF: joint without a name");
    j.name = *nm;
    if (r.joints.count(j.name)) throw std::runtime_error("URDF: joint '" + j.name + "' is not unique");
    const std::string* ty = c.attr("type");
    if (!ty) throw std::runtime_error("URDF: joint '" + j.name + "' has no type");
    if (*ty == "planar") j.type = UJ_PLANAR;
    else if (*ty == "floating") j.type = UJ_FLOATING;
    else if (*ty == "revolute") j.type = UJ_REVOLUTE;
    else if (*ty == "continuous") j.type = UJ_CONTINUOUS;
    else if (*ty == "prismatic") j.type = UJ_PRISMATIC;
    else if (*ty == "fixed") j.type = UJ_FIXED;
    else throw std::runtime_error("URDF: joint '" + j.name + "' has unknown type '" + *ty + "'");
    if (const XmlNode* o = c.child("origin")) {
      if (const std::string* s = o->attr("xyz")) vec3(*s, j.xyz);
      if (const std::string* s = o->attr("rpy")) {
        double rpy[3];
        vec3(*s, rpy);
        rpy_to_quat(rpy, j.quat);
      }
    }
    const XmlNode* p = c.child("parent");
    const XmlNode* ch = c.child("child");
    if (!p || !p->attr("link") || !ch || !ch->attr("link"))
      throw std::runtime_error("Joint [" + j.name + "] is missing a parent and/or child link specification.");
    j.parent = *p->attr("link");
    j.child = *ch->attr("link");
    if (j.type != UJ_FLOATING && j.type != UJ_FIXED) {
      if (const XmlNode* a = c.child("axis")) {
        if (const std::string* s = a->attr("xyz")) vec3(*s, j.axis);
      }
    }
    if (const XmlNode* l = c.child("limit")) {
      j.has_limits = true;
      if (const std::string* s = l->attr("lower")) j.lower = to_double(*s);
      if (const std::string* s = l->attr("upper")) j.upper = to_double(*s);
    } else if (j.type == UJ_REVOLUTE || j.type == UJ_PRISMATIC) {
      throw std::runtime_error("URDF: joint '" + j.name + "' of type revolute/prismatic has no <limit>");
    }
    r.joints[j.name] = j;
  }
  // tree (joint-name order)
  for (auto& kv : r.joints) {
    const UrdfJoint& j = kv.second;
    if (!seen.count(j.child))
      throw std::runtime_error("child link [" + j.child + "] of joint [" + j.name + "] not found");
    if (!seen.count(j.parent))
      throw std::runtime_error("parent link [" + j.parent + "] of joint [" + j.name + "] not found");
    if (r.parent_joint.count(j.child)) throw std::runtime_error("URDF: link '" + j.child + "' has two parents");
    r.parent_joint[j.child] = j.name;
    r.child_joints[j.parent].push_back(j.name);
  }
  std::map<std::string, int> sorted_links(seen.begin(), seen.end());
  for (auto& kv : sorted_links) {
    if (!r.parent_joint.count(kv.first)) {
      if (!r.root.empty()) throw std::runtime_error("Two root links found: [" + r.root + "] and [" + kv.first + "]");
      r.root = kv.first;
    }
  }
  if (r.root.empty()) throw std::runtime_error("No root link found. The robot xml is not a valid tree.");
  return r;
}

}  // namespace pmg
