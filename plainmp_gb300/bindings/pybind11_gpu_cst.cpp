// pybind11 binding of the C ABI, for a maintainer who keeps _plainmp as the only extension: call
// bind_gpu_constraint(cst_m) next to the reference's constraint bindings
// (cpp/plainmp/bindings/constraint.cpp:73-84).  Exposes SphereCollisionCstGpu with the
// reference's exception types (std::invalid_argument -> ValueError, std::runtime_error ->
// RuntimeError).
#include <pybind11/numpy.h>
#include <pybind11/pybind11.h>
#include <pybind11/stl.h>

#include <memory>
#include <stdexcept>
#include <string>
#include <tuple>
#include <vector>

namespace py = pybind11;

#include "pmgpu.h"

// Owning wrapper of the opaque constraint handle (pybind11 binds complete types only).
struct GpuCst {
  pmgpu_cst* h = nullptr;
  GpuCst() = default;
  GpuCst(const GpuCst&) = delete;
  ~GpuCst() { pmgpu_cst_destroy(h); }
};
static void ok_or_throw(int rc) {  // the reference's exception types: ValueError / RuntimeError in Python
  if (rc == PMGPU_ERR_INVALID) throw std::invalid_argument(pmgpu_last_error());
  if (rc != PMGPU_OK) throw std::runtime_error(pmgpu_last_error());
}
using Spec = std::tuple<std::string, py::array_t<double, py::array::c_style | py::array::forcecast>,
                        py::array_t<double, py::array::c_style | py::array::forcecast>, bool>;

// Called next to the other constraint bindings with the constraint submodule (cst_m).
void bind_gpu_constraint(py::module& cst_m) {
py::class_<GpuCst>(cst_m, "SphereCollisionCstGpu")
    // (urdf_xml, control_joint_names, base_type, [(link, relative_positions (3, n), radii (n,),
    //  only_self_collision)], selcol_pairs): SphereCollisionCst's arguments without the SDF
    .def(py::init([](const std::string& urdf, const std::vector<std::string>& joints, int base_type,
                     const std::vector<Spec>& specs, const std::vector<std::pair<std::string, std::string>>& pairs) {
      std::vector<const char*> jn, links, pa, pb;
      std::vector<int32_t> counts;
      std::vector<double> rel, radii;
      std::vector<uint8_t> only;
      for (auto& j : joints) jn.push_back(j.c_str());
      for (auto& [link, r3n, rad, self_only] : specs) {
        const py::ssize_t n = rad.shape(0);
        if (r3n.ndim() != 2 || r3n.shape(0) != 3 || r3n.shape(1) != n) throw std::invalid_argument("relative_positions must be (3, n)");
        links.push_back(link.c_str());
        counts.push_back((int32_t)n);
        only.push_back(self_only ? 1 : 0);
        for (py::ssize_t k = 0; k < n; k++) {
          for (int a = 0; a < 3; a++) rel.push_back(r3n.at(a, k));
          radii.push_back(rad.at(k));
        }
      }
      for (auto& [a, b] : pairs) {
        pa.push_back(a.c_str());
        pb.push_back(b.c_str());
      }
      pmgpu_model* kin = nullptr;
      ok_or_throw(pmgpu_model_create(urdf.c_str(), &kin));
      auto c = std::make_unique<GpuCst>();
      const int rc = pmgpu_cst_create(kin, jn.data(), (int)jn.size(), base_type, (int)links.size(), links.data(), counts.data(),
                                      rel.data(), radii.data(), only.data(), (int)pa.size(), pa.data(), pb.data(), nullptr, 1, &c->h);
      pmgpu_model_destroy(kin);  // the constraint keeps its model alive
      ok_or_throw(rc);
      return c;
    }))
    .def("is_valid_batch", [](GpuCst& c, py::array_t<double, py::array::c_style | py::array::forcecast> q) {
      if (q.ndim() != 2) throw std::invalid_argument("q must be (B, q_dim)");
      py::array_t<uint8_t> out(q.shape(0));
      ok_or_throw(pmgpu_cst_is_valid(c.h, q.data(), q.shape(0), out.mutable_data(), PMGPU_MEM_HOST, nullptr));
      return out;
    });
}
