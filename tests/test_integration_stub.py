"""The bindings INTEGRATION.md shows, built from their committed sources
(plainmp_gb300/bindings/).

* The pybind11 binding (pybind11_gpu_cst.cpp) compiles against include/pmgpu.h, links to the
  in-tree library and works.  Without a GPU its is_valid_batch reports the library's "no CUDA
  device" error; with one it equals the Python mirror's plain method.  Needs pybind11 (skipped
  where it is absent).
* The OMPL adapter (ompl_adapter.hpp) compiles against include/pmgpu.h and a stand-in of the OMPL
  declarations it uses.
* INTEGRATION.md quotes both files' code as it stands.
* A C99 program includes the header, links to the library and calls it (the ABI is plain C).
"""
import importlib.util
import subprocess
import sys
import sysconfig
from pathlib import Path

import numpy as np
import pytest

REPO = Path(__file__).resolve().parent.parent
BINDINGS = REPO / "plainmp_gb300" / "bindings"

MODULE = """#include <pybind11/pybind11.h>
namespace py = pybind11;
void bind_gpu_constraint(py::module& cst_m);
PYBIND11_MODULE(gpu_stub, m) { bind_gpu_constraint(m); }
"""


def doc_block(section: str) -> str:
    """The C++ block of an INTEGRATION.md section."""
    text = (REPO / "INTEGRATION.md").read_text()
    sec = text[text.index(section):]
    start = sec.index("```cpp\n") + len("```cpp\n")
    return sec[start:sec.index("```", start)]


def test_document_quotes_the_sources():
    assert doc_block("## 3. C++ (OMPL") in (BINDINGS / "ompl_adapter.hpp").read_text()
    assert doc_block("## 4. pybind11") in (BINDINGS / "pybind11_gpu_cst.cpp").read_text()


@pytest.fixture(scope="module")
def stub(tmp_path_factory):
    pybind11 = pytest.importorskip("pybind11")
    d = tmp_path_factory.mktemp("stub")
    src = d / "gpu_stub.cpp"
    src.write_text(MODULE)
    so = d / ("gpu_stub" + sysconfig.get_config_var("EXT_SUFFIX"))
    lib_dir = REPO / "plainmp_gb300"
    cmd = ["g++", "-std=c++17", "-O0", "-shared", "-fPIC", "-Wall", f"-I{REPO / 'include'}", f"-I{pybind11.get_include()}",
           f"-I{sysconfig.get_paths()['include']}", str(src), str(BINDINGS / "pybind11_gpu_cst.cpp"), "-o", str(so), f"-L{lib_dir}",
           "-lpmgpu", f"-Wl,-rpath,{lib_dir}"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-3000:]
    spec = importlib.util.spec_from_file_location("gpu_stub", so)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_pybind11_stub_builds_and_runs(stub):
    import plainmp_gb300 as pm
    from plainmp_gb300 import scenes
    from plainmp_gb300 import workloads as W

    robot = W.chain7_robot()
    specs = [(s.parent_link_name, s.relative_positions, s.radii, s.only_self_collision) for s in robot.spheres]
    c = stub.SphereCollisionCstGpu(robot.urdf, robot.control_joints, 0, specs, robot.self_pairs)
    with pytest.raises(ValueError):  # std::invalid_argument from the C ABI: unknown joint name
        stub.SphereCollisionCstGpu(robot.urdf, ["nojoint"], 0, specs, [])
    Q = W.chain7_configs(64, seed=9)
    if pm.device_count() == 0:
        with pytest.raises(RuntimeError, match="no CUDA device"):
            c.is_valid_batch(Q)
        return
    _, mine, _ = scenes.make_constraint(robot, W.Scene(), True, True)  # same spheres and pairs, no SDF
    assert np.array_equal(c.is_valid_batch(Q), mine.is_valid_batch(Q))


# Stand-ins of the OMPL headers the adapter includes (OMPL itself is not installed):
# State::as<T>(), RealVectorStateSpace::StateType::values, MotionValidator's constructor and its two
# pure checkMotion overloads, SpaceInformationPtr.
OMPL_MOTION_VALIDATOR_H = """#pragma once
#include <memory>
#include <utility>
namespace ompl { namespace base {
class State {
 public:
  virtual ~State() = default;
  template <class T> const T* as() const { return static_cast<const T*>(this); }
  template <class T> T* as() { return static_cast<T*>(this); }
};
class SpaceInformation {};
using SpaceInformationPtr = std::shared_ptr<SpaceInformation>;
class MotionValidator {
 public:
  explicit MotionValidator(const SpaceInformationPtr& si) : si_(si) {}
  virtual ~MotionValidator() = default;
  virtual bool checkMotion(const State* s1, const State* s2) const = 0;
  virtual bool checkMotion(const State* s1, const State* s2, std::pair<State*, double>& last_valid) const = 0;
 protected:
  SpaceInformationPtr si_;
};
}}  // namespace ompl::base
"""
OMPL_REAL_VECTOR_H = """#pragma once
#include <ompl/base/MotionValidator.h>
namespace ompl { namespace base {
class RealVectorStateSpace {
 public:
  class StateType : public State { public: double* values = nullptr; };
};
}}  // namespace ompl::base
"""


def test_ompl_adapter_compiles(tmp_path):
    """The OMPL adapter header compiles against include/pmgpu.h (its ABI calls have the header's
    argument lists) and implements both checkMotion overloads."""
    inc = tmp_path / "inc" / "ompl" / "base"
    (inc / "spaces").mkdir(parents=True)
    (inc / "MotionValidator.h").write_text(OMPL_MOTION_VALIDATOR_H)
    (inc / "spaces" / "RealVectorStateSpace.h").write_text(OMPL_REAL_VECTOR_H)
    src = tmp_path / "adapter.cpp"
    src.write_text('#include "ompl_adapter.hpp"\n'
                   "int main() { GpuBoxMotionValidator v(nullptr, nullptr, {0.05}); GpuValidity g{nullptr, 7}; (void)v; (void)g; return 0; }\n")
    r = subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-Wall", f"-I{tmp_path / 'inc'}", f"-I{BINDINGS}",
                        f"-I{REPO / 'include'}", str(src)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr[-3000:]


C_CALLER = r"""
#include <stdio.h>
#include <stdlib.h>
#include "pmgpu.h"

static char* slurp(const char* path) {
  FILE* f = fopen(path, "rb");
  if (!f) return NULL;
  fseek(f, 0, SEEK_END);
  long n = ftell(f);
  fseek(f, 0, SEEK_SET);
  char* s = (char*)malloc((size_t)n + 1);
  if (fread(s, 1, (size_t)n, f) != (size_t)n) n = 0;
  s[n] = 0;
  fclose(f);
  return s;
}

int main(int argc, char** argv) {
  char* urdf = argc > 1 ? slurp(argv[1]) : NULL;
  pmgpu_model* kin = NULL;
  if (!urdf || pmgpu_model_create(urdf, &kin) != PMGPU_OK) return 10;
  const char* joints[7] = {"j1", "j2", "j3", "j4", "j5", "j6", "j7"};
  const char* links[1] = {"link7"};
  const int32_t counts[1] = {1};
  const double rel[3] = {0.0, 0.0, 0.0}, radii[1] = {0.05};
  const uint8_t only[1] = {0};
  pmgpu_cst* cst = NULL;
  if (pmgpu_cst_create(kin, joints, 7, PMGPU_BASE_FIXED, 1, links, counts, rel, radii, only, 0, NULL, NULL, NULL, 1, &cst) != PMGPU_OK)
    return 11;
  pmgpu_model_destroy(kin); /* the constraint keeps its model */
  int q_dim = 0, cst_dim = -1, ns = 0, ng = 0;
  if (pmgpu_cst_dims(cst, &q_dim, &cst_dim, &ns, &ng) != PMGPU_OK) return 12;
  double q[7] = {0, 0, 0, 0, 0, 0, 0};
  uint8_t ok = 7;
  const int rc = pmgpu_cst_is_valid(cst, q, 1, &ok, PMGPU_MEM_HOST, NULL);
  const int rc_null = pmgpu_cst_is_valid(cst, NULL, 1, &ok, PMGPU_MEM_HOST, NULL);
  printf("%d %d %d %d %d %d %d %s\n", q_dim, cst_dim, ns, ng, rc, (int)ok, rc_null, pmgpu_last_error());
  pmgpu_cst_destroy(cst);
  free(urdf);
  return 0;
}
"""


def test_c_caller(tmp_path):
    """A C99 program includes the header, links to the library and calls it: model and constraint
    construction, dimensions, is_valid (PMGPU_ERR_CUDA without a GPU, a valid configuration with
    one: no SDF and no self pairs) and the NULL-argument error."""
    import plainmp_gb300 as pm
    from plainmp_gb300 import workloads as W

    (tmp_path / "caller.c").write_text(C_CALLER)
    (tmp_path / "chain7.urdf").write_text(W.chain7_robot().urdf)
    lib_dir = REPO / "plainmp_gb300"
    exe = tmp_path / "caller"
    r = subprocess.run(["gcc", "-std=c99", "-Wall", "-Wextra", "-pedantic", f"-I{REPO / 'include'}", str(tmp_path / "caller.c"),
                        "-o", str(exe), f"-L{lib_dir}", "-lpmgpu", f"-Wl,-rpath,{lib_dir}"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr[-3000:]
    r = subprocess.run([str(exe), str(tmp_path / "chain7.urdf")], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, (r.returncode, r.stderr[-2000:])
    f = r.stdout.split(" ", 7)
    assert f[:4] == ["7", "0", "1", "1"]  # q_dim, cst_dim (no SDF, no pairs), spheres, groups
    if pm.device_count() == 0:
        assert int(f[4]) == 3  # PMGPU_ERR_CUDA
    else:
        assert int(f[4]) == 0 and f[5] == "1"
    assert int(f[6]) == 1 and f[7].strip() == "q is NULL"  # PMGPU_ERR_INVALID
