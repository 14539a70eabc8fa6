"""CPU tests of the product's host side: the C ABI library loads and exports every symbol that
include/pmgpu.h declares; the C++ URDF reader and tree numbering match the reference's
urdfdom parser (golden dumps); constraint construction (group spheres, farthest-first
reorder, pairs) and SDF construction (pose flags, AABBs) match the oracle bit for bit; errors
map to the reference's exception types.  No compute call runs here."""
import ctypes
import re
from pathlib import Path

import numpy as np
import pytest

from helpers import golden, plainmp_numbering, rpy_matrix

REPO = Path(__file__).resolve().parent.parent


def declared_symbols():
    txt = "\n".join(p.read_text() for p in (REPO / "include").glob("*.h"))
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(pmgpu_[a-z0-9_]+)\s*\(", txt)))


def test_library_exports_every_declared_symbol():
    from plainmp_gb300 import _lib

    lib = ctypes.CDLL(str(_lib.LIB_PATH))
    syms = declared_symbols()
    assert len(syms) > 40
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing


def test_product_path_has_no_oracle_dependency():
    pat = re.compile(r"^\s*(from\s+oracle|import\s+oracle)|pyoracle|liboracle|orc_", re.M)
    for p in list((REPO / "plainmp_gb300").rglob("*.py")) + list((REPO / "plainmp_gb300" / "csrc").glob("*")):
        assert not pat.search(p.read_text()), p


@pytest.mark.parametrize("name", ["chain7", "dualarm", "edge"])
def test_urdf_reader_matches_urdfdom(name):
    from plainmp_gb300 import KinematicModel

    g = golden(f"urdf_{name}.json")
    order, parent, jorder = plainmp_numbering(g)
    kin = KinematicModel(g["urdf"])
    st = kin.structure()
    assert st["link_names"] == order
    assert list(st["link_parent"]) == parent
    assert st["joint_names"] == jorder
    for k, jn in enumerate(jorder):
        j = g["joints"][jn]
        assert st["joint_child"][k] == order.index(j["child"])
        assert st["joint_type"][k] == j["type"]
        assert list(st["joint_axis"][k]) == j["axis"]
        lo, hi = kin.get_joint_position_limits([k])[0]
        if j["type"] == 2:
            assert lo == -np.inf and hi == np.inf
        else:
            assert [lo, hi] == j["limits"]
    for jn, j in g["joints"].items():
        li = order.index(j["child"])
        assert list(st["link_tf7"][li][:3]) == j["xyz"]
        assert list(st["link_tf7"][li][3:]) == j["quat"]  # rpy -> quaternion -> normalise, bit for bit


@pytest.mark.parametrize("name", ["chain7", "dualarm", "edge"])
def test_urdf_reader_matches_oracle(oracle, name):
    from plainmp_gb300 import KinematicModel

    g = golden(f"urdf_{name}.json")
    a = KinematicModel(g["urdf"]).structure()
    b = oracle.Model(g["urdf"]).structure()
    assert np.array_equal(a["link_parent"], b["link_parent"])
    assert np.array_equal(a["link_tf7"], b["link_tf7"])
    assert np.array_equal(a["link_tf_qid"], b["link_tf_qid"])
    assert np.array_equal(a["joint_child"], b["joint_child"])
    assert np.array_equal(a["joint_origin_qid"], b["joint_origin_qid"])


def test_urdf_errors():
    from plainmp_gb300 import KinematicModel

    with pytest.raises(RuntimeError):
        KinematicModel("")
    with pytest.raises(RuntimeError):
        KinematicModel("<robot name='x'><link name='a'/><link name='b'/></robot>")  # two roots
    with pytest.raises(RuntimeError):
        KinematicModel("<robot name='x'><link name='a'/><joint name='j' type='revolute'><parent link='a'/>"
                       "<child link='zz'/><limit lower='0' upper='1'/></joint></robot>")
    with pytest.raises(RuntimeError):
        KinematicModel("<robot name='x'><link name='a'/><link name='b'/><joint name='j' type='revolute'><parent link='a'/>"
                       "<child link='b'/></joint></robot>")  # revolute without limits
    with pytest.raises(RuntimeError):
        KinematicModel("<robot><link name='a'/><joint name='j' type='fixed'><origin xyz='1 2'/></joint></robot>")
    kin = KinematicModel(golden("urdf_chain7.json")["urdf"])
    with pytest.raises(ValueError):
        kin.get_joint_ids(["nope"])
    with pytest.raises(ValueError):
        kin.get_link_ids(["nope"])


def _specs(robot):
    from plainmp_gb300 import SphereAttachmentSpec

    return [SphereAttachmentSpec(s.parent_link_name, s.relative_positions, s.radii, s.only_self_collision) for s in robot.spheres]


@pytest.mark.parametrize("which", ["chain7", "dualarm"])
@pytest.mark.parametrize("reorder", [True, False])
def test_constraint_tables_match_oracle(oracle, which, reorder):
    from plainmp_gb300 import BaseType, KinematicModel, SphereCollisionCst
    from plainmp_gb300 import workloads as W

    robot = W.chain7_robot() if which == "chain7" else W.dualarm_robot()
    kin = KinematicModel(robot.urdf)
    c = SphereCollisionCst(kin, robot.control_joints, BaseType.FIXED, _specs(robot), robot.self_pairs, None, reorder)
    om = oracle.Model(robot.urdf)
    oc = oracle.Cst(om, robot.control_joints, 0, robot.spheres, robot.self_pairs, None, reorder)
    a, b = c.groups(), oc.groups()
    for k in ("link", "radius", "centre", "only_self", "rel", "radii"):
        assert np.array_equal(a[k], b[k]), k
    assert c.q_dim() == oc.q_dim and c.n_spheres == oc.n_spheres
    assert c.cst_dim() == 1  # self pairs only (no SDF yet)


def test_constraint_errors():
    from plainmp_gb300 import BaseType, KinematicModel, SphereCollisionCst
    from plainmp_gb300 import workloads as W

    robot = W.chain7_robot()
    kin = KinematicModel(robot.urdf)
    with pytest.raises(ValueError):
        SphereCollisionCst(kin, ["j1", "nope"], BaseType.FIXED, _specs(robot), [], None, True)
    with pytest.raises(RuntimeError, match="Invalid pair"):
        SphereCollisionCst(kin, robot.control_joints, BaseType.FIXED, _specs(robot), [("link1", "nolink")], None, True)


def test_sdf_construction_matches_oracle(oracle):
    from plainmp_gb300 import BoxSDF, CylinderSDF, GroundSDF, Pose, SphereSDF, UnionSDF

    rng = np.random.default_rng(0)
    for i in range(30):
        pos = rng.standard_normal(3)
        R = np.eye(3) if i == 0 else (rpy_matrix(0.3, 0, 0) if i == 1 else rpy_matrix(*rng.standard_normal(3)))
        pairs = [
            (BoxSDF([0.5, 0.3, 0.6], Pose(pos, R)), oracle.Sdf.box([0.5, 0.3, 0.6], pos, R)),
            (CylinderSDF(0.7, 0.2, Pose(pos, R)), oracle.Sdf.cylinder(0.7, 0.2, pos, R)),
            (SphereSDF(0.5, Pose(pos, R)), oracle.Sdf.sphere(0.5, pos, R)),
        ]
        for mine, ref in pairs:
            lb, ub, aa, za = ref.info()
            assert np.array_equal(mine.lb, lb) and np.array_equal(mine.ub, ub)
            assert mine.pose.axis_aligned == aa and mine.pose.z_axis_aligned == za
            t = rng.standard_normal(3)
            a = float(rng.standard_normal())
            mine.translate(t)
            ref.translate(t)
            mine.rotate_z(a)
            ref.rotate_z(a)
            lb, ub, aa, za = ref.info()
            assert np.array_equal(mine.lb, lb) and np.array_equal(mine.ub, ub)
    g = GroundSDF(1.0)
    assert list(g.lb[2:]) == [0.0] and list(g.ub[2:]) == [0.0]
    with pytest.raises(RuntimeError):
        g.translate([1, 0, 0])
    u = UnionSDF([BoxSDF([1, 1, 1], Pose())])
    u.translate([1.0, 2.0, 3.0])  # members are shared, translated in place


def test_pose_flags_known_answers():  # tests/test_psdf.py:27-39
    from plainmp_gb300 import Pose

    assert Pose(np.zeros(3), np.eye(3)).axis_aligned
    p2 = Pose(np.zeros(3), rpy_matrix(0.3, 0.0, 0.0))
    assert not p2.axis_aligned and p2.z_axis_aligned
    p3 = Pose(np.zeros(3), rpy_matrix(0.3, 0.3, 0.3))
    assert not p3.axis_aligned and not p3.z_axis_aligned


def test_batch_calls_fail_loudly_without_gpu():
    from plainmp_gb300 import CudaError, device_count
    from plainmp_gb300 import scenes
    from plainmp_gb300 import workloads as W

    if device_count() > 0:
        pytest.skip("a GPU is present")
    kin, cst, _ = scenes.make_constraint(W.chain7_robot(), W.chain7_scene())
    with pytest.raises(CudaError):
        cst.is_valid_batch(W.chain7_configs(4))


def test_pose_constraint_construction():
    """LinkPoseCst / LinkPositionBoundCst / composites: dimensions and the reference's errors
    (primitive_link_pose.cpp:16-29, primitive_link_position_bound.cpp:15-32,
    composite_constraint.hpp:24-32); construction is host work."""
    from plainmp_gb300 import (BaseType, IneqCompositeCst, KinematicModel, LinkPoseCst, LinkPositionBoundCst,
                               SphereCollisionCst)
    from plainmp_gb300 import workloads as W

    robot = W.chain7_robot()
    kin = KinematicModel(robot.urdf)
    j = robot.control_joints
    c = LinkPoseCst(kin, j, BaseType.FIXED, [robot.end_link, "link3"], [np.zeros(3), np.zeros(7)])
    assert c.cst_dim() == 10 and c.q_dim() == 7
    assert [p.shape[0] for p in c.get_desired_poses()] == [3, 7]
    assert LinkPoseCst(kin, j, BaseType.PLANAR, ["link2"], [np.zeros(6)]).q_dim() == 10
    assert LinkPoseCst(kin, j, BaseType.FLOATING, ["link2"], [np.zeros(6)]).q_dim() == 13
    with pytest.raises(RuntimeError, match="3 or 6 or 7"):
        LinkPoseCst(kin, j, BaseType.FIXED, ["link2"], [np.zeros(5)])
    with pytest.raises(ValueError):
        LinkPoseCst(kin, j, BaseType.FIXED, ["nolink"], [np.zeros(3)])
    b = LinkPositionBoundCst(kin, j, BaseType.FIXED, robot.end_link, 2, lb=0.1)
    assert b.cst_dim() == 1
    assert LinkPositionBoundCst(kin, j, BaseType.FIXED, robot.end_link, 0, lb=-1.0, ub=1.0).cst_dim() == 2
    with pytest.raises(RuntimeError, match="Axis index"):
        LinkPositionBoundCst(kin, j, BaseType.FIXED, robot.end_link, 3, lb=0.0)
    with pytest.raises(RuntimeError, match="At least one"):
        LinkPositionBoundCst(kin, j, BaseType.FIXED, robot.end_link, 1)
    specs = _specs(robot)
    sc = SphereCollisionCst(kin, j, BaseType.FIXED, specs, [], None, True)
    comp = IneqCompositeCst([sc, b])
    assert comp.cst_dim() == sc.cst_dim() + 1 and comp.q_dim() == 7
    assert "LinkPositionBoundCst: 1" in str(comp)
    other = KinematicModel(robot.urdf)
    with pytest.raises(RuntimeError, match="same kinematic chain"):
        IneqCompositeCst([sc, LinkPositionBoundCst(other, j, BaseType.FIXED, robot.end_link, 2, lb=0.1)])
    assert comp.fused_parts() == (sc, [b])
    assert IneqCompositeCst([sc]).fused_parts() == (sc, [])
    assert IneqCompositeCst([b]).fused_parts() is None  # no collision constraint: the members' own checks
    # the fused C entry point checks its members before any device work
    import ctypes as C

    from plainmp_gb300 import _lib

    q = np.zeros((2, 7))
    out = np.zeros(2, dtype=np.uint8)
    for bad, msg in ((c, "inequality"), (LinkPositionBoundCst(other, j, BaseType.FIXED, robot.end_link, 2, lb=0.1), "same kinematic chain"),
                     (LinkPositionBoundCst(kin, j[:6], BaseType.FIXED, robot.end_link, 2, lb=0.1), "control joints")):
        hs = (C.c_void_p * 1)(bad._h)
        rc = _lib.lib.pmgpu_composite_is_valid_fast(sc._h, hs, 1, q.ctypes.data, 2, out.ctypes.data, None, _lib.MEM_HOST, None)
        assert rc != 0 and msg in _lib.lib.pmgpu_last_error().decode()
    assert _lib.lib.pmgpu_composite_is_valid_fast(sc._h, None, -1, q.ctypes.data, 2, out.ctypes.data, None, _lib.MEM_HOST, None) != 0


def test_sequential_cst_bookkeeping():
    """SequentialCst dimensions (sequential_constraint.cpp:14-61): add_at range check, fixed points
    clear their step's constraints at finalize, the motion-step box adds 2 q_dim rows per step."""
    from plainmp_gb300 import BaseType, KinematicModel, LinkPoseCst
    from plainmp_gb300.sequential import SequentialCst
    from plainmp_gb300 import workloads as W

    robot = W.chain7_robot()
    kin = KinematicModel(robot.urdf)
    c = LinkPoseCst(kin, robot.control_joints, BaseType.FIXED, [robot.end_link], [np.zeros(3)])
    s = SequentialCst(5, 7)
    s.add_globally(c)
    assert s.cst_dim() == 15 and s.x_dim() == 35
    with pytest.raises(RuntimeError, match="out of range"):
        s.add_at(c, 5)
    s.add_fixed_point_at(np.zeros(7), 0)
    s.add_fixed_point_at(np.zeros(7), 4)
    s.add_motion_step_box_constraint(np.full(7, 0.1))
    assert s.cst_dim() == 15 + 14 + 56
    s.finalize()
    assert s.cst_dim() == 9 + 14 + 56
    assert "fixed point: 7" in str(s)


def test_bench_reference_arm_line():
    """bench.py --impl reference (the CPU restatement on the host cores) prints the one JSON line
    of the benchmark contract, with the reference arm's own cpu_baseline and a zero-copy e2e."""
    import json
    import subprocess
    import sys

    r = subprocess.run([sys.executable, str(REPO / "bench.py"), "--impl", "reference", "--steps", "1", "--warmup", "1"],
                       capture_output=True, text=True, timeout=300, cwd=str(REPO))
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for k in ("impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference" and d["metric"] == "configs checked/sec" and d["unit"] == "configs/s"
    assert d["value"] > 0 and d["higher_is_better"] is True
    assert d["cpu_baseline"]["value"] == d["value"] and d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    assert str(d["config"]["batch_configs"]) in d["cpu_baseline"]["sample"]  # the whole batch, every step


def test_bench_reference_arm_loads_no_product_library():
    """The reference arm runs the oracle alone: neither the product package nor its library is
    loaded into its process (the seeded generators come by file path)."""
    import subprocess
    import sys

    code = ("import argparse, sys; sys.path.insert(0, %r); import bench; "
            "bench.run_reference(argparse.Namespace(steps=1, warmup=0, gpus=1)); "
            "maps = open('/proc/self/maps').read(); "
            "assert 'libpmgpu' not in maps, 'product library loaded'; "
            "assert 'liboracle' in maps; "
            "assert not any(m == 'plainmp_gb300' or m.startswith('plainmp_gb300.') for m in sys.modules), 'package imported'; "
            "print('clean')") % str(REPO)
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=300, cwd=str(REPO))
    assert r.returncode == 0, r.stderr[-2000:]
    assert r.stdout.strip().endswith("clean")


def test_output_buffers_are_validated():
    """A preallocated output is written in place, so one of the wrong dtype, shape or layout is
    refused before any device work (a converted copy would receive the results instead, and a
    short buffer would be overrun)."""
    from plainmp_gb300 import BoxMotionValidator, scenes
    from plainmp_gb300 import workloads as W

    _, cst, _ = scenes.make_constraint(W.chain7_robot(), W.chain7_scene())
    Q = W.chain7_configs(8)
    ns = cst.n_spheres
    for bad in (np.zeros(8, np.int32), np.zeros(7, np.uint8), np.zeros(16, np.uint8)[::2], np.zeros((8, 1), np.uint8)):
        with pytest.raises(ValueError):
            cst.is_valid_fast(Q, out=bad)
    for bad in (np.zeros((8, ns), np.float64), np.zeros((8, ns + 1), np.float32), np.zeros((ns, 8), np.float32).T):
        with pytest.raises(ValueError):
            cst.is_valid_fast(Q, distances=True, out=np.zeros(8, np.uint8), dist_out=bad)
    ro = np.zeros(8, np.uint8)
    ro.setflags(write=False)
    with pytest.raises(ValueError):
        cst.is_valid_fast(Q, out=ro)
    s1, s2 = W.chain7_edges(4)
    mv = BoxMotionValidator(cst, [0.05] * 7)
    with pytest.raises(ValueError):
        mv.check_motion_fast(s1, s2, out=np.zeros(3, np.uint8))


def test_bench_issue_rate():
    """The issue-utilisation figure of the bench line: the committed capture's warp instructions per
    launch over a launch time, against 4 warp instructions per SM per cycle."""
    import json
    import sys

    sys.path.insert(0, str(REPO))
    import bench

    assert bench.issue_rate(None, 1.0, 2070.0, 152) is None
    assert bench.issue_rate(1e9, 1.0, None, 152) is None
    r = bench.issue_rate(1258.56e6, 1.0, 2070.0, 152)  # exactly the ceiling for 1 ms at 2070 MHz
    assert abs(r["frac"] - 1.0) < 1e-12 and abs(r["peak"] - 1258.56) < 1e-9
    pj = json.loads((REPO / "profiles" / "k_fast_valid_dualarm65536.traffic.json").read_text())
    per = pj["per_kernel"]
    assert pj["warp_instructions_per_launch"] == sum(v["warp_instructions"] for v in per.values())
    for k, v in per.items():  # the capture's own durations give its issue-active share, roughly
        f = bench.issue_rate(v["warp_instructions"], v["ms"], 2070.0, 152)["frac"]
        assert abs(f * 100 - v["issue_active_pct"]) < 6.0, (k, f)


def test_batch_entry_points_refuse_null_arrays():
    """Every batch entry point of the C ABI refuses a NULL required array of a non-empty batch with
    PMGPU_ERR_INVALID (in device memory it would fault the kernel that reads it), and a negative
    count, before any device work; optional outputs stay optional."""
    import ctypes as C

    from plainmp_gb300 import BaseType, CloudSDF, KinematicModel, LinkPositionBoundCst, _lib, scenes
    from plainmp_gb300 import workloads as W

    lib = _lib.lib
    robot = W.chain7_robot()
    kin, cst, _ = scenes.make_constraint(robot, W.chain7_scene())
    h = cst._h
    b = LinkPositionBoundCst(KinematicModel(robot.urdf), robot.control_joints, BaseType.FIXED, robot.end_link, 2, lb=0.1)
    cloud = CloudSDF(np.zeros((4, 3)), 0.0)
    q = np.zeros((4, 7))
    qf = np.zeros((4, 7), np.float32)
    u8 = np.zeros(16, np.uint8)
    f64 = np.zeros(64)
    f32 = np.zeros(64, np.float32)
    off = np.array([0, 4], np.int64)
    P = lambda a: C.c_void_p(a.ctypes.data)  # noqa: E731
    N = None
    H = _lib.MEM_HOST
    cases = {
        "q": [lambda: lib.pmgpu_cst_is_valid(h, N, 4, P(u8), H, N),
              lambda: lib.pmgpu_cst_evaluate(h, N, 4, P(f64), P(f64), H, N),
              lambda: lib.pmgpu_cst_sphere_distances(h, N, 4, 0, P(f64), N, H, N),
              lambda: lib.pmgpu_cst_is_valid_fast(h, N, 4, P(u8), N, N, H, N),
              lambda: lib.pmgpu_cst_link_poses(h, 3, N, 4, P(f64), H, N),
              lambda: lib.pmgpu_posecst_evaluate(b._h, N, 4, P(f64), P(f64), H, N),
              lambda: lib.pmgpu_posecst_is_valid(b._h, N, 4, P(u8), H, N),
              lambda: lib.pmgpu_ik_cost(h, N, N, N, 4, P(f32), N, H, N),
              lambda: lib.pmgpu_ik_descend(h, N, N, N, 4, 1, C.c_float(0.1), 0, N, N, H, N),
              lambda: lib.pmgpu_traj_cost(h, N, N, P(off), 1, 4, P(f32), N, H, N),
              lambda: lib.pmgpu_cst_update_kintree(h, N, 1),
              lambda: lib.pmgpu_posecst_update_kintree(b._h, N, 1)],
        "out": [lambda: lib.pmgpu_cst_is_valid(h, P(q), 4, N, H, N),
                lambda: lib.pmgpu_cst_is_valid_fast(h, P(q), 4, N, N, N, H, N),
                lambda: lib.pmgpu_posecst_is_valid(b._h, P(q), 4, N, H, N),
                lambda: lib.pmgpu_check_motion(h, P(q), P(q), 4, 1, N, 0.1, N, N, H, N),
                lambda: lib.pmgpu_check_motion_fast(h, P(q), P(q), 4, 1, N, 0.1, N, N, H, N),
                lambda: lib.pmgpu_sdf_evaluate(cloud._h, P(f64), 4, N, H, N)],
        "vals": [lambda: lib.pmgpu_cst_evaluate(h, P(q), 4, N, P(f64), H, N)],
        "jac": [lambda: lib.pmgpu_cst_evaluate(h, P(q), 4, P(f64), N, H, N)],
        "out7": [lambda: lib.pmgpu_cst_link_poses(h, 3, P(q), 4, N, H, N)],
        "cost": [lambda: lib.pmgpu_ik_cost(h, N, P(qf), N, 4, N, N, H, N),
                 lambda: lib.pmgpu_traj_cost(h, N, P(qf), P(off), 1, 4, N, N, H, N)],
        "s1": [lambda: lib.pmgpu_check_motion(h, N, P(q), 4, 1, N, 0.1, P(u8), N, H, N),
               lambda: lib.pmgpu_check_motion_fast(h, N, P(q), 4, 1, N, 0.1, P(u8), N, H, N)],
        "s2": [lambda: lib.pmgpu_check_motion(h, P(q), N, 4, 1, N, 0.1, P(u8), N, H, N)],
        "points": [lambda: lib.pmgpu_sdf_evaluate(cloud._h, N, 4, P(f64), H, N),
                   lambda: lib.pmgpu_sdf_is_outside(cloud._h, N, P(f64), 4, P(u8), H, N),
                   lambda: lib.pmgpu_cloud_nearest(cloud._h, N, 4, P(f64), N, H, N)],
        "radii": [lambda: lib.pmgpu_sdf_is_outside(cloud._h, P(f64), N, 4, P(u8), H, N)],
    }
    for what, calls in cases.items():
        for i, call in enumerate(calls):
            rc = call()
            msg = lib.pmgpu_last_error().decode()
            assert rc == _lib.PMGPU_ERR_INVALID and msg.endswith(f"{what} is NULL"), (what, i, rc, msg)
    for call in (lambda: lib.pmgpu_cst_sphere_distances(h, P(q), -1, 0, N, N, H, N),
                 lambda: lib.pmgpu_check_motion(h, P(q), P(q), -1, 1, N, 0.1, P(u8), N, H, N),
                 lambda: lib.pmgpu_cloud_nearest(cloud._h, P(f64), -1, N, N, H, N)):
        assert call() == _lib.PMGPU_ERR_INVALID and "negative" in lib.pmgpu_last_error().decode()
    # an empty batch needs no arrays; optional outputs may be NULL (the call then reaches the device)
    assert lib.pmgpu_cst_is_valid(h, N, 0, N, H, N) in (_lib.PMGPU_OK, _lib.PMGPU_ERR_CUDA)
    assert lib.pmgpu_cst_sphere_distances(h, P(q), 4, 0, N, N, H, N) in (_lib.PMGPU_OK, _lib.PMGPU_ERR_CUDA)


def test_add_new_link():
    """KinematicModel.add_new_link (kinematics.cpp:292-338 via kinematic_model_wrapper.cpp:31-39): the
    new link gets the next id under the given name; a name given twice raises RuntimeError
    (tests/test_kinematics.py:20-35); an unknown parent raises ValueError (get_link_ids,
    kinematics.cpp:264-276). Host work only."""
    from plainmp_gb300 import KinematicModel
    from plainmp_gb300 import workloads as W

    robot = W.chain7_robot()
    kin = KinematicModel(robot.urdf)
    n = kin.num_links
    i = kin.add_new_link("hahahahah", "link1", [0.1, 0, 0], [0, 0, 0.3], True)
    assert i == n and kin.num_links == n + 1
    assert list(kin.get_link_ids(["hahahahah"])) == [i] and kin.link_name(i) == "hahahahah"
    with pytest.raises(RuntimeError, match="already exists"):
        kin.add_new_link("hahahahah", "link1", [0, 0, 0], [0, 0, 0], True)
    with pytest.raises(ValueError, match="no link named"):
        kin.add_new_link("other", "nolink", [0, 0, 0], [0, 0, 0], True)
    assert kin.num_links == n + 1
    j = kin.add_new_link("child_of_new", "hahahahah", [0, 0, 0.2], [0, 0, 0], False)
    assert j == n + 1


def test_kdtree_and_module_layout():
    """plainmp.kdtree.KDTree (bindings/kdtree.cpp:20-23) and plainmp.constraint.SequentialCst
    (bindings/constraint.cpp:114-125) are where the reference's modules have them; an empty KDTree
    answers sqdist with the largest double, as kdtree.cpp:33-38 does; a query is one 3-vector."""
    import plainmp_gb300 as pm
    from plainmp_gb300.constraint import SequentialCst
    from plainmp_gb300.kdtree import KDTree

    assert pm.KDTree is KDTree and pm.SequentialCst is SequentialCst
    empty = KDTree(np.zeros((0, 3)))
    assert len(empty) == 0 and empty.sqdist([0.0, 0.0, 0.0]) == np.finfo(np.float64).max
    assert np.isnan(empty.query([1.0, 2.0, 3.0])).all()
    tree = KDTree([[0.0, 0.0, 0.0], [1.0, 1.0, 1.0]])  # a list of 3-vectors, as the reference takes
    assert len(tree) == 2
    with pytest.raises(ValueError):
        tree.query([1.0, 2.0])
    with pytest.raises(ValueError):
        KDTree(np.zeros((4, 2)))


def test_class_hierarchy_matches_reference():
    """The reference's base classes (psdf.pyi:36-109, constraint.pyi:9-113): isinstance checks of
    user code hold, and a composite refuses members of the other kind, as the bound member types
    do (bindings/constraint.cpp:105, 109)."""
    import plainmp_gb300 as pm
    from plainmp_gb300 import workloads as W

    for cls in (pm.BoxSDF, pm.CylinderSDF, pm.SphereSDF):
        assert issubclass(cls, pm.ClosedPrimitiveSDFBase) and issubclass(cls, pm.PrimitiveSDFBase)
    for cls in (pm.GroundSDF, pm.CloudSDF):
        assert issubclass(cls, pm.PrimitiveSDFBase) and not issubclass(cls, pm.ClosedPrimitiveSDFBase)
    assert issubclass(pm.UnionSDF, pm.SDFBase) and not issubclass(pm.UnionSDF, pm.PrimitiveSDFBase)
    assert issubclass(pm.SphereCollisionCst, pm.IneqConstraintBase)
    assert issubclass(pm.LinkPositionBoundCst, pm.IneqConstraintBase)
    assert issubclass(pm.LinkPoseCst, pm.EqConstraintBase)
    assert issubclass(pm.EqConstraintBase, pm.ConstraintBase) and issubclass(pm.IneqConstraintBase, pm.ConstraintBase)
    robot = W.chain7_robot()
    kin = pm.KinematicModel(robot.urdf)
    j = robot.control_joints
    pose = pm.LinkPoseCst(kin, j, pm.BaseType.FIXED, [robot.end_link], [np.zeros(3)])
    bound = pm.LinkPositionBoundCst(kin, j, pm.BaseType.FIXED, robot.end_link, 2, lb=0.1)
    assert pm.EqCompositeCst([pose]).cst_dim() == 3 and pm.IneqCompositeCst([bound]).cst_dim() == 1
    with pytest.raises(TypeError):
        pm.EqCompositeCst([bound])
    with pytest.raises(TypeError):
        pm.IneqCompositeCst([pose])


def test_bench_cpu_baseline_rows():
    """bench.py's cpu_baseline: the oracle on all host cores and on one core, over bounded samples
    of the headline batch (a short time limit here)."""
    import sys

    sys.path.insert(0, str(REPO))
    import bench

    robot, scene, q = bench.workload()
    cb = bench.cpu_baseline(robot, scene, q, seconds=0.3)
    assert cb["value"] > 0 and cb["cores"] >= 1 and cb["kind"] == "port"
    assert cb["single_core"]["value"] > 0 and cb["single_core"]["cores"] == 1
    assert cb["value"] >= 0.5 * cb["single_core"]["value"]
    assert isinstance(cb["cpu_model"], str) and cb["cpu_model"]
    assert cb["build"] == "-O3 -ffp-contract=off"
    cc = cb["contract_build"]  # the second build, contraction on, timed in a child process
    assert cc.get("value", 0) > 0, cc
    assert cc["build"] == "-O3 -ffp-contract=fast" and cc["cores"] == cb["cores"]


def test_bench_nvml_poller():
    """bench.py's NVML clock poller: without NVML (or a GPU) it yields no summary, so the
    nvidia-smi sampler's stands; its summary decodes the clock-event reason bits."""
    import sys
    import time

    sys.path.insert(0, str(REPO))
    import bench

    with bench.NvmlPoller(0, "0000-fake-uuid") as nv:
        time.sleep(0.02)
    s = nv.summary()
    assert s is None or (s["samples"] > 0 and s["sm_mhz"] > 0)
    p = bench.NvmlPoller(0)
    p.samples = [(2070.0, 0x0), (2070.0, 0x4), (1995.0, 0x4 | 0x40), (2070.0, 0x1)]
    p.max_mhz = 2070.0
    s = p.summary()
    assert s["sm_mhz"] == 2070.0 and s["samples"] == 4
    assert s["reasons"] == ["hw_thermal_slowdown", "sw_power_cap"]
    assert bench.NvmlPoller(0, "abc").uuid == "GPU-abc" and bench.NvmlPoller(0, "GPU-abc").uuid == "GPU-abc"


def test_bench_traj_cost_check(monkeypatch):
    """bench.py's C4 FP64 check on stand-ins for the device calls: the reference is the smoothing
    term plus the hinge of the FP64 distances, per trajectory, and the reported error is relative."""
    import sys

    sys.path.insert(0, str(REPO))
    import bench
    from plainmp_gb300 import diff
    from plainmp_gb300 import workloads as W

    trajs = W.trajectories(20, seed=3)
    q32 = np.concatenate(trajs, axis=0).astype(np.float32)
    off = np.concatenate([[0], np.cumsum([len(t) for t in trajs])]).astype(np.int64)

    class FakeCst:
        def groups(self):
            return {"only_self": np.zeros(3, bool)}

        def sphere_distances(self, P, high_accuracy=False):
            return np.full((len(P), 4), 0.01) + 0.001 * np.arange(4)  # every sphere inside the 0.03 margin

    def fake_cost(cst, q, o, want_grad=True):
        P = q.astype(np.float64)
        out = []
        for i in range(len(o) - 1):
            T = P[o[i]:o[i + 1]]
            acc = T[2:] - 2 * T[1:-1] + T[:-2]
            d = cst.sphere_distances(T)
            out.append((acc ** 2).sum() + (np.maximum(0.03 - d, 0) ** 2).sum())
        return np.asarray(out, np.float32)

    monkeypatch.setattr(diff, "traj_cost_grad", fake_cost)
    r = bench.traj_cost_check(FakeCst(), q32, off)
    assert r["trajectories"] == 16 and 0 <= r["max_rel_err"] < 1e-6  # FP32 rounding of the cost only


def test_fast_tuning_arguments():
    """The fast kernels' tuning parameters (the autotuner's sphere tile, hard-query grid and edge
    shape): defaults, a round trip and the refusals of unsupported values, all on the host."""
    from plainmp_gb300 import scenes
    from plainmp_gb300 import workloads as W

    _, cst, _ = scenes.make_constraint(W.chain7_robot(), W.chain7_scene())
    assert cst.get_fast_tuning() == (0, 4, 32, 128)
    cst.set_fast_tuning(8, 2, 64, 256)
    assert cst.get_fast_tuning() == (8, 2, 64, 256)
    for bad in ((3, 4, 32, 128), (64, 4, 32, 128), (0, 0, 32, 128), (0, 9, 32, 128), (0, 4, 8, 64), (0, 4, 32, 512)):
        with pytest.raises(ValueError):
            cst.set_fast_tuning(*bad)
    assert cst.get_fast_tuning() == (8, 2, 64, 256)
