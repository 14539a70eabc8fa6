"""GPU parity of the pose constraints (LinkPoseCst, LinkPositionBoundCst) and the composite
constraints against the oracle's FK and get_jacobian restatement (kinematics/algorithm.cpp:
212-344).  Values and joint columns agree within 1e-9 (CUDA vs glibc sin/cos in the FK with
high accuracy); PLANAR/FLOATING base columns are the reference's forward differences with
eps = 1e-7, which amplify 1-ulp differences, and agree within 1e-6.  Validity after
update_kintree(q, False) (Taylor sin/cos) is bit-exact."""
import numpy as np
import pytest

from plainmp_gb300 import BaseType, IneqCompositeCst, KinematicModel, LinkPoseCst, LinkPositionBoundCst, scenes
from plainmp_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def rpy_of(q):
    """Transform::getRPY (transform.hpp:93-120) of a quaternion [x y z w]."""
    x, y, z, w = q
    sarg = -2 * (x * z - w * y)
    if sarg <= -0.99999:
        return np.array([0.0, -np.pi / 2, -2 * np.arctan2(x, y)])
    if sarg >= 0.99999:
        return np.array([0.0, np.pi / 2, 2 * np.arctan2(x, y)])
    return np.array([np.arctan2(2 * (y * z + w * x), w * w - x * x - y * y + z * z), np.arcsin(sarg),
                     np.arctan2(2 * (x * y + w * z), w * w + x * x - y * y - z * z)])


def oracle_pose_cst(oracle, robot, base, links, dims, targets, Q):
    """Per configuration: update_kintree(q) then LinkPoseCst::evaluate_dirty on the oracle model."""
    om, oc, _ = oracle.make_constraint(robot, None, self_collision=False)
    ids = [om.joint_id(j) for j in robot.control_joints]
    lids = [om.link_id(n) for n in links]
    bt = {"FIXED": 0, "FLOATING": 1, "PLANAR": 2}[base]
    vals, jacs = [], []
    for q in Q:
        oc.update_kintree(q, True)
        v, J = [], []
        for lid, d, t in zip(lids, dims, targets):
            p = om.link_pose(lid)
            if d == 3:
                v.append(p[:3] - t)
                J.append(om.link_jacobian(lid, ids, 0, bt))
            elif d == 6:
                v.append(np.concatenate([p[:3] - t[:3], rpy_of(p[3:]) - t[3:]]))
                J.append(om.link_jacobian(lid, ids, 1, bt))
            else:
                v.append(p - t)
                J.append(om.link_jacobian(lid, ids, 2, bt))
        vals.append(np.concatenate(v))
        jacs.append(np.concatenate(J, axis=0))
    return np.array(vals), np.array(jacs)


def robot_with_base(base):
    r = W.chain7_robot()
    return W.Robot(r.urdf, r.control_joints, r.end_link, r.spheres, r.self_pairs, base_type=base)


def configs(base, n, seed):
    rng = np.random.default_rng(seed)
    q = rng.uniform(-np.pi, np.pi, (n, 7))
    nb = {"FIXED": 0, "PLANAR": 3, "FLOATING": 6}[base]
    return np.concatenate([q, rng.uniform(-0.5, 0.5, (n, nb))], axis=1) if nb else q


@pytest.mark.parametrize("base", ["FIXED", "PLANAR", "FLOATING"])
def test_link_pose_cst_matches_oracle(oracle, base):
    robot = robot_with_base(base)
    kin = KinematicModel(robot.urdf)
    links, dims = [robot.end_link, "link3", "link5"], [7, 3, 6]
    rng = np.random.default_rng(9)
    targets = [rng.normal(size=d) for d in dims]
    c = LinkPoseCst(kin, robot.control_joints, BaseType[base], links, targets)
    Q = configs(base, 48, 3)
    vals, jac = c.evaluate_batch(Q)
    rv, rj = oracle_pose_cst(oracle, robot, base, links, dims, targets, Q)
    assert vals.shape == rv.shape and jac.shape == rj.shape
    assert np.abs(vals - rv).max() < 1e-9
    nj = 7
    assert np.abs(jac[:, :, :nj] - rj[:, :, :nj]).max() < 1e-9
    if base != "FIXED":
        assert np.abs(jac[:, :, nj:] - rj[:, :, nj:]).max() < 1e-6
    # single-configuration call
    v1, j1 = c.evaluate(Q[5])
    assert np.array_equal(v1, vals[5]) and np.array_equal(j1, jac[5])


def test_link_position_bound(oracle):
    robot = W.chain7_robot()
    kin = KinematicModel(robot.urdf)
    om, oc, _ = oracle.make_constraint(robot, None, self_collision=False)
    lid = om.link_id(robot.end_link)
    ids = [om.joint_id(j) for j in robot.control_joints]
    Q = W.chain7_configs(512, seed=8)
    for axis, lb, ub in [(2, 0.2, None), (0, None, 0.3), (1, -0.4, 0.4)]:
        b = LinkPositionBoundCst(kin, robot.control_joints, BaseType.FIXED, robot.end_link, axis, lb=lb, ub=ub)
        ok = b.is_valid_batch(Q)
        ref = []
        for q in Q:  # IneqConstraintBase::is_valid: update_kintree(q, false) (Taylor sin/cos)
            oc.update_kintree(q, False)
            p = om.link_pose(lid)[axis]
            ref.append((lb is None or p >= lb) and (ub is None or p <= ub))
        assert np.array_equal(ok.astype(bool), np.array(ref))
        assert 0 < ok.sum() < len(Q)
        vals, jac = b.evaluate_batch(Q[:32])
        for k, q in enumerate(Q[:32]):
            oc.update_kintree(q, True)
            p = om.link_pose(lid)[axis]
            J = om.link_jacobian(lid, ids, 0, 0)[axis]
            rv, rj = [], []
            if lb is not None:
                rv.append(p - lb)
                rj.append(J)
            if ub is not None:
                rv.append(ub - p)
                rj.append(-J)
            assert np.abs(vals[k] - np.array(rv)).max() < 1e-9
            assert np.abs(jac[k] - np.array(rj)).max() < 1e-9


def test_ineq_composite(oracle):
    import torch

    robot, scene = W.chain7_robot(), W.chain7_scene()
    kin, cst, _ = scenes.make_constraint(robot, scene)
    b = LinkPositionBoundCst(kin, robot.control_joints, BaseType.FIXED, robot.end_link, 2, lb=0.0)
    comp = IneqCompositeCst([cst, b])
    Q = W.chain7_configs(2048, seed=12)
    om, oc, _ = oracle.make_constraint(robot, scene)
    lid = om.link_id(robot.end_link)
    ref_s = oc.is_valid(Q, threads=8).astype(bool)
    ref_b = []
    for q in Q:
        oc.update_kintree(q, False)
        ref_b.append(om.link_pose(lid)[2] >= 0.0)
    ref = ref_s & np.array(ref_b)
    assert 0 < ref.sum() < len(Q)
    assert np.array_equal(comp.is_valid_batch(Q).astype(bool), ref)
    assert np.array_equal(comp.is_valid_batch(Q, fast=False).astype(bool), ref)
    Qd = torch.tensor(Q, device="cuda")
    assert np.array_equal(comp.is_valid_batch(Qd).cpu().numpy().astype(bool), ref)
    vals, jac = comp.evaluate_batch(Q[:16])
    v1, j1 = cst.evaluate_batch(Q[:16])
    v2, j2 = b.evaluate_batch(Q[:16])
    assert np.array_equal(vals, np.concatenate([v1, v2], axis=1)) and np.array_equal(jac, np.concatenate([j1, j2], axis=1))
    assert comp.is_valid(Q[0]) == bool(ref[0])


def test_pose_constraint_update_kintree():
    """ConstraintBase.update_kintree of a pose constraint (bindings/constraint.cpp:31-32) sets the
    shared model exactly as the collision constraint's does (primitive.hpp:38-62)."""
    robot = W.chain7_robot()
    kin, cst, _ = scenes.make_constraint(robot, W.chain7_scene())
    b = LinkPositionBoundCst(kin, robot.control_joints, BaseType.FIXED, robot.end_link, 2, lb=0.1)
    q = W.chain7_configs(2, seed=7)
    for high_accuracy in (True, False):
        cst.update_kintree(q[0], high_accuracy)
        ref = kin.debug_get_link_pose(robot.end_link)
        cst.update_kintree(q[1], high_accuracy)
        b.update_kintree(q[0], high_accuracy)
        np.testing.assert_array_equal(kin.debug_get_link_pose(robot.end_link), ref)
        np.testing.assert_array_equal(kin.get_joint_positions(kin.get_joint_ids(robot.control_joints)), q[0])
