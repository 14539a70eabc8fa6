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


def _oracle_bound_ok(oc, om, lid, q, bounds):
    """LinkPositionBoundCst::is_valid_dirty after update_kintree(q, false) (Taylor sin/cos),
    every (axis, lb, ub) of `bounds` on link lid."""
    oc.update_kintree(q, False)
    p = om.link_pose(lid)
    return all((lb is None or p[ax] >= lb) and (ub is None or p[ax] <= ub) for ax, lb, ub in bounds)


def test_ineq_composite_fused_at_bound_edges(oracle):
    """The fused composite path (one launch, one FK) against the oracle, with bounds placed exactly
    on the FP64 link positions of some configurations: those comparisons fall inside the FP32
    error band and are decided by the FP64 recheck, bit for bit (p == lb passes, the next double
    above p as lb fails)."""
    import torch

    robot, scene = W.chain7_robot(), W.chain7_scene()
    kin, cst, _ = scenes.make_constraint(robot, scene)
    Q = W.chain7_configs(4096, seed=21)
    om, oc, _ = oracle.make_constraint(robot, scene)
    lid = om.link_id(robot.end_link)
    pz = []
    for q in Q[:8]:
        oc.update_kintree(q, False)
        pz.append(om.link_pose(lid).copy())
    bounds = [(2, float(pz[0][2]), None),                        # config 0 exactly at lb: passes
              (0, None, float(pz[1][0])),                        # config 1 exactly at ub: passes
              (1, float(np.nextafter(pz[2][1], np.inf)), None)]  # config 2 one double below lb: fails
    mk = [LinkPositionBoundCst(kin, robot.control_joints, BaseType.FIXED, robot.end_link, ax, lb=lb, ub=ub) for ax, lb, ub in bounds]
    comp = IneqCompositeCst([cst] + mk)
    assert comp.fused_parts() is not None
    ref_s = oc.is_valid(Q, threads=8).astype(bool)
    ref = np.array([s and _oracle_bound_ok(oc, om, lid, q, bounds) for s, q in zip(ref_s, Q)])
    assert 0 < ref.sum() < len(Q)
    got, st = comp.is_valid_fast(Q, stats=True)
    assert np.array_equal(got.astype(bool), ref)
    assert st["rechecked_terms"] > 0  # the boundary configurations went to the FP64 recheck
    # the same booleans as the members' own plain checks, and on device tensors
    plain = cst.is_valid_batch(Q).astype(bool)
    for b in mk:
        plain &= b.is_valid_batch(Q).astype(bool)
    assert np.array_equal(plain, ref)
    Qd = torch.tensor(Q, device="cuda")
    assert np.array_equal(comp.is_valid_batch(Qd).cpu().numpy().astype(bool), ref)
    # the members' order does not matter
    comp2 = IneqCompositeCst(mk[::-1] + [cst])
    assert np.array_equal(comp2.is_valid_batch(Q).astype(bool), ref)


def _oracle_edge_waypoints(S1, S2, width, seq):
    """The states checkMotion tests for each edge, in order (motion_validator.cpp:17-79, 89-111):
    none when the step ratio is infinite, else s2 first, then the interior points in the sequence
    table's order (or in plain order past 128 tests); interpolation s1 + (s2 - s1) t."""
    out = []
    for a, b in zip(S1, S2):
        d = b - a
        k = int(np.argmax(np.abs(d) / width))
        if abs(d[k]) < 1e-6:
            out.append([])
            continue
        r = width[k] / abs(d[k])
        n_test = int(np.floor(1 / r)) + 2
        if n_test < seq.shape[0] + 1:
            ts = [seq[n_test - 1][i] * r for i in range(2, n_test)]
        else:
            ts = [i * r for i in range(1, n_test - 1)]
        out.append([b] + [a + (b - a) * t for t in ts])
    return out


def test_composite_motion_validator(oracle):
    """checkMotion with a composite (collision + link-position bound) through the fused edge
    path, against the oracle's composite is_valid at every waypoint the reference would test."""
    from plainmp_gb300 import BoxMotionValidator

    robot, scene = W.chain7_robot(), W.chain7_scene()
    kin, cst, _ = scenes.make_constraint(robot, scene)
    bound = (2, 0.05, None)
    b = LinkPositionBoundCst(kin, robot.control_joints, BaseType.FIXED, robot.end_link, 2, lb=0.05)
    comp = IneqCompositeCst([cst, b])
    s1, s2 = W.chain7_edges(96, seed=4)
    width = np.full(7, 0.05)
    mv = BoxMotionValidator(comp, list(width))
    got = mv.check_motion_fast(s1, s2).astype(bool)
    om, oc, _ = oracle.make_constraint(robot, scene)
    lid = om.link_id(robot.end_link)
    wps = _oracle_edge_waypoints(s1, s2, width, oracle.sequence_table())
    ref = []
    for pts in wps:
        if not pts:
            ref.append(True)
            continue
        P = np.array(pts)
        ok_s = oc.is_valid(P, threads=8).astype(bool)
        ref.append(bool(all(s and _oracle_bound_ok(oc, om, lid, p, [bound]) for s, p in zip(ok_s, P))))
    ref = np.array(ref)
    assert 0 < ref.sum() < len(ref)
    assert np.array_equal(got, ref)
    # the collision constraint alone agrees with the plain edge method; the bound only removes edges
    alone = BoxMotionValidator(cst, list(width)).check_motion_batch(s1, s2).astype(bool)
    assert np.all(got <= alone)
    assert mv.checkMotion(s1[0], s2[0]) == bool(ref[0])
    with pytest.raises(TypeError):
        mv.check_motion_batch(s1, s2)


def test_ineq_composite_fused_bound_beyond_spheres(oracle):
    """A bound on a link no sphere chain reaches (spheres only on links 1-5, bounds on link7): the
    link joins the collision constraint's FK slots, and the fused check still equals the oracle's
    composite, here with a lower and an upper bound on different axes, on a PLANAR base."""
    r = W.chain7_robot()
    keep = {"link1", "link2", "link3", "link4", "link5"}
    robot = W.Robot(r.urdf, r.control_joints, r.end_link, [s for s in r.spheres if s.parent_link_name in keep],
                    [p for p in r.self_pairs if p[0] in keep and p[1] in keep], base_type="PLANAR")
    scene = W.chain7_scene()
    kin, cst, _ = scenes.make_constraint(robot, scene)
    bounds = [(0, -0.3, None), (2, None, 0.45)]
    mk = [LinkPositionBoundCst(kin, robot.control_joints, BaseType.PLANAR, "link7", ax, lb=lb, ub=ub) for ax, lb, ub in bounds]
    comp = IneqCompositeCst([cst] + mk)
    Q = configs("PLANAR", 2048, 31)
    om, oc, _ = oracle.make_constraint(robot, scene)
    lid = om.link_id("link7")
    ref_s = oc.is_valid(Q, threads=8).astype(bool)
    ref = np.array([s and _oracle_bound_ok(oc, om, lid, q, bounds) for s, q in zip(ref_s, Q)])
    assert 0 < ref.sum() < len(Q) and ref.sum() < ref_s.sum()
    assert np.array_equal(comp.is_valid_batch(Q).astype(bool), ref)
    # the collision constraint alone is unchanged by the extra slots
    assert np.array_equal(cst.is_valid_fast(Q).astype(bool), ref_s)
