"""SequentialCst.evaluate on the device batches against the reference's per-step loop restated on
the oracle (sequential_constraint.cpp:63-127), including its waypoint offset that advances only
over steps with constraints."""
import numpy as np
import pytest

from plainmp_gb300 import BaseType, KinematicModel, LinkPoseCst, scenes
from plainmp_gb300 import workloads as W
from plainmp_gb300.sequential import SequentialCst

pytestmark = pytest.mark.gpu


def test_sequential_cst_matches_reference_loop(oracle):
    robot, scene = W.chain7_robot(), W.chain7_scene()
    kin, cst, _ = scenes.make_constraint(robot, scene)
    om, oc, _ = oracle.make_constraint(robot, scene)
    T, d = 12, 7
    rng = np.random.default_rng(4)
    x = rng.uniform(-np.pi, np.pi, T * d)
    goal = rng.normal(size=3)
    pose = LinkPoseCst(kin, robot.control_joints, BaseType.FIXED, [robot.end_link], [goal])
    s = SequentialCst(T, d)
    s.add_globally(cst)
    s.add_at(pose, T - 1)
    s.add_fixed_point_at(x[:d] + 0.01, 0)
    s.add_motion_step_box_constraint(np.full(d, 0.2))
    s.finalize()
    c, J = s.evaluate(x)
    J = J.toarray()
    assert c.shape == (s.cst_dim(),) and J.shape == (s.cst_dim(), s.x_dim())
    # the reference's loop, on the oracle
    lid = om.link_id(robot.end_link)
    ids = [om.joint_id(j) for j in robot.control_joints]
    rc, rJ = np.zeros(s.cst_dim()), np.zeros((s.cst_dim(), s.x_dim()))
    x_head = c_head = 0
    for t in range(T):
        q = x[x_head:x_head + d]
        if t == 0:  # cleared by the fixed point
            continue
        v, jac = oc.evaluate(q[None, :])
        m = v.shape[1]
        rc[c_head:c_head + m] = v[0]
        rJ[c_head:c_head + m, x_head:x_head + d] = jac[0] + 1e-12
        c_head += m
        if t == T - 1:
            oc.update_kintree(q, True)
            rc[c_head:c_head + 3] = om.link_pose(lid)[:3] - goal
            rJ[c_head:c_head + 3, x_head:x_head + d] = om.link_jacobian(lid, ids, 0, 0) + 1e-12
            c_head += 3
        x_head += d
    rc[c_head:c_head + d] = x[:d] - (x[:d] + 0.01)
    rJ[c_head:c_head + d, :d] = np.eye(d)
    c_head += d
    for t in range(T - 1):
        q1, q2 = x[t * d:(t + 1) * d], x[(t + 1) * d:(t + 2) * d]
        rc[c_head:c_head + d] = q1 - q2 + 0.2
        rc[c_head + d:c_head + 2 * d] = q2 - q1 + 0.2
        rJ[c_head:c_head + d, t * d:(t + 1) * d] = np.eye(d)
        rJ[c_head:c_head + d, (t + 1) * d:(t + 2) * d] = -np.eye(d)
        rJ[c_head + d:c_head + 2 * d, t * d:(t + 1) * d] = -np.eye(d)
        rJ[c_head + d:c_head + 2 * d, (t + 1) * d:(t + 2) * d] = np.eye(d)
        c_head += 2 * d
    assert c_head == s.cst_dim()
    assert np.abs(c - rc).max() < 1e-9
    # the collision rows' SDF gradient is a forward difference (h = 1e-6) of FP64 values that
    # carry the 1e-9 libm differences, hence the looser Jacobian bound
    assert np.abs(J - rJ).max() < 1e-6
