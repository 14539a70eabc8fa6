"""CPU tests that pin the oracle (oracle/oracle.cpp) before the device path is compared with it:
golden vectors produced by the reference itself (tests/golden/, see make_golden.py) and the
reference's own known-answer and property tests restated (tests/test_psdf.py,
tests/test_kdtree.py, tests/test_constraints.py of the plainmp project)."""
import math

import numpy as np
import pytest

from helpers import golden, plainmp_numbering, rotz, rpy_matrix


def test_sequence_table_matches_reference_generator(oracle):
    rows = golden("sequence_table.json")["rows"]
    tab = oracle.sequence_table(128)
    for n in range(1, 129):
        assert list(tab[n - 1, :n]) == rows[n - 1]
    # motion_validator.cpp:24-42 and generate_sequence.py:39 known answers
    assert list(tab[7, :8]) == [0, 7, 4, 2, 6, 5, 3, 1]
    assert list(tab[19, :20]) == [0, 19, 10, 5, 15, 17, 13, 8, 3, 18, 16, 14, 12, 11, 9, 7, 6, 4, 2, 1]
    for n in range(2, 129):  # generate_sequence.py:66-73
        assert tab[n - 1, 0] == 0 and tab[n - 1, 1] == n - 1 and sorted(tab[n - 1, :n]) == list(range(n))


@pytest.mark.parametrize("name", ["chain7", "dualarm", "edge"])
def test_oracle_urdf_structure_matches_urdfdom(oracle, name):
    g = golden(f"urdf_{name}.json")
    order, parent, jorder = plainmp_numbering(g)
    m = oracle.Model(g["urdf"])
    assert m.n_link == len(order) and m.n_dof == len(jorder)
    st = m.structure()
    for i, ln in enumerate(order):
        assert m.link_id(ln) == i
    assert list(st["link_parent"]) == parent
    for k, jn in enumerate(jorder):
        assert m.joint_id(jn) == k
        assert st["joint_child"][k] == order.index(g["joints"][jn]["child"])
    # local transforms: origin translation and the urdfdom-normalised quaternion, bit for bit
    for jn, j in g["joints"].items():
        li = order.index(j["child"])
        tf = st["link_tf7"][li]
        assert list(tf[:3]) == j["xyz"]
        assert list(tf[3:]) == j["quat"]
        assert st["link_tf_qid"][li] == (abs(j["quat"][3] - 1.0) < 1e-6)


def test_taylor_sin_cos_known_values(oracle):
    # algorithm.cpp:50-86 evaluated directly: 9th/8th order Taylor of sin/cos with range reduction
    x = np.array([0.0, 0.1, -0.7, 1.5, 1.6, -1.6, 3.0, -3.0, 3.2, -3.2, 7.0, -13.0])
    s, c = oracle.approx_sin_cos(x)
    assert s[0] == 0.0 and c[0] == 1.0
    np.testing.assert_allclose(s, np.sin(x), atol=4e-6)
    np.testing.assert_allclose(c, np.cos(x), atol=3e-5)
    # the reduced branch flips the sign of cos across |x| = pi/2
    xx = 0.1
    s1, c1 = oracle.approx_sin_cos(np.array([xx]))
    ref_s = xx * (1 - xx * xx / 6 + xx ** 4 / 120 - xx ** 6 / 5040 + xx ** 8 / 362880)
    assert abs(s1[0] - ref_s) < 1e-17


def test_pose_alignment_flags(oracle):  # tests/test_psdf.py:27-39
    z = np.zeros(3)
    b = oracle.Sdf.box([1, 1, 1], z, np.eye(3))
    assert b.info()[2] and b.info()[3]
    b = oracle.Sdf.box([1, 1, 1], z, rpy_matrix(0.3, 0.0, 0.0))
    assert not b.info()[2] and b.info()[3]
    b = oracle.Sdf.box([1, 1, 1], z, rpy_matrix(0.3, 0.3, 0.3))
    assert not b.info()[2] and not b.info()[3]


def test_aabb_after_transform(oracle):  # tests/test_psdf.py:89-102
    b = oracle.Sdf.box([1, 1, 1], np.zeros(3), np.eye(3))
    b.translate([1.0, 2.0, 3.0])
    lb, ub, _, _ = b.info()
    np.testing.assert_allclose(lb, [0.5, 1.5, 2.5])
    np.testing.assert_allclose(ub, [1.5, 2.5, 3.5])
    b = oracle.Sdf.box([1, 1, 1], np.zeros(3), np.eye(3))
    b.rotate_z(np.pi * 0.25)
    lb, ub, _, _ = b.info()
    np.testing.assert_allclose(lb, [-0.5 * np.sqrt(2), -0.5 * np.sqrt(2), -0.5])
    np.testing.assert_allclose(ub, [0.5 * np.sqrt(2), 0.5 * np.sqrt(2), 0.5])


def test_ground_known_answer(oracle):  # tests/test_psdf.py:201-207
    g = oracle.Sdf.ground(1.0)
    assert g.evaluate([0.0, 0.0, 0.0])[0] == 1.0
    assert g.evaluate([1.0, 0.0, 0.0])[0] == 1.0


def _closed_sdfs(oracle, rng):
    out = []
    for i in range(10):
        xyz = rng.standard_normal(3)
        ypr = np.zeros(3) if i == 0 else (np.array([0.3, 0, 0]) if i == 1 else rng.standard_normal(3))
        R = rpy_matrix(*ypr)
        out.append(oracle.Sdf.box([1, 1, 1], xyz, R))
        out.append(oracle.Sdf.sphere(1.0, xyz, R))
        out.append(oracle.Sdf.cylinder(1.0, 1.0, xyz, R))
    return out


def _sk_box(p, w, pos, R):
    local = (p - pos) @ R
    d = np.abs(local) - 0.5 * np.asarray(w)
    return np.linalg.norm(np.maximum(d, 0), axis=1) + np.minimum(d.max(axis=1), 0)


def _sk_cyl(p, r, h, pos, R):
    local = (p - pos) @ R
    dr = np.linalg.norm(local[:, :2], axis=1) - r
    dz = np.abs(local[:, 2]) - 0.5 * h
    d = np.stack([dr, dz], axis=1)
    return np.linalg.norm(np.maximum(d, 0), axis=1) + np.minimum(d.max(axis=1), 0)


def test_sdf_values_and_is_outside_consistency(oracle):
    # tests/test_psdf.py:105-198: is_outside(p, r) == (evaluate(p) > r) for closed primitives,
    # values against closed-form SDFs
    rng = np.random.default_rng(0)
    for i in range(20):
        xyz = rng.standard_normal(3) * 0.5
        ypr = np.zeros(3) if i == 0 else (np.array([0.3, 0, 0]) if i == 1 else rng.standard_normal(3))
        R = rpy_matrix(*ypr)
        pts = rng.standard_normal((1000, 3))
        cases = [
            (oracle.Sdf.box([0.5, 0.3, 0.6], xyz, R), _sk_box(pts, [0.5, 0.3, 0.6], xyz, R)),
            (oracle.Sdf.cylinder(0.7, 0.2, xyz, R), _sk_cyl(pts, 0.7, 0.2, xyz, R)),
            (oracle.Sdf.sphere(0.5, xyz, R), np.linalg.norm(pts - xyz, axis=1) - 0.5),
        ]
        for sdf, sk in cases:
            np.testing.assert_allclose(sdf.evaluate(pts), sk, atol=1e-12)
            for r in [0.0] + list(rng.uniform(0, 0.3, 3)) + list(np.linspace(0.0, 2.0, 10)):
                assert np.array_equal(sdf.is_outside(pts, r).astype(bool), sdf.evaluate(pts) > r)


def test_union_and_ground_consistency(oracle):
    rng = np.random.default_rng(1)
    pts = rng.standard_normal((300, 3)) * 2
    b = oracle.Sdf.box([1, 1, 1], rng.standard_normal(3), rpy_matrix(*rng.standard_normal(3)))
    s = oracle.Sdf.sphere(1.0, np.zeros(3), np.eye(3))
    u = oracle.Sdf.union([b, s])
    np.testing.assert_array_equal(u.evaluate(pts), np.minimum(b.evaluate(pts), s.evaluate(pts)))
    for r in np.linspace(0.0, 2.0, 10):
        assert np.array_equal(u.is_outside(pts, r).astype(bool), u.evaluate(pts) > r)
    g = oracle.Sdf.ground(0.3)
    for r in np.linspace(0.0, 2.0, 10):
        assert np.array_equal(g.is_outside(pts, r).astype(bool), g.evaluate(pts) > r)


def test_kdtree_nearest_vs_brute_force(oracle):  # tests/test_kdtree.py:6-20
    rng = np.random.default_rng(2)
    pts = rng.standard_normal((1000, 3))
    c = oracle.Sdf.cloud(pts, 0.0)
    q = rng.standard_normal((1000, 3))
    sq, near = c.nearest(q)
    d2 = ((q[:, None, :] - pts[None, :, :]) ** 2).sum(-1)
    np.testing.assert_allclose(sq, d2.min(1), rtol=1e-12)
    np.testing.assert_allclose(near, pts[d2.argmin(1)])
    # exact: the squared distance equals fl(dx*dx + (dy*dy + dz*dz)) of the nearest point
    d = near - q
    assert np.array_equal(sq, d[:, 0] * d[:, 0] + (d[:, 1] * d[:, 1] + d[:, 2] * d[:, 2]))


def test_cloud_is_outside_consistency(oracle):  # tests/test_psdf.py:209-214
    rng = np.random.default_rng(3)
    c = oracle.Sdf.cloud(rng.random((100, 3)), 0.1)
    pts = rng.standard_normal((1000, 3)) * 1.5
    for r in np.linspace(0.0, 2.0, 10):
        assert np.array_equal(c.is_outside(pts, r).astype(bool), c.evaluate(pts) > r)


def _chain(oracle, scene=True, self_collision=True, base="FIXED"):
    from plainmp_gb300 import workloads as W

    r = W.chain7_robot()
    if base != "FIXED":
        r = W.Robot(r.urdf, r.control_joints, r.end_link, r.spheres, r.self_pairs, base_type=base)
    return oracle.make_constraint(r, W.chain7_scene() if scene else None, self_collision=self_collision)


@pytest.mark.parametrize("base", ["FIXED", "PLANAR", "FLOATING"])
def test_evaluate_is_valid_consistency(oracle, base):  # tests/test_constraints.py:47-53
    m, c, _ = _chain(oracle, base=base)
    rng = np.random.default_rng(4)
    Q = rng.standard_normal((300, c.q_dim)) * (1.0 if base == "FIXED" else 0.5)
    vals, _ = c.evaluate(Q)
    valid = c.is_valid(Q).astype(bool)
    # is_valid uses Taylor sin/cos (FIXED) while evaluate uses libm: they can only disagree
    # when a distance lies within the Taylor error of zero
    agree = np.all(vals > 0, axis=1) == valid
    assert agree.mean() > 0.99


@pytest.mark.parametrize("base", ["FIXED", "PLANAR", "FLOATING"])
def test_jacobian_vs_finite_difference(oracle, base):  # tests/test_constraints.py:22-44
    m, c, _ = _chain(oracle, base=base)
    rng = np.random.default_rng(5)
    eps = 1e-7
    checked = 0
    for _ in range(60):
        q = rng.standard_normal(c.q_dim) * (1.0 if base == "FIXED" else 0.1)
        v0, J = c.evaluate(q[None])
        Jn = np.zeros_like(J[0])
        for i in range(c.q_dim):
            q1 = q.copy()
            q1[i] += eps
            v1, _ = c.evaluate(q1[None])
            Jn[:, i] = (v1[0] - v0[0]) / eps
        # the min switches pieces near kinks; skip rows whose FD crosses one
        ok = np.abs(J[0] - Jn).max(axis=1) < 1e-4
        checked += int(ok.sum())
        assert ok.mean() >= 0.5
    assert checked > 60


def test_empty_constraint_is_valid_and_zero_rows(oracle):  # tests/test_constraints.py:165-175
    m, c, _ = _chain(oracle, scene=False, self_collision=False)
    rng = np.random.default_rng(6)
    Q = rng.standard_normal((30, c.q_dim))
    assert c.is_valid(Q).all()
    assert c.cst_dim == 0


def test_check_motion_matches_waypoint_definition(oracle):
    # motion_validator.cpp:17-79: the edge is valid iff s2 and every s1 + (s2-s1)*k*r,
    # k = 1..n-2, is valid
    from plainmp_gb300 import workloads as W

    m, c, _ = _chain(oracle)
    s1, s2 = W.chain7_edges(64)
    w = np.full(7, 0.05)
    out, n = c.check_motion(s1, s2, 0, w)
    for e in range(64):
        d = s2[e] - s1[e]
        k = int(np.argmax(np.abs(d) / w))
        r = w[k] / abs(d[k])
        n_test = int(math.floor(1 / r) + 2)
        pts = [s2[e]] + [s1[e] + (s2[e] - s1[e]) * (i * r) for i in range(1, n_test - 1)]
        assert bool(out[e]) == bool(c.is_valid(np.array(pts)).all())
