"""GPU parity of the plain FP64 method against the oracle, through the C ABI.

Bar: validity booleans and every FP64 value computed without transcendental functions are
bit-identical to the oracle; values that pass through sin/cos (high_accuracy FK, planar /
floating base poses) agree within 1e-9 (FD base-pose Jacobian columns within 1e-6, since
those divide a 1-ulp libm difference by eps = 1e-7)."""
import numpy as np
import pytest

from plainmp_gb300 import scenes
from plainmp_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def both(oracle, robot, scene, self_collision=True, reorder=True):
    kin, cst, sdf = scenes.make_constraint(robot, scene, self_collision, reorder)
    om, oc, osdf = oracle.make_constraint(robot, scene, self_collision, reorder)
    return (kin, cst, sdf), (om, oc, osdf)


@pytest.fixture(scope="module")
def chain(oracle):
    return both(oracle, W.chain7_robot(), W.chain7_scene())


@pytest.fixture(scope="module")
def dual(oracle):
    return both(oracle, W.dualarm_robot(), W.Scene(cloud=W.box_surface_cloud(), cloud_radius=0.0))


def test_is_valid_chain7_bit_exact(chain):
    (_, cst, _), (_, oc, _) = chain
    Q = W.chain7_configs(4096)
    got = cst.is_valid_batch(Q)
    ref = oc.is_valid(Q, threads=8)
    assert got.dtype == np.uint8
    assert np.array_equal(got, ref)
    assert 0.2 < ref.mean() < 0.8


@pytest.mark.parametrize("self_collision", [False, True])
@pytest.mark.parametrize("reorder", [False, True])
def test_is_valid_variants(oracle, self_collision, reorder):
    (_, cst, _), (_, oc, _) = both(oracle, W.chain7_robot(), W.chain7_scene(), self_collision, reorder)
    Q = W.chain7_configs(1024, seed=3)
    assert np.array_equal(cst.is_valid_batch(Q), oc.is_valid(Q, threads=8))


@pytest.mark.parametrize("B", [0, 1, 2, 31, 33, 129])
def test_is_valid_ragged_sizes(chain, B):
    (_, cst, _), (_, oc, _) = chain
    Q = W.chain7_configs(max(B, 1), seed=7)[:B]
    got = cst.is_valid_batch(Q)
    assert got.shape == (B,)
    if B:
        assert np.array_equal(got, oc.is_valid(Q))


def test_sphere_centres_and_distances_bit_exact(chain):
    (_, cst, _), (_, oc, _) = chain
    Q = W.chain7_configs(256, seed=11)
    d, c = cst.sphere_distances(Q, high_accuracy=False, centres=True)
    rd, rc = oc.sphere_distances(Q, high_accuracy=False, centres=True, threads=8)
    assert np.array_equal(c, rc)
    assert np.array_equal(d, rd)
    d2, c2 = cst.sphere_distances(Q, high_accuracy=True, centres=True)
    rd2, rc2 = oc.sphere_distances(Q, high_accuracy=True, centres=True, threads=8)
    np.testing.assert_allclose(c2, rc2, atol=1e-12, rtol=0)
    np.testing.assert_allclose(d2, rd2, atol=1e-12, rtol=0)


def test_evaluate_chain7(chain):
    (_, cst, _), (_, oc, _) = chain
    Q = W.chain7_configs(512, seed=5)
    v, J = cst.evaluate_batch(Q)
    rv, rJ = oc.evaluate(Q, threads=8)
    assert v.shape == (512, 2) and J.shape == (512, 2, 7)
    np.testing.assert_allclose(v, rv, atol=1e-9, rtol=0)
    np.testing.assert_allclose(J, rJ, atol=1e-9, rtol=0)


@pytest.mark.parametrize("base", ["PLANAR", "FLOATING"])
def test_evaluate_and_is_valid_mobile_base(oracle, base):
    r = W.chain7_robot()
    r = W.Robot(r.urdf, r.control_joints, r.end_link, r.spheres, r.self_pairs, base_type=base)
    (_, cst, _), (_, oc, _) = both(oracle, r, W.chain7_scene())
    rng = np.random.default_rng(9)
    Q = np.concatenate([W.chain7_configs(512, seed=9), rng.normal(0, 0.3, (512, cst.q_dim() - 7))], axis=1)
    v, J = cst.evaluate_batch(Q)
    rv, rJ = oc.evaluate(Q, threads=8)
    np.testing.assert_allclose(v, rv, atol=1e-9, rtol=0)
    nj = 7
    np.testing.assert_allclose(J[:, :, :nj], rJ[:, :, :nj], atol=1e-9, rtol=0)
    np.testing.assert_allclose(J[:, :, nj:], rJ[:, :, nj:], atol=1e-6, rtol=0)
    # is_valid on a non-FIXED base goes through libm sin/cos: booleans may only differ where a
    # distance is within ~1e-12 of its threshold
    got, ref = cst.is_valid_batch(Q), oc.is_valid(Q, threads=8)
    assert (got != ref).sum() == 0


def test_evaluate_dualarm_cloud(dual):
    """evaluate() against the point cloud: the ext row's value is the clamped minimum over spheres
    of the cloud distance (exact nearest point, KD-tree in the oracle) and its Jacobian row the
    forward-difference SDF gradient of the argmin sphere through the attached-point Jacobian
    (primitive_sphere_collision.cpp:256-322, primitive_sdf.hpp:597-603).  Values within 1e-9 on
    every configuration; Jacobian rows within 1e-9 where the argmin sphere is unambiguous (the two
    smallest sphere distances at least 1e-6 apart: a tie may pick either sphere)."""
    import os

    (_, cst, _), (_, oc, _) = dual
    assert not cst.groups()["only_self"].any()  # every sphere takes part in the ext row
    Q = W.dualarm_configs(2048, seed=21)
    v, J = cst.evaluate_batch(Q)
    rv, rJ = oc.evaluate(Q, threads=os.cpu_count() or 8)
    assert v.shape == (2048, 2) and J.shape == (2048, 2, 14)
    np.testing.assert_allclose(v, rv, atol=1e-9, rtol=0)
    d = np.sort(oc.sphere_distances(Q, threads=os.cpu_count() or 8), axis=1)
    near = d[:, 0] < 0.1  # the row is active (below the cutoff): its Jacobian is not zero
    clear = (d[:, 1] - d[:, 0]) > 1e-6
    assert near.sum() > 100 and (near & clear).sum() > 0.9 * near.sum()
    np.testing.assert_allclose(J[clear, 0], rJ[clear, 0], atol=1e-9, rtol=0)
    np.testing.assert_allclose(J[:, 1], rJ[:, 1], atol=1e-9, rtol=0)  # self row: no SDF involved
    assert np.array_equal(cst.is_valid_batch(Q), oc.is_valid(Q, threads=os.cpu_count() or 8))


def test_evaluate_empty_and_self_only(oracle):
    (_, cst, _), (_, oc, _) = both(oracle, W.chain7_robot(), None, self_collision=False)
    Q = W.chain7_configs(17)
    assert cst.cst_dim() == 0
    assert cst.is_valid_batch(Q).all()
    v, J = cst.evaluate_batch(Q)
    assert v.shape == (17, 0) and J.shape == (17, 0, 7)
    (_, cst2, _), (_, oc2, _) = both(oracle, W.chain7_robot(), None, self_collision=True)
    v, J = cst2.evaluate_batch(Q)
    rv, rJ = oc2.evaluate(Q)
    np.testing.assert_allclose(v, rv, atol=1e-9, rtol=0)
    np.testing.assert_allclose(J, rJ, atol=1e-9, rtol=0)


def test_check_motion_chain7_bit_exact(chain):
    (_, cst, _), (_, oc, _) = chain
    from plainmp_gb300 import BoxMotionValidator, EuclideanMotionValidator

    s1, s2 = W.chain7_edges(1024)
    mv = BoxMotionValidator(cst, np.full(7, 0.05))
    got, n = mv.check_motion_batch(s1, s2, return_count=True)
    ref, rn = oc.check_motion(s1, s2, 0, np.full(7, 0.05), threads=8)
    assert np.array_equal(got, ref)
    assert n == rn
    ev = EuclideanMotionValidator(cst, 0.1)
    got = ev.check_motion_batch(s1[:256], s2[:256])
    ref, _ = oc.check_motion(s1[:256], s2[:256], 1, None, 0.1, threads=8)
    assert np.array_equal(got, ref)


def test_link_poses_match_oracle(oracle):
    from plainmp_gb300 import KinematicModel

    r = W.dualarm_robot()
    kin = KinematicModel(r.urdf)
    om = oracle.Model(r.urdf)
    ids = kin.get_joint_ids(r.control_joints)
    q = W.dualarm_configs(1, seed=1)[0]
    for accurate in (False, True):
        kin.set_joint_positions(ids, q, accurate)
        om.set_joint_positions([om.joint_id(n) for n in r.control_joints], q, accurate)
        for l in range(kin.num_links):
            got = kin.link_poses([l])[0]
            ref = om.link_pose(l)
            if accurate:
                np.testing.assert_allclose(got, ref, atol=1e-14, rtol=0)
            else:
                assert np.array_equal(got, ref)
    pose = np.array([0.1, -0.2, 0.3, 0.0, 0.0, np.sin(0.2), np.cos(0.2)])
    kin.set_base_pose(pose)
    om.set_base_pose(pose)
    np.testing.assert_array_equal(kin.get_base_pose(), pose)
    for l in range(kin.num_links):
        np.testing.assert_allclose(kin.link_poses([l])[0], om.link_pose(l), atol=1e-14, rtol=0)


def test_primitive_sdf_evaluate_and_is_outside(oracle):
    from plainmp_gb300 import BoxSDF, CylinderSDF, GroundSDF, Pose, SphereSDF, UnionSDF
    from helpers import rpy_matrix

    rng = np.random.default_rng(21)
    pts = rng.standard_normal((4000, 3))
    for i in range(8):
        pos = rng.standard_normal(3) * 0.5
        R = np.eye(3) if i == 0 else (rpy_matrix(0.3, 0, 0) if i == 1 else rpy_matrix(*rng.standard_normal(3)))
        for mine, ref in [(BoxSDF([0.5, 0.3, 0.6], Pose(pos, R)), oracle.Sdf.box([0.5, 0.3, 0.6], pos, R)),
                          (CylinderSDF(0.7, 0.2, Pose(pos, R)), oracle.Sdf.cylinder(0.7, 0.2, pos, R)),
                          (SphereSDF(0.5, Pose(pos, R)), oracle.Sdf.sphere(0.5, pos, R))]:
            assert np.array_equal(mine.evaluate_points(pts), ref.evaluate(pts))
            for r in (0.0, 1e-7, 0.05, 0.3):
                assert np.array_equal(mine.is_outside_points(pts, r), ref.is_outside(pts, r))
    g, og = GroundSDF(0.2), oracle.Sdf.ground(0.2)
    assert np.array_equal(g.evaluate_points(pts), og.evaluate(pts))
    b1, b2 = BoxSDF([1, 1, 1], Pose([1, 0, 0], np.eye(3))), SphereSDF(0.4, Pose())
    u = UnionSDF([b1, UnionSDF([b2])])
    ou = oracle.Sdf.union([oracle.Sdf.box([1, 1, 1], [1, 0, 0], np.eye(3)), oracle.Sdf.union([oracle.Sdf.sphere(0.4, np.zeros(3), np.eye(3))])])
    assert np.array_equal(u.evaluate_points(pts), ou.evaluate(pts))
    assert np.array_equal(u.is_outside_points(pts, 0.1), ou.is_outside(pts, 0.1))


def test_cloud_nearest_exact(oracle):
    from plainmp_gb300 import CloudSDF

    cloud = W.box_surface_cloud(n_points=20000, seed=3).astype(np.float64)
    mine = CloudSDF(cloud, 0.0)
    ref = oracle.Sdf.cloud(cloud, 0.0)
    rng = np.random.default_rng(4)
    q = np.concatenate([rng.uniform(cloud.min(0) - 0.1, cloud.max(0) + 0.1, (3000, 3)),  # inside the grid
                        rng.uniform(-3, 3, (500, 3)),  # mostly outside the grid
                        cloud[:200] + rng.normal(0, 1e-3, (200, 3)), cloud[200:300]])  # on/near points
    sq, near = mine.nearest(q)
    rsq, _ = ref.nearest(q)
    assert np.array_equal(sq, rsq)
    d = near - q
    assert np.array_equal(sq, d[:, 0] * d[:, 0] + (d[:, 1] * d[:, 1] + d[:, 2] * d[:, 2]))


@pytest.mark.parametrize("cell", [0.0, 0.006, 0.03])
def test_cloud_nearest_cell_sizes(oracle, cell):
    from plainmp_gb300 import CloudSDF

    rng = np.random.default_rng(5)
    cloud = rng.random((3000, 3))
    mine = CloudSDF(cloud, 0.05, cell)
    ref = oracle.Sdf.cloud(cloud, 0.05)
    q = rng.standard_normal((2000, 3)) * 1.5
    assert np.array_equal(mine.nearest(q)[0], ref.nearest(q)[0])
    assert np.array_equal(mine.evaluate_points(q), ref.evaluate(q))
    for r in np.linspace(0, 2, 5):
        assert np.array_equal(mine.is_outside_points(q, r), ref.is_outside(q, r))


def test_kdtree_vs_brute_force():  # tests/test_kdtree.py:6-20
    from plainmp_gb300 import KDTree

    rng = np.random.default_rng(0)
    points = rng.standard_normal((1000, 3))
    tree = KDTree(points)
    Q = rng.standard_normal((1000, 3))
    for q in Q[:200]:  # one query per call, as the reference's test makes them
        nearest = tree.query(q)
        assert np.allclose(nearest, points[np.argmin(np.sum((points - q) ** 2, axis=1))])
        assert np.allclose(np.sum((nearest - q) ** 2), tree.sqdist(q))
    idx = np.argmin(((points[None, :, :] - Q[:, None, :]) ** 2).sum(-1), axis=1)
    np.testing.assert_array_equal(tree.query_batch(Q), points[idx])  # the set's own coordinates
    np.testing.assert_allclose(tree.sqdist_batch(Q), ((points[idx] - Q) ** 2).sum(-1), rtol=1e-12, atol=0)


def test_cloud_edge_cases(oracle):
    from plainmp_gb300 import CloudSDF

    one = CloudSDF(np.array([[0.1, 0.2, 0.3]]), 0.0)
    sq, near = one.nearest(np.array([[1.0, 1.0, 1.0], [0.1, 0.2, 0.3]]))
    np.testing.assert_array_equal(near[0], [0.1, 0.2, 0.3])
    assert sq[1] == 0.0
    dup = CloudSDF(np.tile([[0.5, 0.5, 0.5]], (500, 1)), 0.0)  # every point in one cell
    assert dup.nearest(np.zeros((1, 3)))[0][0] == 0.75


def test_is_valid_dualarm_cloud_bit_exact(dual):
    (_, cst, _), (_, oc, _) = dual
    Q = W.dualarm_configs(512, seed=2)
    got = cst.is_valid_batch(Q)
    ref = oc.is_valid(Q, threads=8)
    assert np.array_equal(got, ref)


def test_sphere_distances_dualarm_cloud_exact(dual):
    (_, cst, _), (_, oc, _) = dual
    Q = W.dualarm_configs(6, seed=4)
    d, c = cst.sphere_distances(Q, centres=True)
    rd, rc = oc.sphere_distances(Q, centres=True, threads=8)
    assert np.array_equal(c, rc)
    assert np.array_equal(d, rd)


def test_update_kintree_and_spheres(chain):
    (kin, cst, _), (om, oc, _) = chain
    q = W.chain7_configs(1, seed=8)[0]
    cst.update_kintree(q, False)
    oc.update_kintree(q, False)
    got = np.array([np.r_[c, r] for c, r in cst.get_all_spheres()])
    ocen = oc.sphere_distances(q[None], centres=True)[1][0]
    assert np.array_equal(got[:, :3], ocen)
    assert len(cst.get_group_spheres()) == cst.n_groups
