"""GPU checks of the differentiable costs (FP32 forward + hand-written adjoint) against the FP64
oracle: central finite differences of the oracle cost (h = 1e-6), the reference's ext-row
Jacobian (SphereCollisionCst.evaluate), and the torch.autograd.Function wrappers.

Gradient tolerance: |g - g_fd|_inf <= 1e-4 * max(1, |g_fd|_inf) per problem.  A central
difference across a kink of the cost (the argmin primitive or sphere switching, a box medial
plane) is not a derivative; such problems are detected by comparing differences at h and h/2
and left out, and the test asserts that they are rare."""
import numpy as np
import pytest

from plainmp_gb300 import diff, scenes
from plainmp_gb300 import workloads as W

pytestmark = pytest.mark.gpu

GRAD_TOL = 1e-4
H = 1e-6


def rel_err(g, ref):
    return np.abs(g - ref).max(axis=1) / np.maximum(1.0, np.abs(ref).max(axis=1))


def central_fd(f, Q, h):
    """(B, d) central differences of a batched scalar function f: (N, d) -> (N,)."""
    B, d = Q.shape
    P = np.repeat(Q[:, None, :], 2 * d, axis=1)
    for j in range(d):
        P[:, 2 * j, j] += h
        P[:, 2 * j + 1, j] -= h
    v = f(P.reshape(-1, d)).reshape(B, 2 * d)
    return (v[:, 0::2] - v[:, 1::2]) / (2 * h)


def smooth_points(f, Q, h=H):
    """FD gradient plus a mask of problems where the FD is a derivative (h and h/2 agree)."""
    g1 = central_fd(f, Q, h)
    g2 = central_fd(f, Q, h / 2)
    return g1, rel_err(g1, g2) < 1e-5


@pytest.fixture(scope="module")
def ik_setup(oracle):
    robot, scene = W.chain7_robot(), W.chain7_scene()
    kin, cst, _ = scenes.make_constraint(robot, scene)
    _, oc, _ = oracle.make_constraint(robot, scene)
    link = kin.get_link_ids([robot.end_link])[0]
    return robot, cst, oc, link


def ik_targets(oc, link, q_star):
    return oc.link_poses(q_star, link, threads=8).astype(np.float32)


def test_link_poses_match_oracle(ik_setup):
    _, cst, oc, link = ik_setup
    Q = W.chain7_configs(256, seed=3)
    got = diff.link_poses(cst, Q, link)
    ref = oc.link_poses(Q, link, threads=8)
    assert np.abs(got - ref).max() < 1e-12


def test_ik_cost_and_gradient_vs_fd(ik_setup, oracle):
    _, cst, oc, link = ik_setup
    q0, q_star = W.ik_problems(256, seed=1)
    q0 = q0.astype(np.float32)
    tgt = ik_targets(oc, link, q_star)
    cost, grad = diff.ik_cost_grad(cst, q0, tgt, link)
    Q64 = q0.astype(np.float64)
    ref = oracle.ik_cost(oc, Q64, tgt, link, threads=8)
    assert np.abs(cost - ref).max() <= 1e-4 * max(1.0, np.abs(ref).max())
    g_fd, ok = smooth_points(lambda P: oracle.ik_cost(oc, P, np.repeat(tgt, P.shape[0] // len(tgt), axis=0), link, threads=8),
                             Q64)
    assert ok.mean() > 0.97, f"{(~ok).sum()} kinked problems"
    err = rel_err(grad.astype(np.float64), g_fd)[ok]
    assert err.max() <= GRAD_TOL, f"max relative gradient error {err.max():.3g}"
    # the hinge is active in a good share of the problems, so the collision adjoint is exercised
    col = oracle.ik_cost(oc, Q64, tgt, -1, threads=8)
    assert (col > 0).mean() > 0.2


@pytest.mark.parametrize("base", ["PLANAR", "FLOATING"])
def test_gradient_with_moving_base(oracle, base):
    """Base columns of the adjoint (x, y, yaw for PLANAR; x, y, z, roll, pitch, yaw for
    FLOATING, q = R_z(yaw) R_y(pitch) R_x(roll)) against central differences."""
    r = W.chain7_robot()
    robot = W.Robot(r.urdf, r.control_joints, r.end_link, r.spheres, r.self_pairs, base_type=base)
    scene = W.chain7_scene()
    kin, cst, _ = scenes.make_constraint(robot, scene)
    _, oc, _ = oracle.make_constraint(robot, scene)
    link = kin.get_link_ids([robot.end_link])[0]
    rng = np.random.default_rng(31)
    nb = 3 if base == "PLANAR" else 6
    q = np.concatenate([rng.uniform(-np.pi, np.pi, (128, 7)), rng.uniform(-0.3, 0.3, (128, nb))], axis=1).astype(np.float32)
    qs = np.concatenate([rng.uniform(-np.pi, np.pi, (128, 7)), rng.uniform(-0.3, 0.3, (128, nb))], axis=1)
    tgt = oc.link_poses(qs, link, threads=8).astype(np.float32)
    cost, grad = diff.ik_cost_grad(cst, q, tgt, link)
    Q64 = q.astype(np.float64)
    ref = oracle.ik_cost(oc, Q64, tgt, link, threads=8)
    assert np.abs(cost - ref).max() <= 1e-4 * max(1.0, np.abs(ref).max())
    g_fd, ok = smooth_points(lambda P: oracle.ik_cost(oc, P, np.repeat(tgt, P.shape[0] // len(tgt), axis=0), link, threads=8),
                             Q64)
    assert ok.mean() > 0.95
    err = rel_err(grad.astype(np.float64), g_fd)[ok]
    assert err.max() <= GRAD_TOL, f"max relative gradient error {err.max():.3g}"


def test_min_distance_matches_reference_ext_row(ik_setup):
    """min_distance's value and gradient against SphereCollisionCst.evaluate's ext row (the
    plain FP64 path, bit-exact with the reference), whose SDF gradient is a forward difference
    with h = 1e-6 (primitive_sphere_collision.cpp:308-315) accurate to about h / curvature radius."""
    _, cst, oc, link = ik_setup
    Q = W.chain7_configs(1024, seed=21).astype(np.float32)
    Q64 = Q.astype(np.float64)
    d, g = diff.min_distance(cst, Q)
    vals, jac = cst.evaluate_batch(Q64)
    v_ref, j_ref = vals[:, 0], jac[:, 0, :]
    assert np.abs(d - v_ref).max() < 1e-5
    # unambiguous argmin: the runner-up sphere is at least 1e-4 further
    ds = np.sort(oc.sphere_distances(Q64, high_accuracy=True, threads=8), axis=1)
    clear = (ds[:, 1] - ds[:, 0] > 1e-4) & (v_ref < 0.1 - 1e-4)
    assert clear.sum() > 200
    err = rel_err(g.astype(np.float64), j_ref)[clear]
    assert err.max() <= 2e-4, f"max relative error vs the reference Jacobian {err.max():.3g}"
    # clamped rows have a zero gradient in both
    far = v_ref >= 0.1
    assert np.all(g[far] == 0) and np.all(j_ref[far] == 0)


def test_ik_autograd_function(ik_setup):
    import torch

    _, cst, oc, link = ik_setup
    q0, q_star = W.ik_problems(512, seed=2)
    tgt = torch.tensor(ik_targets(oc, link, q_star), device="cuda")
    q = torch.tensor(q0, dtype=torch.float32, device="cuda", requires_grad=True)
    cost = diff.ik_cost(cst, q, tgt, link)
    w = torch.linspace(0.5, 1.5, q.shape[0], device="cuda")
    (w * cost).sum().backward()
    c2, g2 = diff.ik_cost_grad(cst, q.detach(), tgt, link)
    assert torch.equal(cost.detach(), c2)
    assert torch.allclose(q.grad, w[:, None] * g2, rtol=0, atol=0)


def test_ik_descend(ik_setup):
    import torch

    _, cst, oc, link = ik_setup
    q0, q_star = W.ik_problems(1024, seed=4)
    tgt = ik_targets(oc, link, q_star)
    qf, cf, hist = diff.ik_descend(cst, q0.astype(np.float32), tgt, link, steps=50, lr=0.05, history=True)
    c0 = diff.ik_cost_grad(cst, q0.astype(np.float32), tgt, link, want_grad=False)
    assert np.array_equal(hist[:, 0], c0)
    assert np.array_equal(cf, diff.ik_cost_grad(cst, qf, tgt, link, want_grad=False))
    assert np.median(cf) < 0.5 * np.median(c0)
    kin = cst.get_kin()
    lo, hi = np.array(kin.get_joint_position_limits(kin.get_joint_ids(cst.get_control_joint_names()))).T
    assert np.all(qf >= lo.astype(np.float32)) and np.all(qf <= hi.astype(np.float32))
    # one step by hand: q1 = clamp(q0 - lr * g0)
    q1, _ = diff.ik_descend(cst, q0[:64].astype(np.float32), tgt[:64], link, steps=1, lr=0.05)
    _, g0 = diff.ik_cost_grad(cst, q0[:64].astype(np.float32), tgt[:64], link)
    man = np.clip(q0[:64].astype(np.float32) - np.float32(0.05) * g0, lo.astype(np.float32), hi.astype(np.float32))
    assert np.abs(q1 - man).max() <= 1e-6
    # device tensors give the same result
    qd, cd = diff.ik_descend(cst, torch.tensor(q0[:64], dtype=torch.float32, device="cuda"),
                             torch.tensor(tgt[:64], device="cuda"), link, steps=50, lr=0.05)
    assert np.array_equal(qd.cpu().numpy(), qf[:64]) and np.array_equal(cd.cpu().numpy(), cf[:64])


@pytest.fixture(scope="module")
def traj_setup(oracle):
    robot = W.planar_chain7_robot()
    scene = W.Scene(cloud=W.box_surface_cloud(), cloud_radius=0.0)
    _, cst, _ = scenes.make_constraint(robot, scene)
    _, oc, _ = oracle.make_constraint(robot, scene)
    return cst, oc


def flat(trajs):
    Q = np.concatenate(trajs, axis=0).astype(np.float32)
    off = np.concatenate([[0], np.cumsum([len(t) for t in trajs])]).astype(np.int64)
    return Q, off


def test_traj_cost_and_gradient_vs_fd(traj_setup, oracle):
    cst, oc = traj_setup
    trajs = W.trajectories(12, seed=5, t_min=1, t_max=30)
    Q, off = flat(trajs)
    cost, grad = diff.traj_cost_grad(cst, Q, off)
    Q64 = Q.astype(np.float64)
    ref = oracle.traj_cost(oc, Q64, off, threads=8)
    assert np.all(np.abs(cost - ref) <= 1e-4 * np.maximum(1.0, np.abs(ref)))
    # FD: the collision part of waypoint u depends on q_u only; the smoothing part is global
    col = lambda P: oracle.ik_cost(oc, P, None, -1, margin=0.03, threads=8)
    g_col, ok = smooth_points(col, Q64)
    g_sm = np.zeros_like(Q64)
    for i in range(len(off) - 1):
        a, b = off[i], off[i + 1]
        for u in range(a, b):
            for j in range(Q.shape[1]):
                P = Q64[a:b].copy()
                P[u - a, j] += H
                fp = oracle.smooth_cost(P)
                P[u - a, j] -= 2 * H
                g_sm[u, j] = (fp - oracle.smooth_cost(P)) / (2 * H)
    g_fd = g_col + g_sm
    assert ok.mean() > 0.95
    err = rel_err(grad.astype(np.float64), g_fd)[ok]
    assert err.max() <= GRAD_TOL, f"max relative gradient error {err.max():.3g}"
    assert (col(Q64) > 0).mean() > 0.1  # the cloud hinge is active somewhere


def test_traj_edge_cases(traj_setup):
    cst, _ = traj_setup
    # empty trajectories, one and two waypoints (no acceleration term), and no trajectories at all
    trajs = [np.zeros((0, 10)), W.trajectories(1, seed=8, t_min=1, t_max=1)[0], W.trajectories(1, seed=9, t_min=2, t_max=2)[0]]
    Q, off = flat(trajs)
    cost, grad = diff.traj_cost_grad(cst, Q, off)
    assert cost[0] == 0.0 and grad.shape == (3, 10)
    col = diff.ik_cost_grad(cst, Q, None, None, margin=0.03, want_grad=True)
    assert np.allclose(cost[1], col[0][0], rtol=1e-6, atol=0) and np.allclose(cost[2], col[0][1:].sum(), rtol=1e-6, atol=1e-7)
    c0 = diff.traj_cost_grad(cst, np.zeros((0, 10), np.float32), np.zeros(1, np.int64), want_grad=False)
    assert c0.shape == (0,)
    with pytest.raises(ValueError):
        diff.traj_cost_grad(cst, Q, np.array([0, 2, 1, 3], np.int64))


def test_traj_autograd_function(traj_setup):
    import torch

    cst, _ = traj_setup
    trajs = W.trajectories(64, seed=11)
    Q, off = flat(trajs)
    q = torch.tensor(Q, device="cuda", requires_grad=True)
    o = torch.tensor(off, device="cuda")
    cost = diff.trajectory_cost(cst, q, o)
    w = torch.linspace(0.5, 1.5, cost.shape[0], device="cuda")
    (w * cost).sum().backward()
    c2, g2 = diff.traj_cost_grad(cst, q.detach(), o)
    assert torch.equal(cost.detach(), c2)
    scale = torch.repeat_interleave(w, o[1:] - o[:-1])
    assert torch.equal(q.grad, scale[:, None] * g2)
