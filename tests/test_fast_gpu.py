"""GPU parity of the FP32 + FP64-recheck fast paths against the oracle (validity identical to
the reference; FP32 per-sphere distances within the stated bound)."""
import numpy as np
import pytest

from plainmp_gb300 import BoxMotionValidator, EuclideanMotionValidator, Pose, SphereSDF, UnionSDF, scenes
from plainmp_gb300 import workloads as W

pytestmark = pytest.mark.gpu

CUTOFF = 0.1
# FP32 distance error bound: 1e-6 + 64 * 2^-24 * (1 + magnitudes), magnitudes below ~20 m here
DIST_TOL = 1e-6 + 64 * 2.0 ** -24 * 21


@pytest.fixture(scope="module")
def chain(oracle):
    r, s = W.chain7_robot(), W.chain7_scene()
    return scenes.make_constraint(r, s), oracle.make_constraint(r, s)


@pytest.fixture(scope="module")
def dual(oracle):
    r, s = W.dualarm_robot(), W.Scene(cloud=W.box_surface_cloud(), cloud_radius=0.0)
    return scenes.make_constraint(r, s), oracle.make_constraint(r, s)


def test_fast_chain7_matches_oracle(chain):
    (_, cst, _), (_, oc, _) = chain
    Q = W.chain7_configs(4096)
    got, st = cst.is_valid_fast(Q, stats=True)
    assert np.array_equal(got, oc.is_valid(Q, threads=8))
    assert np.array_equal(got, cst.is_valid_batch(Q))
    assert st["configs"] == 4096
    assert st["rechecked_terms"] < 4096  # a small fraction of the 56 x 20 + 960 terms per config


@pytest.mark.parametrize("B", [1, 5, 31, 32, 33, 100])
def test_fast_ragged(chain, B):
    (_, cst, _), (_, oc, _) = chain
    Q = W.chain7_configs(B, seed=17)
    assert np.array_equal(cst.is_valid_fast(Q), oc.is_valid(Q))


def test_fast_chain7_distances(chain):
    (_, cst, _), (_, oc, _) = chain
    Q = W.chain7_configs(512, seed=12)
    ok, d32 = cst.is_valid_fast(Q, distances=True)
    ref = np.minimum(oc.sphere_distances(Q, threads=8), CUTOFF)
    assert d32.dtype == np.float32 and d32.shape == (512, 56)
    assert np.abs(d32.astype(np.float64) - ref).max() < DIST_TOL
    assert np.array_equal(ok, oc.is_valid(Q, threads=8))


def test_fast_dualarm_cloud(dual):
    (_, cst, _), (_, oc, _) = dual
    Q = W.dualarm_configs(4096, seed=6)
    got = cst.is_valid_fast(Q)
    assert np.array_equal(got, oc.is_valid(Q, threads=8))
    assert np.array_equal(got, cst.is_valid_batch(Q))


def test_fast_dualarm_full_batch(dual):
    """The benchmark's own batch (65,536 configurations against the 200k-point cloud) through the
    host-memory call (two-stream chunks): fast validity equals the oracle's (the reference's
    is_valid loop with its KD-tree) on every configuration, in both modes, and the plain FP64
    method's; every FP32 distance is finite, at most the cutoff and within the bound of the
    oracle's FP64 KD-tree distance on every 8th configuration."""
    import os

    (_, cst, _), (_, oc, _) = dual
    Q = W.dualarm_configs(65536)
    ref = oc.is_valid(Q, threads=os.cpu_count() or 8)
    ok, d32 = cst.is_valid_fast(Q, distances=True)
    assert int((ok != ref).sum()) == 0
    assert np.array_equal(cst.is_valid_fast(Q), ref)
    assert np.array_equal(cst.is_valid_batch(Q), ref)
    assert d32.shape == (65536, cst.n_spheres) and np.isfinite(d32).all() and (d32 <= np.float32(CUTOFF)).all()
    d64 = np.minimum(oc.sphere_distances(Q[::8], threads=os.cpu_count() or 8), CUTOFF)
    assert np.abs(d32[::8].astype(np.float64) - d64).max() < DIST_TOL


def test_fast_dualarm_cloud_distances(dual):
    (_, cst, _), (_, oc, _) = dual
    Q = W.dualarm_configs(8, seed=7)
    ok, d32 = cst.is_valid_fast(Q, distances=True)
    ref = np.minimum(cst.sphere_distances(Q), CUTOFF)  # plain FP64 grid, exact vs the KD-tree (tested elsewhere)
    assert np.abs(d32.astype(np.float64) - ref).max() < DIST_TOL
    assert np.array_equal(ok, oc.is_valid(Q))


def test_fast_near_boundary_rechecks(oracle):
    """Obstacle spheres placed within 1e-15..1e-9 of tangency to one robot sphere per
    configuration: every such decision is left to the FP64 recheck, which must reproduce the
    reference bit for bit."""
    robot = W.chain7_robot()
    Q = W.chain7_configs(64, seed=31)
    _, oc0, _ = oracle.make_constraint(robot, None, self_collision=False)
    _, cen = oc0.sphere_distances(Q, centres=True)
    order = oc0.groups()["radii"]
    rng = np.random.default_rng(0)
    obstacles = []
    prims = []
    for b in range(64):
        s = int(rng.integers(0, 56))
        c = cen[b, s]
        direction = rng.standard_normal(3)
        direction /= np.linalg.norm(direction)
        R = 0.05 + 0.1 * rng.random()
        delta = [1e-9, -1e-9, 1e-12, -1e-12, 0.0][b % 5]
        pos = c + direction * (R + order[s] + delta)
        obstacles.append(SphereSDF(R, Pose(pos, np.eye(3))))
        prims.append(W.Primitive("sphere", pos, np.eye(3), (R,)))
    scene = W.Scene(prims)
    kin, cst, _ = scenes.make_constraint(robot, None, self_collision=False)
    cst.set_sdf(UnionSDF(obstacles))
    _, oc, _ = oracle.make_constraint(robot, scene, self_collision=False)
    got, st = cst.is_valid_fast(Q, stats=True)
    ref = oc.is_valid(Q)
    assert np.array_equal(got, ref)
    assert np.array_equal(cst.is_valid_batch(Q), ref)
    # tangent terms of configurations without a certain collision went through FP64 (how many
    # depends on the order in which a block's threads meet a certain collision first)
    assert st["rechecked_terms"] > 0


@pytest.mark.parametrize("cloud_radius", [0.0, 0.01])
def test_fast_cloud_near_boundary(oracle, cloud_radius):
    """Per configuration, a cloud of three points at r + radius + delta from three robot sphere
    centres (delta from -3e-3 down to exact tangency and up to +3e-3) plus points on the faces of a
    3 m cube around the robot: the nearest-point field's shortcuts, the warp search and the FP64
    recheck must reproduce the reference's decision, and the FP32 distances stay in bound."""
    robot = W.chain7_robot()
    n = 36
    Q = W.chain7_configs(n, seed=41)
    _, oc0, _ = oracle.make_constraint(robot, None, self_collision=False)
    _, cen = oc0.sphere_distances(Q, centres=True)
    radii = oc0.groups()["radii"]
    rng = np.random.default_rng(5)
    deltas = [-3e-3, -1e-5, -1e-7, -1e-9, 0.0, 1e-9, 1e-7, 1e-5, 3e-3]
    faces = rng.uniform(-1.5, 1.5, (1500, 3))
    ax = rng.integers(0, 3, 1500)
    faces[np.arange(1500), ax] = np.where(rng.random(1500) < 0.5, -1.5, 1.5)
    got, ref, rechecked = [], [], 0
    for b in range(n):
        pts = []
        for k, s in enumerate(rng.choice(56, size=3, replace=False)):
            u = rng.standard_normal(3)
            u /= np.linalg.norm(u)
            pts.append(cen[b, s] + u * (radii[s] + cloud_radius + deltas[(b + k) % len(deltas)]))
        scene = W.Scene(cloud=np.vstack([np.asarray(pts), faces]), cloud_radius=cloud_radius)
        (_, cst, _), (_, oc, _) = scenes.make_constraint(robot, scene, self_collision=False), \
            oracle.make_constraint(robot, scene, self_collision=False)
        q = Q[b:b + 1]
        r = oc.is_valid(q)
        ok, st = cst.is_valid_fast(q, stats=True)
        ok2, d32 = cst.is_valid_fast(q, distances=True)
        assert np.array_equal(ok, r) and np.array_equal(ok2, r), f"configuration {b}"
        dref = np.minimum(oc.sphere_distances(q), CUTOFF)
        assert np.abs(d32.astype(np.float64) - dref).max() < DIST_TOL
        got.append(int(ok[0]))
        ref.append(int(r[0]))
        rechecked += st["rechecked_terms"]
    assert 0 < sum(ref) < n  # both outcomes occur
    assert rechecked > 0


@pytest.mark.parametrize("base,nb", [("PLANAR", 3), ("FLOATING", 6)])
def test_fast_mobile_base(oracle, base, nb):
    r = W.chain7_robot()
    r = W.Robot(r.urdf, r.control_joints, r.end_link, r.spheres, r.self_pairs, base_type=base)
    s = W.chain7_scene()
    (_, cst, _), (_, oc, _) = scenes.make_constraint(r, s), oracle.make_constraint(r, s)
    rng = np.random.default_rng(2)
    Q = np.concatenate([W.chain7_configs(1024, seed=2), rng.normal(0, 0.3, (1024, nb))], axis=1)
    Q[:8, 7:] *= 100.0  # far-away base coordinates and large angles: the FK bound grows with them
    ref = oc.is_valid(Q, threads=8)
    assert np.array_equal(cst.is_valid_fast(Q), ref)
    ok, d32 = cst.is_valid_fast(Q[8:], distances=True)
    assert np.array_equal(ok, ref[8:])


def test_fast_edges_match_oracle(chain):
    (_, cst, _), (_, oc, _) = chain
    s1, s2 = W.chain7_edges(1024)
    w = np.full(7, 0.05)
    mv = BoxMotionValidator(cst, w)
    got, st = mv.check_motion_fast(s1, s2, stats=True)
    ref, _ = oc.check_motion(s1, s2, 0, w, threads=8)
    assert np.array_equal(got, ref)
    assert np.array_equal(got, mv.check_motion_batch(s1, s2))
    ev = EuclideanMotionValidator(cst, 0.1)
    got = ev.check_motion_fast(s1[:300], s2[:300])
    ref, _ = oc.check_motion(s1[:300], s2[:300], 1, None, 0.1, threads=8)
    assert np.array_equal(got, ref)


def test_fast_edges_cuda_graph(chain):
    """All edges in one captured launch sequence: the replayed graph gives the eager booleans,
    for new edge data copied into the captured input buffers too."""
    import torch

    (_, cst, _), _ = chain
    mv = BoxMotionValidator(cst, np.full(7, 0.05))
    s1, s2 = W.chain7_edges(1024, seed=3)
    S1, S2 = torch.tensor(s1, device="cuda"), torch.tensor(s2, device="cuda")
    out = torch.empty(1024, dtype=torch.uint8, device="cuda")
    mv.check_motion_fast(S1, S2, out=out)  # warm-up: workspaces and tables
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side):
        mv.check_motion_fast(S1, S2, out=out)
    torch.cuda.current_stream().wait_stream(side)
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        mv.check_motion_fast(S1, S2, out=out)
    for seed in (3, 4):
        a, b = W.chain7_edges(1024, seed=seed)
        S1.copy_(torch.tensor(a))
        S2.copy_(torch.tensor(b))
        out.fill_(7)
        g.replay()
        torch.cuda.synchronize()
        assert np.array_equal(out.cpu().numpy(), mv.check_motion_batch(a, b))


def test_batched_shortcut(chain):
    """shortcut(): every returned segment is an original segment or a valid edge of the plain
    validator, endpoints are kept and the path gets no longer."""
    (_, cst, _), _ = chain
    mv = BoxMotionValidator(cst, np.full(7, 0.05))
    rng = np.random.default_rng(8)
    # a wandering path through mostly free space: random small steps from a valid start
    start = W.chain7_configs(256, seed=9)[cst.is_valid_batch(W.chain7_configs(256, seed=9)).astype(bool)][0]
    path = start + np.cumsum(rng.normal(0, 0.05, (40, 7)), axis=0)
    out = mv.shortcut(path)
    assert np.array_equal(out[0], path[0]) and np.array_equal(out[-1], path[-1])
    length = lambda p: np.linalg.norm(p[1:] - p[:-1], axis=1).sum()  # noqa: E731
    assert length(out) <= length(path) + 1e-12 and len(out) < len(path)
    orig = {(tuple(a), tuple(b)) for a, b in zip(path[:-1], path[1:])}
    new = [(a, b) for a, b in zip(out[:-1], out[1:]) if (tuple(a), tuple(b)) not in orig]
    if new:
        assert mv.check_motion_batch(np.array([a for a, _ in new]), np.array([b for _, b in new])).all()
    assert np.array_equal(mv.shortcut(path, fast=False), out)


def test_fast_edges_degenerate(chain):
    (_, cst, _), (_, oc, _) = chain
    q = W.chain7_configs(4, seed=40)
    s1 = np.concatenate([q, q[:2]])
    s2 = np.concatenate([q + 1e-8, q[2:] + 0.3])  # zero-length edges are valid without a check
    w = np.full(7, 0.05)
    got = BoxMotionValidator(cst, w).check_motion_fast(s1, s2)
    ref, _ = oc.check_motion(s1, s2, 0, w)
    assert np.array_equal(got, ref)
    assert got[:4].all()


def test_fast_every_launch_shape(dual):
    """Every (configs per block, threads) pair and sphere tile the autotuner may pick, and every
    hard-query grid, gives the same validity and the same FP32 distances (validity-only and with
    distances): the tuning changes the work split, never the arithmetic."""
    from plainmp_gb300._lib import CudaError
    from plainmp_gb300.autotune import SHAPES, sphere_tiles

    (_, cst, _), (_, oc, _) = dual
    Q = W.dualarm_configs(777, seed=21)  # a ragged last block for every shape
    ref = oc.is_valid(Q, threads=8)
    keep, keep_t = cst.get_fast_launch(), cst.get_fast_tuning()
    ran = 0
    try:
        d0 = None
        for cpb, nt in SHAPES:
            cst.set_fast_launch(cpb, nt)
            for st in sphere_tiles(cpb):
                cst.set_fast_tuning(st, 2 + ran % 3, 32, 128)
                try:
                    ok, d = cst.is_valid_fast(Q, distances=True)
                except CudaError as e:  # the block's tables do not fit in shared memory at this shape
                    assert "invalid configuration" in str(e), (cpb, nt, str(e))
                    break
                ran += 1
                assert np.array_equal(ok, ref), (cpb, nt, st)
                assert np.array_equal(cst.is_valid_fast(Q), ref), (cpb, nt, st)
                if d0 is None:
                    d0 = d
                assert np.array_equal(d, d0), (cpb, nt, st)
    finally:
        cst.set_fast_launch(*keep)
        cst.set_fast_tuning(*keep_t)
    assert ran >= 20, ran


def test_fast_edges_every_launch_shape(chain):
    """Every edge-kernel launch shape the autotuner may pick gives the oracle's edge booleans."""
    from plainmp_gb300.autotune import EDGE_SHAPES

    (_, cst, _), (_, oc, _) = chain
    s1, s2 = W.chain7_edges(300, seed=23)
    w = np.full(7, 0.05)
    ref, _ = oc.check_motion(s1, s2, 0, w, threads=8)
    mv = BoxMotionValidator(cst, w)
    keep = cst.get_fast_tuning()
    try:
        for ecpb, ent in EDGE_SHAPES:
            cst.set_fast_tuning(keep[0], keep[1], ecpb, ent)
            assert np.array_equal(mv.check_motion_fast(s1, s2), ref), (ecpb, ent)
    finally:
        cst.set_fast_tuning(*keep)


def test_fma_peak_microbenchmark():
    """The measured FMA throughput used as the roofline denominator is in a plausible range for
    this GPU (FP32 tens of TFLOP/s, FP64 at least a fraction of a TFLOP/s and below FP32)."""
    from plainmp_gb300 import _lib

    f32 = _lib.measure_fma_peak(False)
    f64 = _lib.measure_fma_peak(True)
    assert 10.0 < f32 < 400.0, f32
    assert 0.05 < f64 < f32, (f64, f32)


def test_cloud_stats():
    """The grid's reported sizes are consistent with the cloud and with each other."""
    from plainmp_gb300 import CloudSDF

    pts = W.box_surface_cloud(n_points=20_000, seed=3)
    st = CloudSDF(pts, 0.0).stats()
    assert st["points"] == 20_000
    assert 0 < st["occupied_cells"] <= st["points"]
    assert st["field_cells"] == 64 * st["blocks"]
    assert st["list_entries"] > 0
    # at least the points (FP64 SoA + FP32) and the field (8 + 16 bytes per fine cell)
    assert st["device_bytes"] >= 40 * st["points"] + 24 * st["field_cells"]


def test_fast_host_pipelined_matches_device(dual):
    """A large host-memory batch runs in chunks on two streams (copies overlapping kernels); the
    outcome equals the one-launch device-memory call: validity, distances and recheck counts."""
    import torch

    (_, cst, _), _ = dual
    Q = W.dualarm_configs(20001, seed=23)  # ragged: the last chunk is short
    ok_h, d_h, st_h = cst.is_valid_fast(Q, distances=True, stats=True)
    ok_d, d_d, st_d = cst.is_valid_fast(torch.tensor(Q, device="cuda"), distances=True, stats=True)
    assert np.array_equal(ok_h, ok_d.cpu().numpy())
    assert np.array_equal(d_h, d_d.cpu().numpy())
    # the recheck statistics depend on warp timing (a self pair skips a configuration another warp
    # has already found colliding), so only the outcome is compared, plus the configuration count
    assert st_h["configs"] == st_d["configs"] == len(Q)
    # pinned host buffers, preallocated outputs
    qp = torch.from_numpy(Q).pin_memory()
    op = torch.empty(len(Q), dtype=torch.uint8).pin_memory()
    dp = torch.empty((len(Q), cst.n_spheres), dtype=torch.float32).pin_memory()
    cst.is_valid_fast(qp.numpy(), distances=True, out=op.numpy(), dist_out=dp.numpy())
    assert np.array_equal(op.numpy(), ok_h) and np.array_equal(dp.numpy(), d_h)


def test_fast_non_finite_configurations(chain, dual):
    """Configurations with a NaN or infinite coordinate get the exact FP64 decision (their FP32
    bounds would be NaN and decide nothing): validity equals the plain method and the oracle,
    and their FP32 distances are NaN; every other row is unaffected."""
    for (_, cst, _), (_, oc, _), Q in ((chain[0], chain[1], W.chain7_configs(300, seed=41)),
                                       (dual[0], dual[1], W.dualarm_configs(300, seed=42))):
        Q = Q.copy()
        bad = np.zeros(len(Q), dtype=bool)
        for i, v in ((3, np.nan), (17, np.inf), (18, -np.inf), (150, np.nan), (299, np.nan)):
            Q[i, i % Q.shape[1]] = v
            bad[i] = True
        plain = np.asarray(cst.is_valid_batch(Q))
        assert np.array_equal(plain, oc.is_valid(Q))
        assert np.array_equal(cst.is_valid_fast(Q), plain)
        ok, d = cst.is_valid_fast(Q, distances=True)
        assert np.array_equal(ok, plain)
        assert np.isnan(d[bad]).all()
        ok_clean, d_clean = cst.is_valid_fast(Q[~bad], distances=True)
        assert np.array_equal(d[~bad], d_clean) and np.array_equal(ok[~bad], ok_clean)


def test_fast_degenerate_clouds(oracle):
    """An empty cloud, a single point and 50 coincident points (ties everywhere): validity equals
    the oracle on both paths, and the FP32 distances match the plain FP64 ones (clamped)."""
    robot = W.dualarm_robot()
    Q = W.dualarm_configs(200, seed=44)
    for pts in (np.zeros((0, 3)), np.array([[0.3, 0.0, 0.9]]), np.repeat([[0.4, 0.1, 0.8]], 50, axis=0)):
        scene = W.Scene(cloud=pts.astype(np.float32), cloud_radius=0.01)
        _, cst, _ = scenes.make_constraint(robot, scene)
        _, oc, _ = oracle.make_constraint(robot, scene)
        ref = oc.is_valid(Q, threads=8)
        assert np.array_equal(cst.is_valid_batch(Q), ref), len(pts)
        assert np.array_equal(cst.is_valid_fast(Q), ref), len(pts)
        ok, d = cst.is_valid_fast(Q, distances=True)
        assert np.array_equal(ok, ref), len(pts)
        d_ref = np.minimum(cst.sphere_distances(Q), CUTOFF)
        assert np.abs(d.astype(np.float64) - d_ref).max() < DIST_TOL, len(pts)


def test_fast_queries_beyond_the_cell_lists(oracle):
    """Spheres twice as large (up to 0.16 m) and a 0.05 m cloud radius, no self pairs: hard cloud
    queries reach 0.31 m, so they come from cells both within and beyond the cell lists' 0.25 m,
    and the lists and the whole-warp search both answer.  Validity equals the oracle and the plain
    method in both modes; distances are within the bound of the plain FP64 distances."""
    base = W.dualarm_robot()
    big = [W.SphereSpec(s.parent_link_name, s.relative_positions, s.radii * 2.0, s.only_self_collision) for s in base.spheres]
    robot = W.Robot(base.urdf, base.control_joints, base.end_link, big, base.self_pairs)
    scene = W.Scene(cloud=W.box_surface_cloud(n_points=50_000, seed=9), cloud_radius=0.05)
    _, cst, _ = scenes.make_constraint(robot, scene, self_collision=False)
    _, oc, _ = oracle.make_constraint(robot, scene, self_collision=False)
    Q = W.dualarm_configs(1024, seed=46)
    ref = oc.is_valid(Q, threads=8)
    assert 10 < ref.sum() < len(ref)  # 46 valid
    plain = cst.is_valid_batch(Q)
    assert np.array_equal(plain, ref)
    assert np.array_equal(cst.is_valid_fast(Q), ref)
    ok, d32 = cst.is_valid_fast(Q, distances=True)
    assert np.array_equal(ok, ref)
    d64 = np.minimum(cst.sphere_distances(Q[::4]), CUTOFF)
    assert np.abs(d32[::4].astype(np.float64) - d64).max() < DIST_TOL


def test_fast_refuses_tables_beyond_the_queue_records():
    """The fast path's queue records hold 15 bits of primitive index: a scene of 32,768 primitives
    is refused with a clear error (the plain method still checks it), where 32,767 would only run
    out of shared memory."""
    from plainmp_gb300 import Pose, SphereSDF, UnionSDF

    robot = W.chain7_robot()
    _, cst, _ = scenes.make_constraint(robot, None, self_collision=False)
    far = [SphereSDF(0.01, Pose(np.array([10.0 + 0.001 * i, 0.0, 0.0]), np.eye(3))) for i in range(32768)]
    cst.set_sdf(UnionSDF(far))
    Q = W.chain7_configs(4, seed=47)
    assert cst.is_valid_batch(Q).all()
    with pytest.raises(ValueError, match="32767 primitives"):
        cst.is_valid_fast(Q)


def test_fast_single_calls(chain, dual):
    """One state or one edge per host-memory call, as OMPL's callbacks call, many calls in a row
    through the same staging buffers: every answer equals the oracle's (validity, edges) or the
    plain FP64 distances within DIST_TOL."""
    (_, cst, _), (_, oc, _) = chain
    Q = W.chain7_configs(40, seed=91)
    ref = oc.is_valid(Q).astype(bool)
    got = np.array([bool(cst.is_valid_fast(q[None])[0]) for q in Q])
    assert np.array_equal(got, ref) and 0 < ref.sum() < len(Q)
    s1, s2 = W.chain7_edges(24, seed=92, max_waypoints=6)
    mv = BoxMotionValidator(cst, [0.05] * 7)
    e_ref = oc.check_motion(s1, s2, 0, [0.05] * 7)[0].astype(bool)
    e_got = np.array([bool(mv.check_motion_fast(a[None], b[None])[0]) for a, b in zip(s1, s2)])
    assert np.array_equal(e_got, e_ref) and 0 < e_ref.sum() < len(e_ref)
    # two states per call, with distances, on the cloud scene
    (_, cst2, _), (_, oc2, _) = dual
    Q2 = W.dualarm_configs(30, seed=93)
    ref2 = oc2.is_valid(Q2).astype(bool)
    d_ref = np.minimum(cst2.sphere_distances(Q2), CUTOFF)
    for k in range(0, len(Q2), 2):
        ok, d = cst2.is_valid_fast(Q2[k:k + 2], distances=True)
        assert np.array_equal(ok.astype(bool), ref2[k:k + 2])
        assert np.abs(d.astype(np.float64) - d_ref[k:k + 2]).max() < DIST_TOL
