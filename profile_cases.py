"""Small, self-contained launches for profiling: the fast collision check of 65,536 dual-arm
configurations against the 200k-point box-surface cloud, validity only (``valid``) or with the
per-sphere distances (``dist``), three launches each; one fused IK descent (8192 problems x 50
steps, ``ik``); one trajectory cost + gradient (512 trajectories, ``traj``); three fast edge
pipelines over 1024 chain edges (``edges``); two plain FP64 batches of 8192 dual-arm configurations
(``plain``).
python profile_cases.py [valid|dist|ik|traj|edges|plain|all]"""
import sys
from pathlib import Path

import numpy as np

sys.path.insert(0, str(Path(__file__).resolve().parent))


def fast(distances: bool, n: int = 65536, launches: int = 3):
    import torch

    from plainmp_gb300 import scenes
    from plainmp_gb300 import workloads as W

    _, cst, _ = scenes.make_constraint(W.dualarm_robot(), W.Scene(cloud=W.box_surface_cloud(), cloud_radius=0.0))
    cst.set_fast_launch(16, 256)  # the shape and sphere tile the benchmark's autotuner picks for this workload
    cst.set_fast_tuning(8, 4, 32, 128)
    Q = torch.tensor(W.dualarm_configs(n), device="cuda")
    for _ in range(launches):
        cst.is_valid_fast(Q, distances=distances)
    torch.cuda.synchronize()


def edges(launches: int = 3):
    """C1: 1024 edges (1-120 waypoints) on the 7-joint chain, the fast edge pipeline."""
    import torch

    from plainmp_gb300 import BoxMotionValidator, scenes
    from plainmp_gb300 import workloads as W

    _, cst, _ = scenes.make_constraint(W.chain7_robot(), W.chain7_scene())
    s1, s2 = W.chain7_edges(1024)
    S1, S2 = torch.tensor(s1, device="cuda"), torch.tensor(s2, device="cuda")
    mv = BoxMotionValidator(cst, [0.05] * 7)
    for _ in range(launches):
        mv.check_motion_fast(S1, S2)
    torch.cuda.synchronize()


def plain(n: int = 8192, launches: int = 2):
    """The plain FP64 method (k_is_valid64) on n dual-arm configurations against the 200k-point cloud."""
    import torch

    from plainmp_gb300 import scenes
    from plainmp_gb300 import workloads as W

    _, cst, _ = scenes.make_constraint(W.dualarm_robot(), W.Scene(cloud=W.box_surface_cloud(), cloud_radius=0.0))
    Q = torch.tensor(W.dualarm_configs(n), device="cuda")
    for _ in range(launches):
        cst.is_valid_batch(Q)
    torch.cuda.synchronize()


def ik(steps: int = 50):
    import torch

    from plainmp_gb300 import diff, scenes
    from plainmp_gb300 import workloads as W

    robot, scene = W.chain7_robot(), W.chain7_scene()
    kin, cst, _ = scenes.make_constraint(robot, scene)
    link = kin.get_link_ids([robot.end_link])[0]
    q0, q_star = W.ik_problems(8192)
    tgt = diff.link_poses(cst, torch.tensor(q_star, device="cuda"), link).float()
    Q0 = torch.tensor(q0, dtype=torch.float32, device="cuda")
    for _ in range(2):
        diff.ik_descend(cst, Q0, tgt, link, steps=steps, lr=0.05)
    torch.cuda.synchronize()


def traj():
    import torch

    from plainmp_gb300 import diff, scenes
    from plainmp_gb300 import workloads as W

    _, cst, _ = scenes.make_constraint(W.planar_chain7_robot(), W.Scene(cloud=W.box_surface_cloud(), cloud_radius=0.0))
    trajs = W.trajectories(512)
    Q = torch.tensor(np.concatenate(trajs, axis=0).astype(np.float32), device="cuda")
    off = torch.tensor(np.concatenate([[0], np.cumsum([len(t) for t in trajs])]).astype(np.int64), device="cuda")
    for _ in range(2):
        diff.traj_cost_grad(cst, Q, off)
    torch.cuda.synchronize()


if __name__ == "__main__":
    which = sys.argv[1] if len(sys.argv) > 1 else "all"
    if which in ("valid", "all"):
        fast(False)
    if which in ("dist", "all"):
        fast(True)
    if which in ("ik", "all"):
        ik()
    if which in ("traj", "all"):
        traj()
    if which in ("edges", "all"):
        edges()
    if which in ("plain", "all"):
        plain()
