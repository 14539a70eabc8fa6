"""Seeded synthetic robots, scenes and batches for the collision-checking hot path.

Every workload is generated from fixed numpy seeds, so the device path, the CPU
oracle and the benchmark all see the same bytes.  The shapes follow the five
workloads the hot path is measured on:

* ``chain7``      -- 7-revolute serial chain, 56 spheres, 10 boxes + 5 spheres +
                     5 cylinders in a 1 m cube, 4096 joint configurations.
* ``edges``       -- 1024 straight C-space edges on the chain7 robot/scene, box
                     motion validator with 0.05 rad width, 1..120 waypoints each.
* ``dualarm``     -- 14-DOF dual arm (two chain7 arms on a torso, 0.4 m apart),
                     120 spheres, 200k-point cloud on 12 box surfaces (sigma 2 mm
                     noise, stored as float32), 65536 configurations.
* ``ik``          -- 8192 reachable end-link targets on chain7.
* ``trajectories``-- 512 trajectories of 20..100 waypoints on a planar-base
                     (x, y, yaw) + chain7 robot against the dualarm cloud.

The robot description is produced as URDF text (what ``KinematicModel`` takes)
plus sphere specs mirroring ``SphereAttachmentSpec`` (parent link, 3xN relative
centres, radii, only-self flag) and self-collision link-name pairs.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import List, Optional, Tuple

import numpy as np

PI = math.pi


@dataclass
class SphereSpec:
    parent_link_name: str
    relative_positions: np.ndarray  # (3, n) float64
    radii: np.ndarray  # (n,) float64
    only_self_collision: bool = False


@dataclass
class Primitive:
    kind: str  # "box" | "sphere" | "cylinder"
    position: np.ndarray  # (3,)
    rotation: np.ndarray  # (3, 3)
    size: Tuple[float, ...]  # box: (wx, wy, wz); sphere: (r,); cylinder: (r, h)


@dataclass
class Robot:
    urdf: str
    control_joints: List[str]
    end_link: str
    spheres: List[SphereSpec]
    self_pairs: List[Tuple[str, str]]
    base_type: str = "FIXED"  # FIXED | PLANAR | FLOATING


@dataclass
class Scene:
    primitives: List[Primitive] = field(default_factory=list)
    cloud: Optional[np.ndarray] = None  # (N, 3) float32
    cloud_radius: float = 0.0


def _fmt(x: float) -> str:
    return repr(float(x))


def _random_rotation(rng: np.random.Generator) -> np.ndarray:
    a = rng.standard_normal((3, 3))
    qm, rm = np.linalg.qr(a)
    qm = qm @ np.diag(np.sign(np.diag(rm)))
    if np.linalg.det(qm) < 0:
        qm[:, 0] = -qm[:, 0]
    return qm


def _chain_params(seed: int = 0, n: int = 7):
    """Offsets (n+1, 3) -- the last one only bounds the last link's spheres --,
    unit axes (n, 3), per-link sphere centres (n, 8, 3) and radii (n, 8)."""
    rng = np.random.default_rng(seed)
    offsets = rng.uniform(0.05, 0.35, size=(n + 1, 3))
    axes = rng.standard_normal((n, 3))
    axes /= np.linalg.norm(axes, axis=1, keepdims=True)
    centres = np.empty((n, 8, 3))
    radii = np.empty((n, 8))
    for k in range(n):
        nxt = offsets[k + 1]
        lo = np.minimum(0.0, nxt)
        hi = np.maximum(0.0, nxt)
        centres[k] = rng.uniform(lo, hi, size=(8, 3))
        radii[k] = rng.uniform(0.03, 0.08, size=8)
    return offsets, axes, centres, radii


def _chain_xml(prefix: str, root: str, offsets, axes, mirror_y: bool, first_origin=None) -> str:
    lines = []
    n = axes.shape[0]
    parent = root
    for k in range(n):
        off = offsets[k].copy()
        ax = axes[k].copy()
        if mirror_y:
            off[1] = -off[1]
            ax = np.array([-ax[0], ax[1], -ax[2]])  # reflection acts on axes as a pseudovector
        if k == 0 and first_origin is not None:
            off = np.asarray(first_origin, dtype=float)
        link = f"{prefix}link{k + 1}"
        lines.append(f'  <link name="{link}"/>')
        lines.append(
            f'  <joint name="{prefix}j{k + 1}" type="revolute">\n'
            f'    <parent link="{parent}"/>\n    <child link="{link}"/>\n'
            f'    <origin xyz="{_fmt(off[0])} {_fmt(off[1])} {_fmt(off[2])}" rpy="0 0 0"/>\n'
            f'    <axis xyz="{_fmt(ax[0])} {_fmt(ax[1])} {_fmt(ax[2])}"/>\n'
            f'    <limit lower="{_fmt(-PI)}" upper="{_fmt(PI)}" effort="10" velocity="1"/>\n'
            f"  </joint>"
        )
        parent = link
    return "\n".join(lines)


def _chain_spheres(prefix: str, centres, radii, mirror_y: bool) -> List[SphereSpec]:
    out = []
    for k in range(centres.shape[0]):
        c = centres[k].copy()
        if mirror_y:
            c[:, 1] = -c[:, 1]
        out.append(SphereSpec(f"{prefix}link{k + 1}", np.ascontiguousarray(c.T), radii[k].copy()))
    return out


def chain7_robot(seed: int = 0) -> Robot:
    """7-revolute serial chain rooted at ``base_link`` (identity joint origins)."""
    offsets, axes, centres, radii = _chain_params(seed)
    body = _chain_xml("", "base_link", offsets, axes, mirror_y=False)
    urdf = f'<?xml version="1.0"?>\n<robot name="chain7">\n  <link name="base_link"/>\n{body}\n</robot>\n'
    spheres = _chain_spheres("", centres, radii, mirror_y=False)
    pairs = [(f"link{i}", f"link{j}") for i in range(1, 8) for j in range(i + 2, 8)]
    return Robot(urdf, [f"j{k}" for k in range(1, 8)], "link7", spheres, pairs)


def chain7_scene(seed: int = 0, center=(0.55, 0.55, 0.55)) -> Scene:
    """10 boxes, 5 spheres, 5 cylinders, uniformly random poses in a 1 m cube
    centred at ``center``; sizes U[0.05, 0.3] m (box widths, sphere and cylinder
    diameters, cylinder heights)."""
    rng = np.random.default_rng(seed + 1000)
    c = np.asarray(center, dtype=float)
    prims: List[Primitive] = []
    for kind, count in (("box", 10), ("sphere", 5), ("cylinder", 5)):
        for _ in range(count):
            pos = c + rng.uniform(-0.5, 0.5, size=3)
            rot = _random_rotation(rng)
            if kind == "box":
                size = tuple(float(v) for v in rng.uniform(0.05, 0.3, size=3))
            elif kind == "sphere":
                size = (0.5 * float(rng.uniform(0.05, 0.3)),)
            else:
                size = (0.5 * float(rng.uniform(0.05, 0.3)), float(rng.uniform(0.05, 0.3)))
            prims.append(Primitive(kind, pos, rot, size))
    return Scene(prims)


def chain7_configs(n: int = 4096, seed: int = 0) -> np.ndarray:
    rng = np.random.default_rng(seed + 2000)
    return rng.uniform(-PI, PI, size=(n, 7))


def chain7_edges(n: int = 1024, seed: int = 0, width: float = 0.05, max_waypoints: int = 120):
    """Straight C-space edges (s1, s2).  s1 and a direction come from a random
    config pair; the edge length is rescaled so the number of checked waypoints
    of the box validator, floor(max|dq|/width) + 1, is uniform in 1..120."""
    rng = np.random.default_rng(seed + 3000)
    s1 = rng.uniform(-PI, PI, size=(n, 7))
    s2r = rng.uniform(-PI, PI, size=(n, 7))
    target = rng.integers(1, max_waypoints + 1, size=n)
    d = s2r - s1
    dmax = np.abs(d).max(axis=1, keepdims=True)
    # max|dq| in [ (k-1)*w + 0.25w, (k-1)*w + 0.75w ] so floor(.)+1 == k robustly
    length = (target[:, None] - 1 + rng.uniform(0.25, 0.75, size=(n, 1))) * width
    s2 = s1 + d / dmax * length
    return s1, s2


def dualarm_robot(seed: int = 0) -> Robot:
    """Two chain7 arms (the right one mirrored in y) on a fixed torso, bases
    0.4 m apart; 112 arm spheres + 8 torso spheres; self pairs are the 49
    cross-arm link pairs plus torso vs links 3..7 of each arm."""
    offsets, axes, centres, radii = _chain_params(seed)
    rng = np.random.default_rng(seed + 4000)
    parts = ['<?xml version="1.0"?>', '<robot name="dualarm">', '  <link name="torso"/>']
    for side, y in (("l_", 0.2), ("r_", -0.2)):
        parts.append(f'  <link name="{side}base"/>')
        parts.append(
            f'  <joint name="{side}mount" type="fixed">\n    <parent link="torso"/>\n'
            f'    <child link="{side}base"/>\n    <origin xyz="0 {_fmt(y)} 0" rpy="0 0 0"/>\n  </joint>'
        )
        parts.append(_chain_xml(side, f"{side}base", offsets, axes, mirror_y=(side == "r_")))
    parts.append("</robot>")
    urdf = "\n".join(parts) + "\n"
    spheres = _chain_spheres("l_", centres, radii, False) + _chain_spheres("r_", centres, radii, True)
    torso_c = rng.uniform([-0.1, -0.15, -0.5], [0.1, 0.15, -0.05], size=(8, 3))
    torso_r = rng.uniform(0.03, 0.08, size=8)
    spheres.append(SphereSpec("torso", np.ascontiguousarray(torso_c.T), torso_r))
    pairs = [(f"l_link{i}", f"r_link{j}") for i in range(1, 8) for j in range(1, 8)]
    pairs += [("torso", f"{s}link{k}") for s in ("l_", "r_") for k in range(3, 8)]
    joints = [f"l_j{k}" for k in range(1, 8)] + [f"r_j{k}" for k in range(1, 8)]
    return Robot(urdf, joints, "l_link7", spheres, pairs)


def box_surface_cloud(n_points: int = 200_000, n_boxes: int = 12, seed: int = 0,
                      center=(0.6, 0.0, 0.8), extent: float = 1.5, sigma: float = 0.002) -> np.ndarray:
    """Points uniform (area-weighted) on the surfaces of random boxes inside a
    cube of side ``extent``, plus N(0, sigma^2) noise, as float32 (N, 3)."""
    rng = np.random.default_rng(seed + 5000)
    c = np.asarray(center, dtype=float)
    boxes = []
    for _ in range(n_boxes):
        w = rng.uniform(0.1, 0.5, size=3)
        pos = c + rng.uniform(-0.5 * extent + 0.5 * w.max(), 0.5 * extent - 0.5 * w.max(), size=3)
        rot = _random_rotation(rng)
        boxes.append((w, pos, rot))
    faces = []  # (area, box index, axis, sign)
    for bi, (w, _, _) in enumerate(boxes):
        for ax in range(3):
            a1, a2 = [i for i in range(3) if i != ax]
            for s in (-1.0, 1.0):
                faces.append((w[a1] * w[a2], bi, ax, s))
    areas = np.array([f[0] for f in faces])
    choice = rng.choice(len(faces), size=n_points, p=areas / areas.sum())
    pts = np.empty((n_points, 3))
    uv = rng.uniform(-0.5, 0.5, size=(n_points, 3))
    for fi, (_, bi, ax, s) in enumerate(faces):
        m = choice == fi
        if not m.any():
            continue
        w, pos, rot = boxes[bi]
        local = uv[m] * w
        local[:, ax] = 0.5 * s * w[ax]
        pts[m] = local @ rot.T + pos
    pts += rng.normal(0.0, sigma, size=pts.shape)
    return pts.astype(np.float32)


def dualarm_configs(n: int = 65536, seed: int = 0) -> np.ndarray:
    rng = np.random.default_rng(seed + 6000)
    return rng.uniform(-PI, PI, size=(n, 14))


def ik_problems(n: int = 8192, seed: int = 0):
    """Initial configs and reachable end-link targets (target = FK(q*) of a
    random q*; the FK is evaluated by the caller's KinematicModel)."""
    rng = np.random.default_rng(seed + 7000)
    q_star = rng.uniform(-PI, PI, size=(n, 7))
    q0 = q_star + rng.normal(0.0, 0.3, size=(n, 7))
    return q0, q_star


def planar_chain7_robot(seed: int = 0) -> Robot:
    """chain7 with a PLANAR base: q = [7 joints, x, y, yaw] as in
    ``ConstraintBase::update_kintree``."""
    r = chain7_robot(seed)
    return Robot(r.urdf, r.control_joints, r.end_link, r.spheres, r.self_pairs, base_type="PLANAR")


def trajectories(n: int = 512, seed: int = 0, t_min: int = 20, t_max: int = 100):
    """Uneven-length trajectories (list of (T_i, 10) float64) on the planar-base
    chain: straight lines between random endpoints plus smooth noise."""
    rng = np.random.default_rng(seed + 8000)
    out = []
    lens = rng.integers(t_min, t_max + 1, size=n)
    for T in lens:
        a = np.concatenate([rng.uniform(-PI, PI, 7), rng.uniform(-1.0, 1.0, 2), rng.uniform(-PI, PI, 1)])
        b = np.concatenate([rng.uniform(-PI, PI, 7), rng.uniform(-1.0, 1.0, 2), rng.uniform(-PI, PI, 1)])
        t = np.linspace(0.0, 1.0, T)[:, None]
        traj = a + (b - a) * t + 0.05 * rng.standard_normal((T, 10))
        out.append(traj)
    return out
