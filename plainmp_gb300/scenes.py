"""Instantiate the synthetic workloads (plainmp_gb300.workloads) as device objects."""
from __future__ import annotations

from typing import List, Optional

from . import workloads as W
from .constraint import SphereAttachmentSpec, SphereCollisionCst
from .kinematics import BaseType, KinematicModel
from .psdf import BoxSDF, CloudSDF, CylinderSDF, Pose, SDFBase, SphereSDF, UnionSDF


def primitives_sdf(scene: W.Scene) -> Optional[UnionSDF]:
    sdfs: List[SDFBase] = []
    for p in scene.primitives:
        pose = Pose(p.position, p.rotation)
        if p.kind == "box":
            sdfs.append(BoxSDF(list(p.size), pose))
        elif p.kind == "sphere":
            sdfs.append(SphereSDF(p.size[0], pose))
        else:
            sdfs.append(CylinderSDF(p.size[0], p.size[1], pose))
    return UnionSDF(sdfs) if sdfs else None


def make_constraint(robot: W.Robot, scene: Optional[W.Scene] = None, self_collision: bool = True, reorder: bool = True,
                    cell_size: float = 0.0):
    kin = KinematicModel(robot.urdf)
    specs = [SphereAttachmentSpec(s.parent_link_name, s.relative_positions, s.radii, s.only_self_collision) for s in robot.spheres]
    cst = SphereCollisionCst(kin, robot.control_joints, BaseType[robot.base_type], specs,
                             robot.self_pairs if self_collision else [], None, reorder)
    sdf = None
    if scene is not None:
        if scene.cloud is not None:
            sdf = CloudSDF(scene.cloud.astype("float64"), scene.cloud_radius, cell_size)
        else:
            sdf = primitives_sdf(scene)
        if sdf is not None:
            cst.set_sdf(sdf)
    return kin, cst, sdf
