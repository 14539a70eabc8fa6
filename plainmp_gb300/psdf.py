"""Primitive SDFs mirroring plainmp.psdf (src/plainmp/psdf.pyi,
cpp/plainmp/bindings/primitive.cpp:18-111).  Evaluation runs on the device."""
from __future__ import annotations

import ctypes as C
from typing import List, Optional

import numpy as np

from ._lib import Batch, check, dptr, f64, lib

UNION, BOX, CYLINDER, SPHERE, GROUND, CLOUD = range(6)


class Pose:
    """Pose(position=[0,0,0], rotation=eye(3)) (primitive_sdf.hpp:30-75)."""

    def __init__(self, position=None, rotation=None) -> None:
        self.position = np.zeros(3) if position is None else f64(position, (3,)).copy()
        self.rotation = np.eye(3) if rotation is None else f64(rotation, (3, 3)).copy()

    def _flags(self):
        aa, za = C.c_int(), C.c_int()
        r = f64(self.rotation, (3, 3))
        check(lib.pmgpu_pose_flags(dptr(r), C.byref(aa), C.byref(za), None))
        return bool(aa.value), bool(za.value)

    @property
    def axis_aligned(self) -> bool:
        return self._flags()[0]

    @property
    def z_axis_aligned(self) -> bool:
        return self._flags()[1]

    def translate(self, translation) -> None:
        self.position = self.position + f64(translation, (3,))

    def rotate_z(self, angle: float) -> None:
        c, s = np.cos(angle), np.sin(angle)
        rz = np.array([[c, -s, 0.0], [s, c, 0.0], [0.0, 0.0, 1.0]])
        self.rotation = rz @ self.rotation

    def __copy__(self):
        return Pose(self.position, self.rotation)

    def __deepcopy__(self, memo):
        return Pose(self.position, self.rotation)


class SDFBase:
    _h: C.c_void_p

    @classmethod
    def _wrap(cls, h: C.c_void_p):
        obj = cls.__new__(cls)
        obj._h = h
        obj._members = []
        return obj

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib.pmgpu_sdf_destroy(h)
            self._h = None

    def _info(self):
        kind = C.c_int()
        lb, ub, pos, rot = np.empty(3), np.empty(3), np.empty(3), np.empty(9)
        aa, za = C.c_int(), C.c_int()
        check(lib.pmgpu_sdf_info(self._h, C.byref(kind), dptr(lb), dptr(ub), C.byref(aa), C.byref(za), dptr(pos), dptr(rot)))
        return kind.value, lb, ub, bool(aa.value), bool(za.value), pos, rot.reshape(3, 3)

    def clone(self):
        h = C.c_void_p()
        check(lib.pmgpu_sdf_clone(self._h, C.byref(h)))
        return type(self)._wrap(h)

    def translate(self, translation) -> None:
        t = f64(translation, (3,))
        check(lib.pmgpu_sdf_translate(self._h, dptr(t)))

    def rotate_z(self, angle: float) -> None:
        check(lib.pmgpu_sdf_rotate_z(self._h, float(angle)))

    def evaluate_batch(self, points) -> np.ndarray:
        """points (3, N) -> (N,) signed distances (on the device)."""
        p = f64(points)
        if p.ndim != 2 or p.shape[0] != 3:
            raise ValueError("points must be (3, N)")
        return self.evaluate_points(np.ascontiguousarray(p.T))

    def evaluate_points(self, points):
        """points (N, 3) numpy array or torch CUDA tensor -> (N,) signed distances."""
        b = Batch(points)
        n = b.shape[0]
        out, optr = b.empty((n,), np.float64)
        check(lib.pmgpu_sdf_evaluate(self._h, b.ptr, n, optr, b.mem, b.stream))
        return out

    def evaluate(self, point) -> float:
        return float(self.evaluate_points(f64(point, (1, 3)))[0])

    def is_outside_points(self, points, radii):
        b = Batch(points)
        n = b.shape[0]
        r = Batch(radii) if not np.isscalar(radii) else Batch(np.full(n, float(radii)))
        out, optr = b.empty((n,), np.uint8)
        check(lib.pmgpu_sdf_is_outside(self._h, b.ptr, r.ptr, n, optr, b.mem, b.stream))
        return out

    def is_outside(self, point, radius: float) -> bool:
        return bool(self.is_outside_points(f64(point, (1, 3)), np.array([float(radius)]))[0])


class PrimitiveSDFBase(SDFBase):
    @property
    def lb(self) -> np.ndarray:
        return self._info()[1]

    @property
    def ub(self) -> np.ndarray:
        return self._info()[2]


class ClosedPrimitiveSDFBase(PrimitiveSDFBase):
    """plainmp.psdf.ClosedPrimitiveSDFBase: the bounded primitives (box, cylinder, sphere), which
    carry a pose."""


class _HasPose:
    @property
    def pose(self) -> Pose:
        _, _, _, _, _, pos, rot = self._info()
        return Pose(pos, rot)


class BoxSDF(ClosedPrimitiveSDFBase, _HasPose):
    def __init__(self, size, pose: Optional[Pose] = None) -> None:
        pose = pose or Pose()
        h = C.c_void_p()
        w = f64(size, (3,))
        check(lib.pmgpu_sdf_box_create(dptr(w), dptr(f64(pose.position, (3,))), dptr(f64(pose.rotation, (3, 3))), C.byref(h)))
        self._h = h
        self._members = []


class CylinderSDF(ClosedPrimitiveSDFBase, _HasPose):
    def __init__(self, radius: float, height: float, pose: Optional[Pose] = None) -> None:
        pose = pose or Pose()
        h = C.c_void_p()
        check(lib.pmgpu_sdf_cylinder_create(float(radius), float(height), dptr(f64(pose.position, (3,))),
                                            dptr(f64(pose.rotation, (3, 3))), C.byref(h)))
        self._h = h
        self._members = []


class SphereSDF(ClosedPrimitiveSDFBase, _HasPose):
    def __init__(self, radius: float, pose: Optional[Pose] = None) -> None:
        pose = pose or Pose()
        h = C.c_void_p()
        check(lib.pmgpu_sdf_sphere_create(float(radius), dptr(f64(pose.position, (3,))), dptr(f64(pose.rotation, (3, 3))), C.byref(h)))
        self._h = h
        self._members = []


class GroundSDF(PrimitiveSDFBase):
    def __init__(self, height: float) -> None:
        h = C.c_void_p()
        check(lib.pmgpu_sdf_ground_create(float(height), C.byref(h)))
        self._h = h
        self._members = []


class CloudSDF(PrimitiveSDFBase):
    """CloudSDF(points (N, 3), radius): exact nearest-point distance through a device grid."""

    def __init__(self, points, radius: float, cell_size: float = 0.0) -> None:
        p = f64(points)
        if p.ndim != 2 or p.shape[1] != 3:
            raise ValueError("points must be (N, 3)")
        h = C.c_void_p()
        check(lib.pmgpu_sdf_cloud_create(dptr(p), p.shape[0], float(radius), float(cell_size), C.byref(h)))
        self._h = h
        self._members = []

    def nearest(self, points):
        """(squared distance (N,), nearest point (N, 3)) for N query points (KDTree.sqdist/query)."""
        b = Batch(points)
        n = b.shape[0]
        sq, sp = b.empty((n,), np.float64)
        near, npt = b.empty((n, 3), np.float64)
        check(lib.pmgpu_cloud_nearest(self._h, b.ptr, n, sp, npt, b.mem, b.stream))
        return sq, near

    def stats(self) -> dict:
        """Sizes of the device grid: points, occupied fine cells, blocks, field cells, candidate-list
        entries and device bytes (the grid is built first if it is not yet)."""
        out = np.zeros(6, dtype=np.int64)
        check(lib.pmgpu_sdf_cloud_stats(self._h, out.ctypes.data_as(C.POINTER(C.c_int64))))
        keys = ("points", "occupied_cells", "blocks", "field_cells", "list_entries", "device_bytes")
        return {k: int(v) for k, v in zip(keys, out)}


class UnionSDF(SDFBase):
    def __init__(self, sdf_list: List[SDFBase]) -> None:
        arr = (C.c_void_p * max(len(sdf_list), 1))(*[s._h for s in sdf_list])
        h = C.c_void_p()
        check(lib.pmgpu_sdf_union_create(arr, len(sdf_list), C.byref(h)))
        self._h = h
        self._members = list(sdf_list)

    def add(self, sdf: SDFBase, clone: bool = False) -> None:
        check(lib.pmgpu_sdf_union_add(self._h, sdf._h, int(bool(clone))))
        if not clone:
            self._members.append(sdf)

    def merge(self, other: "UnionSDF", clone: bool = False) -> None:
        for m in list(other._members):
            self.add(m, clone)


__all__ = ["Pose", "SDFBase", "PrimitiveSDFBase", "BoxSDF", "CylinderSDF", "SphereSDF", "GroundSDF", "CloudSDF", "UnionSDF"]
