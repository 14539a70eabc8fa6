"""KinematicModel and BaseType, mirroring plainmp.kinematics (src/plainmp/kinematics.pyi,
cpp/plainmp/bindings/kinematics.cpp:26-45) on top of the C ABI."""
from __future__ import annotations

import ctypes as C
from enum import IntEnum
from typing import List, Sequence, Tuple

import numpy as np

from ._lib import check, cstrs, dptr, f64, lib


class BaseType(IntEnum):
    FIXED = 0
    FLOATING = 1
    PLANAR = 2


class KinematicModel:
    """KinematicModel(urdf_string): the URDF text (not a path), as in the reference."""

    def __init__(self, urdf_string: str) -> None:
        h = C.c_void_p()
        check(lib.pmgpu_model_create(urdf_string.encode(), C.byref(h)))
        self._h = h
        self._urdf = urdf_string

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib.pmgpu_model_destroy(h)
            self._h = None

    # ---- structure
    def _counts(self) -> Tuple[int, int, int]:
        nl, nj, root = C.c_int(), C.c_int(), C.c_int()
        check(lib.pmgpu_model_counts(self._h, C.byref(nl), C.byref(nj), C.byref(root)))
        return nl.value, nj.value, root.value

    @property
    def num_links(self) -> int:
        return self._counts()[0]

    @property
    def num_dof(self) -> int:
        return self._counts()[1]

    def get_joint_ids(self, joint_names: Sequence[str]) -> List[int]:
        out = np.empty(len(joint_names), dtype=np.int64)
        check(lib.pmgpu_model_get_joint_ids(self._h, cstrs(joint_names), len(joint_names), out.ctypes.data_as(C.POINTER(C.c_int64))))
        return [int(v) for v in out]

    def get_link_ids(self, link_names: Sequence[str]) -> List[int]:
        out = np.empty(len(link_names), dtype=np.int64)
        check(lib.pmgpu_model_get_link_ids(self._h, cstrs(link_names), len(link_names), out.ctypes.data_as(C.POINTER(C.c_int64))))
        return [int(v) for v in out]

    def get_joint_position_limits(self, joint_ids: Sequence[int]) -> List[Tuple[float, float]]:
        ids = np.asarray(joint_ids, dtype=np.int64)
        lo = np.empty(len(ids))
        hi = np.empty(len(ids))
        check(lib.pmgpu_model_get_joint_position_limits(self._h, ids.ctypes.data_as(C.POINTER(C.c_int64)), len(ids), dptr(lo), dptr(hi)))
        return [(float(a), float(b)) for a, b in zip(lo, hi)]

    def link_name(self, link_id: int) -> str:
        buf = C.create_string_buffer(512)
        check(lib.pmgpu_model_link_name(self._h, link_id, buf, 512))
        return buf.value.decode()

    def joint_name(self, joint_id: int) -> str:
        buf = C.create_string_buffer(512)
        check(lib.pmgpu_model_joint_name(self._h, joint_id, buf, 512))
        return buf.value.decode()

    def structure(self) -> dict:
        """Link parents, initial local transforms and joint records (for tests)."""
        nl, nj, root = self._counts()
        par = np.empty(nl, dtype=np.int32)
        tf = np.empty((nl, 7))
        tfq = np.empty(nl, dtype=np.int32)
        jc = np.empty(max(nj, 1), dtype=np.int32)
        jt = np.empty(max(nj, 1), dtype=np.int32)
        ja = np.empty((max(nj, 1), 3))
        jq = np.empty(max(nj, 1), dtype=np.int32)
        i32 = C.POINTER(C.c_int32)
        check(lib.pmgpu_model_structure(self._h, par.ctypes.data_as(i32), dptr(tf), tfq.ctypes.data_as(i32), jc.ctypes.data_as(i32),
                                        jt.ctypes.data_as(i32), dptr(ja), jq.ctypes.data_as(i32)))
        return {
            "link_names": [self.link_name(i) for i in range(nl)],
            "joint_names": [self.joint_name(i) for i in range(nj)],
            "link_parent": par, "link_tf7": tf, "link_tf_qid": tfq, "root": root,
            "joint_child": jc[:nj], "joint_type": jt[:nj], "joint_axis": ja[:nj], "joint_origin_qid": jq[:nj],
        }

    # ---- state
    def set_joint_positions(self, joint_ids: Sequence[int], positions, accurate: bool = True) -> None:
        ids = np.asarray(joint_ids, dtype=np.int64)
        q = f64(positions)
        if q.shape != (len(ids),):
            raise ValueError("positions must match joint_ids")
        check(lib.pmgpu_model_set_joint_positions(self._h, ids.ctypes.data_as(C.POINTER(C.c_int64)), len(ids), dptr(q), int(bool(accurate))))

    def get_joint_positions(self, joint_ids: Sequence[int]) -> List[float]:
        ids = np.asarray(joint_ids, dtype=np.int64)
        q = np.empty(len(ids))
        check(lib.pmgpu_model_get_joint_positions(self._h, ids.ctypes.data_as(C.POINTER(C.c_int64)), len(ids), dptr(q)))
        return [float(v) for v in q]

    def set_base_pose(self, pose_vec) -> None:
        """pose_vec: [x, y, z, qx, qy, qz, qw]"""
        p = f64(pose_vec, (7,))
        check(lib.pmgpu_model_set_base_pose(self._h, dptr(p)))

    def get_base_pose(self) -> np.ndarray:
        p = np.empty(7)
        check(lib.pmgpu_model_get_base_pose(self._h, dptr(p)))
        return p

    def debug_get_link_pose(self, link_name: str) -> np.ndarray:
        """[x, y, z, qx, qy, qz, qw] of a link in the current state (device FK)."""
        return self.link_poses([self.get_link_ids([link_name])[0]])[0]

    def link_poses(self, link_ids: Sequence[int]) -> np.ndarray:
        ids = np.asarray(link_ids, dtype=np.int64)
        out = np.empty((len(ids), 7))
        check(lib.pmgpu_model_link_poses(self._h, ids.ctypes.data_as(C.POINTER(C.c_int64)), len(ids), dptr(out)))
        return out

    def add_new_link(self, link_name: str, parent_link_name: str, position, rpy, consider_rotation: bool) -> int:
        p = f64(position, (3,))
        r = f64(rpy, (3,))
        out = C.c_int64()
        check(lib.pmgpu_model_add_new_link(self._h, link_name.encode(), parent_link_name.encode(), dptr(p), dptr(r),
                                           int(bool(consider_rotation)), C.byref(out)))
        return int(out.value)
