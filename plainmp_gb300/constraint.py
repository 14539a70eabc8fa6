"""SphereCollisionCst mirroring plainmp.constraint (src/plainmp/constraint.pyi:9-38,76-94,
cpp/plainmp/bindings/constraint.cpp:65-84) on top of the C ABI.

Single-configuration methods keep the reference's signatures (``is_valid(q) -> bool``,
``evaluate(q) -> (vals, jac)``, ``update_kintree(q, high_accuracy)``); the ``*_batch``
methods take a (B, q_dim) numpy array (host memory) or a torch CUDA tensor (device memory,
enqueued on torch's current stream) and are the GB300 hot path.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import List, Optional, Sequence, Tuple

import numpy as np

from ._lib import Batch, check, cstrs, dptr, f64, lib
from .kinematics import BaseType, KinematicModel
from .psdf import SDFBase


class ConstraintBase:
    """plainmp.constraint.ConstraintBase (bindings/constraint.cpp:31-35): update_kintree(q,
    high_accuracy), evaluate(q) -> (values, jacobian), get_kin(), get_control_joint_names().  Every
    constraint below provides them; the *_batch methods are the batched forms."""


class EqConstraintBase(ConstraintBase):
    """plainmp.constraint.EqConstraintBase (bindings/constraint.cpp:36-37): values meant to be zero."""


class IneqConstraintBase(ConstraintBase):
    """plainmp.constraint.IneqConstraintBase (bindings/constraint.cpp:38-39): values meant to be
    non-negative, with is_valid(q)."""


@dataclass
class SphereAttachmentSpec:
    """SphereAttachmentSpec(parent_link_name, relative_positions (3, n), radii (n,), only_self_collision)."""

    parent_link_name: str
    relative_positions: np.ndarray
    radii: np.ndarray
    only_self_collision: bool = False

    def __post_init__(self):
        self.relative_positions = f64(self.relative_positions)
        self.radii = f64(self.radii).reshape(-1)
        if self.relative_positions.ndim != 2 or self.relative_positions.shape[0] != 3:
            raise ValueError("relative_positions must be (3, n)")
        if self.relative_positions.shape[1] != self.radii.shape[0]:
            raise ValueError("relative_positions and radii disagree on the sphere count")


class SphereCollisionCst(IneqConstraintBase):
    def __init__(self, kin: KinematicModel, control_joint_names: Sequence[str], base_type: BaseType,
                 sphere_specs: Sequence[SphereAttachmentSpec], selcol_pairs: Sequence[Tuple[str, str]],
                 fixed_sdf: Optional[SDFBase] = None, reorder_spheres: bool = True) -> None:
        self._kin = kin
        self._fixed = fixed_sdf
        self._sdf = None
        self.control_joint_names = list(control_joint_names)
        self.base_type = BaseType(int(base_type))
        counts = np.array([s.radii.shape[0] for s in sphere_specs], dtype=np.int32)
        rel = (np.concatenate([s.relative_positions.T for s in sphere_specs], axis=0) if sphere_specs else np.zeros((0, 3)))
        rel = f64(rel)
        radii = f64(np.concatenate([s.radii for s in sphere_specs]) if sphere_specs else np.zeros(0))
        only = np.array([1 if s.only_self_collision else 0 for s in sphere_specs], dtype=np.uint8)
        h = C.c_void_p()
        check(lib.pmgpu_cst_create(
            kin._h, cstrs(self.control_joint_names), len(self.control_joint_names), int(self.base_type),
            len(sphere_specs), cstrs([s.parent_link_name for s in sphere_specs]),
            counts.ctypes.data_as(C.POINTER(C.c_int32)), dptr(rel), dptr(radii), only.ctypes.data_as(C.POINTER(C.c_uint8)),
            len(selcol_pairs), cstrs([a for a, _ in selcol_pairs]), cstrs([b for _, b in selcol_pairs]),
            fixed_sdf._h if fixed_sdf is not None else None, int(bool(reorder_spheres)), C.byref(h)))
        self._h = h

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib.pmgpu_cst_destroy(h)
            self._h = None

    # ---- structure
    def _dims(self):
        a, b, c, d = C.c_int(), C.c_int(), C.c_int(), C.c_int()
        check(lib.pmgpu_cst_dims(self._h, C.byref(a), C.byref(b), C.byref(c), C.byref(d)))
        return a.value, b.value, c.value, d.value

    def q_dim(self) -> int:
        return self._dims()[0]

    def cst_dim(self) -> int:
        return self._dims()[1]

    @property
    def n_spheres(self) -> int:
        return self._dims()[2]

    @property
    def n_groups(self) -> int:
        return self._dims()[3]

    def groups(self) -> dict:
        """Constructed group table (post-reorder order)."""
        ng, ns = self.n_groups, self.n_spheres
        i32 = C.POINTER(C.c_int32)
        link = np.empty(max(ng, 1), dtype=np.int32)
        rad = np.empty(max(ng, 1))
        ctr = np.empty((max(ng, 1), 3))
        only = np.empty(max(ng, 1), dtype=np.int32)
        rel = np.empty((max(ns, 1), 3))
        sr = np.empty(max(ns, 1))
        check(lib.pmgpu_cst_groups(self._h, link.ctypes.data_as(i32), dptr(rad), dptr(ctr), only.ctypes.data_as(i32), dptr(rel), dptr(sr)))
        return {"link": link[:ng], "radius": rad[:ng], "centre": ctr[:ng], "only_self": only[:ng], "rel": rel[:ns], "radii": sr[:ns]}

    def get_kin(self) -> KinematicModel:
        return self._kin

    def get_control_joint_names(self) -> List[str]:
        return list(self.control_joint_names)

    def set_sdf(self, sdf: Optional[SDFBase]) -> None:
        check(lib.pmgpu_cst_set_sdf(self._h, sdf._h if sdf is not None else None))
        self._sdf = sdf

    def get_sdf(self) -> Optional[SDFBase]:
        return self._sdf

    # ---- single configuration (reference signatures)
    def update_kintree(self, q, high_accuracy: bool = True) -> None:
        qq = f64(q, (self.q_dim(),))
        check(lib.pmgpu_cst_update_kintree(self._h, dptr(qq), int(bool(high_accuracy))))

    def is_valid(self, q) -> bool:
        """IneqConstraintBase.is_valid: also leaves the model in q's state, as the reference does."""
        qq = f64(q, (1, self.q_dim()))
        ok = bool(self.is_valid_batch(qq)[0])
        self.update_kintree(qq[0], high_accuracy=self.base_type != BaseType.FIXED)
        return ok

    def evaluate(self, q) -> Tuple[np.ndarray, np.ndarray]:
        qq = f64(q, (1, self.q_dim()))
        vals, jac = self.evaluate_batch(qq)
        self.update_kintree(qq[0], high_accuracy=True)
        return vals[0], jac[0]

    def get_all_spheres(self) -> List[Tuple[np.ndarray, float]]:
        n = self.n_spheres
        out = np.empty((max(n, 1), 4))
        check(lib.pmgpu_cst_get_all_spheres(self._h, dptr(out)))
        return [(out[i, :3].copy(), float(out[i, 3])) for i in range(n)]

    def get_group_spheres(self) -> List[Tuple[np.ndarray, float]]:
        n = self.n_groups
        out = np.empty((max(n, 1), 4))
        check(lib.pmgpu_cst_get_group_spheres(self._h, dptr(out)))
        return [(out[i, :3].copy(), float(out[i, 3])) for i in range(n)]

    # ---- batches (the device hot path)
    def _batch(self, Q):
        b = Batch(Q)
        if len(b.shape) != 2 or b.shape[1] != self.q_dim():
            raise ValueError(f"expected a (B, {self.q_dim()}) batch, got {b.shape}")
        return b

    def is_valid_batch(self, Q):
        """Plain FP64 method: (B,) uint8 validity, bit-exact with the reference."""
        b = self._batch(Q)
        out, optr = b.empty((b.shape[0],), np.uint8)
        check(lib.pmgpu_cst_is_valid(self._h, b.ptr, b.shape[0], optr, b.mem, b.stream))
        return out

    def evaluate_batch(self, Q):
        """(vals (B, cst_dim), jac (B, cst_dim, q_dim)) in FP64."""
        b = self._batch(Q)
        m, d = self.cst_dim(), self.q_dim()
        vals, vptr = b.empty((b.shape[0], m), np.float64)
        jac, jptr = b.empty((b.shape[0], m, d), np.float64)
        check(lib.pmgpu_cst_evaluate(self._h, b.ptr, b.shape[0], vptr, jptr, b.mem, b.stream))
        return vals, jac

    def sphere_distances(self, Q, high_accuracy: bool = False, centres: bool = False):
        """Per-sphere signed distance (B, n_spheres) in FP64 (and centres (B, n_spheres, 3))."""
        b = self._batch(Q)
        ns = self.n_spheres
        dist, dptr_ = b.empty((b.shape[0], ns), np.float64)
        cen, cptr = b.empty((b.shape[0], ns, 3), np.float64) if centres else (None, None)
        check(lib.pmgpu_cst_sphere_distances(self._h, b.ptr, b.shape[0], int(bool(high_accuracy)), dptr_, cptr, b.mem, b.stream))
        return (dist, cen) if centres else dist

    def set_fast_launch(self, configs_per_block: int, threads_per_block: int) -> None:
        """Launch shape of the fast kernel (see plainmp_gb300.autotune)."""
        check(lib.pmgpu_cst_set_fast_launch(self._h, int(configs_per_block), int(threads_per_block)))

    def get_fast_launch(self) -> Tuple[int, int]:
        a, b = C.c_int(), C.c_int()
        check(lib.pmgpu_cst_get_fast_launch(self._h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def set_fast_tuning(self, sphere_tile: int = 0, hq_blocks_per_sm: int = 4, edge_configs_per_block: int = 32,
                        edge_threads: int = 128) -> None:
        """The fast kernels' other tuning parameters (see plainmp_gb300.autotune): spheres of one
        configuration per warp row of sphere tasks (0: the least), blocks per SM of the hard
        cloud-query kernel, and the edge kernel's waypoints and threads per block."""
        check(lib.pmgpu_cst_set_fast_tuning(self._h, int(sphere_tile), int(hq_blocks_per_sm), int(edge_configs_per_block),
                                             int(edge_threads)))

    def get_fast_tuning(self) -> Tuple[int, int, int, int]:
        v = [C.c_int() for _ in range(4)]
        check(lib.pmgpu_cst_get_fast_tuning(self._h, *(C.byref(x) for x in v)))
        return tuple(x.value for x in v)

    def is_valid_fast(self, Q, distances: bool = False, stats: bool = False, out=None, dist_out=None):
        """FP32 + FP64-recheck path: validity identical to is_valid_batch; optional FP32
        per-sphere signed distances clamped at the reference's 0.1 m cutoff (B, n_spheres) and
        recheck statistics.  out / dist_out may be preallocated buffers (e.g. pinned host
        arrays) in the same memory space as Q."""
        b = self._batch(Q)
        if out is not None:
            optr = b.out(out, (b.shape[0],), np.uint8)
        else:
            out, optr = b.empty((b.shape[0],), np.uint8)
        if distances and dist_out is not None:
            dist, dp = dist_out, b.out(dist_out, (b.shape[0], self.n_spheres), np.float32)
        else:
            dist, dp = b.empty((b.shape[0], self.n_spheres), np.float32) if distances else (None, None)
        st = np.zeros(4, dtype=np.int64)
        check(lib.pmgpu_cst_is_valid_fast(self._h, b.ptr, b.shape[0], optr, dp, C.c_void_p(st.ctypes.data) if stats else None,
                                          b.mem, b.stream))
        res = [out]
        if distances:
            res.append(dist)
        if stats:
            res.append({"configs": int(st[0]), "rechecked_terms": int(st[1]), "rechecked_configs": int(st[2])})
        return res[0] if len(res) == 1 else tuple(res)


# ------------------------------------------------------------------ pose constraints, composites
class _PoseCstBase:
    """Shared part of LinkPoseCst / LinkPositionBoundCst (one C handle type, pmgpu_posecst)."""

    def __init__(self, kin: KinematicModel, control_joint_names: Sequence[str], base_type: BaseType):
        self._kin = kin
        self.control_joint_names = list(control_joint_names)
        self.base_type = BaseType(int(base_type))
        self._h = None

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib.pmgpu_posecst_destroy(h)
            self._h = None

    def _dims(self):
        qd, cd, eq = C.c_int(), C.c_int(), C.c_int()
        check(lib.pmgpu_posecst_dims(self._h, C.byref(qd), C.byref(cd), C.byref(eq)))
        return qd.value, cd.value, bool(eq.value)

    def q_dim(self) -> int:
        return self._dims()[0]

    def cst_dim(self) -> int:
        return self._dims()[1]

    def get_kin(self) -> KinematicModel:
        return self._kin

    def get_control_joint_names(self) -> List[str]:
        return list(self.control_joint_names)

    def update_kintree(self, q, high_accuracy: bool = True) -> None:
        """ConstraintBase.update_kintree (primitive.hpp:38-62) on the shared model state."""
        qq = f64(q, (self.q_dim(),))
        check(lib.pmgpu_posecst_update_kintree(self._h, dptr(qq), int(bool(high_accuracy))))

    def _batch(self, Q):
        b = Batch(Q)
        if len(b.shape) != 2 or b.shape[1] != self.q_dim():
            raise ValueError(f"expected a (B, {self.q_dim()}) batch, got {b.shape}")
        return b

    def evaluate_batch(self, Q):
        """ConstraintBase.evaluate for every row of Q: (vals (B, cst_dim), jac (B, cst_dim, q_dim)), FP64."""
        b = self._batch(Q)
        m, d = self.cst_dim(), self.q_dim()
        vals, vp = b.empty((b.shape[0], m), np.float64)
        jac, jp = b.empty((b.shape[0], m, d), np.float64)
        check(lib.pmgpu_posecst_evaluate(self._h, b.ptr, b.shape[0], vp, jp, b.mem, b.stream))
        return vals, jac

    def evaluate(self, q) -> Tuple[np.ndarray, np.ndarray]:
        qq = f64(q, (1, self.q_dim()))
        vals, jac = self.evaluate_batch(qq)
        return vals[0], jac[0]


class LinkPoseCst(_PoseCstBase, EqConstraintBase):
    """LinkPoseCst(kin, control_joint_names, base_type, link_names, poses): poses of 3 (position),
    6 (position + RPY) or 7 (position + quaternion xyzw) values (constraints/primitive_link_pose.cpp)."""

    def __init__(self, kin: KinematicModel, control_joint_names: Sequence[str], base_type: BaseType, link_names: Sequence[str],
                 poses: Sequence[np.ndarray]):
        super().__init__(kin, control_joint_names, base_type)
        if len(link_names) != len(poses):
            raise ValueError("one pose per link")
        self._poses = [f64(p).reshape(-1) for p in poses]
        dims = np.array([p.shape[0] for p in self._poses], dtype=np.int32)
        flat = np.ascontiguousarray(np.concatenate(self._poses) if self._poses else np.zeros(1))
        h = C.c_void_p()
        check(lib.pmgpu_linkpose_create(kin._h, cstrs(self.control_joint_names), len(self.control_joint_names), int(self.base_type),
                                        cstrs(list(link_names)), len(link_names), dptr(flat),
                                        dims.ctypes.data_as(C.POINTER(C.c_int32)), C.byref(h)))
        self._h = h

    def get_desired_poses(self) -> List[np.ndarray]:
        return [p.copy() for p in self._poses]


class LinkPositionBoundCst(_PoseCstBase, IneqConstraintBase):
    """LinkPositionBoundCst(kin, control_joint_names, base_type, link_name, axis, lb, ub): lb <= p[axis] <= ub
    for the link's world position, either bound optional (constraints/primitive_link_position_bound.cpp)."""

    def __init__(self, kin: KinematicModel, control_joint_names: Sequence[str], base_type: BaseType, link_name: str, axis: int,
                 lb: Optional[float] = None, ub: Optional[float] = None):
        super().__init__(kin, control_joint_names, base_type)
        h = C.c_void_p()
        check(lib.pmgpu_linkbound_create(kin._h, cstrs(self.control_joint_names), len(self.control_joint_names), int(self.base_type),
                                         link_name.encode(), int(axis), int(lb is not None), float(lb or 0.0), int(ub is not None),
                                         float(ub or 0.0), C.byref(h)))
        self._h = h

    def is_valid_batch(self, Q):
        """(B,) uint8: the link position within the bounds after update_kintree(q, False)."""
        b = self._batch(Q)
        out, optr = b.empty((b.shape[0],), np.uint8)
        check(lib.pmgpu_posecst_is_valid(self._h, b.ptr, b.shape[0], optr, b.mem, b.stream))
        return out

    def is_valid(self, q) -> bool:
        return bool(self.is_valid_batch(f64(q, (1, self.q_dim())))[0])


class _CompositeBase:
    """CompositeConstraintBase (constraints/composite_constraint.hpp:21-86): constraints on one
    kinematic model.  The batched calls evaluate each member on the same batch and stack the rows.
    The reference drives the shared model with the first member's q mapping; the batched path
    requires every member to have the same control joints and base type, so the mappings agree."""

    _member = ConstraintBase

    def __init__(self, constraints):
        self.constraints = list(constraints)
        if not self.constraints:
            raise ValueError("a composite constraint needs at least one constraint")
        for c in self.constraints:  # the reference binds the member type (bindings/constraint.cpp:105, 109)
            if not isinstance(c, self._member):
                raise TypeError(f"{type(self).__name__} takes {self._member.__name__} members, got {type(c).__name__}")
        k0 = self.constraints[0].get_kin()
        for c in self.constraints:
            if c.get_kin() is not k0:
                raise RuntimeError("All constraints must have the same kinematic chain")
            if (c.get_control_joint_names() != self.constraints[0].get_control_joint_names()
                    or c.base_type != self.constraints[0].base_type):
                raise ValueError("batched composite constraints need the same control joints and base type")

    def q_dim(self) -> int:
        return self.constraints[0].q_dim()

    def cst_dim(self) -> int:
        return sum(c.cst_dim() for c in self.constraints)

    def evaluate_batch(self, Q):
        """(vals (B, cst_dim), jac (B, cst_dim, q_dim)): the members' rows stacked in order."""
        parts = [c.evaluate_batch(Q) for c in self.constraints]
        if _is_torch(parts[0][0]):
            import torch

            return torch.cat([p[0] for p in parts], dim=1), torch.cat([p[1] for p in parts], dim=1)
        return np.concatenate([p[0] for p in parts], axis=1), np.concatenate([p[1] for p in parts], axis=1)

    def evaluate(self, q):
        vals, jac = self.evaluate_batch(f64(q, (1, self.q_dim())))
        return vals[0], jac[0]

    def __str__(self) -> str:
        lines = ["Composite constraint:", f"total dim: {self.cst_dim()}"]
        lines += [f"  - {type(c).__name__}: {c.cst_dim()}" for c in self.constraints]
        return "\n".join(lines) + "\n"


def _is_torch(x) -> bool:
    return type(x).__module__.startswith("torch")


class EqCompositeCst(_CompositeBase):
    """EqCompositeCst(constraints) of equality constraints (LinkPoseCst)."""

    _member = EqConstraintBase


class IneqCompositeCst(_CompositeBase):
    """IneqCompositeCst(constraints): is_valid = AND over the members after update_kintree(q, False)
    (composite_constraint.hpp:98-105)."""

    _member = IneqConstraintBase

    def fused_parts(self):
        """(collision constraint, [bounds]) when the members are one SphereCollisionCst and any
        number of LinkPositionBoundCst: the fast path then checks all of them in one launch on one
        FK (pmgpu_composite_is_valid_fast); else None."""
        sph = [c for c in self.constraints if isinstance(c, SphereCollisionCst)]
        bnd = [c for c in self.constraints if isinstance(c, LinkPositionBoundCst)]
        if len(sph) != 1 or len(sph) + len(bnd) != len(self.constraints):
            return None
        return sph[0], bnd

    def is_valid_fast(self, Q, stats: bool = False, out=None):
        """Fused FP32 + FP64-recheck check of a SphereCollisionCst and LinkPositionBoundCst members
        (fused_parts): (B,) uint8 identical to the AND of the members' plain checks; stats as
        SphereCollisionCst.is_valid_fast."""
        parts = self.fused_parts()
        if parts is None:
            raise TypeError("is_valid_fast needs one SphereCollisionCst and LinkPositionBoundCst members")
        sph, bnd = parts
        b = sph._batch(Q)
        if out is not None:
            optr = b.out(out, (b.shape[0],), np.uint8)
        else:
            out, optr = b.empty((b.shape[0],), np.uint8)
        hs = (C.c_void_p * max(len(bnd), 1))(*[c._h for c in bnd])
        st = np.zeros(4, dtype=np.int64)
        check(lib.pmgpu_composite_is_valid_fast(sph._h, hs, len(bnd), b.ptr, b.shape[0], optr,
                                                C.c_void_p(st.ctypes.data) if stats else None, b.mem, b.stream))
        if stats:
            return out, {"configs": int(st[0]), "rechecked_terms": int(st[1]), "rechecked_configs": int(st[2])}
        return out

    def is_valid_batch(self, Q, fast: bool = True):
        """(B,) uint8 AND of the members' validity.  fast: one fused launch when fused_parts
        applies (same booleans), else each SphereCollisionCst member on its FP32 + FP64-recheck
        path; not fast: every member's plain FP64 method."""
        if fast and self.fused_parts() is not None:
            return self.is_valid_fast(Q)
        ok = None
        for c in self.constraints:
            if isinstance(c, SphereCollisionCst):
                r = c.is_valid_fast(Q) if fast else c.is_valid_batch(Q)
            else:
                r = c.is_valid_batch(Q)
            ok = r if ok is None else (ok & r)
        return ok

    def is_valid(self, q) -> bool:
        return bool(self.is_valid_batch(f64(q, (1, self.q_dim())))[0])


# plainmp.constraint also holds SequentialCst (bindings/constraint.cpp:114-125)
from .sequential import SequentialCst  # noqa: E402,F401
