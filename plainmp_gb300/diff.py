"""Differentiable costs on the GPU: batched collision-aware IK and trajectory smoothing.

The forward value and the gradient come from the library's FP32 kernels (include/pmgpu.h,
"differentiable costs"); the gradient is a hand-written reverse-mode adjoint through the FK
chain and the SDF, not autograd.  ``IKCost`` and ``TrajectoryCost`` wrap them as
``torch.autograd.Function``s: the forward pass evaluates the cost only and the backward pass
recomputes FK and runs the adjoint, so nothing per link or per waypoint is kept between the two.

Terms (all FP32):
    d_s       min over primitives of SDF.evaluate(c_s) - r_s (the SphereCollisionCst ext-row
              value, constraints/primitive_sphere_collision.cpp:256-322)
    hinge     w_col * sum_s max(0, margin - d_s)^2
    pose      w_pos * ||p - p*||^2 + w_rot * ||log(R*^T R)||^2 of one link
    smoothing w_smooth * sum_t sum_d w_d^2 (q[t+1] - 2 q[t] + q[t-1])_d^2, the acceleration cost
              of smoothcost_fullmat (src/plainmp/nlp_solver/sqp_based_solver.py:74-97)
The reference computes the matching constraint values and Jacobians in FP64 for its CPU solvers
(src/plainmp/ik.py:42-156); ``min_distance`` returns that ext-row value with an analytic gradient.
"""
from __future__ import annotations

import ctypes as C
from typing import Optional, Sequence, Union

import numpy as np

from ._lib import Batch, check, lib

COST_SUM = 0
COST_MIN_DISTANCE = 1


class CostParams(C.Structure):
    """pmgpu_cost_params."""

    _fields_ = [
        ("mode", C.c_int32),
        ("pose_link", C.c_int32),
        ("w_pos", C.c_float),
        ("w_rot", C.c_float),
        ("w_col", C.c_float),
        ("margin", C.c_float),
        ("cutoff", C.c_float),
        ("w_smooth", C.c_float),
        ("dof_weights", C.POINTER(C.c_float)),
    ]


def _link_id(cst, link: Union[None, int, str]) -> int:
    if link is None:
        return -1
    if isinstance(link, str):
        return int(cst.get_kin().get_link_ids([link])[0])
    return int(link)


def make_params(cst, mode: int = COST_SUM, pose_link: Union[None, int, str] = None, w_pos: float = 1.0,
                w_rot: float = 0.1, w_col: float = 1.0, margin: float = 0.02, cutoff: float = 0.1,
                w_smooth: float = 1.0, dof_weights: Optional[Sequence[float]] = None):
    """A pmgpu_cost_params (and the array its dof_weights points at, to keep alive)."""
    p = CostParams()
    p.mode = mode
    p.pose_link = _link_id(cst, pose_link)
    p.w_pos, p.w_rot, p.w_col, p.margin, p.cutoff, p.w_smooth = w_pos, w_rot, w_col, margin, cutoff, w_smooth
    keep = None
    if dof_weights is not None:
        keep = np.ascontiguousarray(np.asarray(dof_weights, dtype=np.float32).reshape(-1))
        if keep.shape[0] != cst.q_dim():
            raise ValueError(f"dof_weights has {keep.shape[0]} entries, q_dim is {cst.q_dim()}")
        p.dof_weights = keep.ctypes.data_as(C.POINTER(C.c_float))
    return p, keep


def _pair(b: Batch, target):
    if target is None:
        return None, None
    tb = Batch(target, np.float32)
    if tb.mem != b.mem:
        raise ValueError("q and target must both be host arrays or both CUDA tensors")
    if tb.shape != (b.shape[0], 7):
        raise ValueError(f"target must be (B, 7) [x y z qx qy qz qw], got {tb.shape}")
    return tb, tb.ptr


def ik_cost_grad(cst, q, target=None, pose_link=None, want_grad: bool = True, **weights):
    """Cost (B,) and, if want_grad, its gradient (B, q_dim) for a batch of configurations.
    q and target are numpy arrays (host) or CUDA tensors (device, torch's current stream)."""
    b = Batch(q, np.float32)
    if len(b.shape) != 2 or b.shape[1] != cst.q_dim():
        raise ValueError(f"q must be (B, {cst.q_dim()}), got {b.shape}")
    tb, tp = _pair(b, target)
    p, keep = make_params(cst, pose_link=pose_link, **weights)
    cost, cp = b.empty((b.shape[0],), np.float32)
    grad, gp = b.empty((b.shape[0], cst.q_dim()), np.float32) if want_grad else (None, None)
    check(lib.pmgpu_ik_cost(cst._h, C.byref(p), b.ptr, tp, b.shape[0], cp, gp, b.mem, b.stream))
    del keep, tb
    return (cost, grad) if want_grad else cost


def min_distance(cst, q, cutoff: float = 0.1, want_grad: bool = True):
    """min(cutoff, min_s d_s) per configuration and its gradient: the value and Jacobian row of
    SphereCollisionCst's ext row, with an analytic SDF gradient in place of the reference's
    forward difference."""
    b = Batch(q, np.float32)
    p, _ = make_params(cst, mode=COST_MIN_DISTANCE, cutoff=cutoff)
    cost, cp = b.empty((b.shape[0],), np.float32)
    grad, gp = b.empty((b.shape[0], cst.q_dim()), np.float32) if want_grad else (None, None)
    check(lib.pmgpu_ik_cost(cst._h, C.byref(p), b.ptr, None, b.shape[0], cp, gp, b.mem, b.stream))
    return (cost, grad) if want_grad else cost


def ik_descend(cst, q, target, pose_link, steps: int = 50, lr: float = 0.05, clamp: bool = True, history: bool = False,
               **weights):
    """`steps` gradient-descent steps per problem in one kernel launch.  Returns (q_final,
    final cost[, cost history (B, steps)]); q itself is not modified."""
    b = Batch(q, np.float32)
    if len(b.shape) != 2 or b.shape[1] != cst.q_dim():
        raise ValueError(f"q must be (B, {cst.q_dim()}), got {b.shape}")
    qo, qp = b.empty(b.shape, np.float32)
    if b.mem == 1:
        qo.copy_(b.keep)
    else:
        qo[...] = b.keep
    tb, tp = _pair(b, target)
    p, keep = make_params(cst, pose_link=pose_link, **weights)
    cost, cp = b.empty((b.shape[0],), np.float32)
    hist, hp = b.empty((b.shape[0], steps), np.float32) if history else (None, None)
    check(lib.pmgpu_ik_descend(cst._h, C.byref(p), qp, tp, b.shape[0], int(steps), float(lr), int(bool(clamp)), cp, hp, b.mem,
                               b.stream))
    del keep, tb
    return (qo, cost, hist) if history else (qo, cost)


def traj_cost_grad(cst, q, offsets, want_grad: bool = True, **weights):
    """Per-trajectory cost (n_traj,) and, if want_grad, the gradient (n_waypoints, q_dim) of
    trajectories stored back to back in q (n_waypoints, q_dim) with int64 offsets (n_traj + 1)."""
    b = Batch(q, np.float32)
    if len(b.shape) != 2 or b.shape[1] != cst.q_dim():
        raise ValueError(f"q must be (n_waypoints, {cst.q_dim()}), got {b.shape}")
    ob = Batch(offsets, np.int64)
    if ob.mem != b.mem:
        raise ValueError("q and offsets must both be host arrays or both CUDA tensors")
    n_traj = ob.shape[0] - 1
    if n_traj < 0:
        raise ValueError("offsets needs n_traj + 1 entries")
    p, keep = make_params(cst, margin=weights.pop("margin", 0.03), **weights)
    cost, cp = b.empty((n_traj,), np.float32)
    grad, gp = b.empty(b.shape, np.float32) if want_grad else (None, None)
    check(lib.pmgpu_traj_cost(cst._h, C.byref(p), b.ptr, ob.ptr, n_traj, b.shape[0], cp, gp, b.mem, b.stream))
    del keep, ob
    return (cost, grad) if want_grad else cost


def link_poses(cst, q, link: Union[int, str]):
    """FP64 world poses (B, 7) [x y z qx qy qz qw] of one link (sin/cos FK)."""
    b = Batch(q, np.float64)
    out, op = b.empty((b.shape[0], 7), np.float64)
    check(lib.pmgpu_cst_link_poses(cst._h, _link_id(cst, link), b.ptr, b.shape[0], op, b.mem, b.stream))
    return out


def _torch():
    import torch

    return torch


class IKCost:
    """torch.autograd.Function: cost (B,) of q (B, q_dim) against targets (B, 7)."""

    _fn = None

    @classmethod
    def apply(cls, q, target, cst, pose_link, weights):
        if cls._fn is None:
            torch = _torch()

            class _F(torch.autograd.Function):
                @staticmethod
                def forward(ctx, q, target, cst, pose_link, weights):
                    ctx.cst, ctx.pose_link, ctx.weights = cst, pose_link, weights
                    ctx.save_for_backward(q, target)
                    return ik_cost_grad(cst, q, target, pose_link, want_grad=False, **weights)

                @staticmethod
                def backward(ctx, g):
                    q, target = ctx.saved_tensors
                    _, grad = ik_cost_grad(ctx.cst, q, target, ctx.pose_link, want_grad=True, **ctx.weights)
                    return (g[:, None] * grad).to(q.dtype), None, None, None, None

            cls._fn = _F
        return cls._fn.apply(q, target, cst, pose_link, weights)


class TrajectoryCost:
    """torch.autograd.Function: per-trajectory cost (n_traj,) of back-to-back waypoints q
    (n_waypoints, q_dim) with offsets (n_traj + 1); FK is recomputed in the backward pass."""

    _fn = None

    @classmethod
    def apply(cls, q, offsets, cst, weights):
        if cls._fn is None:
            torch = _torch()

            class _F(torch.autograd.Function):
                @staticmethod
                def forward(ctx, q, offsets, cst, weights):
                    ctx.cst, ctx.weights = cst, weights
                    ctx.save_for_backward(q, offsets)
                    return traj_cost_grad(cst, q, offsets, want_grad=False, **dict(weights))

                @staticmethod
                def backward(ctx, g):
                    q, offsets = ctx.saved_tensors
                    _, grad = traj_cost_grad(ctx.cst, q, offsets, want_grad=True, **dict(ctx.weights))
                    # d cost_i / d q_u for u in trajectory i: scale each waypoint row by g[i]
                    counts = offsets[1:] - offsets[:-1]
                    scale = torch.repeat_interleave(g, counts, output_size=q.shape[0])
                    return (scale[:, None] * grad).to(q.dtype), None, None, None

            cls._fn = _F
        return cls._fn.apply(q, offsets, cst, weights)


def ik_cost(cst, q, target, pose_link, **weights):
    """Differentiable IK cost (B,) of CUDA tensors q (B, q_dim) and target (B, 7)."""
    return IKCost.apply(q, target, cst, pose_link, weights)


def trajectory_cost(cst, q, offsets, **weights):
    """Differentiable per-trajectory cost (n_traj,) of CUDA tensors q (n_waypoints, q_dim) and
    offsets (n_traj + 1, int64)."""
    return TrajectoryCost.apply(q, offsets, cst, weights)
