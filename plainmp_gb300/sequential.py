"""SequentialCst (constraints/sequential_constraint.cpp:14-151; bindings/constraint.cpp:114-125):
constraints over a trajectory x = [q_0, ..., q_{T-1}] for the SQP smoother, with the values and
the sparse Jacobian of SequentialCst::evaluate.

Each constraint object attached to several time steps is evaluated once, as one device batch
over those waypoints (``evaluate_batch``), instead of once per waypoint; the rows are then laid
out as the reference lays them out:

* per time step t with constraints, in insertion order, the constraint's rows; the Jacobian block
  sits at the columns of the waypoint that step reads, every entry + 1e-12 (the reference's way of
  keeping the sparsity pattern);
* the fixed points (rows x_t - q_fixed, identity blocks);
* the motion-step box rows q_t - q_{t+1} + w and q_{t+1} - q_t + w.

The reference reads step t's waypoint at an offset that advances only over steps that carry
constraints (sequential_constraint.cpp:63-96: ``x_head`` is not advanced on ``continue``), so once
``finalize`` has cleared the constraints of fixed-point steps, later steps read earlier waypoints.
That offset is reproduced as-is; the fixed-point and box rows use t * q_dim.
"""
from __future__ import annotations

from typing import List, Optional

import numpy as np


class SequentialCst:
    def __init__(self, T: int, q_dim: int):
        self.T = int(T)
        self.q_dim_ = int(q_dim)
        self._seq: List[list] = [[] for _ in range(self.T)]
        self._fixed: List[Optional[np.ndarray]] = [None] * self.T
        self._msbox: Optional[np.ndarray] = None
        self._cst_dim = 0
        self._finalized = False

    # ---- construction (sequential_constraint.cpp:14-61)
    def add_globally(self, constraint) -> None:
        for t in range(self.T):
            self.add_at(constraint, t)

    def add_at(self, constraint, t: int) -> None:
        if t >= self.T or t < 0:
            raise RuntimeError("t is out of range")
        self._finalized = False
        self._seq[t].append(constraint)
        self._cst_dim += constraint.cst_dim()

    def add_fixed_point_at(self, q, t: int) -> None:
        if t >= self.T or t < 0:
            raise RuntimeError("t is out of range")
        self._fixed[t] = np.asarray(q, dtype=np.float64).reshape(-1).copy()
        self._cst_dim += self._fixed[t].shape[0]

    def add_motion_step_box_constraint(self, box_width) -> None:
        w = np.asarray(box_width, dtype=np.float64).reshape(-1)
        self._cst_dim += w.shape[0] * 2 * max(self.T - 1, 0)
        self._msbox = w.copy()

    def finalize(self) -> None:
        for t in range(self.T):
            if self._fixed[t] is not None:
                self._cst_dim -= sum(c.cst_dim() for c in self._seq[t])
                self._seq[t] = []
        self._finalized = True

    def x_dim(self) -> int:
        return self.T * self.q_dim_

    def cst_dim(self) -> int:
        return self._cst_dim

    # ---- evaluation (sequential_constraint.cpp:63-127)
    def evaluate(self, x):
        """(c (cst_dim,), jac (cst_dim, x_dim) scipy.sparse.csc_matrix) for x (x_dim,)."""
        import scipy.sparse as sp

        x = np.ascontiguousarray(np.asarray(x, dtype=np.float64).reshape(-1))
        if x.shape[0] != self.x_dim():
            raise ValueError(f"x must have {self.x_dim()} entries")
        d = self.q_dim_
        X = x.reshape(self.T, d)
        # the waypoint each constrained step reads, and its row offset
        plan = []  # (t, x_head, [(constraint, c_head)])
        x_head = c_head = 0
        for t in range(self.T):
            if not self._seq[t]:
                continue
            items = []
            for c in self._seq[t]:
                items.append((c, c_head))
                c_head += c.cst_dim()
            plan.append((x_head, items))
            x_head += d
        # one batch per distinct constraint over the waypoints it is evaluated at
        jobs = {}
        for xh, items in plan:
            for c, ch in items:
                jobs.setdefault(id(c), (c, []))[1].append((xh, ch))
        c_vec = np.zeros(self.cst_dim())
        rows, cols, vals = [], [], []
        for c, uses in jobs.values():
            xh = np.array([u[0] for u in uses])
            ch = np.array([u[1] for u in uses])
            Q = x[(xh[:, None] + np.arange(d)[None, :])]
            v, J = c.evaluate_batch(Q)
            v, J = _np(v), _np(J)
            m = v.shape[1]
            c_vec[(ch[:, None] + np.arange(m)[None, :]).reshape(-1)] = v.reshape(-1)
            r = ch[:, None, None] + np.arange(m)[None, :, None]
            k = xh[:, None, None] + np.arange(d)[None, None, :]
            rows.append(np.broadcast_to(r, J.shape).reshape(-1))
            cols.append(np.broadcast_to(k, J.shape).reshape(-1))
            vals.append((J + 1e-12).reshape(-1))
        head = c_head
        for t in range(self.T):
            if self._fixed[t] is not None:
                c_vec[head:head + d] = X[t] - self._fixed[t]
                rows.append(np.arange(head, head + d))
                cols.append(t * d + np.arange(d))
                vals.append(np.ones(d))
                head += d
        if self._msbox is not None:
            w = self._msbox
            for t in range(self.T - 1):
                q1, q2 = X[t], X[t + 1]
                c_vec[head:head + d] = q1 - q2 + w
                c_vec[head + d:head + 2 * d] = q2 - q1 + w
                i = np.arange(d)
                rows += [head + i, head + i, head + d + i, head + d + i]
                cols += [t * d + i, (t + 1) * d + i, t * d + i, (t + 1) * d + i]
                vals += [np.ones(d), -np.ones(d), -np.ones(d), np.ones(d)]
                head += 2 * d
        if rows:
            R, Cc, V = np.concatenate(rows), np.concatenate(cols), np.concatenate(vals)
        else:
            R = Cc = np.zeros(0, dtype=np.int64)
            V = np.zeros(0)
        jac = sp.csc_matrix((V, (R, Cc)), shape=(self.cst_dim(), self.x_dim()))
        return c_vec, jac

    def __str__(self) -> str:
        lines = ["Sequential constraint:", f"total dim: {self.cst_dim()}"]
        for t in range(self.T):
            lines.append(f"  - time {t}")
            for c in self._seq[t]:
                lines.append(f"    - {type(c).__name__}: {c.cst_dim()}")
            if self._fixed[t] is not None:
                lines.append(f"    - fixed point: {self.q_dim_}")
        if self._msbox is not None:
            lines.append(f"  - motion step box constraint  : {self.q_dim_ * 2 * (self.T - 1)}")
        return "\n".join(lines) + "\n"


def _np(a):
    if type(a).__module__.startswith("torch"):
        return a.detach().cpu().numpy()
    return np.asarray(a)
