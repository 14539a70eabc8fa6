"""Motion validators mirroring plainmp's OMPL validators (cpp/plainmp/ompl/motion_validator.hpp:22-63):
``BoxMotionValidator(width)`` and ``EuclideanMotionValidator(resolution)``, both answering
``checkMotion(s1, s2)`` against an inequality constraint.  ``check_motion_batch`` is the
device hot path over E edges."""
from __future__ import annotations

import ctypes as C
from typing import Sequence

import numpy as np

from ._lib import Batch, check, f64, lib
from .constraint import IneqCompositeCst, SphereCollisionCst

BOX = 0
EUCLIDEAN = 1


class _ValidatorBase:
    """cst: a SphereCollisionCst, or an IneqCompositeCst of one SphereCollisionCst and
    LinkPositionBoundCst members (the composite is checked at every waypoint by the fast path)."""

    kind = BOX

    def __init__(self, cst) -> None:
        self.cst = cst
        self._parts = None
        if isinstance(cst, IneqCompositeCst):
            self._parts = cst.fused_parts()
            if self._parts is None:
                raise TypeError("a composite validator needs one SphereCollisionCst and LinkPositionBoundCst members")
        elif not isinstance(cst, SphereCollisionCst):
            raise TypeError(f"expected SphereCollisionCst or IneqCompositeCst, got {type(cst).__name__}")
        self._width = np.zeros(cst.q_dim())
        self._res = 0.0
        self._dev_width = {}  # device -> width tensor, made once so device calls copy nothing from the host

    def _width_arg(self, b: Batch) -> Batch:
        if b.mem == 0:
            return Batch(self._width)
        dev = b.keep.device
        if dev not in self._dev_width:
            self._dev_width[dev] = _to_device_like(self._width, b)
        return Batch(self._dev_width[dev])

    def _edges(self, S1, S2):
        b1, b2 = Batch(S1), Batch(S2)
        d = self.cst.q_dim()
        if b1.shape != b2.shape or len(b1.shape) != 2 or b1.shape[1] != d:
            raise ValueError(f"s1 and s2 must both be (E, {d})")
        if b1.mem != b2.mem:
            raise ValueError("s1 and s2 must live in the same memory space")
        return b1, b2

    def check_motion_batch(self, S1, S2, return_count: bool = False):
        """Plain FP64 method, one device thread per edge: (E,) uint8."""
        if self._parts is not None:
            raise TypeError("the plain edge method takes a SphereCollisionCst; a composite goes through check_motion_fast")
        b1, b2 = self._edges(S1, S2)
        E = b1.shape[0]
        out, optr = b1.empty((E,), np.uint8)
        w = self._width_arg(b1)
        cnt = C.c_int64(0)
        check(lib.pmgpu_check_motion(self.cst._h, b1.ptr, b2.ptr, E, self.kind, w.ptr, float(self._res), optr, C.byref(cnt), b1.mem,
                                     b1.stream))
        return (out, int(cnt.value)) if return_count else out

    def check_motion_fast(self, S1, S2, stats: bool = False, out=None):
        """FP32 + FP64-recheck persistent work-queue path: (E,) uint8 identical to the plain method.
        With CUDA tensors and stats=False the call only enqueues work on torch's current stream
        (no host synchronisation, no host copies), so it can be captured in a CUDA graph after one
        warm-up call; `out` may be a preallocated (E,) uint8 buffer in the same memory space."""
        b1, b2 = self._edges(S1, S2)
        E = b1.shape[0]
        if out is not None:
            optr = b1.out(out, (b1.shape[0],), np.uint8)
        else:
            out, optr = b1.empty((E,), np.uint8)
        w = self._width_arg(b1)
        st = np.zeros(4, dtype=np.int64)
        sp = C.c_void_p(st.ctypes.data) if stats else None
        if self._parts is None:
            check(lib.pmgpu_check_motion_fast(self.cst._h, b1.ptr, b2.ptr, E, self.kind, w.ptr, float(self._res), optr, sp, b1.mem,
                                              b1.stream))
        else:
            sph, bnd = self._parts
            hs = (C.c_void_p * max(len(bnd), 1))(*[c._h for c in bnd])
            check(lib.pmgpu_composite_check_motion_fast(sph._h, hs, len(bnd), b1.ptr, b2.ptr, E, self.kind, w.ptr, float(self._res),
                                                        optr, sp, b1.mem, b1.stream))
        if stats:
            return out, {"waypoints": int(st[0]), "rechecked_terms": int(st[1]), "edges": int(st[2])}
        return out

    def shortcut(self, points, fast: bool = True):
        """Shortcut a path with all candidate edges checked in one batch.

        The reference shortcuts through OMPL's randomised PathSimplifier::partialShortcutPath
        (ompl/ompl_thin_wrap.hpp:130-170), one checkMotion per candidate.  Here every pair (i, j),
        j > i + 1, of the path's waypoints is a candidate edge; all are checked at once
        (check_motion_fast, or the plain method), and the returned path is the shortest (sum of
        Euclidean segment lengths) through valid candidates and the original segments, found by
        a forward pass over the waypoints.  Deterministic; the endpoints are kept.  points: (n, q_dim)."""
        P = f64(points)
        n = P.shape[0]
        if P.ndim != 2 or P.shape[1] != self.cst.q_dim():
            raise ValueError(f"points must be (n, {self.cst.q_dim()})")
        if n <= 2:
            return P.copy()
        ii, jj = np.triu_indices(n, k=2)
        ok = self.check_motion_fast(P[ii], P[jj]) if fast else self.check_motion_batch(P[ii], P[jj])
        ok = np.asarray(ok.cpu() if hasattr(ok, "cpu") else ok).astype(bool)
        best = np.full(n, np.inf)
        prev = np.full(n, -1)
        best[0] = 0.0
        seg = np.linalg.norm(P[1:] - P[:-1], axis=1)
        by_end = {}
        for a, b, v in zip(ii, jj, ok):
            if v:
                by_end.setdefault(int(b), []).append(int(a))
        for j in range(1, n):
            best[j], prev[j] = best[j - 1] + seg[j - 1], j - 1
            for i in by_end.get(j, []):
                c = best[i] + float(np.linalg.norm(P[j] - P[i]))
                if c < best[j]:
                    best[j], prev[j] = c, i
        idx = [n - 1]
        while idx[-1] != 0:
            idx.append(int(prev[idx[-1]]))
        return P[idx[::-1]].copy()

    def checkMotion(self, s1, s2) -> bool:  # noqa: N802 (OMPL's name)
        d = self.cst.q_dim()
        if self._parts is not None:
            return bool(self.check_motion_fast(f64(s1, (1, d)), f64(s2, (1, d)))[0])
        return bool(self.check_motion_batch(f64(s1, (1, d)), f64(s2, (1, d)))[0])


def _to_device_like(arr: np.ndarray, b: Batch):
    return b.torch.as_tensor(arr, dtype=b.torch.float64, device=b.keep.device)


class BoxMotionValidator(_ValidatorBase):
    kind = BOX

    def __init__(self, cst: SphereCollisionCst, width: Sequence[float]) -> None:
        super().__init__(cst)
        w = f64(width).reshape(-1)
        if w.shape[0] != cst.q_dim():
            raise RuntimeError("box dimension and space dimension mismatch")
        self._width = w


class EuclideanMotionValidator(_ValidatorBase):
    kind = EUCLIDEAN

    def __init__(self, cst: SphereCollisionCst, resolution: float) -> None:
        super().__init__(cst)
        self._res = float(resolution)
