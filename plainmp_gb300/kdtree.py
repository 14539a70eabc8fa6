"""Mirror of plainmp.kdtree: KDTree(points) with query(p) and sqdist(p) (bindings/kdtree.cpp:20-23).

The reference builds a 3-d tree on the CPU (collision/kdtree.cpp:20-96).  Here the same points go
into the device cloud grid of a CloudSDF of radius 0, and every query is that grid's exact FP64
nearest search, the one the cloud SDF uses.  query / sqdist take one point, as the reference's do
(each is a device batch of one); query_batch / sqdist_batch take (N, 3) arrays or CUDA tensors.
"""
from __future__ import annotations

import numpy as np

from .psdf import CloudSDF

# KDTree::sqdist of an empty tree: the initial best squared distance, never improved
# (kdtree.cpp:33-38)
_EMPTY_SQDIST = float(np.finfo(np.float64).max)


def _one(p) -> np.ndarray:
    q = np.asarray(p, dtype=np.float64)
    if q.shape != (3,):
        raise ValueError(f"a query is one 3-vector, got shape {q.shape}")
    return q.reshape(1, 3)


class KDTree:
    """Nearest point of a fixed point set (kdtree.cpp:20-38)."""

    def __init__(self, points) -> None:
        p = np.asarray(points, dtype=np.float64)
        if p.size == 0:
            p = p.reshape(0, 3)
        if p.ndim != 2 or p.shape[1] != 3:
            raise ValueError("points must be (N, 3)")
        self._n = p.shape[0]
        self._cloud = CloudSDF(p, 0.0)

    def __len__(self) -> int:
        return self._n

    def query(self, p) -> np.ndarray:
        """The point of the set nearest to p (KDTree::query, kdtree.cpp:26-31); NaN for an empty set."""
        q = _one(p)
        if self._n == 0:
            return np.full(3, np.nan)
        return self._cloud.nearest(q)[1][0]

    def sqdist(self, p) -> float:
        """Squared distance from p to the nearest point (KDTree::sqdist, kdtree.cpp:33-38); the
        largest double for an empty set, as the reference returns."""
        q = _one(p)
        if self._n == 0:
            return _EMPTY_SQDIST
        return float(self._cloud.nearest(q)[0][0])

    def query_batch(self, points):
        """query for N points at once: (N, 3) nearest points, in the memory space of `points`."""
        return self._cloud.nearest(points)[1]

    def sqdist_batch(self, points):
        """sqdist for N points at once: (N,) squared distances, in the memory space of `points`."""
        return self._cloud.nearest(points)[0]
