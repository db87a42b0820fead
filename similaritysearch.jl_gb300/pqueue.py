"""Result containers (mirror of src/pqueue/knnsorted.jl and src/iddist.jl).

``KnnSorted`` is the bounded, always-sorted k-NN queue the reference's
``search`` fills.  The GPU computes whole result lists; ``search(idx, ctx, q,
res)`` then pushes them into ``res`` in (distance, id) order, which leaves the
queue in the state the reference's own push sequence would.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass(frozen=True)
class IdDist:
    """(id::UInt32, dist::Float32) -- src/iddist.jl:23-26"""
    id: int
    dist: float


class AbstractMetricQueue:
    """Any per-query result container (src/pqueue/pqueue.jl)."""


class AbstractKnnQueue(AbstractMetricQueue):
    """Fixed-k containers (KnnSorted, KnnHeap)."""


class AbstractRadiusQueue(AbstractMetricQueue):
    """Radius-bounded, growable containers (RadiusSorted, RadiusHeap)."""


class RadiusSorted(AbstractRadiusQueue):
    """Every (id, dist) with dist <= radius, kept sorted by distance
    (src/pqueue/radiussorted.jl:28-52).  A host container: the GPU index
    answers fixed-k queries only and rejects it."""

    def __init__(self, radius: float):
        self.radius = np.float32(radius)
        self.ids: list[int] = []
        self.dists: list[float] = []

    def __len__(self):
        return len(self.ids)

    def push_item(self, i: int, dist: float) -> bool:
        dist = np.float32(dist)
        if dist > self.radius:
            return False
        pos = len(self.dists)
        while pos > 0 and self.dists[pos - 1] > dist:
            pos -= 1
        self.ids.insert(pos, int(i))
        self.dists.insert(pos, float(dist))
        return True


class KnnSorted(AbstractKnnQueue):
    """Sorted bounded queue; insert after equal distances, reject d >= frontier
    when full (knnsorted.jl:68-101,140-168)."""

    def __init__(self, ids=None, dists=None, k: int | None = None):
        if ids is None:
            ids = np.zeros(k, dtype=np.uint32)
            dists = np.zeros(k, dtype=np.float32)
        self.ids = ids
        self.dists = dists
        self.sp = 0   # 0-based start of the active range
        self.ep = -1  # 0-based end (inclusive)
        self.maxlen = len(ids)

    def __len__(self):
        return self.ep - self.sp + 1

    def maxlength(self):
        return self.maxlen

    def _sort_last(self):
        ids, d, sp, ep = self.ids, self.dists, self.sp, self.ep
        if sp == ep:
            return
        iid, idist = ids[ep], d[ep]
        if d[ep - 1] <= idist:
            return
        lo, hi = sp, ep - 1
        while lo < hi:
            mid = (lo + hi) >> 1
            if d[mid] <= idist:
                lo = mid + 1
            else:
                hi = mid
        ids[lo + 1:ep + 1] = ids[lo:ep].copy()
        d[lo + 1:ep + 1] = d[lo:ep].copy()
        ids[lo], d[lo] = iid, idist

    def push_item(self, i: int, dist: float) -> bool:
        dist = np.float32(dist)
        if len(self) < self.maxlen:
            if self.ep == len(self.ids) - 1:
                n = len(self)
                self.ids[:n] = self.ids[self.sp:self.ep + 1].copy()
                self.dists[:n] = self.dists[self.sp:self.ep + 1].copy()
                self.sp, self.ep = 0, n - 1
            self.ep += 1
            self.ids[self.ep] = i
            self.dists[self.ep] = dist
            self._sort_last()
            return True
        if dist >= self.dists[self.ep]:
            return False
        self.ids[self.ep] = i
        self.dists[self.ep] = dist
        self._sort_last()
        return True

    def items(self):
        return [IdDist(int(self.ids[i]), float(self.dists[i])) for i in range(self.sp, self.ep + 1)]

    def nearest(self) -> IdDist:
        return IdDist(int(self.ids[self.sp]), float(self.dists[self.sp]))

    def frontier(self) -> IdDist:
        return IdDist(int(self.ids[self.ep]), float(self.dists[self.ep]))

    def covradius(self) -> float:
        return float("inf") if len(self) < self.maxlen else float(self.dists[self.ep])


def knnqueue(kind, ids_or_k, dists=None):
    """knnqueue(KnnSorted, k) or knnqueue(KnnSorted, ids, dists) -- pqueue.jl:229-247"""
    if kind is not KnnSorted:
        raise TypeError("only KnnSorted queues are produced by the GPU index")
    if dists is None:
        return KnnSorted(k=int(ids_or_k))
    return KnnSorted(ids_or_k, dists)
