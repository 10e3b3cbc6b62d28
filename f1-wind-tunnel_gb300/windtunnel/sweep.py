"""Aero-map sweep: the case list and its split over ranks.

The reference sweeps front x rear ride height (src/ui/aeromap.ts:15-16) in
serpentine order (aeromap.ts:79-84), re-voxelizing per point and letting the
flow settle before averaging (aeromap.ts:86-100).  Here every point is its own
lattice; cases are independent, so several GPUs run disjoint subsets of them
with no data exchange (replicas).  Only the timing is reduced across ranks.
"""
from dataclasses import dataclass

FRONT_MM = (10.0, 22.5, 35.0, 47.5, 60.0)
REAR_MM = (10.0, 22.5, 35.0, 47.5, 60.0)
# aeromap.ts:15-16 grid of the reference UI (metres)
REFERENCE_FRONT = (0.08, 0.11, 0.14, 0.17, 0.2)
REFERENCE_REAR = (0.1, 0.14, 0.18, 0.22, 0.26)


@dataclass(frozen=True)
class SweepPoint:
    index: int   # position in the serpentine order
    i: int       # front index
    j: int       # rear index
    front: float  # ride height, metres
    rear: float


def serpentine(nf, nr):
    """aeromap.ts:79-84: rows in order, every odd row's columns reversed."""
    order = []
    for i in range(nf):
        cols = list(range(nr))
        if i % 2:
            cols.reverse()
        order.extend((i, j) for j in cols)
    return order


def aero_map_points(front_mm=FRONT_MM, rear_mm=REAR_MM):
    return [SweepPoint(k, i, j, front_mm[i] / 1000.0, rear_mm[j] / 1000.0)
            for k, (i, j) in enumerate(serpentine(len(front_mm), len(rear_mm)))]


def shard(points, rank, world):
    """Round-robin split of the cases over ranks (balanced to within one case)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad rank/world")
    return [p for p in points if p.index % world == rank]
