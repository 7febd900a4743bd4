"""Spatial queries on a world's published state (QueryIndex.swift of the reference's runtime): objects containing a
point, intersecting a rectangle or a circle, and the first hit of a segment. Bodies are tested exactly (polygon,
circle, capsule); a bubble is a circle of its effective radius (its exact contour is the hit test's business); sensors
and force fields take no part. Collective answers come in ascending unsigned id order, and a query filter acts like an
object's collision filter (the answer is what such an object would collide with; None narrows nothing).

This is host code over host state, as in the reference: a uniform grid over the objects' boxes, cell size the median
box extent, objects spanning 16 or more cells in one axis on a separate list checked by every query, and a full scan
for queries covering more than 4096 cells. Arithmetic is float32, the reference's Float."""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

F = np.float32
SCAN_LIMIT = 4096
LARGE_SPAN = 16


@dataclass(frozen=True)
class RaycastHit:
    object_id: int
    point: tuple
    normal: tuple        # unit, pointing out of the object; the reversed ray when the segment starts inside
    fraction: float      # along the segment from start (0) to end (1)


def _pt(p):
    return np.array([F(p[0]), F(p[1])], np.float32)


def _length(v):
    return F(math.sqrt(float(F(v[0] * v[0] + v[1] * v[1]))))


def distance_to_segment(p, a, b):
    e = b - a
    sq = F(e[0] * e[0] + e[1] * e[1])
    t = max(F(0), min(F(1), F(F((p[0] - a[0]) * e[0]) + F((p[1] - a[1]) * e[1])) / sq)) if sq > 0 else F(0)
    return _length(p - (a + e * t))


def polygon_contains(ring, p) -> bool:
    """Crossing parity (PlacementGeometry.polygonContains)."""
    inside = False
    j = len(ring) - 1
    for i in range(len(ring)):
        a, b = ring[i], ring[j]
        if (a[1] > p[1]) != (b[1] > p[1]) and p[0] <= (b[0] - a[0]) * (p[1] - a[1]) / (b[1] - a[1]) + a[0]:
            inside = not inside
        j = i
    return inside


def contains(shape, p) -> bool:
    """PlacementGeometry.contains: circle and capsule by distance (boundary inside), polygon by parity."""
    if shape[0] == "circle":
        d = p - shape[1]
        return bool(F(d[0] * d[0] + d[1] * d[1]) <= shape[2] * shape[2])
    if shape[0] == "capsule":
        return bool(distance_to_segment(p, shape[1], shape[2]) <= shape[3])
    return polygon_contains(shape[1], p)


def shape_box(shape):
    """The axis-aligned box (low, high) of a shape."""
    if shape[0] == "circle":
        r = shape[2]
        return shape[1] - r, shape[1] + r
    if shape[0] == "capsule":
        a, b, r = shape[1], shape[2], shape[3]
        return np.minimum(a, b) - r, np.maximum(a, b) + r
    ring = np.array(shape[1], np.float32)
    return ring.min(axis=0), ring.max(axis=0)


def _segments_intersect(a, b, c, d) -> bool:
    def cross(p, q, r):
        return F(F((q[0] - p[0]) * (r[1] - p[1])) - F((q[1] - p[1]) * (r[0] - p[0])))

    def on(p, q, r):
        return min(p[0], q[0]) <= r[0] <= max(p[0], q[0]) and min(p[1], q[1]) <= r[1] <= max(p[1], q[1])
    d1, d2, d3, d4 = cross(a, b, c), cross(a, b, d), cross(c, d, a), cross(c, d, b)
    if ((d1 > 0 > d2) or (d1 < 0 < d2)) and ((d3 > 0 > d4) or (d3 < 0 < d4)):
        return True
    return (d1 == 0 and on(a, b, c)) or (d2 == 0 and on(a, b, d)) or (d3 == 0 and on(c, d, a)) or \
        (d4 == 0 and on(c, d, b))


def _segment_distance(a, b, c, d):
    if _segments_intersect(a, b, c, d):
        return F(0)
    return min(distance_to_segment(a, c, d), distance_to_segment(b, c, d), distance_to_segment(c, a, b),
               distance_to_segment(d, a, b))


def _in_rect(lo, hi, p) -> bool:
    return lo[0] <= p[0] <= hi[0] and lo[1] <= p[1] <= hi[1]


def _intersects_rect(shape, lo, hi) -> bool:
    corners = [lo, _pt((hi[0], lo[1])), hi, _pt((lo[0], hi[1]))]
    if shape[0] == "circle":
        return bool(_length(shape[1] - np.minimum(np.maximum(shape[1], lo), hi)) <= shape[2])
    if shape[0] == "capsule":
        a, b, r = shape[1], shape[2], shape[3]
        if _in_rect(lo, hi, a) or _in_rect(lo, hi, b):
            return True
        return any(_segment_distance(a, b, corners[k], corners[(k + 1) % 4]) <= r for k in range(4))
    ring = shape[1]
    if any(_in_rect(lo, hi, v) for v in ring) or any(polygon_contains(ring, c) for c in corners):
        return True
    return any(_segments_intersect(ring[i], ring[(i + 1) % len(ring)], corners[k], corners[(k + 1) % 4])
               for i in range(len(ring)) for k in range(4))


def _intersects_circle(shape, center, radius) -> bool:
    if shape[0] == "circle":
        reach = radius + shape[2]
        d = center - shape[1]
        return bool(F(d[0] * d[0] + d[1] * d[1]) <= reach * reach)
    if shape[0] == "capsule":
        return bool(distance_to_segment(center, shape[1], shape[2]) <= radius + shape[3])
    ring = shape[1]
    if polygon_contains(ring, center):
        return True
    return any(distance_to_segment(center, ring[i], ring[(i + 1) % len(ring)]) <= radius for i in range(len(ring)))


def _ray_circle(start, direction, center, radius):
    """Entry of the ray into a circle from outside."""
    offset = start - center
    a = F(direction[0] * direction[0] + direction[1] * direction[1])
    if not a > 0:
        return None
    b = F(offset[0] * direction[0] + offset[1] * direction[1])
    c = F(F(offset[0] * offset[0] + offset[1] * offset[1]) - radius * radius)
    disc = F(b * b - a * c)
    if not disc >= 0:
        return None
    t = F((-b - F(math.sqrt(float(disc)))) / a)
    if not (0 <= t <= 1):
        return None
    point = offset + direction * t
    length = _length(point)
    return t, (point / length if length > 0 else np.zeros(2, np.float32))


def _ray_segment(start, direction, a, b, outward=None):
    edge = b - a
    den = F(direction[0] * edge[1] - direction[1] * edge[0])
    if den == 0:
        return None
    delta = a - start
    t = F(F(delta[0] * edge[1] - delta[1] * edge[0]) / den)
    u = F(F(delta[0] * direction[1] - delta[1] * direction[0]) / den)
    if not (0 <= t <= 1 and 0 <= u <= 1):
        return None
    normal = outward if outward is not None else _pt((-edge[1], edge[0]))
    length = _length(normal)
    if not length > 0:
        return None
    normal = normal / length
    if outward is None and F(normal[0] * direction[0] + normal[1] * direction[1]) > 0:
        normal = -normal
    return t, normal


def _ray_shape(shape, start, direction):
    best = None

    def consider(hit):
        nonlocal best
        if hit is not None and (best is None or hit[0] < best[0]):
            best = hit
    if shape[0] == "circle":
        return _ray_circle(start, direction, shape[1], shape[2])
    if shape[0] == "capsule":
        a, b, r = shape[1], shape[2], shape[3]
        consider(_ray_circle(start, direction, a, r))
        consider(_ray_circle(start, direction, b, r))
        axis = b - a
        length = _length(axis)
        if not length > 0:
            return best
        side = _pt((-axis[1], axis[0])) / length * r
        for sign in (F(1), F(-1)):
            consider(_ray_segment(start, direction, a + side * sign, b + side * sign, side * sign))
        return best
    ring = shape[1]
    for i in range(len(ring)):
        consider(_ray_segment(start, direction, ring[i], ring[(i + 1) % len(ring)]))
    return best


def _segment_may_touch(start, direction, lo, hi) -> bool:
    """Slab test of the segment against a box."""
    near, far = F(0), F(1)
    for axis in range(2):
        if direction[axis] == 0:
            if start[axis] < lo[axis] or start[axis] > hi[axis]:
                return False
        else:
            t1, t2 = F((lo[axis] - start[axis]) / direction[axis]), F((hi[axis] - start[axis]) / direction[axis])
            if t1 > t2:
                t1, t2 = t2, t1
            near, far = max(near, t1), min(far, t2)
            if near > far:
                return False
    return True


class QueryIndex:
    """Queries over one published state. `objects` are (id, CollisionFilter, shape) with shapes as
    ("circle", centre, r), ("capsule", a, b, r) or ("polygon", ring) in world coordinates (float32)."""

    def __init__(self, objects):
        built = []
        for oid, filt, shape in objects:
            lo, hi = shape_box(shape)
            built.append((int(oid), filt, shape, lo, hi))
        built.sort(key=lambda e: e[0] & 0xFFFFFFFFFFFFFFFF)
        self.entries = built
        extents = sorted(float(max(hi[0] - lo[0], hi[1] - lo[1])) for _, _, _, lo, hi in built)
        median = extents[len(extents) // 2] if extents else 1.0
        self.cell_size = F(median) if math.isfinite(median) and median > 1e-3 else F(1)
        self.cells: dict = {}
        self.large: list = []
        for index, (_, _, _, lo, hi) in enumerate(built):
            (x0, y0), (x1, y1) = self._cell(lo), self._cell(hi)
            if x1 - x0 >= LARGE_SPAN or y1 - y0 >= LARGE_SPAN:
                self.large.append(index)
                continue
            for x in range(x0, x1 + 1):
                for y in range(y0, y1 + 1):
                    self.cells.setdefault((x, y), []).append(index)

    def _cell(self, p):
        def one(v):
            scaled = math.floor(float(F(v / self.cell_size))) if math.isfinite(float(v)) else 0
            return int(max(-1_000_000, min(1_000_000, scaled)))
        return one(p[0]), one(p[1])

    def _candidates(self, lo, hi) -> list:
        (x0, y0), (x1, y1) = self._cell(lo), self._cell(hi)
        if (x1 - x0 + 1) * (y1 - y0 + 1) > SCAN_LIMIT:
            return list(range(len(self.entries)))
        found = set(self.large)
        for x in range(x0, x1 + 1):
            for y in range(y0, y1 + 1):
                found.update(self.cells.get((x, y), ()))
        return sorted(found)

    @staticmethod
    def _accepts(entry, filt) -> bool:
        return filt is None or filt.accepts(entry[1])

    def objects_at(self, point, filt=None) -> list:
        if not (math.isfinite(point[0]) and math.isfinite(point[1])):
            return []
        p = _pt(point)
        return [self.entries[i][0] for i in self._candidates(p, p)
                if self._accepts(self.entries[i], filt) and contains(self.entries[i][2], p)]

    def objects_in_rect(self, lo, hi, filt=None) -> list:
        lo, hi = _pt(lo), _pt(hi)
        return [self.entries[i][0] for i in self._candidates(lo, hi)
                if self._accepts(self.entries[i], filt) and _intersects_rect(self.entries[i][2], lo, hi)]

    def objects_in_circle(self, center, radius, filt=None) -> list:
        if not (math.isfinite(center[0]) and math.isfinite(center[1]) and math.isfinite(radius) and radius >= 0):
            return []
        c, r = _pt(center), F(radius)
        return [self.entries[i][0] for i in self._candidates(c - r, c + r)
                if self._accepts(self.entries[i], filt) and _intersects_circle(self.entries[i][2], c, r)]

    def raycast(self, start, end, filt=None) -> RaycastHit | None:
        """First hit along start -> end; a segment starting inside an object hits it at fraction 0; ties go to the
        smaller id."""
        if not all(math.isfinite(v) for v in (*start, *end)):
            return None
        s, e = _pt(start), _pt(end)
        direction = e - s
        best = None
        for i in self._candidates(np.minimum(s, e), np.maximum(s, e)):
            entry = self.entries[i]
            if not self._accepts(entry, filt) or not _segment_may_touch(s, direction, entry[3], entry[4]):
                continue
            if contains(entry[2], s):
                length = _length(direction)
                hit = (F(0), -direction / length if length > 0 else np.zeros(2, np.float32))
            else:
                hit = _ray_shape(entry[2], s, direction)
            if hit is not None and (best is None or hit[0] < best[1]):
                best = (i, hit[0], hit[1])
        if best is None:
            return None
        i, t, normal = best
        point = s + direction * t
        return RaycastHit(self.entries[i][0], (float(point[0]), float(point[1])), (float(normal[0]), float(normal[1])),
                          float(t))
