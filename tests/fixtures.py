"""Small worlds restating the reference's own test scenes (the scene, not recorded outputs):
 - broadphase equality scene (NativeMetalBroadPhaseTests.swift:9-35): 35 bubbles at spacings 0.2 / 1.9 / 7, radii
   1.5 / 0.5, ids -17..16 and Int.max, contact stiffness 0 so nothing moves;
 - dense truncation scene (:55-85): 128 + 12 bubbles on an 8-column grid of spacing 0.1, radius 1;
 - segment candidate scene (:87-110);
 - bounce against a one-sided wall (NativeMetalSubstepKernelTests.swift:884-916), pair bounce (:957-979),
   constant force with damping (:793-814), static press (ContactLawReferenceTests.swift:129).
"""
from __future__ import annotations

import numpy as np

from bubblephysics_gb300 import _native as N
from bubblephysics_gb300.scenes import polygon_edges
from bubblephysics_gb300.spec import WorldSpec, make_bubbles

INT64_MAX = 2**63 - 1
INT64_MIN = -(2**63)


def broadphase_scene(spacing: float) -> WorldSpec:
    ids, centers, radii = [], [], []
    for i in range(35):
        ids.append(INT64_MAX if i == 34 else i - 17)
        centers.append(((i % 7 - 3) * spacing, (i // 7 - 2) * spacing))
        radii.append(1.5 if i % 3 == 0 else 0.5)
    order = np.argsort(np.array(ids, dtype=np.int64), kind="stable")
    b = make_bubbles(np.array(centers)[order], np.array(radii)[order], ids=np.array(ids, np.int64)[order],
                     masses=1.0, stiffness=0.0)
    return WorldSpec(bubbles=b)


def broadphase_expected(spec: WorldSpec):
    """Brute-force pair keys with reach 1.25 (r_a + r_b), the expectation of the reference test."""
    b = spec.bubbles
    keys = []
    for i in range(len(b)):
        for j in range(i + 1, len(b)):
            reach = np.float32(b["radius"][i]) * np.float32(1.25) + np.float32(b["radius"][j]) * np.float32(1.25)
            d = np.abs(b["center"][i] - b["center"][j])
            if d[0] <= reach and d[1] <= reach:
                keys.append((0, int(b["id"][i]), int(b["id"][j])))
    return sorted(keys)


def dense_scene(limit: int = 128) -> WorldSpec:
    count = limit + 12
    centers = [((i % 8) * 0.1, (i // 8) * 0.1) for i in range(count)]
    b = make_bubbles(np.array(centers), 1.0, ids=np.arange(1, count + 1), masses=1.0, stiffness=0.0)
    return WorldSpec(bubbles=b, candidate_limit=limit)


def segment_scene() -> WorldSpec:
    b = make_bubbles([(0.0, 0.0)], 1.0, ids=[INT64_MAX], masses=1.0, stiffness=229.0)
    segs = np.zeros(3, N.SEGMENT_DTYPE)
    segs["category"] = 1
    segs["mask"] = 0xFFFFFFFF
    segs[0]["id"] = INT64_MIN
    segs[0]["a"] = (-2, -0.5)
    segs[0]["b"] = (2, -0.5)
    segs[0]["flags"] = N.SEGMENT_ALLOWED_SIDE
    segs[0]["allowed_side"] = 1.0
    segs[1]["id"] = 10
    segs[1]["a"] = (0.9, -0.9)
    segs[1]["b"] = (2, -2)
    segs[2]["id"] = 11
    segs[2]["a"] = (10, -10)
    segs[2]["b"] = (12, -12)
    return WorldSpec(bubbles=b, segments=segs)


def floor_wall(y: float = 0.0, half_width: float = 1000.0, thickness: float = 50.0, first_id: int = 1000):
    """A static rectangle above y (its bottom edge at y faces -y), as one-sided polygon edges."""
    poly = [(-half_width, y), (half_width, y), (half_width, y + thickness), (-half_width, y + thickness)]
    return polygon_edges(poly, first_id, owner_id=900)


def bounce_scene(speed: float, start_distance: float = 80.0) -> WorldSpec:
    b = make_bubbles([(100.0, -start_distance)], 12.0, velocities=[(0.0, speed)], masses=0.36, stiffness=229.0)
    return WorldSpec(bubbles=b, segments=floor_wall())


def pair_bounce_scene() -> WorldSpec:
    b = make_bubbles([(0.0, 0.0), (60.0, 0.0)], 12.0, velocities=[(600.0, 0.0), (-400.0, 0.0)],
                     masses=[0.36, 1.5], stiffness=229.0)
    return WorldSpec(bubbles=b)


def constant_force_scene(gamma: float, step: float = 1.0 / 60) -> WorldSpec:
    b = make_bubbles([(0.0, 0.0)], 12.0, velocities=[(10.0, -4.0)], masses=0.5, stiffness=229.0, damping=gamma)
    return WorldSpec(bubbles=b, global_force=(3.0, 0.0), time_step=step)


def press_scene(force_value: float = 20000.0) -> WorldSpec:
    """Bubble r = 24, m = 1, K_c = 229 pressed against the floor wall by a constant force, starting at equilibrium."""
    from clr import equilibrium_distance
    d = equilibrium_distance(force_value, 229.0, 24.0)
    b = make_bubbles([(0.0, -d)], 24.0, masses=1.0, stiffness=229.0)
    return WorldSpec(bubbles=b, segments=floor_wall(), global_force=(0.0, force_value))
