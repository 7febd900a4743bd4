"""Spatial queries on the published state (queries.QueryIndex through world.query_index), against the reference's own
cases (QueryIndexTests.swift:17-268): exact point, rectangle and circle answers for a bubble (circle of its effective
radius), a rotated square, a circle and a vertical capsule; a polygon whose local origin is not its centroid; sorted
overlapping answers; query filters; raycasts with point, normal and fraction (capsule side and cap, starting inside,
misses, degenerate input); the empty state; and the grid against brute force on 400 bubbles with one large body."""
import math

import numpy as np
import pytest

from bubblephysics_gb300 import world as W
from bubblephysics_gb300.world import (BubbleDescriptor, Capsule, Circle, CollisionFilter, PhysicsMaterial, Polygon,
                                       RigidBodyDescriptor, SensorDescriptor, WorldTransaction)

REGION = (-100.0, -100.0, 100.0, 100.0)


def bubble(i, x, y, r=5.0, filt=CollisionFilter()):
    return BubbleDescriptor(i, (x, y), r, 1.0, "soft", filter=filt)


def box(half):
    return Polygon(((-half, -half), (half, -half), (half, half), (-half, half)))


def stage(tx):
    state, rec, ev = W.stage([(1, WorldTransaction().update_physics_material("soft", PhysicsMaterial(1e9)))],
                             W._State(), REGION)
    state, rec, ev = W.stage([(2, tx)], state, REGION)
    assert rec, ev
    return state


def scene(extra=(), circle_filter=CollisionFilter(), radii=None, state_hook=None):
    """Bubble 1 (0,0) r5; a square of half side 5 turned by pi/4 at (30,0); circle 3 r4 at (-30,0); capsule 4 at
    (0,30) with a vertical axis (half length 6, radius 2)."""
    tx = (WorldTransaction().add(bubble(1, 0, 0))
          .add(RigidBodyDescriptor(2, box(5.0), (30.0, 0.0), angle=math.pi / 4))
          .add(RigidBodyDescriptor(3, Circle(4.0), (-30.0, 0.0), filter=circle_filter))
          .add(RigidBodyDescriptor(4, Capsule(6.0, 2.0), (0.0, 30.0), angle=math.pi / 2)))
    for obj in extra:
        tx = tx.add(obj)
    state = stage(tx)
    if state_hook:
        state_hook(state)
    return W.query_index(state, radii)


def test_point_query_is_exact_for_every_shape():
    q = scene()
    cases = [((3, 3), [1]), ((4, 4), []), ((36, 0), [2]), ((34.5, 4.5), []), ((-28, 2), [3]), ((-27, 3.4), []),
             ((0, 37), [4]), ((1.9, 37.9), []), ((1.9, 28), [4]), ((0, -60), [])]
    for point, expected in cases:
        assert q.objects_at(point) == expected, point


@pytest.mark.parametrize("angle,in_arm,in_other,notch,centroid", [
    (0.0, (58, 51), (51, 58), (58, 58), (53.2, 53.2)),
    (math.pi / 2, (49, 58), (42, 51), (42, 58), (46.8, 53.2))])
def test_point_query_uses_the_local_origin_not_the_centroid(angle, in_arm, in_other, notch, centroid):
    ell = Polygon(((0, 0), (10, 0), (10, 2), (2, 2), (2, 10), (0, 10)))
    q = scene(extra=[RigidBodyDescriptor(5, ell, (50.0, 50.0), angle=angle)])
    assert q.objects_at(in_arm) == [5] and q.objects_at(in_other) == [5]
    assert q.objects_at(notch) == [] and q.objects_at(centroid) == []


def test_point_query_uses_the_effective_radius():
    q = scene(radii={1: 2.0})
    assert q.objects_at((1.5, 0)) == [1] and q.objects_at((3, 0)) == []


def test_overlapping_answers_are_sorted_by_id():
    q = scene(extra=[bubble(9, 1, 0), bubble(7, -1, 0)])
    assert q.objects_at((0, 0)) == [1, 7, 9]


def test_rectangle_query_is_exact_for_every_shape():
    q = scene()
    cases = [((4, 4), (6, 6), []), ((3, 3), (6, 6), [1]), ((5.5, -10), (6, 10), []), ((-1, -1), (1, 1), [1]),
             ((34, 4), (36, 6), []), ((29, -1), (31, 1), [2]), ((36, -1), (40, 1), [2]), ((-27, 3.4), (-25, 5), []),
             ((-27, 2.5), (-25, 5), [3]), ((1.9, 37.9), (5, 40), []), ((1, 37), (5, 40), [4]),
             ((-100, -100), (100, 100), [1, 2, 3, 4]), ((50, 50), (60, 60), [])]
    for lo, hi, expected in cases:
        assert q.objects_in_rect(lo, hi) == expected, (lo, hi)


def test_circle_query_is_exact_for_every_shape():
    q = scene()
    cases = [((8, 0), 2.9, []), ((8, 0), 3.1, [1]), ((34.5, 4.5), 1, []), ((34.5, 4.5), 2, [2]), ((30, 0), 0.5, [2]),
             ((-30, 9), 4.9, []), ((-30, 9), 5.1, [3]), ((3, 39), 2, []), ((3, 39), 2.5, [4]), ((5, 30), 2, []),
             ((3.9, 30), 2, [4]), ((0, 0), 200, [1, 2, 3, 4]), ((0, 0), -1, [])]
    for center, radius, expected in cases:
        assert q.objects_in_circle(center, radius) == expected, (center, radius)


def test_filters_narrow_every_query():
    def twin(state):  # the reference puts bubble 8 at bubble 1's centre past the stager
        other = W._Bubble(bubble(8, 0, 0, filt=CollisionFilter(2, 0b1)), np.zeros(2, np.float32), np.zeros(2, np.float32))
        state.bubbles[8] = other
    q = scene(state_hook=twin)
    probe, rejected = CollisionFilter(1, 2), CollisionFilter(4, 2)
    assert q.objects_at((0, 0)) == [1, 8] and q.objects_at((0, 0), CollisionFilter()) == [1, 8]
    assert q.objects_at((0, 0), probe) == [8] and q.objects_at((0, 0), rejected) == []
    assert q.objects_in_rect((-1, -1), (1, 1), probe) == [8] and q.objects_in_rect((-1, -1), (1, 1), rejected) == []
    assert q.objects_in_circle((0, 0), 1, probe) == [8] and q.objects_in_circle((0, 0), 1, rejected) == []
    assert q.raycast((-20, 0), (20, 0), probe).object_id == 8 and q.raycast((-20, 0), (20, 0), rejected) is None
    assert q.raycast((-20, 0), (20, 0)).object_id == 1  # a tie goes to the smaller id


def test_sensors_are_not_queryable():
    state = stage(WorldTransaction().add(SensorDescriptor(20, Circle(5.0), (60.0, 60.0))))
    q = W.query_index(state)
    assert q.objects_at((60, 60)) == [] and q.objects_in_circle((60, 60), 10) == [] and q.raycast((50, 60), (70, 60)) is None


def test_raycast_returns_the_first_hit_with_point_normal_and_fraction():
    q = scene()
    first = q.raycast((-50, 0), (50, 0))
    assert first.object_id == 3 and first.point == pytest.approx((-34, 0), abs=1e-4)
    assert first.normal == pytest.approx((-1, 0), abs=1e-4) and first.fraction == pytest.approx(0.16, abs=1e-4)
    diamond = q.raycast((60, 2), (0, 2))
    assert diamond.object_id == 2 and diamond.point[0] == pytest.approx(35.0711, abs=1e-3)
    assert diamond.normal == pytest.approx((0.7071, 0.7071), abs=1e-3)
    assert diamond.fraction == pytest.approx((60 - 35.0711) / 60, abs=1e-4)


def test_raycast_hits_the_capsule_side_and_cap():
    q = scene()
    side = q.raycast((10, 30), (-10, 30))
    assert side.object_id == 4 and side.point[0] == pytest.approx(2, abs=1e-4)
    assert side.normal[0] == pytest.approx(1, abs=1e-4) and side.fraction == pytest.approx(0.4, abs=1e-4)
    cap = q.raycast((0, 50), (0, 0))
    assert cap.object_id == 4 and cap.point[1] == pytest.approx(38, abs=1e-4)
    assert cap.normal[1] == pytest.approx(1, abs=1e-4) and cap.fraction == pytest.approx(0.24, abs=1e-4)


def test_raycast_filter_skips_filtered_objects():
    q = scene(circle_filter=CollisionFilter(2, 0xFFFFFFFF))
    assert q.raycast((-50, 0), (50, 0)).object_id == 3
    hit = q.raycast((-50, 0), (50, 0), CollisionFilter(1, 1))
    assert hit.object_id == 1 and hit.point[0] == pytest.approx(-5, abs=1e-4) and hit.fraction == pytest.approx(0.45, abs=1e-4)


def test_raycast_misses_and_degenerate_input():
    q = scene()
    assert q.raycast((-50, 15), (50, 15)) is None and q.raycast((-50, 0), (-40, 0)) is None
    assert q.raycast((0, 0), (math.nan, 0)) is None and q.raycast((math.inf, 0), (0, 0)) is None
    assert q.raycast((0, 15), (0, 15)) is None


def test_raycast_starting_inside_reports_fraction_zero():
    q = scene()
    hit = q.raycast((1, 0), (20, 0))
    assert hit.object_id == 1 and hit.fraction == 0 and hit.point == (1.0, 0.0)
    assert hit.normal[0] == pytest.approx(-1, abs=1e-5)
    degenerate = q.raycast((1, 0), (1, 0))
    assert degenerate.object_id == 1 and degenerate.fraction == 0


def test_empty_state_answers_empty():
    q = W.query_index(W._State())
    assert q.objects_at((0, 0)) == [] and q.objects_in_circle((0, 0), 5) == [] and q.raycast((-1, 0), (1, 0)) is None


def test_grid_answers_match_brute_force_on_many_objects():
    tx, expected = WorldTransaction(), {}
    for k in range(400):
        x, y, r = (k % 20) * 9.0 - 90, (k // 20) * 9.0 - 90, 3.0 + k % 3
        tx = tx.add(bubble(k + 1, x, y, r, CollisionFilter(0b01, 0b01)))
        expected[k + 1] = (np.array([x, y], np.float32), np.float32(r))
    tx = tx.add(RigidBodyDescriptor(1000, box(80.0), (0.0, 0.0), filter=CollisionFilter(0b10, 0b10)))
    q = W.query_index(stage(tx))
    for probe in ((0, 0), (13.5, -22.2), (-85, 40), (99, 99), (4.4, 4.4)):
        p = np.array(probe, np.float32)
        want = [i for i, (c, r) in expected.items() if np.hypot(*(c - p)) <= r]
        if abs(probe[0]) <= 80 and abs(probe[1]) <= 80:
            want.append(1000)
        assert q.objects_at(probe) == sorted(want), probe
    c = np.array((10, 10), np.float32)
    want = sorted([i for i, (cc, r) in expected.items() if np.hypot(*(cc - c)) <= r + 20] + [1000])
    assert q.objects_in_circle((10, 10), 20) == want


def test_world_builds_the_index_once_per_publication():
    w = W.BubbleWorld(W.WorldConfiguration(REGION))
    assert w.objects_at((0, 0)) == [] and w.objects_in_circle((0, 0), 1) == []
    assert w.query_index_build_count == 1
    w.advance(1.0 / 60)
    w.objects_at((0, 0))
    w.raycast((0, 0), (1, 0))
    assert w.query_index_build_count == 2
