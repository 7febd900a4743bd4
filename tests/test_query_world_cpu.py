"""Synchronous queries answer from the published state, against QueryWorldTests.swift:12-114, through the world API on a
stand-in device world that forwards to the oracle. The scene is the reference test's: a 600 x 300 region, bubble 1
(radius 10, K_c 1e4) flying right from (100, 100) at 60 units/s for 30 steps, a static square 2 (half 15) at
(300, 100), a static circle 3 (radius 12) at (400, 100) and a static horizontal capsule 4 (half length 20, radius 8)
at (500, 100)."""
import math

import pytest

from bubblephysics_gb300 import world as W
from bubblephysics_gb300.world import (BubbleDescriptor, BubbleWorld, Capsule, Circle, CollisionFilter, PhysicsMaterial,
                                       Polygon, RigidBodyDescriptor, WorldConfiguration, WorldTransaction)
from test_world_api_oracle_cpu import OracleBackedWorld

STEP = 1.0 / 60


@pytest.fixture(autouse=True)
def oracle_backed(monkeypatch):
    monkeypatch.setattr(W, "World", OracleBackedWorld)
    monkeypatch.setattr(W, "default_context", lambda: None)


def make_scene(circle_filter=CollisionFilter()):
    world = BubbleWorld(WorldConfiguration((0.0, 0.0, 600.0, 300.0)))
    world.submit(WorldTransaction().update_physics_material(1, PhysicsMaterial(1e4))
                 .add(BubbleDescriptor(1, (100.0, 100.0), 10.0, 1.0, 1, velocity=(60.0, 0.0)))
                 .add(RigidBodyDescriptor(2, Polygon(((-15.0, -15.0), (15.0, -15.0), (15.0, 15.0), (-15.0, 15.0))),
                                          (300.0, 100.0)))
                 .add(RigidBodyDescriptor(3, Circle(12.0), (400.0, 100.0), filter=circle_filter))
                 .add(RigidBodyDescriptor(4, Capsule(20.0, 8.0), (500.0, 100.0))))
    for _ in range(30):
        frame = world.advance(STEP)
        assert world.diagnostics.last_advance_issue is None
    return world, frame


def test_point_rectangle_and_circle_queries_answer_from_the_published_state():
    world, frame = make_scene()
    position = frame.objects[1].position
    assert math.dist(position, (100.0, 100.0)) > 11
    assert world.objects_at(position) == [1] and world.objects_at((100.0, 100.0)) == []
    assert world.objects_at((310.0, 110.0)) == [2] and world.objects_at((316.0, 100.0)) == []
    assert world.objects_at((408.0, 108.0)) == [3]  # 11.3 < 12
    assert world.objects_at((409.0, 109.0)) == []   # 12.7: in the box, out of the circle
    assert world.objects_at((525.0, 100.0)) == [4] and world.objects_at((530.0, 100.0)) == []
    assert world.objects_in((0.0, 0.0, 600.0, 300.0)) == [1, 2, 3, 4]
    assert world.objects_in((280.0, 80.0, 320.0, 120.0)) == [2]
    assert world.objects_in_circle((450.0, 100.0), 40.0) == [3, 4]
    assert world.objects_in_circle((450.0, 100.0), 0.1) == []


def test_an_asymmetric_polygon_answers_the_same_in_queries_and_in_the_hit_test():
    """QueryWorldTests.swift:45-66: an L whose centroid is far from its local origin, turned by pi/2."""
    world = BubbleWorld(WorldConfiguration((0.0, 0.0, 600.0, 300.0)))
    world.submit(WorldTransaction().update_physics_material(1, PhysicsMaterial(1e4))
                 .add(RigidBodyDescriptor(5, Polygon(((0.0, 0.0), (10.0, 0.0), (10.0, 2.0), (2.0, 2.0), (2.0, 10.0),
                                                      (0.0, 10.0))), (300.0, 100.0), angle=math.pi / 2))
                 .add(BubbleDescriptor(1, (50.0, 50.0), 5.0, 1.0, 1)))
    world.advance(STEP)
    world.advance(STEP)
    cases = (((299.0, 108.0), 5), ((292.0, 101.0), 5), ((292.0, 108.0), None), ((296.8, 103.2), None),
             ((320.0, 100.0), None))
    requests = [world.request_hit_test(p) for p, _ in cases]
    world.advance(STEP)
    for (point, expected), request in zip(cases, requests):
        assert world.objects_at(point) == ([expected] if expected else []), point
        assert request.result == expected, point


def test_a_raycast_finds_the_first_hit_and_a_filter_narrows_it():
    world, _ = make_scene(circle_filter=CollisionFilter(2, 0xFFFFFFFF))
    hit = world.raycast((350.0, 100.0), (600.0, 100.0))
    assert hit.object_id == 3 and abs(hit.point[0] - 388) <= 1e-3 and abs(hit.normal[0] + 1) <= 1e-3
    assert abs(hit.fraction - (388 - 350) / 250) <= 1e-4
    only_1 = CollisionFilter(1, 1)
    filtered = world.raycast((350.0, 100.0), (600.0, 100.0), only_1)
    assert filtered.object_id == 4 and abs(filtered.point[0] - 472) <= 1e-3
    assert world.objects_at((400.0, 100.0), only_1) == [] and world.objects_at((400.0, 100.0)) == [3]


def test_a_removed_object_leaves_the_queries_with_the_step_that_publishes_the_removal():
    world, _ = make_scene()
    world.submit(WorldTransaction().remove(2))
    assert world.objects_at((300.0, 100.0)) == [2]  # the published state
    world.advance(STEP)
    assert world.objects_at((300.0, 100.0)) == []


def test_the_index_is_built_once_per_publication_on_the_first_query():
    world, _ = make_scene()
    assert world.query_index_build_count == 0
    world.objects_at((300.0, 100.0))
    world.objects_in((0.0, 0.0, 10.0, 10.0))
    world.objects_in_circle((450.0, 100.0), 40.0)
    world.raycast((0.0, 100.0), (600.0, 100.0))
    assert world.query_index_build_count == 1
    world.advance(STEP)
    assert world.query_index_build_count == 1
    world.objects_at((300.0, 100.0))
    world.objects_at((301.0, 100.0))
    assert world.query_index_build_count == 2


def test_a_world_without_any_step_answers_empty():
    world = BubbleWorld(WorldConfiguration((0.0, 0.0, 600.0, 300.0)))
    assert world.objects_at((10.0, 10.0)) == [] and world.raycast((0.0, 0.0), (100.0, 100.0)) is None
