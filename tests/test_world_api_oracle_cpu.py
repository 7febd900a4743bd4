"""The world API's sensor, hit-test and contour plumbing on the CPU: BubbleWorld runs on a stand-in device world that
forwards every call to the oracle, so the host logic (pair bookkeeping across rebuilds and removals, event filtering,
contour-derived bubble states, hit-test answers) is checked here; the same scenes run on the CUDA path in
test_gpu_world_api.py."""
import numpy as np
import pytest

from bubblephysics_gb300 import _native as N
from bubblephysics_gb300 import world as W
from bubblephysics_gb300.world import (BubbleDescriptor, BubbleWorld, Circle, PhysicsMaterial, Polygon,
                                       RigidBodyDescriptor, SensorDescriptor, WorldConfiguration, WorldTransaction)
from oracle.oracle import OracleWorld

REGION = (0.0, 0.0, 400.0, 400.0)


class OracleBackedWorld:
    """The calls BubbleWorld makes on a device world, answered by the oracle."""

    def __init__(self, spec, context=None):
        self.o = OracleWorld(spec)
        self.objects = spec.bubble_count + len(spec.bodies)
        self.sensors, self.vertices, self.state, self.allowed = [], None, None, None

    def step(self, steps):
        return self.o.step(steps)

    def bubbles(self):
        return self.o.bubbles()

    def contacts(self):
        return self.o.contacts()

    def set_sensors(self, sensors, vertices=None, state=None, allowed=None):
        self.sensors, self.vertices, self.allowed = list(sensors), vertices, allowed
        self.state = np.zeros(len(sensors) * self.objects, np.uint8) if state is None else np.array(state, np.uint8)

    def sensor_events(self):
        return self.o.sensor_events(self.sensors, self.vertices, self.state, self.allowed)

    def contours(self, max_edge, surface_tension, clearance):
        return (*self.o.contours(max_edge, surface_tension, clearance), 0.0)

    def hit_test(self, points, max_edge, surface_tension, clearance):
        return self.o.hit_test(points, max_edge, surface_tension, clearance)

    def close(self):
        pass


@pytest.fixture
def oracle_backed(monkeypatch):
    monkeypatch.setattr(W, "World", OracleBackedWorld)
    monkeypatch.setattr(W, "default_context", lambda: None)


def sensor_world():
    world = BubbleWorld(WorldConfiguration(REGION))
    tx = WorldTransaction().update_physics_material("soft", PhysicsMaterial(229.0))
    tx = tx.add(BubbleDescriptor(1, (100.0, 200.0), 10.0, 1.0, "soft", velocity=(120.0, 0.0)))
    tx = tx.add(SensorDescriptor(50, Circle(20.0), (200.0, 200.0)))
    tx = tx.add(SensorDescriptor(60, Polygon(((-10, -30), (10, -30), (10, 30), (-10, 30))), (300.0, 200.0),
                                 reports_enter=False))
    world.submit(tx)
    return world


def test_sensor_events_follow_the_published_positions(oracle_backed):
    world = sensor_world()
    seen, prev = [], None
    for _ in range(135):
        frame = world.advance(1.0 / 60)
        d = np.array(frame.objects[1].position, np.float32) - np.float32(200.0)
        inside = bool(d[0] * d[0] + d[1] * d[1] <= np.float32(900.0))
        for e in frame.events:
            if e.kind.endswith("Sensor"):
                seen.append((e.kind, e.objects))
                if e.objects[0] == 50:
                    assert inside == (e.kind == "enteredSensor") and prev is not None and prev != inside
        prev = inside
    assert seen == [("enteredSensor", (50, 1)), ("exitedSensor", (50, 1)), ("exitedSensor", (60, 1))]
    assert world._sensor_pairs == set()


def test_sensor_pairs_survive_a_rebuild_and_end_with_the_bubble(oracle_backed):
    world = sensor_world()
    kinds = []
    for _ in range(45):
        kinds += [e.kind for e in world.advance(1.0 / 60).events if e.kind.endswith("Sensor")]
    assert kinds == ["enteredSensor"] and world._sensor_pairs == {(50, 1)}
    world.submit(WorldTransaction().add(BubbleDescriptor(2, (50.0, 50.0), 8.0, 1.0, "soft")))
    assert not [e for e in world.advance(1.0 / 60).events if e.kind.endswith("Sensor")]
    world.submit(WorldTransaction().remove(1))
    frame = world.advance(1.0 / 60)
    assert [(e.kind, e.objects) for e in frame.events if e.kind.endswith("Sensor")] == [("exitedSensor", (50, 1))]
    assert world._sensor_pairs == set()


def test_removing_a_sensor_ends_its_pairs(oracle_backed):
    world = sensor_world()
    for _ in range(45):
        world.advance(1.0 / 60)
    world.submit(WorldTransaction().remove(50))
    frame = world.advance(1.0 / 60)
    assert [(e.kind, e.objects) for e in frame.events if e.kind.endswith("Sensor")] == [("exitedSensor", (50, 1))]


def test_contour_states_and_hit_test(oracle_backed):
    world = BubbleWorld(WorldConfiguration(REGION))
    tx = WorldTransaction().update_physics_material("soft", PhysicsMaterial(229.0))
    tx = tx.add(BubbleDescriptor(1, (150.0, 200.0), 12.0, 1.0, "soft", velocity=(150.0, 0.0)))
    tx = tx.add(BubbleDescriptor(2, (250.0, 200.0), 12.0, 1.0, "soft", velocity=(-150.0, 0.0)))
    tx = tx.add(BubbleDescriptor(3, (100.0, 350.0), 10.0, 1.0, "soft"))
    tx = tx.add(RigidBodyDescriptor(1000, Circle(30.0), (320.0, 80.0), layer=2))
    world.submit(tx)
    pressed = []
    for _ in range(40):
        frame = world.advance(1.0 / 60)
        pressed.append(min(frame.objects[1].effective_radius, frame.objects[2].effective_radius))
    free = frame.objects[3]
    assert abs(free.effective_radius - 10.0) <= 1e-3
    lo, hi, c = np.array(free.bounds[:2]), np.array(free.bounds[2:]), np.array(free.position)
    assert np.all(lo >= c - 10.0 - 1e-3) and np.all(lo <= c - 9.9)
    assert np.all(hi <= c + 10.0 + 1e-3) and np.all(hi >= c + 9.9)
    assert min(pressed) < 11.9
    assert world.hit_test(free.position) == 3 and world.hit_test((320.0, 80.0)) == 1000
    assert world.hit_test((10.0, 390.0)) is None
    print(f"\nsmallest effective radius of the pressed pair: {min(pressed):.3f}")


def test_without_contours_a_bubble_state_is_its_circle(oracle_backed):
    world = BubbleWorld(WorldConfiguration(REGION, contours=False))
    world.submit(WorldTransaction().update_physics_material("soft", PhysicsMaterial(229.0))
                 .add(BubbleDescriptor(3, (100.0, 350.0), 10.0, 1.0, "soft")))
    o = world.advance(1.0 / 60).objects[3]
    assert o.effective_radius == 10.0 and o.bounds == (90.0, 340.0, 110.0, 360.0)


def test_bodies_and_object_filters(oracle_backed):
    """A kinematic body crosses two sensors; the second one's object filter takes only bubble 1, so it reports nothing
    of the body."""
    world = BubbleWorld(WorldConfiguration(REGION))
    tx = WorldTransaction().update_physics_material("soft", PhysicsMaterial(229.0))
    tx = tx.add(BubbleDescriptor(1, (50.0, 50.0), 8.0, 1.0, "soft"))
    tx = tx.add(RigidBodyDescriptor(700, Circle(10.0), (100.0, 300.0), motion_role=W.MotionRole.KINEMATIC,
                                    velocity=(120.0, 0.0)))
    tx = tx.add(SensorDescriptor(80, Circle(20.0), (200.0, 300.0)))
    tx = tx.add(SensorDescriptor(81, Circle(20.0), (200.0, 300.0), filter=W.ObjectFilter(frozenset({1}))))
    world.submit(tx)
    seen = []
    for _ in range(100):
        seen += [(e.kind, e.objects) for e in world.advance(1.0 / 60).events if e.kind.endswith("Sensor")]
    assert seen == [("enteredSensor", (80, 700)), ("exitedSensor", (80, 700))]
