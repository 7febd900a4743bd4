"""Events follow the objects' interests and fit the event buffer, through the world API on a stand-in device world
that forwards to the oracle: EventInterestTests.swift:5-52 (no contact event without interest, a removed bubble leaves
its sensor and a re-added one enters again), the event buffer of EventCompactor.swift:11-37 (step events beyond
eventBufferCapacity are counted as dropped; a dropped contactEnded comes with the next step) and
NativeMetalEventCompactionTests.swift:93-191 (overflow reported, removed pairs' exits within the buffer, a wrap event
needs interest, a polygon sensor ignores distant collinear edges)."""
import pytest

from bubblephysics_gb300 import world as W
from bubblephysics_gb300.world import (BubbleDescriptor, BubbleWorld, Circle, EventInterest, PhysicsMaterial,
                                       SensorDescriptor, WorldConfiguration, WorldTransaction)
from test_world_api_oracle_cpu import OracleBackedWorld

STEP = 1.0 / 60


@pytest.fixture(autouse=True)
def oracle_backed(monkeypatch):
    monkeypatch.setattr(W, "World", OracleBackedWorld)
    monkeypatch.setattr(W, "default_context", lambda: None)


def test_no_contact_event_is_published_without_interest():
    """EventInterestTests.swift:5-21: two overlapping bubbles, neither asking for contact events."""
    world = BubbleWorld(WorldConfiguration((-20.0, -20.0, 20.0, 20.0)))
    world.submit(WorldTransaction().update_physics_material(1, PhysicsMaterial(1e9))
                 .add(BubbleDescriptor(1, (-0.5, 0.0), 1.0, 1.0, 1)).add(BubbleDescriptor(2, (0.5, 0.0), 1.0, 1.0, 1)))
    frame = world.advance(STEP)
    assert not any(e.kind.startswith("contact") for e in frame.events)
    assert frame.event_overflow.dropped_count == 0


def test_a_removed_bubble_leaves_its_sensor_and_a_re_added_one_enters_again():
    """EventInterestTests.swift:27-51: the last bubble of the world is removed and added again."""
    world = BubbleWorld(WorldConfiguration((-20.0, -20.0, 20.0, 20.0)))
    body = BubbleDescriptor(1, (0.0, 0.0), 1.0, 1.0, 1)
    world.submit(WorldTransaction().update_physics_material(1, PhysicsMaterial(1e9)).add(body)
                 .add(SensorDescriptor(9, Circle(3.0), (0.0, 0.0))))
    assert any(e.kind == "enteredSensor" and e.objects == (9, 1) for e in world.advance(STEP).events)
    world.submit(WorldTransaction().remove(1))
    assert any(e.kind == "exitedSensor" and e.objects == (9, 1) for e in world.advance(STEP).events)
    world.submit(WorldTransaction().add(body))
    assert any(e.kind == "enteredSensor" and e.objects == (9, 1) for e in world.advance(STEP).events)


def test_lifecycle_events_follow_the_interests_in_operation_order():
    """didAdd / didRemove / didReplace come only for objects that ask for them (TransactionStager.swift:237, 412, 435),
    in the order of the operations."""
    told = frozenset({EventInterest.DID_ADD, EventInterest.DID_REMOVE, EventInterest.DID_REPLACE})
    world = BubbleWorld(WorldConfiguration((-50.0, -50.0, 50.0, 50.0)))
    world.submit(WorldTransaction().update_physics_material(1, PhysicsMaterial(229.0))
                 .add(BubbleDescriptor(1, (0.0, 0.0), 1.0, 1.0, 1, event_interest=told))
                 .add(BubbleDescriptor(2, (10.0, 0.0), 1.0, 1.0, 1)))
    assert [(e.kind, e.objects) for e in world.advance(STEP).events] == [("didAdd", (1,))]
    world.submit(WorldTransaction().remove(2).replace(1, BubbleDescriptor(1, (0.0, 5.0), 1.0, 1.0, 1)).remove(1))
    assert [(e.kind, e.objects) for e in world.advance(STEP).events] == [("didReplace", (1,))]


def test_step_events_beyond_the_buffer_are_dropped_and_a_dropped_end_comes_next_step():
    """Three pairs touch and part at once with room for two events per step: one begin is dropped (its pair begins
    on the next step while it lasts), and the ends that did not fit come with the following steps."""
    contact = frozenset({EventInterest.CONTACT})
    world = BubbleWorld(WorldConfiguration((-200.0, -200.0, 200.0, 200.0), event_buffer_capacity=2))
    tx = WorldTransaction().update_physics_material(1, PhysicsMaterial(229.0))
    for k in range(3):
        y = 40.0 * k
        tx = tx.add(BubbleDescriptor(10 + k, (-1.05, y), 1.0, 1.0, 1, velocity=(30.0, 0.0), event_interest=contact))
        tx = tx.add(BubbleDescriptor(20 + k, (1.05, y), 1.0, 1.0, 1, velocity=(-30.0, 0.0)))
    world.submit(tx)
    began, ended, dropped = [], [], 0
    for _ in range(30):
        frame = world.advance(STEP)
        began += [e.objects for e in frame.events if e.kind == "contactBegan"]
        ended += [e.objects for e in frame.events if e.kind == "contactEnded"]
        dropped += frame.event_overflow.dropped_count
        assert len(frame.events) <= 2
    assert dropped > 0
    assert sorted(set(began)) == [(10, 20), (11, 21), (12, 22)]
    assert sorted(ended) == [(10, 20), (11, 21), (12, 22)]  # each end delivered once, late or not


def sensor_world(capacity=1024, region=(-20.0, -20.0, 20.0, 20.0), step=STEP):
    world = BubbleWorld(WorldConfiguration(region, fixed_time_step=step, event_buffer_capacity=capacity))
    world.submit(WorldTransaction().update_physics_material(1, PhysicsMaterial(1e9)))
    return world


def test_event_buffer_overflow_is_reported_instead_of_silently_dropped():
    """NativeMetalEventCompactionTests.swift:113-121: two bubbles enter a sensor with room for one event."""
    world = sensor_world(capacity=1)
    world.submit(WorldTransaction().add(BubbleDescriptor(1, (-1.0, 0.0), 1.0, 1.0, 1))
                 .add(BubbleDescriptor(2, (1.0, 0.0), 1.0, 1.0, 1))
                 .add(SensorDescriptor(9, Circle(3.0), (0.0, 0.0), reports_exit=False)))
    frame = world.advance(STEP)
    assert len(frame.events) == 1 and frame.event_overflow.dropped_count == 1


def test_the_exits_of_removed_pairs_respect_the_event_buffer():
    """NativeMetalEventCompactionTests.swift:93-111: both observed bubbles go at once with room for one event; the
    lost exit is counted and not delivered later."""
    from dataclasses import replace
    world = sensor_world(capacity=2)
    world.submit(WorldTransaction().add(BubbleDescriptor(1, (-1.0, 0.0), 1.0, 1.0, 1))
                 .add(BubbleDescriptor(2, (1.0, 0.0), 1.0, 1.0, 1)).add(SensorDescriptor(9, Circle(3.0), (0.0, 0.0))))
    world.advance(STEP)
    world.configuration = replace(world.configuration, event_buffer_capacity=1)
    world.submit(WorldTransaction().remove(1).remove(2))
    removed = world.advance(STEP)
    assert [e.kind for e in removed.events] == ["exitedSensor"] and removed.events[0].objects[0] == 9
    assert removed.event_overflow.dropped_count == 1
    cleared = world.advance(STEP)
    assert not cleared.events and cleared.event_overflow.dropped_count == 0


def test_a_wrap_event_needs_interest():
    """NativeMetalEventCompactionTests.swift:168-176: one step of 0.25 s takes the bubble across the region's edge."""
    world = sensor_world(region=(0.0, 0.0, 10.0, 10.0), step=0.25)
    world.submit(WorldTransaction().add(BubbleDescriptor(1, (9.0, 5.0), 1.0, 1.0, 1, velocity=(20.0, 0.0),
                                                         region_exit_policy=W.RegionExitPolicy.WRAP,
                                                         event_interest=frozenset({EventInterest.DID_WRAP}))))
    assert [(e.kind, e.objects) for e in world.advance(0.25).events] == [("didWrap", (1,))]


def test_a_polygon_sensor_ignores_distant_collinear_edges():
    """NativeMetalEventCompactionTests.swift:178-191: a triangle whose base lies on the line of the sensor's lower
    edge, 5 units beyond its corner, does not enter it."""
    from bubblephysics_gb300.world import Polygon, RigidBodyDescriptor
    world = sensor_world()
    world.submit(WorldTransaction()
                 .add(SensorDescriptor(9, Polygon(((-2.0, -2.0), (2.0, -2.0), (2.0, 2.0), (-2.0, 2.0))), (0.0, 0.0),
                                       reports_exit=False))
                 .add(RigidBodyDescriptor(3, Polygon(((-0.5, -2.0), (0.5, -2.0), (0.0, -1.0))), (7.0, 0.0)))
                 .add(BubbleDescriptor(1, (-15.0, 15.0), 1.0, 1.0, 1)))
    assert not world.advance(STEP).events
