"""The world API mirror on the GPU: BubbleWorld.advance steps exactly like the plain world path, transactions apply at
step boundaries, contact events begin and end, region exits remove bubbles, and a failed step stops the world and
publishes nothing (BubbleWorld.swift:285-420, CompleteStep.swift:5-7)."""
import numpy as np
import pytest

from bubblephysics_gb300 import _native as N
from bubblephysics_gb300.solver import World
from bubblephysics_gb300.world import (BubbleDescriptor, BubbleWorld, Capsule, Circle, EventInterest, MotionRole,
                                       PhysicsMaterial, Polygon, RegionExitPolicy, RigidBodyDescriptor,
                                       WorldConfiguration, WorldFailureReason, WorldTransaction)

pytestmark = pytest.mark.gpu

REGION = (0.0, 0.0, 400.0, 400.0)


def populated(seed=3, n=40):
    rng = np.random.default_rng(seed)
    tx = WorldTransaction().update_physics_material("soft", PhysicsMaterial(229.0))
    tx = tx.add(RigidBodyDescriptor(1000, Circle(30.0), (200.0, 200.0)))
    tx = tx.add(RigidBodyDescriptor(1001, Capsule(25.0, 8.0), (100.0, 300.0), angle=0.3))
    tx = tx.add(RigidBodyDescriptor(1002, Polygon(((-20, -20), (20, -20), (20, 20), (-20, 20))), (300.0, 100.0)))
    tx = tx.add(RigidBodyDescriptor(1003, Circle(12.0), (80.0, 80.0), motion_role=MotionRole.KINEMATIC,
                                    velocity=(4.0, 2.0)))
    placed = 0
    for i in range(400):
        p = rng.uniform(30, 370, 2)
        if np.hypot(*(p - (200, 200))) < 60 or np.hypot(*(p - (300, 100))) < 50 or np.hypot(*(p - (100, 300))) < 50 \
                or np.hypot(*(p - (80, 80))) < 40:
            continue
        tx = tx.add(BubbleDescriptor(1 + placed, tuple(p), float(rng.uniform(6, 12)), 1.0, "soft",
                                     velocity=tuple(rng.normal(0, 30, 2)), region_exit_policy=RegionExitPolicy.WRAP))
        placed += 1
        if placed == n:
            break
    return tx


def test_advance_steps_like_the_plain_world_path(ctx):
    world = BubbleWorld(WorldConfiguration(REGION), ctx)
    world.submit(populated())
    frame = world.advance(1.0 / 60)
    assert frame.step_index == 1 and len(frame.transaction_receipts) == 1
    spec, ids, _ = world._spec(world._state)  # the device world the next steps run on
    plain = World(spec, ctx)
    for _ in range(6):
        frame = world.advance(1.0 / 60)
    status, _ = plain.step(6)
    assert status == N.OK and frame.step_index == 7
    out = plain.bubbles()
    for i, oid in enumerate(ids):
        assert frame.objects[oid].position == tuple(map(float, out[i]["center"]))
        assert frame.objects[oid].velocity == tuple(map(float, out[i]["velocity"]))


def test_transactions_apply_at_the_step_boundary(ctx):
    world = BubbleWorld(WorldConfiguration(REGION), ctx)
    world.submit(populated())
    world.advance(1.0 / 60)
    before = world.last_frame.objects[1].velocity
    token = world.submit(WorldTransaction().apply_impulse(1, (50.0, 0.0)).remove(2))
    assert world.last_frame.objects[1].velocity == before  # nothing happens before the next step
    frame = world.advance(1.0 / 60)
    assert [r.token for r in frame.transaction_receipts] == [token]
    assert 2 not in frame.objects and frame.objects[1].velocity != before
    assert frame.transaction_receipts[0].removed_object_ids == (2,)
    assert not any(e.kind == "didRemove" for e in frame.events)  # bubble 2 asked for no lifecycle events


def test_contact_events_begin_and_end(ctx):
    world = BubbleWorld(WorldConfiguration(REGION), ctx)
    tx = WorldTransaction().update_physics_material("soft", PhysicsMaterial(229.0))
    tx = tx.add(BubbleDescriptor(1, (150.0, 200.0), 12.0, 1.0, "soft", velocity=(120.0, 0.0),
                                 event_interest=frozenset({EventInterest.CONTACT})))
    tx = tx.add(BubbleDescriptor(2, (250.0, 200.0), 12.0, 1.0, "soft", velocity=(-120.0, 0.0)))
    world.submit(tx)
    kinds = []
    for _ in range(120):
        frame = world.advance(1.0 / 60)
        kinds += [(e.kind, e.objects) for e in frame.events if e.kind.startswith("contact")]
    assert ("contactBegan", (1, 2)) in kinds and ("contactEnded", (1, 2)) in kinds
    assert kinds.index(("contactBegan", (1, 2))) < kinds.index(("contactEnded", (1, 2)))


def test_region_exit_removes_the_bubble(ctx):
    world = BubbleWorld(WorldConfiguration(REGION), ctx)
    tx = WorldTransaction().update_physics_material("soft", PhysicsMaterial(229.0))
    tx = tx.add(BubbleDescriptor(1, (390.0, 200.0), 5.0, 1.0, "soft", velocity=(900.0, 0.0),
                                 event_interest=frozenset({EventInterest.DID_EXIT_SIMULATION_REGION})))
    tx = tx.add(BubbleDescriptor(2, (100.0, 200.0), 5.0, 1.0, "soft"))
    world.submit(tx)
    events = []
    for _ in range(5):
        events += list(world.advance(1.0 / 60).events)
    assert any(e.kind == "didExitSimulationRegion" and e.objects == (1,) for e in events)
    assert 1 not in world.last_frame.objects and 2 in world.last_frame.objects


def test_a_failed_step_stops_the_world(ctx):
    # the reference's fast bounce against a one-sided wall (NativeMetalSubstepKernelTests.swift:884-916) with every
    # substep split 2000 ways: the step needs more than the frame limit of 1024 substeps, fails and publishes nothing
    world = BubbleWorld(WorldConfiguration((-1000.0, -100.0, 1000.0, 100.0), substep_split_multiplier=2000.0), ctx)
    tx = WorldTransaction().update_physics_material("soft", PhysicsMaterial(229.0))
    tx = tx.add(RigidBodyDescriptor(50, Polygon(((-1000.0, -25.0), (1000.0, -25.0), (1000.0, 25.0), (-1000.0, 25.0))),
                                    (0.0, 25.0)))
    tx = tx.add(BubbleDescriptor(1, (100.0, -20.0), 12.0, 0.36, "soft", velocity=(0.0, 3000.0)))
    world.submit(tx)
    frame = world.advance(1.0 / 60)
    assert world.diagnostics.failure_reason == WorldFailureReason.SUBSTEP_LIMIT_EXCEEDED
    assert frame.step_index == 0
    assert world.advance(1.0) is frame


def sensor_world(ctx):
    """One bubble crossing a circle sensor (both kinds of event) and a polygon sensor that reports exits only."""
    from bubblephysics_gb300.world import SensorDescriptor
    world = BubbleWorld(WorldConfiguration(REGION), ctx)
    tx = WorldTransaction().update_physics_material("soft", PhysicsMaterial(229.0))
    tx = tx.add(BubbleDescriptor(1, (100.0, 200.0), 10.0, 1.0, "soft", velocity=(120.0, 0.0)))
    tx = tx.add(SensorDescriptor(50, Circle(20.0), (200.0, 200.0)))
    tx = tx.add(SensorDescriptor(60, Polygon(((-10, -30), (10, -30), (10, 30), (-10, 30))), (300.0, 200.0),
                                 reports_enter=False))
    world.submit(tx)
    return world


def test_sensor_events_follow_the_published_positions(ctx):
    world = sensor_world(ctx)
    seen, prev = [], None
    for step in range(135):  # x from 100 to 370, inside the region
        frame = world.advance(1.0 / 60)
        p = np.array(frame.objects[1].position, np.float32)
        d = p - np.float32(200.0)
        inside = bool(d[0] * d[0] + d[1] * d[1] <= np.float32(30.0) * np.float32(30.0))
        for e in frame.events:
            if e.kind.endswith("Sensor"):
                seen.append((e.kind, e.objects))
                if e.objects[0] == 50:
                    assert inside == (e.kind == "enteredSensor") and prev is not None and prev != inside
                assert e.point == tuple(map(float, frame.objects[1].position))
        prev = inside
    assert seen == [("enteredSensor", (50, 1)), ("exitedSensor", (50, 1)), ("exitedSensor", (60, 1))]


def test_sensor_state_survives_a_rebuild_and_removal_ends_the_pair(ctx):
    world = sensor_world(ctx)
    kinds = []
    for _ in range(45):  # inside the circle sensor by now
        kinds += [e.kind for e in world.advance(1.0 / 60).events if e.kind.endswith("Sensor")]
    assert kinds == ["enteredSensor"] and world._sensor_pairs == {(50, 1)}
    world.submit(WorldTransaction().add(BubbleDescriptor(2, (50.0, 50.0), 8.0, 1.0, "soft")))  # rebuilds the device world
    frame = world.advance(1.0 / 60)
    assert not [e for e in frame.events if e.kind.endswith("Sensor")]
    world.submit(WorldTransaction().remove(1))
    frame = world.advance(1.0 / 60)
    assert [(e.kind, e.objects) for e in frame.events if e.kind.endswith("Sensor")] == [("exitedSensor", (50, 1))]
    assert world._sensor_pairs == set()


def test_hit_test_and_contour_shapes(ctx):
    world = BubbleWorld(WorldConfiguration(REGION), ctx)
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
    lo, hi = np.array(free.bounds[:2]), np.array(free.bounds[2:])
    assert np.all(lo >= np.array(free.position) - 10.0 - 1e-3) and np.all(lo <= np.array(free.position) - 9.9)
    assert np.all(hi <= np.array(free.position) + 10.0 + 1e-3) and np.all(hi >= np.array(free.position) + 9.9)
    assert min(pressed) < 11.9  # the pair met and pressed in
    assert world.hit_test(free.position) == 3 and world.hit_test((320.0, 80.0)) == 1000
    assert world.hit_test((10.0, 390.0)) is None


def test_body_sensor_events_and_object_filters(ctx):
    from bubblephysics_gb300.world import ObjectFilter, SensorDescriptor
    world = BubbleWorld(WorldConfiguration(REGION), ctx)
    tx = WorldTransaction().update_physics_material("soft", PhysicsMaterial(229.0))
    tx = tx.add(BubbleDescriptor(1, (50.0, 50.0), 8.0, 1.0, "soft"))
    tx = tx.add(RigidBodyDescriptor(700, Circle(10.0), (100.0, 300.0), motion_role=MotionRole.KINEMATIC,
                                    velocity=(120.0, 0.0)))
    tx = tx.add(SensorDescriptor(80, Circle(20.0), (200.0, 300.0)))
    tx = tx.add(SensorDescriptor(81, Circle(20.0), (200.0, 300.0), filter=ObjectFilter(frozenset({1}))))
    world.submit(tx)
    seen = []
    for _ in range(100):
        seen += [(e.kind, e.objects) for e in world.advance(1.0 / 60).events if e.kind.endswith("Sensor")]
    assert seen == [("enteredSensor", (80, 700)), ("exitedSensor", (80, 700))]
