"""Host logic of the world API mirror (BubbleWorld / WorldTransaction / WorldFrame, Sources/BubblePhysicsPublic):
transaction staging and rejection, the fixed-step clock of advance(by:) (FixedStepDriver.swift) and contact-event
compaction from contact records (NativePublicWorld.swift:340-391). None of this needs a GPU: a world without bubbles
never builds a device world."""
import numpy as np
import pytest

from bubblephysics_gb300 import _native as N
from bubblephysics_gb300 import world as W
from bubblephysics_gb300.world import (BubbleDescriptor, BubbleWorld, Circle, EventInterest, MotionRole,
                                       PhysicsMaterial, RigidBodyDescriptor, TransactionRejectionReason as R,
                                       WorldConfiguration, WorldTransaction)

REGION = (0.0, 0.0, 200.0, 200.0)


def soft():
    return WorldTransaction().update_physics_material("soft", PhysicsMaterial(229.0))


def bubble(i, x, y, **kw):
    return BubbleDescriptor(i, (x, y), 10.0, 1.0, "soft", **kw)


def test_transaction_builder_returns_copies_in_order():
    a = WorldTransaction()
    b = a.add(bubble(1, 5, 5))
    c = b.remove(1)
    assert a.operations == () and len(b.operations) == 1 and [op[0] for op in c.operations] == ["add", "remove"]


@pytest.mark.parametrize("tx,reason", [
    (soft().add(bubble(1, 10, 10)).add(bubble(1, 50, 50)), R.DUPLICATE_OBJECT_ID),
    (WorldTransaction().add(bubble(1, 10, 10)), R.PHYSICS_MATERIAL_NOT_FOUND),
    (soft().add(bubble(1, 500, 10)), R.INVALID_PLACEMENT),
    (soft().add(bubble(1, 10, 10)).add(bubble(2, 10, 10)), R.INVALID_PLACEMENT),
    (soft().add(RigidBodyDescriptor(7, Circle(20.0), (100, 100))).add(bubble(1, 105, 100)), R.INVALID_PLACEMENT),
    (soft().add(BubbleDescriptor(1, (10, 10), 10.0, 1e-3, "soft", drive_policy=W.BubbleDrivePolicy(1000.0))),
     R.INVALID_VALUE),
    (soft().remove(99), R.OBJECT_NOT_FOUND),
    (soft().add(RigidBodyDescriptor(7, Circle(5.0), (50, 50), motion_role=MotionRole.DYNAMIC)), R.UNSUPPORTED_OPERATION),
    (soft().operation("mergeBubbles", (1, 2)), R.UNSUPPORTED_OPERATION),
])
def test_rejections_are_atomic(tx, reason):
    state, receipts, events = W.stage([(1, tx)], W._State(), REGION)
    assert receipts == [] and state.bubbles == {} and state.bodies == {} and state.materials == {}
    assert len(events) == 1 and events[0].kind == "transactionRejected" and events[0].rejection.reason == reason


def test_staging_applies_transactions_in_order_against_the_staged_state():
    told = frozenset({EventInterest.DID_ADD, EventInterest.DID_REMOVE})  # lifecycle events follow the interests
    txs = [(1, soft().add(bubble(1, 10, 10, event_interest=told)).add(bubble(2, 50, 50, event_interest=told))
            .add(bubble(3, 90, 90))),
           (2, WorldTransaction().remove(2).apply_impulse(1, (3.0, 0.0)).remove(3)),
           (3, WorldTransaction().remove(2))]
    state, receipts, events = W.stage(txs, W._State(), REGION)
    assert [r.token for r in receipts] == [1, 2]
    assert receipts[0].created_object_ids == (1, 2, 3) and receipts[1].removed_object_ids == (2, 3)
    assert sorted(state.bubbles) == [1]
    assert np.array_equal(state.bubbles[1].velocity, np.array([3.0, 0.0], np.float32))
    kinds = [e.kind for e in events]
    assert kinds == ["didAdd", "didAdd", "didRemove", "transactionRejected"]


def test_advance_runs_a_fixed_step_clock_with_a_backlog_cap():
    w = BubbleWorld(WorldConfiguration(REGION, fixed_time_step=0.01, maximum_backlog=0.05))
    frame = w.advance(0.035)
    assert frame.step_index == 3 and w.diagnostics.steps_in_last_advance == 3
    assert abs(w.diagnostics.backlog_seconds - 0.005) < 1e-9
    frame = w.advance(1.0)  # capped at 0.05 of backlog: 5 steps, the rest discarded
    assert frame.step_index == 8 and w.diagnostics.discarded_backlog_seconds == pytest.approx(0.955)
    same = w.advance(0.0)
    assert same is frame
    w.pause()
    assert w.advance(1.0) is frame
    w.resume()
    assert w.advance(float("nan")) is frame


def test_steps_per_advance_are_limited():
    w = BubbleWorld(WorldConfiguration(REGION, fixed_time_step=0.01, maximum_backlog=1.0))
    w.advance(0.5)
    assert w.diagnostics.steps_in_last_advance == 8 and w.last_frame.step_index == 8


def contacts(*records):
    out = np.zeros(len(records), N.CONTACT_DTYPE)
    for i, (a, b, kind, pen, imp, normal, point) in enumerate(records):
        out[i]["participants"] = (a, b)
        out[i]["kind"], out[i]["penetration"], out[i]["impulse"] = kind, pen, imp
        out[i]["normal"], out[i]["point"] = normal, point
    return out


def test_contact_events_begin_and_end_per_pair():
    step = 1.0 / 60
    c1 = contacts((5, 3, 0, 0.5, 0.2, (1.0, 0.0), (4.0, 0.0)), (7, 900, 1, 0.1, 0.0, (0.0, 1.0), (7.0, 1.0)))
    events, history = W.contact_transitions(c1, {900: 42}, {3}, set(), step, set())
    assert [(e.kind, e.objects) for e in events] == [("contactBegan", (3, 5))]  # (7, 42) has no interested object
    began = events[0]
    assert began.normal == (-1.0, 0.0) and began.impulse == pytest.approx(0.2 / step, rel=1e-6)
    events, history = W.contact_transitions(c1, {900: 42}, {3}, history, step, set())
    assert events == []  # still in contact: nothing new
    events, history = W.contact_transitions(contacts(), {}, {3}, history, step, set())
    assert [(e.kind, e.objects) for e in events] == [("contactEnded", (3, 5))] and history == set()


def test_contact_pairs_order_by_unsigned_ids():
    c = contacts((-1, 2, 0, 0.5, 0.0, (1.0, 0.0), (0.0, 0.0)), (1, 2, 0, 0.5, 0.0, (1.0, 0.0), (0.0, 0.0)))
    events, _ = W.contact_transitions(c, {}, {1, 2, -1}, set(), 1.0, set())
    # -1 is 0xFFFF...FFFF as an ObjectID: the largest id
    assert [e.objects for e in events] == [(1, 2), (2, -1)]


def test_event_compactor_cases_of_the_reference():
    """EventCompactorTests.swift:50-99: events sorted by pair; a begin for a pair already in the history is skipped;
    a removed object ends its contacts for the remaining partner only; a contact between two removed objects gives no
    event and leaves the history; an end for a removed object is not duplicated."""
    hit = lambda a, b: (a, b, 0, 0.5, 2.0, (1.0, 0.0), (1.0, 0.0))
    everyone = {1, 2, 3, 4}
    events, history = W.contact_transitions(contacts(hit(3, 4), hit(1, 2)), {}, everyone, set(), 1.0, set())
    assert [(e.kind, e.objects) for e in events] == [("contactBegan", (1, 2)), ("contactBegan", (3, 4))]
    assert history == {(1, 2), (3, 4)}
    events, history = W.contact_transitions(contacts(hit(1, 2)), {}, everyone, {(1, 2)}, 1.0, set())
    assert events == [] and history == {(1, 2)}
    events, history = W.contact_transitions(contacts(hit(3, 4)), {}, everyone, {(1, 2), (3, 4)}, 1.0, {2})
    assert [(e.kind, e.objects) for e in events] == [("contactEnded", (1, 2))] and history == {(3, 4)}
    events, history = W.contact_transitions(contacts(), {}, everyone, {(2, 3)}, 1.0, {2, 3})
    assert events == [] and history == set()
    events, history = W.contact_transitions(contacts(), {}, everyone, {(1, 2)}, 1.0, {2})
    assert [(e.kind, e.objects) for e in events] == [("contactEnded", (1, 2))] and history == set()


def test_sensors_stage_like_objects():
    sensor = W.SensorDescriptor(50, Circle(20.0), (100.0, 100.0))
    state, receipts, _ = W.stage([(1, soft().add(sensor).add(bubble(1, 100, 100)))], W._State(), REGION)
    assert receipts[0].created_object_ids == (50, 1) and state.sensors[50] == sensor  # a sensor overlaps freely
    for make in (lambda: W.Polygon(((0, 0), (1, 0))), lambda: Circle(0.0),  # refused when they are made
                 lambda: W.SensorDescriptor(51, Circle(5.0), (float("nan"), 0))):
        with pytest.raises(ValueError):
            make()
    _, _, ev = W.stage([(3, WorldTransaction().add(W.SensorDescriptor(1, Circle(5.0), (0, 0))))], state, REGION)
    assert ev[0].rejection.reason == R.DUPLICATE_OBJECT_ID
    moved = W.SensorDescriptor(50, W.Polygon(((-5, -5), (5, -5), (0, 5))), (30.0, 30.0))
    replaced, rec, _ = W.stage([(4, WorldTransaction().replace(50, moved))], state, REGION)
    assert rec[0].replaced_object_ids == (50,) and replaced.sensors[50] == moved
    removed, rec, _ = W.stage([(5, WorldTransaction().remove(50))], state, REGION)
    assert rec[0].removed_object_ids == (50,) and removed.sensors == {} and 50 in state.sensors


def test_sensor_records_and_carried_overlap_state():
    world = BubbleWorld(WorldConfiguration(REGION))
    state, _, _ = W.stage([(1, soft().add(W.SensorDescriptor(9, W.Polygon(((0, 0), (4, 0), (0, 4))), (11.0, 12.0), 0.5,
                                                                 filter=W.ObjectFilter(frozenset({20, 500})),
                                                                 reports_enter=False))
                               .add(W.SensorDescriptor(4, Circle(7.0), (50.0, 60.0))))], W._State(), REGION)
    world._sensor_pairs = {(4, 30), (9, 10), (9, 500), (9, 99)}  # 99 is no longer an object of the device world
    records, verts, carried, allowed = world._sensor_records(state, [10, 20, 30, 500])  # three bubbles, one body
    assert [r.id for r in records] == [4, 9]
    assert records[0].radius == 7.0 and records[0].vertex_count == 0
    assert records[1].vertex_offset == 0 and records[1].vertex_count == 3 and records[1].angle == 0.5
    assert all(r.flags == N.SENSOR_ENTER_EVENTS | N.SENSOR_EXIT_EVENTS for r in records)  # filtered on the host
    assert verts.tolist() == [[0, 0], [4, 0], [0, 4]]
    assert carried.tolist() == [0, 0, 1, 0, 1, 0, 0, 1]
    assert allowed.tolist() == [1, 1, 1, 1, 0, 1, 0, 1]


def test_set_layer():
    state, _, _ = W.stage([(1, soft().add(bubble(1, 10, 10)).add(W.SensorDescriptor(5, Circle(3.0), (10, 50))))],
                          W._State(), REGION)
    layered, rec, _ = W.stage([(2, WorldTransaction().set_layer(1, 7))], state, REGION)
    assert rec and layered.bubbles[1].desc.layer == 7 and state.bubbles[1].desc.layer == 0
    assert W.stage([(3, WorldTransaction().set_layer(1, -5))], state, REGION)[0].bubbles[1].desc.layer == -5  # Int32
    for tx, reason in ((WorldTransaction().set_layer(1, 2 ** 31), R.INVALID_VALUE),
                       (WorldTransaction().set_layer(5, 1), R.INCOMPATIBLE_OBJECT_KIND),
                       (WorldTransaction().set_layer(8, 1), R.OBJECT_NOT_FOUND)):
        _, rec, ev = W.stage([(3, tx)], state, REGION)
        assert rec == [] and ev[0].rejection.reason == reason


def test_object_states_of_bodies_follow_their_shape_and_rotation():
    """ObjectStateTests.swift:42-145: a static square's bounds are its own box (92 / 198 for half 8 at (100, 190));
    a square turned by pi/4 reaches 10 sqrt(2); a kinematic body moves and turns with its drive, also in a world
    without bubbles."""
    import math as _m
    from bubblephysics_gb300.world import Polygon
    w = BubbleWorld(WorldConfiguration((0.0, 0.0, 400.0, 400.0)))
    sq = lambda h: Polygon(((-h, -h), (h, -h), (h, h), (-h, h)))
    w.submit(WorldTransaction().add(RigidBodyDescriptor(4, sq(8.0), (100.0, 190.0)))
             .add(RigidBodyDescriptor(7, sq(10.0), (100.0, 100.0), angle=_m.pi / 4))
             .add(RigidBodyDescriptor(3, sq(10.0), (100.0, 150.0), motion_role=MotionRole.KINEMATIC,
                                      velocity=(0.0, -5.0), angular_velocity=1.0)))
    for _ in range(30):
        frame = w.advance(1.0 / 60)
    assert frame.step_index == 30
    wall = frame.objects[4]
    assert wall.position == (100.0, 190.0) and wall.bounds[0] == pytest.approx(92, abs=1e-3)
    assert wall.bounds[3] == pytest.approx(198, abs=1e-3)
    turned = frame.objects[7]
    assert turned.bounds[0] == pytest.approx(100 - 10 * _m.sqrt(2), abs=1e-3)
    assert turned.bounds[3] == pytest.approx(100 + 10 * _m.sqrt(2), abs=1e-3)
    spinning = frame.objects[3]
    assert spinning.kind == "polygon" and spinning.rotation != 0 and spinning.angular_velocity != 0
    assert spinning.position[1] < 150.0
    for state in frame.objects.values():
        lo, hi = state.bounds[:2], state.bounds[2:]
        assert lo[0] < hi[0] and lo[1] < hi[1] and lo[0] <= state.position[0] <= hi[0]


@pytest.mark.parametrize("kwargs", [dict(radius=-1.0), dict(radius=0.0), dict(radius=float("nan")), dict(mass=0.0),
                                    dict(position=(float("nan"), 0.0)), dict(velocity=(float("inf"), 0.0))])
def test_a_bubble_with_invalid_values_is_refused_when_it_is_made(kwargs):
    """ModelValidationTests.swift:113-125: the descriptor checks its own values, as the reference's init throws."""
    values = dict(position=(0.0, 0.0), radius=1.0, mass=1.0, velocity=(0.0, 0.0)) | kwargs
    with pytest.raises(ValueError):
        BubbleDescriptor(1, values["position"], values["radius"], values["mass"], "soft", velocity=values["velocity"])
