"""Host logic of the world API mirror (BubbleWorld / WorldTransaction / WorldFrame, Sources/BubblePhysicsPublic):
transaction staging and rejection, the fixed-step clock of advance(by:) (FixedStepDriver.swift) and contact-event
compaction from contact records (NativePublicWorld.swift:340-391). None of this needs a GPU: a world without bubbles
never builds a device world."""
import numpy as np
import pytest

from bubblephysics_gb300 import _native as N
from bubblephysics_gb300 import world as W
from bubblephysics_gb300.world import (BubbleDescriptor, BubbleWorld, Circle, MotionRole,
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
    (soft().add(BubbleDescriptor(1, (10, 10), -1.0, 1.0, "soft")), R.INVALID_VALUE),
    (soft().remove(99), R.OBJECT_NOT_FOUND),
    (soft().add(RigidBodyDescriptor(7, Circle(5.0), (50, 50), motion_role=MotionRole.DYNAMIC)), R.UNSUPPORTED_OPERATION),
    (soft().operation("mergeBubbles", (1, 2)), R.UNSUPPORTED_OPERATION),
])
def test_rejections_are_atomic(tx, reason):
    state, receipts, events = W.stage([(1, tx)], W._State(), REGION)
    assert receipts == [] and state.bubbles == {} and state.bodies == {} and state.materials == {}
    assert len(events) == 1 and events[0].kind == "transactionRejected" and events[0].rejection.reason == reason


def test_staging_applies_transactions_in_order_against_the_staged_state():
    txs = [(1, soft().add(bubble(1, 10, 10)).add(bubble(2, 50, 50))),
           (2, WorldTransaction().remove(2).apply_impulse(1, (3.0, 0.0))),
           (3, WorldTransaction().remove(2))]
    state, receipts, events = W.stage(txs, W._State(), REGION)
    assert [r.token for r in receipts] == [1, 2]
    assert receipts[0].created_object_ids == (1, 2) and receipts[1].removed_object_ids == (2,)
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
