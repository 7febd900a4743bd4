"""contactBegan / contactEnded through the world API (ContactEventTests.swift:46-300), on a stand-in device world that
forwards to the oracle. Scenes follow PhysicsSceneBuilders.swift:14-50: region 600 x 300, bubbles r 8 and mass 1 of
a soft material (K_c 2000, gamma 10), a static floor box whose top is y = 10, a force of (0, -400) on every bubble.
One began per lasting contact (unit normal from the first object to the second, positive finite impulse, point in the
pair's box), no events for pairs nobody is interested in; the began arrives in the first step of contact; its impulse
is the wall law's force at the end of the step times the step (2 %); a gap within the separation tolerance is no
contact; in a corner the point leans toward the deeper edge; the end arrives in the first step after separation and
goes to the remaining partner when one side is removed; a pair added again after everything was removed begins
again. The dynamic-body and merge cases belong to the rigid solver and to merges."""
import math

import numpy as np
import pytest

from bubblephysics_gb300 import world as W
from bubblephysics_gb300.world import (BubbleDescriptor, BubbleWorld, EventInterest, MotionRole, PhysicsMaterial,
                                       Polygon, RigidBodyDescriptor, WorldConfiguration, WorldTransaction)
from test_world_api_oracle_cpu import OracleBackedWorld

FLOOR = 100
CONTACT = frozenset({EventInterest.CONTACT})


@pytest.fixture(autouse=True)
def oracle_backed(monkeypatch):
    monkeypatch.setattr(W, "World", OracleBackedWorld)
    monkeypatch.setattr(W, "default_context", lambda: None)


def world(gravity=True):
    w = BubbleWorld(WorldConfiguration((0.0, 0.0, 600.0, 300.0), global_force=(0.0, -400.0) if gravity else (0.0, 0.0)))
    return w, WorldTransaction().update_physics_material("b", PhysicsMaterial(2000.0, 10.0))


def box(i, x, y, hx, hy, role=MotionRole.STATIC, interest=frozenset()):
    return RigidBodyDescriptor(i, Polygon(((-hx, -hy), (hx, -hy), (hx, hy), (-hx, hy))), (x, y), motion_role=role,
                               event_interest=interest)


def floor(interest=frozenset()):
    return box(FLOOR, 300.0, 5.0, 300.0, 5.0, interest=interest)


def bubble(i, x, y, interest=frozenset()):
    return BubbleDescriptor(i, (x, y), 8.0, 1.0, "b", event_interest=interest)


def run(w, steps, each=None):
    events, frame = [], None
    for k in range(steps):
        frame = w.advance(1.0 / 60)
        assert w.diagnostics.last_advance_issue is None
        events += frame.events
        if each:
            each(k, frame)
    return frame, events


def began(events, pair=None):
    out = [e for e in events if e.kind == "contactBegan"]
    return out if pair is None else [e for e in out if set(e.objects) == set(pair)]


def ended(events, pair=None):
    out = [e for e in events if e.kind == "contactEnded"]
    return out if pair is None else [e for e in out if set(e.objects) == set(pair)]


def assert_single_began(events, frame, pair, hint=None):
    b = began(events, pair)
    assert len(b) == 1 and ended(events, pair) == []
    e = b[0]
    assert abs(math.hypot(*e.normal) - 1) <= 1e-3 and e.impulse > 0 and math.isfinite(e.impulse)
    first, second = frame.objects[e.objects[0]], frame.objects[e.objects[1]]
    d = np.array(hint) if hint else np.array(second.position) - np.array(first.position)
    d = d / np.hypot(*d)
    assert float(np.dot(e.normal, d)) > 0.7
    lo = np.minimum(first.bounds[:2], second.bounds[:2]) - 1
    hi = np.maximum(first.bounds[2:], second.bounds[2:]) + 1
    assert np.all(np.array(e.point) >= lo) and np.all(np.array(e.point) <= hi)


def test_began_bubble_and_static_polygon():
    w, tx = world()
    w.submit(tx.add(floor()).add(bubble(1, 150, 18.3, CONTACT)))
    frame, events = run(w, 90)
    assert_single_began(events, frame, (1, FLOOR), hint=(0, -1))


def test_began_bubble_and_bubble_without_events_for_uninterested_pairs():
    w, tx = world()
    w.submit(tx.add(floor()).add(bubble(2, 150, 18.3)).add(bubble(1, 150, 34.6, CONTACT)))
    frame, events = run(w, 90)
    assert_single_began(events, frame, (1, 2))
    assert all(set(e.objects) == {1, 2} for e in began(events))


def test_began_kinematic_polygon_and_bubble():
    w, tx = world()
    w.submit(tx.add(box(2, 150, 50, 40, 4, MotionRole.KINEMATIC)).add(bubble(1, 150, 62.3, CONTACT)))
    frame, events = run(w, 90)
    assert_single_began(events, frame, (1, 2))


def first_steps(w, steps, pair, touching):
    seen = {"began": None, "touch": None}

    def each(k, frame):
        if seen["touch"] is None and touching(frame):
            seen["touch"] = k
        if seen["began"] is None and began(frame.events, pair):
            seen["began"] = k
    run(w, steps, each)
    return seen


def test_began_arrives_in_the_first_step_of_contact_with_the_floor():
    w, tx = world()
    w.submit(tx.add(floor()).add(bubble(1, 150, 40, CONTACT)))
    seen = first_steps(w, 40, (1, FLOOR), lambda f: f.objects[1].bounds[1] <= 10.05)
    assert seen["touch"] is not None and seen["began"] == seen["touch"]


def test_began_arrives_in_the_first_step_of_contact_between_bubbles():
    w, tx = world()
    w.submit(tx.add(floor()).add(bubble(2, 150, 18.3)).add(bubble(1, 150, 60, CONTACT)))
    seen = first_steps(w, 60, (1, 2), lambda f: math.dist(f.objects[1].position, f.objects[2].position) <= 16.05)
    assert seen["touch"] is not None and seen["began"] == seen["touch"]


def test_began_impulse_is_the_step_end_contact_force_times_the_step():
    w, tx = world()
    w.submit(tx.add(floor()).add(bubble(1, 150, 40, CONTACT)))
    found = {}

    def each(k, frame):
        b = began(frame.events, (1, FLOOR))
        if b and not found:
            found["impulse"], found["d"] = b[0].impulse, frame.objects[1].position[1] - 10
    run(w, 40, each)
    eps = 1 - found["d"] / 8
    expected = 2000 * eps / ((1 - eps) * (1 - eps)) / 60
    assert eps > 0 and abs(found["impulse"] - expected) <= 0.02 * expected + 1e-4


def test_no_began_for_a_gap_within_the_separation_tolerance():
    w, tx = world(gravity=False)
    w.submit(tx.add(bubble(1, 100, 100, CONTACT)).add(bubble(2, 116.001, 100)))
    _, events = run(w, 6)
    assert began(events) == [] and ended(events) == []


def test_began_point_leans_toward_the_deeper_edge_in_a_corner():
    def corner_point(position):
        w, tx = world(gravity=False)
        corner = RigidBodyDescriptor(FLOOR, Polygon(((0, 0), (100, 0), (100, 10), (10, 10), (10, 60), (0, 60))),
                                     (100.0, 100.0))
        w.submit(tx.add(corner).add(bubble(1, *position, CONTACT)))
        _, events = run(w, 2)
        b = began(events, (1, FLOOR))
        assert len(b) == 1
        return b[0].point
    floor_deeper, wall_deeper = corner_point((117.5, 116.0)), corner_point((116.0, 117.5))
    assert floor_deeper[0] > 115 and floor_deeper[1] < 112
    assert wall_deeper[0] < 112 and wall_deeper[1] > 114.5


def test_ended_arrives_in_the_first_step_after_separation():
    w, tx = world()
    w.submit(tx.add(floor()).add(bubble(1, 150, 18.3, CONTACT)))
    run(w, 30)
    w.submit(WorldTransaction().apply_impulse(1, (0.0, 300.0)))
    seen = {"ended": None, "separated": None, "events": []}

    def each(k, frame):
        seen["events"] += frame.events
        if seen["separated"] is None and frame.objects[1].bounds[1] > 10.05:
            seen["separated"] = k
        if seen["ended"] is None and ended(frame.events):
            seen["ended"] = k
    run(w, 20, each)
    assert len(ended(seen["events"], (1, FLOOR))) == 1 and seen["ended"] == seen["separated"]


def test_ended_goes_to_the_remaining_partner_when_the_other_is_removed():
    w, tx = world()
    w.submit(tx.add(floor()).add(bubble(1, 150, 18.3, CONTACT)))
    _, events = run(w, 30)
    assert len(began(events)) == 1
    w.submit(WorldTransaction().remove(FLOOR))
    removal = w.advance(1.0 / 60)
    e = ended(removal.events)
    assert len(e) == 1 and set(e[0].objects) == {1, FLOOR}


def test_ended_goes_to_the_static_partner_when_the_only_bubble_is_removed():
    w, tx = world()
    w.submit(tx.add(floor(CONTACT)).add(bubble(1, 150, 18.3)))
    _, events = run(w, 30)
    assert len(began(events)) == 1
    w.submit(WorldTransaction().remove(1))
    e = ended(w.advance(1.0 / 60).events)
    assert len(e) == 1 and set(e[0].objects) == {1, FLOOR}


def test_a_pair_added_again_after_removing_everything_begins_again():
    w, tx = world()
    w.submit(tx.add(floor()).add(bubble(1, 150, 18.3, CONTACT)))
    _, events = run(w, 30)
    assert len(began(events)) == 1
    w.submit(WorldTransaction().remove(1).remove(FLOOR))
    run(w, 2)
    w.submit(WorldTransaction().add(floor()).add(bubble(1, 150, 17.0, CONTACT)))
    _, again = run(w, 30)
    assert len(began(again, (1, FLOOR))) == 1
    w.submit(WorldTransaction().apply_impulse(1, (0.0, 300.0)))
    _, launched = run(w, 20)
    assert len(ended(launched, (1, FLOOR))) == 1
