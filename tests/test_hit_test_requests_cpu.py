"""The asynchronous hit test (BubbleWorld.hitTest) through the world API on a stand-in device world that forwards to
the oracle, against the reference's own cases (BubbleWorldCompletionTests.swift:380-507): requests reach the next step
in order and each gets its own answer on that step's state; a paused world keeps them waiting until the first step
after resume; a failed world answers waiting and later requests with None at once; a cancelled request leaves the
queue before the step."""
import math

import pytest

from bubblephysics_gb300 import world as W
from bubblephysics_gb300.world import (BubbleDescriptor, BubbleWorld, Circle, PhysicsMaterial, RigidBodyDescriptor,
                                       WorldConfiguration, WorldFailureReason, WorldTransaction)
from test_world_api_oracle_cpu import OracleBackedWorld


@pytest.fixture(autouse=True)
def oracle_backed(monkeypatch):
    monkeypatch.setattr(W, "World", OracleBackedWorld)
    monkeypatch.setattr(W, "default_context", lambda: None)


def scene():
    world = BubbleWorld(WorldConfiguration((-100.0, -100.0, 100.0, 100.0)))
    world.submit(WorldTransaction().update_physics_material("m", PhysicsMaterial(229.0))
                 .add(BubbleDescriptor(5, (0.0, 0.0), 5.0, 1.0, "m", velocity=(60.0, 0.0)))
                 .add(RigidBodyDescriptor(7, Circle(4.0), (40.0, 0.0))))
    return world


def test_requests_reach_the_next_step_in_order_with_their_own_answers():
    world = scene()
    requests = [world.request_hit_test(p) for p in ((5.5, 0.0), (-5.5, 0.0), (40.0, 1.0))]
    assert world.pending_hit_test_count == 3 and not any(r.done for r in requests)
    world.advance(1.0 / 60)  # the bubble moved one unit: (5.5, 0) is inside, (-5.5, 0) is not
    assert [r.result for r in requests] == [5, None, 7] and all(r.done for r in requests)
    assert world.pending_hit_test_count == 0


def test_a_paused_world_keeps_requests_waiting():
    world = scene()
    world.pause()
    request = world.request_hit_test((40.0, 0.0))
    world.advance(1.0)
    assert not request.done and world.pending_hit_test_count == 1
    world.resume()
    world.advance(1.0 / 60)
    assert request.done and request.result == 7


def test_a_failed_world_answers_none_at_once():
    world = BubbleWorld(WorldConfiguration((-100.0, -100.0, 100.0, 100.0), substep_split_multiplier=2000.0))
    world.submit(WorldTransaction().update_physics_material("m", PhysicsMaterial(229.0))
                 .add(BubbleDescriptor(1, (0.0, 0.0), 12.0, 0.36, "m", velocity=(0.0, 100.0)))
                 .add(RigidBodyDescriptor(2, Circle(20.0), (0.0, 50.0))))
    waiting = world.request_hit_test((0.0, 0.0))
    for _ in range(60):
        world.advance(1.0 / 60)
        if world.diagnostics.failure_reason is not None:
            break
    assert world.diagnostics.failure_reason is not None
    assert waiting.done and waiting.result is None and world.pending_hit_test_count == 0
    later = world.request_hit_test((0.0, 50.0))
    assert later.done and later.result is None


def test_a_cancelled_request_leaves_before_the_step():
    world = scene()
    cancelled, kept = world.request_hit_test((0.0, 0.0)), world.request_hit_test((40.0, 0.0))
    cancelled.cancel()
    assert cancelled.done and cancelled.result is None and world.pending_hit_test_count == 1
    world.advance(1.0 / 60)
    assert kept.result == 7


def test_non_finite_points_answer_none_at_once():
    world = scene()
    assert world.request_hit_test((math.nan, 0.0)).done and world.pending_hit_test_count == 0


def test_a_world_without_bubbles_answers_from_its_bodies():
    world = BubbleWorld(WorldConfiguration((-100.0, -100.0, 100.0, 100.0)))
    world.submit(WorldTransaction().add(RigidBodyDescriptor(7, Circle(4.0), (40.0, 0.0)))
                 .add(RigidBodyDescriptor(9, Circle(4.0), (41.0, 0.0))))
    request = world.request_hit_test((40.5, 0.0))
    world.advance(1.0 / 60)
    assert request.result == 9
