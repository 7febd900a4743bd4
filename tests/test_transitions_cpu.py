"""Parameter transitions (ParameterTransition, MotionControllers.swift:215-275) through the world API on a stand-in
device world that forwards to the oracle, against the reference's own cases (RegionPolicyTests.swift:222-262): a
material's contact stiffness or damping moves linearly and is published a quarter of the way after a quarter of the
duration; a bubble whose radius shrinks leaves the region by its transitioned collider and its transition is dropped
with it. Also the curves, the global force as a vector transition and the staging rules."""
import math

import numpy as np
import pytest

from bubblephysics_gb300 import world as W
from bubblephysics_gb300.world import (BubbleDescriptor, BubbleWorld, ParameterTransition, PhysicsMaterial,
                                       TransactionRejectionReason as R, WorldConfiguration, WorldTransaction)
from test_world_api_oracle_cpu import OracleBackedWorld


@pytest.fixture(autouse=True)
def oracle_backed(monkeypatch):
    monkeypatch.setattr(W, "World", OracleBackedWorld)
    monkeypatch.setattr(W, "default_context", lambda: None)


def small_world():
    return BubbleWorld(WorldConfiguration((0.0, 0.0, 10.0, 10.0), fixed_time_step=0.25, maximum_backlog=10.0))


@pytest.mark.parametrize("parameter,start,expected", [("contactStiffness", 229.0, 229 + (0.5 - 229) * 0.25),
                                                      ("damping", 1.0, 1 + (0.5 - 1) * 0.25)])
def test_material_transitions_advance_the_published_value(parameter, start, expected):
    world = small_world()
    token = world.submit(WorldTransaction().update_physics_material("m", PhysicsMaterial(229.0, 1.0))
                         .start_transition(ParameterTransition(("physicsMaterial", "m", parameter), 0.5, 1.0)))
    frame = world.advance(0.25)
    assert frame.step_index == 1 and [r.token for r in frame.transaction_receipts] == [token]
    m = world.physics_materials["m"]
    value = m.contact_stiffness if parameter == "contactStiffness" else m.damping
    assert value == pytest.approx(expected, abs=1e-3)


def test_removal_uses_the_transitioning_collider_and_drops_the_transition():
    world = small_world()
    world.submit(WorldTransaction().update_physics_material("m", PhysicsMaterial(229.0))
                 .add(BubbleDescriptor(1, (9.0, 5.0), 1.0, 1.0, "m", velocity=(4.0, 0.0)))
                 .start_transition(ParameterTransition(("bubbleRadius", 1), 0.5, 10.0)))
    first = world.advance(0.25)
    assert first.objects[1].position[0] == pytest.approx(10.0, abs=1e-4)
    second = world.advance(0.25)  # x = 11 with radius 0.975: the whole collider left the region
    assert 1 not in second.objects and world._state.transitions == {} and world._state.transition_progress == {}


def test_curves():
    assert W.transition_curve("linear", 0.3) == pytest.approx(0.3)
    assert W.transition_curve("easeIn", 0.5) == pytest.approx(0.25)
    assert W.transition_curve("easeOut", 0.5) == pytest.approx(0.75)
    assert W.transition_curve("easeInOut", 0.5) == pytest.approx(0.5)
    assert W.transition_curve(("cubicBezier", 0.0, 0.0, 1.0, 1.0), 0.3) == pytest.approx(0.3, abs=1e-5)
    assert W.transition_curve(("cubicBezier", 0.4, 0.0, 0.6, 1.0), 1.0) == 1


def test_global_force_moves_as_a_vector_and_finishes_at_the_target():
    world = small_world()
    world.submit(WorldTransaction().start_transition(ParameterTransition(("globalForce",), (8.0, -4.0), 0.5)))
    world.advance(0.25)
    assert world.global_force == pytest.approx((4.0, -2.0))
    world.advance(0.25)
    assert world.global_force == pytest.approx((8.0, -4.0)) and world._state.transitions == {}


def test_a_growing_bubble_takes_its_radius_into_the_step():
    world = BubbleWorld(WorldConfiguration((-100.0, -100.0, 100.0, 100.0)))
    world.submit(WorldTransaction().update_physics_material("m", PhysicsMaterial(229.0, 1.0))
                 .add(BubbleDescriptor(1, (0.0, 0.0), 6.0, 1.0, "m"))
                 .start_transition(ParameterTransition(("bubbleRadius", 1), 12.0, 1.0, "easeInOut")))
    radii = []
    for _ in range(70):
        world.advance(1.0 / 60)
        radii.append(world._state.bubbles[1].desc.radius)
    assert radii[0] > 6.0 and all(b >= a for a, b in zip(radii, radii[1:])) and radii[-1] == 12.0


def test_staging_rules():
    world = small_world()
    world.submit(WorldTransaction().update_physics_material("m", PhysicsMaterial(229.0)))
    world.advance(0.25)
    cases = [(ParameterTransition(("globalForce",), 3.0, 1.0), R.INCOMPATIBLE_TRANSITION_VALUE),
             (ParameterTransition(("bubbleRadius", 9), 1.0, 1.0), R.OBJECT_NOT_FOUND),
             (ParameterTransition(("physicsMaterial", "none", "damping"), 1.0, 1.0), R.PHYSICS_MATERIAL_NOT_FOUND),
             (ParameterTransition(("physicsMaterial", "m", "damping"), 1.0, math.nan), R.INVALID_VALUE),
             (ParameterTransition(("physicsMaterial", "m", "damping"), 1.0, -1.0), R.INVALID_VALUE),
             (ParameterTransition(("physicsMaterial", "m", "damping"), 1.0, 1.0, ("cubicBezier", 0.8, 0, 0.2, 1)),
              R.INVALID_VALUE)]
    for tr, reason in cases:
        _, rec, ev = W.stage([(5, WorldTransaction().start_transition(tr))], world._state, (0.0, 0.0, 10.0, 10.0))
        assert rec == [] and ev[0].rejection.reason == reason, tr
