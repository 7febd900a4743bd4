"""Transitions and collision filters on the model side, against TransitionTests.swift:17-58 (a new transition on the
same parameter replaces the running one from the current value; every curve reaches its end and simulation time is
independent of how it is partitioned; stiffness and damping move together) and CollisionFilterTests.swift:17-47 (the
default filter collides with everything; a collision needs each category in the other's mask; descriptors carry their
filter and default to the default one)."""
import numpy as np
import pytest

from bubblephysics_gb300 import world as W
from bubblephysics_gb300.world import (BubbleDescriptor, CollisionFilter, ParameterTransition, PhysicsMaterial, Polygon,
                                       RigidBodyDescriptor, WorldTransaction)

REGION = (-20.0, -20.0, 20.0, 20.0)


def staged(tx, state=None):
    state, receipts, events = W.stage([(1, tx)], state or W._State(), REGION)
    assert receipts, events
    return state


def initial(damping=0.0):
    return staged(WorldTransaction().update_physics_material(1, PhysicsMaterial(200.0, damping))
                  .add(BubbleDescriptor(1, (0.0, 0.0), 1.0, 1.0, 1)))


def test_a_new_transition_on_the_same_parameter_replaces_the_running_one():
    state = staged(WorldTransaction().start_transition(ParameterTransition(("physicsMaterial", 1, "damping"), 10.0, 2.0)),
                   initial(damping=2.0))
    W.advance_transitions(state, 0.5)
    assert state.materials[1].damping == 4.0
    state = staged(WorldTransaction().start_transition(ParameterTransition(("physicsMaterial", 1, "damping"), 0.0, 1.0)),
                   state)
    W.advance_transitions(state, 0.5)
    assert state.materials[1].damping == 2.0
    W.advance_transitions(state, 0.5)
    assert state.materials[1].damping == 0.0 and not state.transitions


@pytest.mark.parametrize("curve", ["linear", "easeIn", "easeOut", "easeInOut", ("cubicBezier", 0.2, 0.0, 0.8, 1.0)])
def test_every_curve_reaches_its_end_and_time_is_partition_independent(curve):
    tx = WorldTransaction().start_transition(ParameterTransition(("globalForce",), (8.0, 4.0), 1.0, curve))
    a = staged(tx, initial())
    b = staged(tx, initial())
    W.advance_transitions(a, 0.5)
    for _ in range(4):
        W.advance_transitions(b, 0.125)
    assert a.global_force == b.global_force
    W.advance_transitions(a, 0.5)
    assert tuple(a.global_force) == (8.0, 4.0)


def test_stiffness_and_damping_transitions_move_together():
    state = staged(WorldTransaction()
                   .start_transition(ParameterTransition(("physicsMaterial", 1, "contactStiffness"), 400.0, 1.0))
                   .start_transition(ParameterTransition(("physicsMaterial", 1, "damping"), 0.6, 1.0)), initial())
    W.advance_transitions(state, 0.5)
    assert state.materials[1].contact_stiffness == 300.0 and abs(state.materials[1].damping - 0.3) <= 1e-6
    W.advance_transitions(state, 0.5)
    assert state.materials[1].contact_stiffness == 400.0 and state.materials[1].damping == float(np.float32(0.6))


def test_the_default_filter_collides_with_everything_including_itself():
    default, other = CollisionFilter(), CollisionFilter(0x80000000, 0x1)
    assert default.collides_with(default)
    assert default.collides_with(other) == bool(other.mask & default.category)
    assert default.mask == 0xFFFFFFFF and default.category != 0


def test_a_collision_needs_each_category_in_the_others_mask():
    a, b, one_sided = CollisionFilter(0b01, 0b10), CollisionFilter(0b10, 0b01), CollisionFilter(0b10, 0b00)
    assert a.collides_with(b) and b.collides_with(a)
    assert not a.collides_with(one_sided) and not one_sided.collides_with(a)
    assert not a.collides_with(a)


def test_descriptors_carry_their_filter_and_default_to_the_default_filter():
    f = CollisionFilter(4, 8)
    assert BubbleDescriptor(1, (0.0, 0.0), 1.0, 1.0, 1, filter=f).filter == f
    assert RigidBodyDescriptor(2, Polygon(((0.0, 0.0), (1.0, 0.0), (0.0, 1.0))), (0.0, 0.0), filter=f).filter == f
    assert BubbleDescriptor(3, (0.0, 0.0), 1.0, 1.0, 1).filter == CollisionFilter()
