"""The host's part of a step for moving objects (MotionControllers.prepare and .feedback), against
MotionControllersPrepareTests.swift:8-160 and MotionControllersFeedbackTests.swift:8-62, on bubbles and kinematic
bodies (the cases on dynamic rigid bodies need the rigid solver, which is not built here). The host leaves a
force-driven bubble's velocity alone (forces, bands, motors and damping act on the device in every substep), zeroes a
static one, sets a path-driven one from its path, moves radius and material transitions, and reports feedback for
driven bubbles only, in id order."""
from dataclasses import replace

import numpy as np

from bubblephysics_gb300 import _native as N
from bubblephysics_gb300 import world as W
from bubblephysics_gb300.world import (BubbleDescriptor, BubbleDrivePolicy, BubbleWorld, Circle, DriveBlockingContact,
                                       ForceFieldDescriptor, KinematicDrive, MotionRole as M, MotorDrive,
                                       ParameterTransition, PathDrive, PhysicsMaterial, Polygon, RigidBodyDescriptor,
                                       WorldConfiguration, WorldTransaction)

REGION = (-1000.0, -1000.0, 1000.0, 1000.0)
DURATION = 1.0 / 60


def staged(tx, global_force=(0.0, 0.0)):
    state = W._State()
    state.global_force = global_force
    state, receipts, events = W.stage([(1, tx)], state, REGION)
    assert receipts, events
    return state


def test_force_driven_bubbles_keep_their_velocity_static_ones_stop_and_path_driven_ones_follow_the_path():
    """MotionControllersPrepareTests.swift:84-120."""
    start, policy = (30.0, -20.0), BubbleDrivePolicy(100.0)
    tx = WorldTransaction().update_physics_material(1, PhysicsMaterial(229.0, 0.6))
    for oid, x in ((11, 0.0), (12, 50.0), (13, 100.0), (14, 150.0), (15, 200.0)):
        tx = tx.add(BubbleDescriptor(oid, (x, 0.0), 1.0, 2.0, 1, velocity=start, drive_policy=policy))
    tx = tx.add(ForceFieldDescriptor(90, (0.0, 0.0), "directional", Circle(1000.0), force=(0.0, 40.0))) \
        .set_motor_drive(12, MotorDrive((5.0, 5.0), 3.0)).begin_player_drive(13, (103.0, 54.0)) \
        .set_path_drive(14, PathDrive(((150.0, 500.0),), 5.0)).set_motion(15, M.STATIC)
    state = staged(tx, global_force=(4.0, -10.0))
    W.advance_transitions(state, DURATION)
    W.prepare_paths(state, DURATION)
    for oid in (11, 12, 13):
        assert np.allclose(state.bubbles[oid].velocity, start, atol=1e-4) and state.bubbles[oid].angular_velocity == 0
    assert np.allclose(state.bubbles[14].velocity, (0.0, 5.0), atol=1e-4)
    assert tuple(state.bubbles[15].velocity) == (0.0, 0.0)


def test_the_collision_radius_follows_the_radius_transition():
    """MotionControllersPrepareTests.swift:122-136: half way through a transition from 12 to 24 over 2 s."""
    state = staged(WorldTransaction().update_physics_material(1, PhysicsMaterial(229.0))
                   .add(BubbleDescriptor(1, (0.0, 0.0), 12.0, 1.0, 1))
                   .start_transition(ParameterTransition(("bubbleRadius", 1), 24.0, 2.0)))
    W.advance_transitions(state, 1.0)
    assert abs(state.bubbles[1].desc.radius - 18.0) <= 1e-4


def test_a_material_parameter_transition_keeps_the_contact_stiffness():
    """MotionControllersPrepareTests.swift:35-47."""
    state = staged(WorldTransaction().update_physics_material(7, PhysicsMaterial(229.0, 0.1))
                   .start_transition(ParameterTransition(("physicsMaterial", 7, "damping"), 0.5, 1.0)))
    W.advance_transitions(state, DURATION)
    assert state.materials[7].damping != 0.1 and state.materials[7].contact_stiffness == 229.0


def test_a_kinematic_body_takes_its_velocity_from_its_drive_not_from_the_global_force():
    """MotionControllersPrepareTests.swift:138-160."""
    state = staged(WorldTransaction().add(RigidBodyDescriptor(1, Polygon(((0.0, 0.0), (2.0, 0.0), (2.0, 2.0),
                                                                          (0.0, 2.0))), (0.0, 0.0),
                                                              motion_role=M.KINEMATIC))
                   .set_kinematic_drive(1, KinematicDrive.velocity((600.0, 0.0), 1.5)), global_force=(0.0, -10.0))
    W.prepare_kinematic(state, DURATION)
    body = state.bodies[1]
    assert np.allclose(body.velocity, (600.0, 0.0), atol=1e-2) and abs(body.angular_velocity - 1.5) <= 1e-3


def feedback_world():
    world = BubbleWorld(WorldConfiguration(REGION))
    world._segment_owner = {}
    return world


def test_feedback_lists_only_driven_bubbles_in_id_order():
    """MotionControllersFeedbackTests.swift:24-41: a player-driven bubble without a target and dynamic bubbles give
    no entry; nothing changes without a blocker."""
    tx = WorldTransaction().update_physics_material(1, PhysicsMaterial(229.0))
    for oid in list(range(1, 61)) + [900, 300]:
        tx = tx.add(BubbleDescriptor(oid, (float(oid % 50) * 5, float(oid // 50) * 5), 1.0, 1.0, 1,
                                     drive_policy=BubbleDrivePolicy(10.0)))
    for oid in (900, 5, 300, 41):
        tx = tx.begin_player_drive(oid, (3.0, 4.0))
    tx = tx.set_path_drive(17, PathDrive(((40.0, 40.0),), 5.0))
    state = staged(tx)
    state.bubbles[8].desc = replace(state.bubbles[8].desc, motion_role=M.PLAYER_DRIVEN)  # no target
    before = {oid: (b.velocity.copy(), b.path_stopped) for oid, b in state.bubbles.items()}
    starts = {oid: b.position.copy() for oid, b in state.bubbles.items()}
    feedback = feedback_world()._drive_feedback(state, np.zeros(0, N.CONTACT_DTYPE), starts)
    assert [f.object_id for f in feedback] == [5, 17, 41, 300, 900]
    assert {f.object_id: f.target for f in feedback}[5] == (3.0, 4.0)
    assert {f.object_id: f.target for f in feedback}[17] == (40.0, 40.0)
    assert all(np.array_equal(b.velocity, before[oid][0]) and b.path_stopped == before[oid][1]
               for oid, b in state.bubbles.items())


def test_a_blocked_path_bubble_stops_and_only_its_record_changes():
    """MotionControllersFeedbackTests.swift:43-62: a contact whose normal (from the obstacle to the bubble) stands
    against the drive blocks both the path and the player drive; only the path stops for good."""
    tx = WorldTransaction().update_physics_material(1, PhysicsMaterial(229.0))
    for oid in range(1, 31):
        tx = tx.add(BubbleDescriptor(oid, (float(oid) * 5, 0.0), 1.0, 1.0, 1, drive_policy=BubbleDrivePolicy(10.0)))
    tx = tx.set_path_drive(12, PathDrive(((100.0, 0.0),), 5.0)).begin_player_drive(20, (200.0, 0.0))
    state = staged(tx)
    state.bubbles[12].velocity = np.array([3.0, 0.0], np.float32)
    contacts = np.zeros(2, N.CONTACT_DTYPE)
    for c, oid in zip(contacts, (12, 20)):  # a pair's normal runs from its first participant to its second
        c["participants"], c["kind"], c["normal"], c["point"] = (oid, 2), 0, (1.0, 0.0), (1.0, 1.0)
    starts = {oid: b.position.copy() for oid, b in state.bubbles.items()}
    velocities = {oid: b.velocity.copy() for oid, b in state.bubbles.items()}
    feedback = {f.object_id: f for f in feedback_world()._drive_feedback(state, contacts, starts)}
    blocker = DriveBlockingContact(2, (1.0, 1.0), (-1.0, 0.0))
    assert feedback[12].blocking_contact == blocker and feedback[12].is_stopped
    assert state.bubbles[12].path_stopped and state.bubbles[12].path_blocker == blocker
    assert tuple(state.bubbles[12].velocity) == (0.0, 0.0)
    assert feedback[20].blocking_contact == blocker and not feedback[20].is_stopped
    assert all(np.array_equal(b.velocity, velocities[oid]) for oid, b in state.bubbles.items() if oid != 12)
