"""Motion roles at staging, against the reference's own cases: KinematicStagingTests.swift:37-90 (kinematic is for
bodies only: a kinematic bubble is refused on add, replace and setMotion; a kinematic polygon carries its drive; a
drive for another role or a missing object is refused; leaving the kinematic role discards the drive; a non-finite
drive is refused) and DynamicRigidExclusionTests.swift:62-160 (bubbles and dynamic bodies never share a world: judged
on the state after the whole transaction and reported at its last operation; static and kinematic bodies share it;
one rejected transaction does not stop the next). Worlds of dynamic bodies alone need the rigid solver, which is not
built here: they are refused as unsupported."""
import math

import pytest

from bubblephysics_gb300 import world as W
from bubblephysics_gb300.world import (BubbleDescriptor, Circle, MotionRole as M, PhysicsMaterial, Polygon,
                                       RigidBodyDescriptor, TransactionRejectionReason as R, WorldTransaction)

REGION = (-100.0, -100.0, 100.0, 100.0)
EXCLUSION = R.UNSUPPORTED_BUBBLE_WITH_DYNAMIC_RIGID_BODY


def bubble(i, role=M.DYNAMIC, at=(-50.0, 0.0)):
    return BubbleDescriptor(i, at, 2.0, 2.0, "soft", motion_role=role)


def body(i, role, at=(50.0, 0.0)):
    return RigidBodyDescriptor(i, Circle(3.0), at, motion_role=role)


def square(i, role):
    return RigidBodyDescriptor(i, Polygon(((0, 0), (2, 0), (2, 2), (0, 2))), (5.0, 0.0), motion_role=role)


def initial(tx=WorldTransaction()):
    tx = WorldTransaction(WorldTransaction().update_physics_material("soft", PhysicsMaterial(1e9)).operations + tx.operations)
    state, rec, ev = W.stage([(1, tx)], W._State(), REGION)
    assert rec, ev
    return state


def outcome(state, *txs):
    new, rec, ev = W.stage([(10 + k, tx) for k, tx in enumerate(txs)], state, REGION)
    return new, rec, [e.rejection for e in ev if e.kind == "transactionRejected"]


def rejected(state, tx, reason, index=0, detail=None):
    new, rec, rej = outcome(state, tx)
    assert rec == [] and len(rej) == 1 and (rej[0].operation_index, rej[0].reason) == (index, reason), rej
    if detail is not None:
        assert rej[0].detail == detail
    assert new is state


def accepted(state, tx):
    new, rec, rej = outcome(state, tx)
    assert len(rec) == 1 and rej == [], rej
    return new


def test_kinematic_bubble_is_refused_on_add_replace_and_set_motion():
    rejected(initial(), WorldTransaction().add(bubble(1, M.KINEMATIC)), R.UNSUPPORTED_MOTION_ROLE, detail=(1, M.KINEMATIC))
    seeded = initial(WorldTransaction().add(bubble(1)))
    rejected(seeded, WorldTransaction().replace(1, bubble(1, M.KINEMATIC)), R.UNSUPPORTED_MOTION_ROLE, detail=(1, M.KINEMATIC))
    rejected(seeded, WorldTransaction().set_motion(1, M.KINEMATIC), R.UNSUPPORTED_MOTION_ROLE, detail=(1, M.KINEMATIC))


def test_kinematic_polygon_carries_its_drive():
    seeded = initial(WorldTransaction().add(square(2, M.STATIC)))
    kinematic = accepted(seeded, WorldTransaction().set_motion(2, M.KINEMATIC))
    assert kinematic.bodies[2].desc.motion_role == M.KINEMATIC
    driven = accepted(kinematic, WorldTransaction().set_kinematic_drive(2, (1.0, 0.0), 0.5))
    assert driven.bodies[2].desc.velocity == (1.0, 0.0) and driven.bodies[2].desc.angular_velocity == 0.5


def test_drive_for_another_role_or_a_missing_object_is_refused():
    seeded = initial(WorldTransaction().add(square(2, M.STATIC)).add(bubble(1)))
    rejected(seeded, WorldTransaction().set_kinematic_drive(2, (3.0, 3.0)), R.INCOMPATIBLE_MOTION_ROLE, detail=2)
    rejected(seeded, WorldTransaction().set_kinematic_drive(1, (3.0, 3.0)), R.INCOMPATIBLE_MOTION_ROLE, detail=1)
    rejected(seeded, WorldTransaction().set_kinematic_drive(9, (3.0, 3.0)), R.OBJECT_NOT_FOUND)


def test_leaving_the_kinematic_role_discards_the_drive():
    seeded = initial(WorldTransaction().add(square(2, M.KINEMATIC)).set_kinematic_drive(2, (1.0, 0.0)))
    assert seeded.bodies[2].desc.velocity == (1.0, 0.0)
    static = accepted(seeded, WorldTransaction().set_motion(2, M.STATIC))
    assert static.bodies[2].desc.velocity == (0.0, 0.0) and static.bodies[2].desc.angular_velocity == 0.0


@pytest.mark.parametrize("velocity,omega", [((math.nan, 0.0), 0.0), ((0.0, math.inf), 0.0), ((1.0, 0.0), math.nan)])
def test_non_finite_drive_is_refused(velocity, omega):
    seeded = initial(WorldTransaction().add(square(2, M.KINEMATIC)))
    rejected(seeded, WorldTransaction().set_kinematic_drive(2, velocity, omega), R.INVALID_VALUE)


@pytest.mark.parametrize("role", W.DYNAMIC_ROLES)
def test_dynamic_body_next_to_bubbles_is_refused_either_way(role):
    rejected(initial(WorldTransaction().add(bubble(1))), WorldTransaction().add(body(100, role)), EXCLUSION)


def test_static_and_kinematic_bodies_share_a_world_with_bubbles():
    with_bubble = initial(WorldTransaction().add(bubble(1)))
    accepted(with_bubble, WorldTransaction().add(body(100, M.STATIC)))
    accepted(with_bubble, WorldTransaction().add(body(100, M.KINEMATIC)))
    with_bodies = initial(WorldTransaction().add(body(100, M.STATIC)).add(body(101, M.KINEMATIC, (60.0, 0.0))))
    accepted(with_bodies, WorldTransaction().add(bubble(1)))


def test_replacing_or_turning_a_body_dynamic_next_to_bubbles_is_refused():
    state = initial(WorldTransaction().add(bubble(1)).add(body(100, M.STATIC)))
    rejected(state, WorldTransaction().replace(100, body(100, M.DYNAMIC)), EXCLUSION)
    accepted(state, WorldTransaction().replace(100, body(100, M.KINEMATIC)))
    for role in (M.DYNAMIC, M.MOTOR_DRIVEN, M.PATH_DRIVEN):
        rejected(state, WorldTransaction().set_motion(100, role), EXCLUSION)
    accepted(state, WorldTransaction().set_motion(100, M.KINEMATIC))
    accepted(initial(WorldTransaction().add(bubble(1))), WorldTransaction().set_motion(1, M.STATIC))


def test_the_rule_looks_at_the_state_after_the_whole_transaction():
    empty = initial()
    rejected(empty, WorldTransaction().add(bubble(1)).add(body(100, M.DYNAMIC)), EXCLUSION, index=1)
    rejected(empty, WorldTransaction().add(bubble(1)).add(body(100, M.DYNAMIC)).set_global_force((0.0, -1.0)), EXCLUSION,
             index=2)
    accepted(empty, WorldTransaction().add(bubble(1)).add(body(100, M.DYNAMIC)).remove(100))


def test_a_rejection_does_not_stop_the_next_transaction():
    state = initial(WorldTransaction().add(bubble(1)))
    new, rec, rej = outcome(state, WorldTransaction().add(body(100, M.DYNAMIC)), WorldTransaction().add(body(101, M.STATIC)))
    assert [r.token for r in rec] == [11] and [(r.operation_index, r.reason) for r in rej] == [(0, EXCLUSION)]
    assert 100 not in new.bodies and 101 in new.bodies


def test_worlds_of_dynamic_bodies_alone_need_the_rigid_solver():
    rejected(initial(), WorldTransaction().add(body(100, M.DYNAMIC)), R.UNSUPPORTED_OPERATION)
