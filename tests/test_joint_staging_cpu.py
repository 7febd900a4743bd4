"""Joint staging in the world API against the reference's own cases (JointStagingTests.swift:78-140): a joint with a
bubble at either end is rejected as unsupportedJointBody for every kind, a rejected joint leaves the batch's state
unchanged, huge finite anchors, angles and distance parameters are rejected at staging (1e6 still passes the joint's
checks), removing a body removes its joints, and removing an unknown joint is jointNotFound. The reference's states
hold dynamic bodies next to bubbles (its stager does not check that; its stepper does), so the states here are built
directly; this world then rejects a transaction that leaves a dynamic body at its end, as its stepper would."""
import numpy as np

from bubblephysics_gb300 import world as W
from bubblephysics_gb300.rigid import Joint
from bubblephysics_gb300.world import (BubbleDescriptor, MotionRole as M, PhysicsMaterial, Polygon,
                                       RigidBodyDescriptor, TransactionRejectionReason as R, WorldTransaction)

REGION = (-100.0, -100.0, 100.0, 100.0)


def state_with(bubbles=(), boxes=()):
    state = W._State()
    state.materials[1] = PhysicsMaterial(1e9)
    for i, x in bubbles:
        desc = BubbleDescriptor(i, (x, 0.0), 2.0, 2.0, 1)
        state.bubbles[i] = W._Bubble(desc, np.asarray(desc.position, np.float32).copy(), np.zeros(2, np.float32))
    for i, x, role in boxes:
        desc = RigidBodyDescriptor(i, Polygon(((-1, -1), (1, -1), (1, 1), (-1, 1))), (x, 0.0), motion_role=role)
        state.bodies[i] = W._Body.of(desc)
    return state


def distance(jid, a, b):
    return Joint(jid, a, b, "distance", anchor_b=(0.0, 5.0), length=5.0)


def hinge(jid, a, b):
    return Joint(jid, a, b, "hinge")


def weld(jid, a, b):
    return Joint(jid, a, b, "weld")


def rejection(tx, state):
    _, receipts, events = W.stage([(7, tx)], state, REGION)
    assert not receipts
    (event,) = [e for e in events if e.kind == "transactionRejected"]
    return event.rejection


def test_a_joint_with_a_bubble_is_rejected_for_every_kind():
    state = state_with(bubbles=[(1, 0.0), (3, 10.0)], boxes=[(2, 5.0, M.DYNAMIC)])
    cases = [(hinge(1, 1, 2), 1), (hinge(1, 2, 1), 1), (weld(4, 1, 2), 4), (weld(5, 1, None), 5), (hinge(6, 1, 3), 6),
             (distance(1, 1, 2), 1), (distance(2, 1, None), 2), (distance(3, 1, 3), 3)]
    for joint, jid in cases:
        r = rejection(WorldTransaction().add_joint(joint), state)
        assert (r.operation_index, r.reason, r.detail) == (0, R.UNSUPPORTED_JOINT_BODY, jid), joint


def test_a_rejected_joint_transaction_leaves_the_state_unchanged():
    state = state_with(bubbles=[(3, 10.0)], boxes=[(1, 0.0, M.DYNAMIC), (2, 5.0, M.DYNAMIC)])
    bad = WorldTransaction().add_joint(distance(1, 1, 2)).add_joint(distance(2, 1, 3))
    after, receipts, events = W.stage([(7, bad)], state, REGION)
    assert after is state and not after.joints and not receipts
    (event,) = events
    assert (event.rejection.operation_index, event.rejection.reason, event.rejection.detail) == \
        (1, R.UNSUPPORTED_JOINT_BODY, 2)


def test_huge_finite_joint_values_are_rejected_at_staging():
    state = state_with(boxes=[(1, 0.0, M.DYNAMIC), (2, 5.0, M.DYNAMIC)])
    huge = 3e38
    cases = [(Joint(1, 1, 2, "weld", anchor_a=(huge, 0.0)), "joint.anchorA"),
             (Joint(1, 1, None, "weld", anchor_b=(0.0, -huge)), "joint.anchorB"),
             (Joint(1, 1, 2, "weld", reference_angle=huge), "joint.referenceAngle"),
             (Joint(1, 1, 2, "distance", length=huge), "joint.length"),
             (Joint(1, 1, 2, "distance", length=5.0, softness=huge), "joint.softness"),
             (Joint(1, 1, 2, "distance", length=5.0, damping=huge), "joint.damping"),
             (Joint(1, 1, 2, "hinge", limits=(-huge, 0.0)), "hinge.lower"),
             (Joint(1, 1, 2, "hinge", limits=(0.0, huge)), "hinge.upper"),
             (Joint(1, 1, 2, "hinge", motor=(huge, 1.0)), "hinge.motor.targetAngularVelocity")]
    for joint, name in cases:
        r = rejection(WorldTransaction().add_joint(joint), state)
        assert (r.operation_index, r.reason, r.detail) == (0, R.INVALID_VALUE, name), name
    # 1e6 passes the joint's checks; the transaction then ends with dynamic bodies, which this world does not step
    ok = Joint(1, 1, 2, "distance", anchor_a=(1e6, -1e6), length=1e6, softness=1e6, damping=1e6)
    r = rejection(WorldTransaction().add_joint(ok), state)
    assert (r.reason, r.detail) == (R.UNSUPPORTED_OPERATION, "validate")


def test_joint_ids_ends_and_removal():
    state = state_with(boxes=[(1, 0.0, M.DYNAMIC), (2, 5.0, M.STATIC), (3, -5.0, M.STATIC), (4, 9.0, M.PATH_DRIVEN)])
    assert W._add_joint(hinge(1, 1, 2), state) is None
    assert W._add_joint(hinge(1, 1, 3), state) == (R.DUPLICATE_JOINT_ID, 1)
    assert W._add_joint(weld(2, 2, 3), state) == (R.UNSUPPORTED_JOINT_BODY, 2)     # no movable body
    assert W._add_joint(weld(3, 1, 4), state) == (R.UNSUPPORTED_JOINT_BODY, 3)     # a path-driven end
    assert W._add_joint(weld(4, 1, 99), state) == (R.OBJECT_NOT_FOUND, 99)
    assert W._add_joint(weld(5, 1, 1), state) == (R.INVALID_VALUE, "joint.bodies")
    assert W._add_joint(distance(6, 1, None), state) is None
    reason, touched = W._apply(("removeJoint", 9), state, REGION)
    assert reason == (R.JOINT_NOT_FOUND, 9)
    reason, touched = W._apply(("remove", 1), state, REGION)  # the body takes both its joints with it
    assert reason is None and sorted(touched["removed_joints"]) == [1, 6] and not state.joints
