"""The staging of transactions against the reference's own cases, TransactionStagerTests.swift:25-620, on this path's
`stage` (the state, receipts and events of one step boundary). The scene is the reference test's: a region of
200 x 200 about the origin, a bubble material of K_c 1e9, bubbles of radius 2 and mass 2. Cases on merges, splits,
joints, dynamic rigid bodies and material kinds have no counterpart here (those operations are rejected as
unsupported; bodies take no material)."""
import math

import numpy as np

from bubblephysics_gb300 import world as W
from bubblephysics_gb300.world import (BubbleDescriptor, BubbleDrivePolicy, Capsule, Circle, ForceFieldDescriptor,
                                       MotionRole as M, ParameterTransition, Polygon, PhysicsMaterial,
                                       RigidBodyDescriptor, SensorDescriptor, TransactionRejectionReason as R,
                                       WorldTransaction)

REGION = (-100.0, -100.0, 100.0, 100.0)
OUTSIDE = W.STATIC_OUTSIDE


def resources():
    return WorldTransaction().update_physics_material(1, PhysicsMaterial(1e9)).update_render_material(1)


def bubble(i, role=M.DYNAMIC, position=(0.0, 0.0), policy=None, mass=2.0):
    return BubbleDescriptor(i, position, 2.0, mass, 1, motion_role=role, drive_policy=policy)


def stage(tx, state=None, token=1):
    return W.stage([(token, tx)], state or W._State(), REGION)


def staged(tx, state=None):
    state, receipts, events = stage(tx, state)
    assert receipts, events
    return state


def rejection(tx, state=None):
    _, receipts, events = stage(tx, state)
    assert not receipts
    rejected = [e for e in events if e.kind == "transactionRejected"]
    assert len(rejected) == 1
    return rejected[0].rejection


def test_a_rejected_transaction_publishes_no_partial_object_or_resource_change():
    """TransactionStagerTests.swift:25-34: the rejection names the failing operation's index."""
    initial = W._State()
    r = rejection(resources().add(bubble(1)).remove(999), initial)
    assert r.operation_index == 3 and r.reason == R.OBJECT_NOT_FOUND
    assert not initial.bubbles and not initial.materials


def test_accepted_transactions_apply_in_submission_order_at_one_step_boundary():
    """TransactionStagerTests.swift:36-47."""
    txs = [resources().add(bubble(1)), WorldTransaction().apply_impulse(1, (6.0, 0.0)),
           WorldTransaction().set_global_force((0.0, -5.0))]
    state, receipts, _ = W.stage(list(zip([30, 10, 20], txs)), W._State(), REGION)
    assert tuple(state.bubbles[1].velocity) == (3.0, 0.0)
    assert tuple(state.global_force) == (0.0, -5.0)
    assert [r.token for r in receipts] == [30, 10, 20]


def test_an_invalid_command_has_a_structured_rejection_and_the_next_transaction_applies():
    """TransactionStagerTests.swift:49-64."""
    initial = staged(resources().add(bubble(1)))
    bad = WorldTransaction().set_global_force((7.0, 8.0)).apply_impulse(1, (math.nan, 0.0))
    state, receipts, events = W.stage([(3, bad), (4, WorldTransaction().set_global_force((1.0, 2.0)))], initial, REGION)
    assert [(e.kind, e.token, e.rejection.operation_index, e.rejection.reason, e.rejection.detail) for e in events] == \
        [("transactionRejected", 3, 1, R.INVALID_VALUE, "impulse")]
    assert [r.token for r in receipts] == [4]
    assert tuple(state.global_force) == (1.0, 2.0) and tuple(initial.global_force) == (0.0, 0.0)
    assert tuple(state.bubbles[1].velocity) == (0.0, 0.0)


def test_missing_materials_are_rejected():
    """TransactionStagerTests.swift:82-89 (the material-kind cases aside)."""
    assert rejection(WorldTransaction().add(bubble(1))).reason == R.PHYSICS_MATERIAL_NOT_FOUND


def test_duplicate_ids_and_static_geometry_outside_the_region_are_atomic():
    """TransactionStagerTests.swift:91-97: a static bubble must lie wholly in the region, at add and at setMotion."""
    assert rejection(resources().add(bubble(1)).add(bubble(1))).reason == R.DUPLICATE_OBJECT_ID
    for tx in (resources().add(bubble(1, M.STATIC, (100.0, 0.0))),
               resources().add(bubble(1, position=(100.0, 0.0))).set_motion(1, M.STATIC)):
        r = rejection(tx)
        assert (r.reason, r.detail) == (R.INVALID_VALUE, OUTSIDE)


def test_a_completed_radius_transition_cannot_make_a_bubble_static_outside_the_region():
    """TransactionStagerTests.swift:99-115: region 20 x 20, a bubble at (8, 0) grown to radius 3 in one second may
    not turn static."""
    region = (-10.0, -10.0, 10.0, 10.0)
    state, receipts, _ = W.stage([(1, resources().add(BubbleDescriptor(1, (8.0, 0.0), 1.0, 1.0, 1))
                                   .start_transition(ParameterTransition(("bubbleRadius", 1), 3.0, 1.0)))],
                                 W._State(), region)
    assert receipts
    W.advance_transitions(state, 1.0)
    assert state.bubbles[1].desc.radius == 3.0 and not state.transitions
    _, receipts, events = W.stage([(2, WorldTransaction().set_motion(1, M.STATIC))], state, region)
    assert not receipts and (events[0].rejection.reason, events[0].rejection.detail) == (R.INVALID_VALUE, OUTSIDE)
    assert state.bubbles[1].desc.motion_role == M.DYNAMIC


def test_drive_lifecycle_and_invalid_roles():
    """TransactionStagerTests.swift:117-128."""
    initial = staged(resources().add(bubble(1, policy=BubbleDrivePolicy(30.0))))
    driven = staged(WorldTransaction().begin_player_drive(1, (2.0, 3.0)).update_player_drive(1, (4.0, 5.0)), initial)
    assert driven.bubbles[1].desc.motion_role == M.PLAYER_DRIVEN and driven.bubbles[1].drive_target == (4.0, 5.0)
    ended = staged(WorldTransaction().end_player_drive(1), driven)
    assert ended.bubbles[1].desc.motion_role == M.DYNAMIC and ended.bubbles[1].drive_target is None
    r = rejection(WorldTransaction().update_player_drive(1, (0.0, 0.0)), initial)
    assert (r.reason, r.detail) == (R.DRIVE_NOT_ACTIVE, 1)
    r = rejection(WorldTransaction().apply_impulse(1, (1.0, 0.0)), driven)
    assert (r.reason, r.detail) == (R.INCOMPATIBLE_MOTION_ROLE, 1)


def test_a_transition_replaces_the_one_on_its_target_and_an_invalid_one_is_atomic():
    """TransactionStagerTests.swift:130-140."""
    initial = staged(resources().add(bubble(1)))
    first = ParameterTransition(("bubbleRadius", 1), 4.0, 2.0)
    second = ParameterTransition(("bubbleRadius", 1), 7.0, 3.0)
    changed = staged(WorldTransaction().start_transition(first).start_transition(second), initial)
    assert changed.transitions[("bubbleRadius", 1)] == second
    r = rejection(WorldTransaction().start_transition(first)
                  .start_transition(ParameterTransition(("globalForce",), 3.0, 1.0)), initial)
    assert r.reason == R.INCOMPATIBLE_TRANSITION_VALUE and r.operation_index == 1
    assert not initial.transitions


def test_commands_reject_invalid_numbers_and_unsupported_object_kinds():
    """TransactionStagerTests.swift:176-195."""
    initial = staged(resources().add(bubble(1, policy=BubbleDrivePolicy(30.0))))
    assert rejection(WorldTransaction().set_global_force((math.inf, 0.0)), initial).reason == R.INVALID_VALUE
    assert rejection(WorldTransaction().begin_player_drive(1, (0.0, math.nan)), initial).reason == R.INVALID_VALUE
    cases = [(WorldTransaction().begin_player_drive(1, (0.0, 0.0)).begin_player_drive(1, (0.0, 0.0)),
              R.DRIVE_ALREADY_ACTIVE),
             (WorldTransaction().end_player_drive(1), R.DRIVE_NOT_ACTIVE),
             (WorldTransaction().set_motion(1, M.PLAYER_DRIVEN), R.DRIVE_NOT_ACTIVE),
             (WorldTransaction().replace(1, bubble(2)), R.REPLACEMENT_ID_MISMATCH)]
    for tx, reason in cases:
        assert rejection(tx, initial).reason == reason
    ranges = staged(WorldTransaction().add(SensorDescriptor(2, Circle(1.0), (0.0, 0.0)))
                    .add(ForceFieldDescriptor(3, (0.0, 0.0), "directional", Circle(1.0), force=(1.0, 0.0))), initial)
    for tx, oid in ((WorldTransaction().apply_impulse(2, (1.0, 0.0)), 2),
                    (WorldTransaction().begin_player_drive(3, (1.0, 0.0)), 3),
                    (WorldTransaction().set_motion(2, M.DYNAMIC), 2)):
        r = rejection(tx, ranges)
        assert (r.reason, r.detail) == (R.INCOMPATIBLE_OBJECT_KIND, oid)


def test_transition_targets_validate_their_values_and_removed_objects_lose_their_schedules():
    """TransactionStagerTests.swift:211-234."""
    initial = staged(resources().add(bubble(1)))
    scheduled = staged(WorldTransaction()
                       .start_transition(ParameterTransition(("globalForce",), (0.0, -3.0), 0.0))
                       .start_transition(ParameterTransition(("physicsMaterial", 1, "damping"), 2.0, 1.0))
                       .start_transition(ParameterTransition(("bubbleRadius", 1), 3.0, 1.0)), initial)
    assert len(scheduled.transitions) == 3
    removed, receipts, _ = stage(WorldTransaction().remove(1), scheduled)
    W._drop_transitions_of(removed, {i for r in receipts for i in r.removed_object_ids})
    assert len(removed.transitions) == 2 and ("bubbleRadius", 1) not in removed.transitions
    cases = [(ParameterTransition(("globalForce",), (0.0, 0.0), math.nan), "transition.duration"),
             (ParameterTransition(("globalForce",), (0.0, 0.0), -1.0), "transition.duration"),
             (ParameterTransition(("physicsMaterial", 1, "restitution"), 2.0, 1.0), "transition.material"),
             (ParameterTransition(("bubbleRadius", 1), 0.0, 1.0), "transition.radius"),
             (ParameterTransition(("globalForce",), (0.0, 0.0), 1.0, ("cubicBezier", 1.0, 0.0, 0.0, 1.0)),
              "transition.curve")]
    for transition, detail in cases:
        r = rejection(WorldTransaction().start_transition(transition), initial)
        assert (r.reason, r.detail) == (R.INVALID_VALUE, detail), transition


def test_a_rejected_batch_leaks_no_events_receipts_or_shared_resource_updates():
    """TransactionStagerTests.swift:236-248."""
    initial = staged(resources().add(bubble(1)))
    tx = WorldTransaction().remove(1).add(bubble(2)).update_render_material(1) \
        .update_physics_material(1, PhysicsMaterial(1e9)).remove(999)
    state, receipts, events = stage(tx, initial)
    assert set(state.bubbles) == {1} and state.materials == initial.materials
    assert not receipts and [e.kind for e in events] == ["transactionRejected"]


def test_a_static_motion_change_validates_an_already_scheduled_radius_transition():
    """TransactionStagerTests.swift:250-256."""
    initial = staged(resources().add(bubble(1)))
    r = rejection(WorldTransaction().start_transition(ParameterTransition(("bubbleRadius", 1), 200.0, 1.0))
                  .set_motion(1, M.STATIC), initial)
    assert (r.reason, r.detail) == (R.INVALID_VALUE, OUTSIDE)


def test_an_invalid_polygon_rolls_back_the_valid_object_and_resource_changes():
    """TransactionStagerTests.swift:258-270: a static polygon at (100, 100) reaches out of the region."""
    initial = W._State()
    outside = RigidBodyDescriptor(2, Polygon(((0.0, 0.0), (2.0, 0.0), (0.0, 2.0))), (100.0, 100.0))
    tx = resources().add(bubble(1)).update_physics_material(2, PhysicsMaterial(1e9)).add(outside)
    state, receipts, events = stage(tx, initial)
    assert not state.bubbles and not state.bodies and not state.materials and not receipts
    r = events[0].rejection
    assert (r.operation_index, r.reason, r.detail) == (4, R.INVALID_VALUE, OUTSIDE)


def test_circle_and_capsule_bodies_are_staged_and_published_with_their_kind_and_bounds():
    """TransactionStagerTests.swift:272-294 (as kinematic bodies: dynamic ones need the rigid solver)."""
    circle = RigidBodyDescriptor(1, Circle(2.0), (10.0, 20.0), motion_role=M.KINEMATIC)
    capsule = RigidBodyDescriptor(2, Capsule(3.0, 1.0), (-10.0, 5.0), angle=math.pi / 2, motion_role=M.KINEMATIC)
    state = staged(resources().add(circle).add(capsule))
    lo, hi = W.shape_box(W._body_shape(state.bodies[1]))
    assert tuple(lo) == (8.0, 18.0) and tuple(hi) == (12.0, 22.0)
    lo, hi = W.shape_box(W._body_shape(state.bodies[2]))
    assert np.allclose(lo, (-11.0, 1.0), atol=1e-5) and np.allclose(hi, (-9.0, 9.0), atol=1e-5)


def test_a_static_circle_outside_the_region_is_rejected_at_staging():
    """TransactionStagerTests.swift:296-302."""
    r = rejection(resources().add(RigidBodyDescriptor(1, Circle(5.0), (98.0, 0.0))))
    assert (r.reason, r.detail) == (R.INVALID_VALUE, OUTSIDE)


def test_a_very_soft_material_and_a_large_radius_are_not_rejected():
    """TransactionStagerTests.swift:412-447: staging holds no stiffness-to-size ratio against a bubble."""
    state = staged(WorldTransaction().update_physics_material(1, PhysicsMaterial(1e-3))
                   .add(BubbleDescriptor(1, (0.0, 0.0), 90.0, 1e-3, 1)))
    assert state.bubbles[1].desc.radius == 90.0


def test_add_and_replace_reject_a_band_bubble_with_too_small_a_mass():
    """TransactionStagerTests.swift:449-463: K_band <= m / (16 dt^2) at dt = 1/60."""
    light = bubble(1, policy=BubbleDrivePolicy(60.0), mass=0.1)
    r = rejection(resources().add(light))
    assert (r.reason, r.detail) == (R.INVALID_VALUE, "drive.bandStiffness")
    initial = staged(resources().add(bubble(1)))
    r = rejection(WorldTransaction().replace(1, light), initial)
    assert (r.reason, r.detail) == (R.INVALID_VALUE, "drive.bandStiffness")


def test_begin_player_drive_is_rejected_for_a_bubble_without_a_drive_policy_or_a_body():
    """TransactionStagerTests.swift:503-525 and 599-620."""
    initial = staged(resources().add(bubble(1)).add(RigidBodyDescriptor(5, Polygon(((0.0, 10.0), (4.0, 10.0),
                                                                                    (4.0, 14.0)), ), (0.0, 0.0))))
    for oid in (1, 5):
        r = rejection(WorldTransaction().begin_player_drive(oid, (1.0, 0.0)), initial)
        assert (r.reason, r.detail) == (R.INCOMPATIBLE_OBJECT_KIND, oid)
    assert initial.bubbles[1].desc.motion_role == M.DYNAMIC


def test_replacing_a_grabbed_bubble_ends_the_drive():
    """TransactionStagerTests.swift:527-597 (the replace case): the new descriptor comes in its own role, without the
    old drive."""
    initial = staged(resources().add(bubble(1, policy=BubbleDrivePolicy(30.0))))
    driven = staged(WorldTransaction().begin_player_drive(1, (5.0, 0.0)), initial)
    for policy in (BubbleDrivePolicy(30.0), None):
        replaced = staged(WorldTransaction().replace(1, bubble(1, policy=policy)), driven)
        assert replaced.bubbles[1].desc.motion_role == M.DYNAMIC and replaced.bubbles[1].drive_target is None
