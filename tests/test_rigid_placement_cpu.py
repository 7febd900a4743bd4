"""Placement on the body's side, against RigidPlacementTests.swift:59-173, on this path's `stage`: a body may not cover
the centre of a bubble it collides with, whichever of the two enters the world (boundary included, for every shape),
also by a replace and within one transaction in either order (reported at the second operation); filters that never
collide take no part, and only colliding bubbles are reported; the coincident-centre tolerance is
max(1e-4 min(r_a, r_b), 1e-4)."""
import pytest

from bubblephysics_gb300 import world as W
from bubblephysics_gb300.world import (BubbleDescriptor, Capsule, Circle, CollisionFilter, MotionRole, PhysicsMaterial,
                                       PlacementIssue as P, Polygon, RigidBodyDescriptor,
                                       TransactionRejectionReason as R, WorldTransaction)

REGION = (-100.0, -100.0, 100.0, 100.0)


def resources():
    return WorldTransaction().update_physics_material(1, PhysicsMaterial(1e9))


def bubble(i, at, radius=2.0, filt=CollisionFilter()):
    return BubbleDescriptor(i, at, radius, 2.0, 1, filter=filt)


def rect(lo, hi):
    return Polygon(((lo[0], lo[1]), (hi[0], lo[1]), (hi[0], hi[1]), (lo[0], hi[1])))


def body(i, shape, at=(0.0, 0.0), role=MotionRole.STATIC, filt=CollisionFilter()):
    return RigidBodyDescriptor(i, shape, at, motion_role=role, filter=filt)


def state(*txs):
    s = W._State()
    for tx in txs:
        s, receipts, events = W.stage([(1, tx)], s, REGION)
        assert receipts, events
    return s


def rejected(tx, against, index, bubble_id, issue=P.INSIDE_RIGID_BODY):
    after, receipts, events = W.stage([(2, tx)], against, REGION)
    assert not receipts and set(after.bubbles) == set(against.bubbles) and set(after.bodies) == set(against.bodies)
    r = events[0].rejection
    assert (r.operation_index, r.reason, r.detail) == (index, R.INVALID_PLACEMENT, (bubble_id, issue))


def accepted(tx, against):
    _, receipts, events = W.stage([(2, tx)], against, REGION)
    assert receipts, events


def test_an_added_body_covering_a_bubble_centre_is_rejected_for_every_shape_and_role():
    initial = state(resources().add(bubble(1, (10.0, 10.0))))
    for shape, at in ((rect((-5, -5), (5, 5)), (10.0, 10.0)), (Circle(5.0), (12.0, 10.0)), (Capsule(8.0, 1.0), (10.0, 10.5))):
        rejected(WorldTransaction().add(body(100, shape, at)), initial, 0, 1)
    rejected(WorldTransaction().add(body(100, Circle(5.0), (10.0, 10.0), MotionRole.KINEMATIC)), initial, 0, 1)


def test_a_body_away_from_bubble_centres_is_accepted():
    initial = state(resources().add(bubble(1, (10.0, 10.0))))
    accepted(WorldTransaction().add(body(100, Circle(5.0), (16.0, 10.0))), initial)  # only the centre counts
    accepted(WorldTransaction().add(body(100, rect((20, 20), (30, 30)))), initial)


@pytest.mark.parametrize("shape, centre", [(rect((0, 0), (4, 4)), (0.0, 2.0)), (rect((0, 0), (4, 4)), (4.0, 2.0)),
                                           (rect((0, 0), (4, 4)), (2.0, 0.0)), (rect((0, 0), (4, 4)), (2.0, 4.0)),
                                           (rect((0, 0), (4, 4)), (0.0, 0.0)), (Circle(5.0), (5.0, 0.0)),
                                           (Capsule(4.0, 1.0), (0.0, 1.0))])
def test_a_centre_on_the_boundary_counts_as_inside(shape, centre):
    rejected(WorldTransaction().add(bubble(1, centre)), state(resources().add(body(100, shape))), 0, 1)
    rejected(WorldTransaction().add(body(100, shape)), state(resources().add(bubble(1, centre))), 0, 1)


def test_a_replaced_body_covering_a_bubble_centre_is_rejected():
    initial = state(resources().add(bubble(1, (10.0, 10.0))).add(body(100, rect((40, 40), (50, 50)))))
    rejected(WorldTransaction().replace(100, body(100, rect((5, 5), (15, 15)))), initial, 0, 1)
    accepted(WorldTransaction().replace(100, body(100, rect((60, 60), (70, 70)))), initial)


def test_a_body_and_a_bubble_in_one_transaction_are_rejected_in_either_order():
    initial = state(resources())
    rejected(WorldTransaction().add(bubble(1, (10.0, 10.0))).add(body(100, Circle(5.0), (10.0, 10.0))), initial, 1, 1)
    rejected(WorldTransaction().add(body(100, Circle(5.0), (10.0, 10.0))).add(bubble(1, (10.0, 10.0))), initial, 1, 1)


def test_a_body_its_filter_excludes_may_cover_the_bubble_centre():
    bubble_only, body_only = CollisionFilter(0b01, 0b01), CollisionFilter(0b10, 0b10)
    initial = state(resources().add(bubble(1, (10.0, 10.0), filt=bubble_only)))
    accepted(WorldTransaction().add(body(100, Circle(5.0), (10.0, 10.0), filt=body_only)), initial)
    accepted(WorldTransaction().add(bubble(1, (10.0, 10.0), filt=bubble_only)),
             state(resources().add(body(100, Circle(5.0), (10.0, 10.0), filt=body_only))))
    rejected(WorldTransaction().add(body(100, Circle(5.0), (10.0, 10.0), filt=bubble_only)), initial, 0, 1)


def test_only_bubbles_colliding_with_the_body_are_reported():
    initial = state(resources().add(bubble(1, (10.0, 10.0), filt=CollisionFilter(0b01, 0b01)))
                    .add(bubble(2, (11.0, 10.0))))
    rejected(WorldTransaction().add(body(100, Circle(5.0), (10.0, 10.0), filt=CollisionFilter(0b10, 0b11))), initial, 0, 2)


def test_the_coincident_centre_tolerance_is_the_constant_1e_minus_4():
    initial = state(resources().add(bubble(1, (10.0, 10.0), radius=0.5)))
    rejected(WorldTransaction().add(bubble(2, (10.00008, 10.0), radius=0.5)), initial, 0, 2, P.COINCIDENT_CENTER)
    accepted(WorldTransaction().add(bubble(2, (10.0002, 10.0), radius=0.5)), initial)
