"""Where a bubble's centre may stand (PlacementGeometry.swift:43-200), against the reference's own cases
(PlacementValidationTests.swift:100-279): the region (also with the wrap policy, edge included), bodies the bubble
collides with (polygon, rotated polygon, circle, capsule; boundary included), the coincident-centre tolerance
max(1e-4 min(r), 1e-4) against colliding bubbles (also those created earlier in the same transaction), the order
region > body > coincident centre, replace excluding the replaced bubble, and filters that never collide taking no
part. Merges and splits are out of scope with them."""
import math

import pytest

from bubblephysics_gb300 import world as W
from bubblephysics_gb300.world import (BubbleDescriptor, Capsule, Circle, CollisionFilter, MotionRole, PhysicsMaterial,
                                       PlacementIssue as P, Polygon, RegionExitPolicy, RigidBodyDescriptor,
                                       TransactionRejectionReason as R, WorldTransaction)

REGION = (-100.0, -100.0, 100.0, 100.0)
GHOST = CollisionFilter(2, 0)


def bubble(i, x, y, r=2.0, filt=CollisionFilter(), policy=RegionExitPolicy.REMOVE):
    return BubbleDescriptor(i, (x, y), r, 2.0, "soft", filter=filt, region_exit_policy=policy)


def rect(i, lo, hi, pos=(0.0, 0.0), angle=0.0, filt=CollisionFilter(), role=MotionRole.STATIC):
    pts = ((lo[0], lo[1]), (hi[0], lo[1]), (hi[0], hi[1]), (lo[0], hi[1]))
    return RigidBodyDescriptor(i, Polygon(pts), pos, angle=angle, filter=filt, motion_role=role)


def staged(tx):
    state, rec, ev = W.stage([(1, WorldTransaction().update_physics_material("soft", PhysicsMaterial(1852.0)))],
                             W._State(), REGION)
    state, rec, ev = W.stage([(2, tx)], state, REGION)
    assert rec, ev
    return state


def rejection(state, tx):
    _, rec, ev = W.stage([(3, tx)], state, REGION)
    return None if rec else ev[0].rejection


def test_coincident_centre_is_rejected():
    state = staged(WorldTransaction().add(bubble(1, 10, 10)))
    r = rejection(state, WorldTransaction().add(bubble(2, 10, 10, r=5)))
    assert (r.operation_index, r.reason, r.detail) == (0, R.INVALID_PLACEMENT, (2, P.COINCIDENT_CENTER))


def test_coincident_tolerance_edges():
    state = staged(WorldTransaction().add(bubble(1, 10, 10)))  # tolerance max(1e-4 * 2, 1e-4) = 2e-4
    assert rejection(state, WorldTransaction().add(bubble(2, 10.0001, 10))).detail == (2, P.COINCIDENT_CENTER)
    assert rejection(state, WorldTransaction().add(bubble(2, 10.01, 10))) is None


def test_coincident_with_a_bubble_of_the_same_transaction():
    state = staged(WorldTransaction())
    r = rejection(state, WorldTransaction().add(bubble(1, 5, 5)).add(bubble(2, 5, 5)))
    assert (r.operation_index, r.detail) == (1, (2, P.COINCIDENT_CENTER))


@pytest.mark.parametrize("body,inside", [
    (rect(100, (-20, -20), (20, 20)), (5.0, 5.0)),
    (RigidBodyDescriptor(101, Circle(15.0), (50.0, 0.0)), (55.0, 4.0)),
    (RigidBodyDescriptor(102, Capsule(10.0, 4.0), (0.0, -50.0)), (8.0, -52.0))], ids=["polygon", "circle", "capsule"])
def test_inside_a_rigid_body_is_rejected(body, inside):
    state = staged(WorldTransaction().add(body))
    assert rejection(state, WorldTransaction().add(bubble(2, *inside))).detail == (2, P.INSIDE_RIGID_BODY)
    assert rejection(state, WorldTransaction().add(bubble(900, 60, 60))) is None


@pytest.mark.parametrize("policy", [RegionExitPolicy.REMOVE, RegionExitPolicy.WRAP])
def test_outside_the_region_is_rejected_whatever_the_policy(policy):
    state = staged(WorldTransaction())
    for point in ((100.5, 0.0), (0.0, -101.0), (-300.0, 300.0)):
        assert rejection(state, WorldTransaction().add(bubble(2, *point, policy=policy))).detail == (2, P.OUTSIDE_REGION)
    assert rejection(state, WorldTransaction().add(bubble(1, 100, 100))) is None  # the edge belongs to the region


def test_region_before_body_before_coincident_centre():
    source, gate = CollisionFilter(0b01, 0b01), CollisionFilter(0b10, 0b10)
    # a moving body may reach out of the region (a static one may not); the reference uses a dynamic one
    state = staged(WorldTransaction().add(bubble(1, 0, 0, filt=source))
                   .add(rect(10, (-10, -10), (150, 10), filt=gate, role=MotionRole.KINEMATIC)))
    probe = CollisionFilter(0b11)
    issue = lambda p: W.placement_issue(p, 2.0, probe, state, REGION)
    assert issue((120.0, 0.0)) == P.OUTSIDE_REGION and issue((0.0, 0.0)) == P.INSIDE_RIGID_BODY
    assert issue((0.0, 30.0)) is None


def test_replace_at_a_bad_placement_is_rejected_with_the_same_causes():
    state = staged(WorldTransaction().add(bubble(1, -30, 0)).add(bubble(2, 30, 0)).add(rect(100, (-5, 40), (5, 50))))
    for point, issue in (((30.0, 0.0), P.COINCIDENT_CENTER), ((0.0, 45.0), P.INSIDE_RIGID_BODY),
                         ((150.0, 0.0), P.OUTSIDE_REGION)):
        assert rejection(state, WorldTransaction().replace(1, bubble(1, *point))).detail == (1, issue)
        assert tuple(state.bubbles[1].position) == (-30.0, 0.0)


def test_replace_excludes_the_replaced_bubble():
    state = staged(WorldTransaction().add(bubble(1, 10, 10)))
    assert rejection(state, WorldTransaction().replace(1, bubble(1, 10, 10, r=5))) is None


def test_valid_placements_including_partial_overlap():
    state = staged(WorldTransaction().add(bubble(1, 0, 0, r=10)))
    tx = WorldTransaction().add(bubble(2, 12, 0, r=5)).add(bubble(3, -30, 0.01)).add(bubble(4, -30, 0.02))
    assert rejection(state, tx) is None


def test_the_issue_table_of_the_reference():
    tx = (WorldTransaction().add(bubble(1, 0, 30)).add(rect(100, (-60, -60), (-40, -40)))
          .add(rect(101, (-4, -1), (4, 1), pos=(20.0, 0.0), angle=math.pi / 2))
          .add(RigidBodyDescriptor(102, Circle(3.0), (0.0, -20.0)))
          .add(RigidBodyDescriptor(103, Capsule(5.0, 1.0), (30.0, 30.0)))
          .add(RigidBodyDescriptor(104, Circle(3.0), (-20.0, 0.0), filter=GHOST)))
    state = staged(tx)
    default = CollisionFilter()
    cases = [((200, 0), set(), default, P.OUTSIDE_REGION), ((-50, -50), set(), default, P.INSIDE_RIGID_BODY),
             ((-50, -50), {100}, default, None), ((-50, -50), set(), GHOST, None),
             ((20, 3.5), set(), default, P.INSIDE_RIGID_BODY), ((23.5, 0), set(), default, None),
             ((0, -18), set(), default, P.INSIDE_RIGID_BODY), ((34, 30.5), set(), default, P.INSIDE_RIGID_BODY),
             ((-20, 0), set(), default, None), ((0, 30), set(), default, P.COINCIDENT_CENTER),
             ((0, 30), {1}, default, None), ((0, 30.005), set(), default, None)]
    for point, excluding, filt, expected in cases:
        assert W.placement_issue(point, 2.0, filt, state, REGION, frozenset(excluding)) == expected, point


def test_filters_that_never_collide_take_no_part():
    state = staged(WorldTransaction().add(bubble(1, 10, 10)).add(rect(100, (-60, -60), (-40, -40))))
    for tx in (WorldTransaction().add(bubble(2, 10, 10, filt=GHOST)),
               WorldTransaction().add(bubble(2, -50, -50, filt=GHOST)),
               WorldTransaction().add(bubble(2, 0, 0, filt=GHOST)).add(bubble(3, 0, 0, filt=GHOST)),
               WorldTransaction().add(bubble(2, 30, 30, filt=GHOST)).replace(2, bubble(2, 10, 10, filt=GHOST))):
        assert rejection(state, tx) is None


def test_a_body_may_not_cover_a_colliding_bubble():
    state = staged(WorldTransaction().add(bubble(7, 5, 5)).add(bubble(3, -5, -5)))
    r = rejection(state, WorldTransaction().add(rect(100, (-20, -20), (20, 20))))
    assert r.detail == (3, P.INSIDE_RIGID_BODY)  # the smallest id inside
