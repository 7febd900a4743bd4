"""Collision filters at world level (CollisionFilterWorldTests.swift:16-70), through the world API on a stand-in device
world that forwards to the oracle: bubbles with disjoint masks pass through each other while default ones collide;
a collision needs both masks to take the other's category; a bubble with a disjoint mask passes a static wall and a
kinematic body that stop a default bubble. Scenes follow PhysicsSceneBuilders.swift:14-50 (region 600 x 300, K_c
1e4, mass 1). The dynamic-body cases belong to the rigid solver."""
import pytest

from bubblephysics_gb300 import world as W
from bubblephysics_gb300.world import (BubbleDescriptor, BubbleWorld, CollisionFilter, MotionRole, PhysicsMaterial,
                                       Polygon, RigidBodyDescriptor, WorldConfiguration, WorldTransaction)
from test_world_api_oracle_cpu import OracleBackedWorld

ONLY_CATEGORY_2 = CollisionFilter(1, 1 << 1)
# KinematicMotionTests.trackTolerance: a velocity drive follows an exact double-precision track, re-anchored every
# step (MotionControllers.swift:124-134).
TRACK_TOLERANCE = 1e-4


@pytest.fixture(autouse=True)
def oracle_backed(monkeypatch):
    monkeypatch.setattr(W, "World", OracleBackedWorld)
    monkeypatch.setattr(W, "default_context", lambda: None)


def world():
    w = BubbleWorld(WorldConfiguration((0.0, 0.0, 600.0, 300.0), contours=False))
    return w, WorldTransaction().update_physics_material("b", PhysicsMaterial(1e4))


def bubble(i, x, y, vx, r=8.0, filt=CollisionFilter()):
    return BubbleDescriptor(i, (x, y), r, 1.0, "b", velocity=(vx, 0.0), filter=filt)


def box(i, x, y, hx, hy, role=MotionRole.STATIC, filt=CollisionFilter()):
    return RigidBodyDescriptor(i, Polygon(((-hx, -hy), (hx, -hy), (hx, hy), (-hx, hy))), (x, y), motion_role=role,
                               filter=filt)


def run(w, steps):
    for _ in range(steps):
        frame = w.advance(1.0 / 60)
        assert w.diagnostics.last_advance_issue is None
    return frame


def x(frame, oid):
    return frame.objects[oid].position[0]


def test_disjoint_masks_pass_through_each_other_while_defaults_collide():
    w, tx = world()
    w.submit(tx.add(bubble(1, 100, 100, 60, 10, ONLY_CATEGORY_2)).add(bubble(2, 200, 100, -60, 10, ONLY_CATEGORY_2))
             .add(bubble(3, 100, 200, 60, 10)).add(bubble(4, 200, 200, -60, 10)))
    f = run(w, 90)
    assert x(f, 1) > x(f, 2) + 20 and x(f, 3) < x(f, 4)


def test_a_collision_needs_both_masks():
    w, tx = world()
    w.submit(tx.add(bubble(1, 100, 100, 60, 10, CollisionFilter(1, 0xFFFFFFFF)))
             .add(bubble(2, 200, 100, -60, 10, CollisionFilter(2, 4))))
    f = run(w, 90)
    assert x(f, 1) > x(f, 2) + 20


def test_a_disjoint_mask_passes_a_static_wall_that_stops_a_default_bubble():
    w, tx = world()
    w.submit(tx.add(box(10, 300, 100, 5, 60, filt=CollisionFilter(1, 1))).add(box(11, 300, 220, 5, 60))
             .add(bubble(1, 200, 100, 80, 8, ONLY_CATEGORY_2)).add(bubble(2, 200, 220, 80, 8)))
    f = run(w, 120)
    assert x(f, 1) > 310 and x(f, 2) < 295


def test_a_disjoint_mask_passes_a_kinematic_body_that_stops_a_default_bubble():
    w, tx = world()
    w.submit(tx.add(box(11, 200, 120, 10, 20, MotionRole.KINEMATIC)).add(box(13, 200, 260, 10, 20, MotionRole.KINEMATIC))
             .add(bubble(2, 100, 120, 80, 10, ONLY_CATEGORY_2)).add(bubble(4, 100, 260, 80, 10)))
    f = run(w, 120)
    assert x(f, 2) > 225 and x(f, 4) < 190


def test_a_kinematic_box_pushes_twenty_bubbles_and_stays_on_its_track():
    """KinematicMotionTests.swift:18-44: a kinematic box at 12 units/s pushes a 4 x 5 block of bubbles; it stays on
    its prescribed track (within TRACK_TOLERANCE), the bubbles move on by more than 10 on average and none passes
    through the box."""
    w = BubbleWorld(WorldConfiguration((0.0, 0.0, 800.0, 300.0), contours=False))
    tx = WorldTransaction().update_physics_material("b", PhysicsMaterial(1e4))
    tx = tx.add(box(1000, 20, 104, 8, 40, MotionRole.KINEMATIC)).set_kinematic_drive(1000, (12.0, 0.0), 0.0)
    for k in range(20):
        tx = tx.add(bubble(k + 1, 50 + (k % 4) * 12.0, 80 + (k // 4) * 12.0, 0.0, 5.0))
    w.submit(tx)
    worst = 0.0
    for _ in range(240):
        frame = w.advance(1.0 / 60)
        assert w.diagnostics.last_advance_issue is None
        bx, by = frame.objects[1000].position
        worst = max(worst, ((bx - (20 + 12 * frame.simulation_time)) ** 2 + (by - 104) ** 2) ** 0.5)
    assert worst <= TRACK_TOLERANCE
    xs = [frame.objects[k].position[0] for k in range(1, 21)]
    assert sum(xs) / 20 - 68 > 10
    assert all(v > frame.objects[1000].bounds[2] - 1 for v in xs)
