"""The candidate limit's margin on the stress-300 scene, through the world API on a stand-in device world that
forwards to the oracle, against ContactCandidateMarginTests.swift:11-25: over 300 steps no object overflows its k = 128
candidates and the largest count seen stays at most half of k, on stress-300 and on the mixed scene. The stress-300 scene restates Stress300Scene
(PublicWorldStressBenchmark.swift:681-827): a 375 x 700 region framed by four 1-unit static walls, 300 grid slots of
15 columns (spacing 23 x 33.5) jittered by the scene's linear congruential generator (Knuth's MMIX constants, seed
0x2B60F5), radius 12.42 (0.78 + 0.44 u), mass max(1, 0.02 r^2), K_c 229, less the slots under the start of a kinematic
triangle that drives two laps of five waypoints at 200 units/s."""
import math

import numpy as np
import pytest

from bubblephysics_gb300 import world as W
from bubblephysics_gb300.world import (BubbleDescriptor, BubbleWorld, Capsule, Circle, KinematicDrive, MotionRole,
                                       PathDrive, PhysicsMaterial, Polygon, RigidBodyDescriptor, WorldConfiguration,
                                       WorldTransaction)
from test_world_api_oracle_cpu import OracleBackedWorld

HEIGHT = 700.0
WAYPOINTS = ((187.5, 350.0), (65.0, 105.0), (310.0, 595.0), (310.0, 105.0), (65.0, 595.0))
TRIANGLE = ((-46.0, 34.0), (46.0, 34.0), (0.0, -52.0))


@pytest.fixture(autouse=True)
def oracle_backed(monkeypatch):
    monkeypatch.setattr(W, "World", OracleBackedWorld)
    monkeypatch.setattr(W, "default_context", lambda: None)


class Lcg:
    """A 64-bit linear congruential generator (Knuth's MMIX multiplier and increment); a unit draw is the top 24 bits."""

    def __init__(self, seed):
        self.state = seed or 1

    def unit(self):
        self.state = (self.state * 6364136223846793005 + 1442695040888963407) & 0xFFFFFFFFFFFFFFFF
        return np.float32(self.state >> 40) / np.float32(1 << 24)


def distance_to_triangle(p, center):
    corners = [np.float32(v) + np.asarray(center, np.float32) for v in np.asarray(TRIANGLE, np.float32)]
    cross = lambda a, b: a[0] * b[1] - a[1] * b[0]
    signs = [cross(corners[(k + 1) % 3] - corners[k], p - corners[k]) for k in range(3)]
    if all(s >= 0 for s in signs) or all(s <= 0 for s in signs):
        return 0.0
    out = []
    for k in range(3):
        a, b = corners[k], corners[(k + 1) % 3]
        t = max(0.0, min(1.0, float(np.dot(p - a, b - a) / np.dot(b - a, b - a))))
        out.append(float(np.hypot(*(p - (a + (b - a) * np.float32(t))))))
    return min(out)


def stress300():
    rng = Lcg(0x2B60F5)
    dx, dy = np.float32(345.0) / np.float32(15), np.float32(33.5)
    base = min(dx, dy) * np.float32(0.54)
    tx = WorldTransaction().update_physics_material(1, PhysicsMaterial(229.0))
    placed = 0
    for index in range(300):
        column, row = index % 15, index // 15
        jx = (rng.unit() - np.float32(0.5)) * dx * np.float32(0.12)
        jy = (rng.unit() - np.float32(0.5)) * dy * np.float32(0.12)
        radius = base * (np.float32(0.78) + rng.unit() * np.float32(0.44))
        p = np.array([15 + (np.float32(column) + np.float32(0.5)) * dx + jx,
                      15 + (np.float32(row) + np.float32(0.5)) * dy + jy], np.float32)
        if distance_to_triangle(p, WAYPOINTS[0]) > base * np.float32(1.22) + 1:
            mass = max(1.0, float(radius * radius * np.float32(0.02)))
            tx = tx.add(BubbleDescriptor(index + 1, tuple(map(float, p)), float(radius), mass, 1))
            placed += 1
    for k, pts in enumerate((((0, 0), (1, 0), (1, HEIGHT), (0, HEIGHT)),
                             ((374, 0), (375, 0), (375, HEIGHT), (374, HEIGHT)),
                             ((0, 0), (375, 0), (375, 1), (0, 1)),
                             ((0, HEIGHT - 1), (375, HEIGHT - 1), (375, HEIGHT), (0, HEIGHT)))):
        tx = tx.add(RigidBodyDescriptor(10_001 + k, Polygon(tuple((float(x), float(y)) for x, y in pts)), (0.0, 0.0)))
    lap = WAYPOINTS[1:] + WAYPOINTS[:1]
    tx = tx.add(RigidBodyDescriptor(10_000, Polygon(TRIANGLE), WAYPOINTS[0], motion_role=MotionRole.KINEMATIC))
    tx = tx.set_kinematic_drive(10_000, KinematicDrive.path(PathDrive(lap + lap, 200.0)))
    return tx, placed


def test_stress300_keeps_the_candidate_limit_with_a_twofold_margin():
    tx, placed = stress300()
    assert placed == 287  # the reference's count for this scene (StressSubstepReportTests.swift:55)
    world = BubbleWorld(WorldConfiguration((0.0, 0.0, 375.0, HEIGHT), contours=False))
    world.submit(tx)
    maximum = 0
    for step in range(300):
        world.advance(1.0 / 60)
        assert world.diagnostics.last_advance_issue is None, step
        maximum = max(maximum, world.diagnostics.maximum_contact_candidates_per_object)
        assert world.diagnostics.contact_candidate_overflow == 0, step
    assert 0 < maximum and maximum * 2 <= 128, maximum
    assert math.hypot(*(np.asarray(world.last_frame.objects[10_000].position) - WAYPOINTS[0])) > 1  # the triangle drove


def mixed():
    """MixedScene (PublicWorldStressBenchmark.swift:982-1088): 200 bubbles on a 20-column grid in the lower band, 55
    kinematic bodies spinning in place on an 11 x 5 grid (rectangle, circle, capsule, triangle in turn, scaled
    0.8-1.2), 5 kinematic bars sliding at 80 units/s and turning every 150 steps, and four 1-unit walls."""
    rng = Lcg(0x4D1C5E)
    spacing, body_spacing = np.float32(345.0) / np.float32(20), np.float32(345.0) / np.float32(11)
    tx = WorldTransaction().update_physics_material(1, PhysicsMaterial(229.0))
    for index in range(200):
        radius = spacing * np.float32(0.4) * (np.float32(0.78) + rng.unit() * np.float32(0.44))
        p = (float(15 + (np.float32(index % 20) + np.float32(0.5)) * spacing),
             float(15 + (np.float32(index // 20) + np.float32(0.5)) * spacing))
        tx = tx.add(BubbleDescriptor(index + 1, p, float(radius), max(1.0, float(radius * radius * np.float32(0.02))), 1))
    for index in range(55):
        scale = np.float32(0.8) + rng.unit() * np.float32(0.4)
        rng.unit(), rng.unit()  # two draws of a linear velocity the scene no longer uses
        spin = float((rng.unit() - np.float32(0.5)) * np.float32(6))
        p = (float(15 + (np.float32(index % 11) + np.float32(0.5)) * body_spacing),
             (450.0, 500.0, 550.0, 600.0, 650.0)[index // 11])
        s = float(scale)
        shape = (Polygon(((-9 * s, -6 * s), (9 * s, -6 * s), (9 * s, 6 * s), (-9 * s, 6 * s))), Circle(8 * s),
                 Capsule(6 * s, 5 * s), Polygon(((-9 * s, 7 * s), (9 * s, 7 * s), (0.0, -9 * s))))[index % 4]
        tx = tx.add(RigidBodyDescriptor(1001 + index, shape, p, motion_role=MotionRole.KINEMATIC))
        tx = tx.set_kinematic_drive(1001 + index, KinematicDrive.velocity((0.0, 0.0), spin))
    for index, y in enumerate((210.0, 260.0, 310.0, 360.0, 410.0)):
        tx = tx.add(RigidBodyDescriptor(2001 + index, Polygon(((-30.0, -4.0), (30.0, -4.0), (30.0, 4.0), (-30.0, 4.0))),
                                        (100.0, y), motion_role=MotionRole.KINEMATIC))
        tx = tx.set_kinematic_drive(2001 + index, KinematicDrive.velocity((80.0, 0.0), 0.0))
    for k, pts in enumerate((((0, 0), (1, 0), (1, HEIGHT), (0, HEIGHT)),
                             ((374, 0), (375, 0), (375, HEIGHT), (374, HEIGHT)),
                             ((0, 0), (375, 0), (375, 1), (0, 1)),
                             ((0, HEIGHT - 1), (375, HEIGHT - 1), (375, HEIGHT), (0, HEIGHT)))):
        tx = tx.add(RigidBodyDescriptor(10_001 + k, Polygon(tuple((float(x), float(y)) for x, y in pts)), (0.0, 0.0)))
    return tx


def mixed_step(step):
    if step == 0 or step % 150:
        return None
    direction = 1.0 if (step // 150) % 2 == 0 else -1.0
    tx = WorldTransaction()
    for index in range(5):
        tx = tx.set_kinematic_drive(2001 + index, KinematicDrive.velocity((direction * 80.0, 0.0), 0.0))
    return tx


def test_the_mixed_scene_keeps_the_candidate_limit_with_a_twofold_margin():
    """ContactCandidateMarginTests.swift:27-47: body rows are candidates too."""
    world = BubbleWorld(WorldConfiguration((0.0, 0.0, 375.0, HEIGHT), contours=False))
    world.submit(mixed())
    maximum = 0
    for step in range(300):
        tx = mixed_step(step)
        if tx is not None:
            world.submit(tx)
        frame = world.advance(1.0 / 60)
        assert world.diagnostics.last_advance_issue is None, step
        maximum = max(maximum, world.diagnostics.maximum_contact_candidates_per_object)
        assert world.diagnostics.contact_candidate_overflow == 0, step
    assert len(frame.objects) == 264  # 200 bubbles, 60 bodies and 4 walls
    assert 0 < maximum and maximum * 2 <= 128, maximum
