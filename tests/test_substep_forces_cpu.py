"""Forces evaluated in every substep (SubstepForceTests.swift:16-160), through the world API on a stand-in device
world that forwards to the oracle: a head-on pair, a wall bounce, a band pulling a bubble into a crowd and a radial
field give the same state after 1 s with a four times finer substep split (positions within 1, velocities within 2 %
of the scene's top speed, at least three times the substeps); the band drags a bubble behind a target moving at
100 units/s at that speed (1 %) with the stretch u m gamma / K_band (1 %); a force limit caps the band only when set.
Scenes follow ForceSceneSupport.swift (K_c 229, bubble "2" r 24 m 1, 7168 r 148)."""
import math

import numpy as np
import pytest

from bubblephysics_gb300 import world as W
from bubblephysics_gb300.world import (BubbleDescriptor, BubbleDrivePolicy, BubbleWorld, Circle, ForceFieldDescriptor,
                                       PhysicsMaterial, Polygon, RigidBodyDescriptor, WorldConfiguration,
                                       WorldTransaction)
from test_world_api_oracle_cpu import OracleBackedWorld

DT = 1.0 / 60
TWO = (24.0, 1.0)
B7168 = (148.0, float(np.float32((7168 / 2) ** (1 / 2.25))))


@pytest.fixture(autouse=True)
def oracle_backed(monkeypatch):
    monkeypatch.setattr(W, "World", OracleBackedWorld)
    monkeypatch.setattr(W, "default_context", lambda: None)


def force_world(damping, half=2000.0, split=1.0):
    w = BubbleWorld(WorldConfiguration((-half, -half, half, half), substep_split_multiplier=split, contours=False))
    return w, WorldTransaction().update_physics_material("m", PhysicsMaterial(229.0, damping))


def bubble(i, x, y, kind=TWO, velocity=(0.0, 0.0), policy=None):
    return BubbleDescriptor(i, (x, y), kind[0], kind[1], "m", velocity=velocity, drive_policy=policy)


def split_invariance(damping, ids, build, before=None, frames=60):
    results, substeps = [], []
    for split in (1.0, 4.0):
        w, tx = force_world(damping, split=split)
        w.submit(build(tx))
        count, top = 0, 0.0
        for k in range(frames):
            if before is not None and before(k) is not None:
                w.submit(before(k))
            frame = w.advance(DT)
            assert w.diagnostics.last_advance_issue is None
            count += w.diagnostics.last_step_substeps
            top = max([top] + [math.hypot(*frame.objects[i].velocity) for i in ids])
        results.append((frame, top))
        substeps.append(count)
    (natural, top), (split4, _) = results
    assert substeps[0] >= frames and substeps[1] >= 3 * substeps[0] and top > 1
    for i in ids:
        assert math.dist(natural.objects[i].position, split4.objects[i].position) <= 1
        assert math.dist(natural.objects[i].velocity, split4.objects[i].velocity) <= 0.02 * top


def test_head_on_pair_is_split_invariant():
    split_invariance(1.0, [1, 2], lambda tx: tx.add(bubble(1, 300 - 24 - 30, 0, velocity=(100.0, 0.0)))
                     .add(bubble(2, 300 + 24 + 30, 0, velocity=(-100.0, 0.0))))


def test_wall_bounce_is_split_invariant():
    wall = RigidBodyDescriptor(2, Polygon(((360, -1900), (361, -1900), (361, 1900), (360, 1900))), (0.0, 0.0))
    split_invariance(1.0, [1], lambda tx: tx.add(bubble(1, 360 - 24 - 20, 0, velocity=(100.0, 0.0))).add(wall))


def test_band_pulling_into_a_crowd_is_split_invariant():
    def build(tx):
        for row in range(4):
            for col in range(4):
                tx = tx.add(bubble(1 + row * 4 + col, 80 + col * 50.0, row * 50.0 - 75))
        return tx.add(bubble(100, 0, 0, policy=BubbleDrivePolicy(22.0))).begin_player_drive(100, (0.0, 0.0))
    split_invariance(1.0, [100] + list(range(1, 17)), build,
                     before=lambda k: WorldTransaction().update_player_drive(100, (k * 100 / 60, 0.0)))


def test_radial_field_is_split_invariant():
    split_invariance(0.0, [1], lambda tx: tx.add(bubble(1, 100, 0, velocity=(0.0, 100.0)))
                     .add(ForceFieldDescriptor(2, (0.0, 0.0), "radial", Circle(400.0), strength=-500.0)))


def drag(kind, damping, u, seconds, maximum_force=None):
    start = -3000.0
    w, tx = force_world(damping, half=5000.0)
    w.submit(tx.add(bubble(1, start, 0, kind, policy=BubbleDrivePolicy(22.0, maximum_force))).begin_player_drive(1, (start, 0.0)))
    frames, xs = seconds * 60, []
    for k in range(frames):
        if k:
            w.submit(WorldTransaction().update_player_drive(1, (float(np.float32(start + np.float32(u / 60) * k)), 0.0)))
        xs.append(w.advance(DT).objects[1].position[0])
        assert w.diagnostics.last_advance_issue is None
    tail = 300
    velocity = (xs[-1] - xs[-1 - tail]) / (tail / 60)
    stretch = np.mean([start + u / 60 * k - 0.5 * (xs[k] + xs[k - 1]) for k in range(frames - tail, frames)])
    return velocity, stretch


@pytest.mark.parametrize("kind,damping", [(TWO, 1.0), (TWO, 5.0), (B7168, 1.0)], ids=["2-1", "2-5", "7168-1"])
def test_band_drags_at_the_target_speed_with_stretch_proportional_to_mass(kind, damping):
    v, s = drag(kind, damping, 100.0, 60)
    expected = 100 * kind[1] * damping / 22
    assert abs(v - 100) <= 1 and abs(s - expected) <= 0.01 * expected, (v, s, expected)


def test_a_force_limit_caps_the_band_only_when_set():
    capped, _ = drag(TWO, 1.0, 300.0, 20, maximum_force=100.0)
    free, _ = drag(TWO, 1.0, 300.0, 20)
    assert abs(capped - 100) <= 1 and abs(free - 300) <= 3
