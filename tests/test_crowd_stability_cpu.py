"""A growing crowd pulled by the band (CrowdStabilityTests.swift:5-137), through the world API on a stand-in device world
that forwards to the oracle: 150 bubbles (30 of kind 128, 120 of kind "2"; K_c 229, gamma 1) placed at half radius in a
640 x 1280 frame of static walls grow to full radius in 2 s while the band (K 22, no force limit) pulls three of them in
turn to the lower-left corner, 5 s each. Every step stays healthy, every centre stays inside the frame and apart from
the others, and the contours sampled every second do not enter one another by more than 0.02, for the reference's
full minute. The reference places the crowd with its own seeded generator; this placement is seeded synthetic data
under the same rules."""
import numpy as np
import pytest

from bubblephysics_gb300 import world as W
from bubblephysics_gb300.world import (BubbleDescriptor, BubbleDrivePolicy, BubbleWorld, ParameterTransition,
                                       PhysicsMaterial, Polygon, RigidBodyDescriptor, WorldConfiguration,
                                       WorldTransaction)
from test_world_api_oracle_cpu import OracleBackedWorld

INTERIOR, THICK = (320.0, 640.0), 48.0
TWO, B128 = (24.0, 1.0), (64.0, float(np.float32((128 / 2) ** (1 / 2.25))))
SECONDS = 60


@pytest.fixture(autouse=True)
def oracle_backed(monkeypatch):
    monkeypatch.setattr(W, "World", OracleBackedWorld)
    monkeypatch.setattr(W, "default_context", lambda: None)


def placements(seed=1):
    rng = np.random.default_rng(seed)
    placed = []
    for index, kind in enumerate([B128] * 30 + [TWO] * 120):
        half = kind[0] / 2
        limit = np.array(INTERIOR) - (half + 1)
        for attempt in range(10_000):
            p = rng.uniform(-limit, limit)
            if all(np.hypot(*(q - p)) > k[0] / 2 + half + 1 for _, k, q in placed):
                break
        placed.append((index + 1, kind, p))
    return placed


def penetration(inner, outer):
    """The deepest vertex of `inner` inside the polygon `outer` (0 when none is inside)."""
    deepest = 0.0
    a, b = outer, np.roll(outer, -1, axis=0)
    for p in inner:
        crosses = ((a[:, 1] > p[1]) != (b[:, 1] > p[1])) & \
            (p[0] < (b[:, 0] - a[:, 0]) * (p[1] - a[:, 1]) / np.where(b[:, 1] == a[:, 1], 1, b[:, 1] - a[:, 1]) + a[:, 0])
        if crosses.sum() % 2:
            e = b - a
            t = np.clip(((p - a) * e).sum(1) / np.maximum((e * e).sum(1), 1e-12), 0, 1)
            deepest = max(deepest, float(np.hypot(*(p - (a + e * t[:, None])).T).min()))
    return deepest


def test_growing_crowd_pulled_by_the_band_stays_stable():
    crowd = placements()
    ix, iy = INTERIOR
    ox, oy = ix + THICK, iy + THICK
    world = BubbleWorld(WorldConfiguration((-ox, -oy, ox, oy)))
    tx = WorldTransaction().update_physics_material("m", PhysicsMaterial(229.0, 1.0))
    for k, ((lx, ly), (hx, hy)) in enumerate([((-ox, -oy), (-ix, oy)), ((ix, -oy), (ox, oy)), ((-ix, -oy), (ix, -iy)),
                                              ((-ix, iy), (ix, oy))]):
        tx = tx.add(RigidBodyDescriptor(9001 + k, Polygon(((lx, ly), (hx, ly), (hx, hy), (lx, hy))), (0.0, 0.0)))
    for oid, kind, p in crowd:
        tx = tx.add(BubbleDescriptor(oid, tuple(p), kind[0] / 2, kind[1], "m", drive_policy=BubbleDrivePolicy(22.0)))
        tx = tx.start_transition(ParameterTransition(("bubbleRadius", oid), kind[0], 2.0))
    world.submit(tx)
    pullers, corner = [1, 31, 32], (-ix, -iy)
    samples = 0
    for step in range(SECONDS * 60):
        if step % 300 == 0:
            cycle = step // 300
            pull = WorldTransaction()
            if cycle > 0:
                pull = pull.end_player_drive(pullers[(cycle - 1) % 3])
            world.submit(pull.begin_player_drive(pullers[cycle % 3], corner))
        frame = world.advance(1.0 / 60)
        assert world.diagnostics.last_advance_issue is None and world.diagnostics.failure_reason is None, step
        pos = np.array([frame.objects[oid].position for oid, _, _ in crowd])
        assert np.isfinite(pos).all() and (np.abs(pos[:, 0]) < ix).all() and (np.abs(pos[:, 1]) < iy).all(), step
        d = np.hypot(*(pos[:, None, :] - pos[None, :, :]).transpose(2, 0, 1))
        assert (d[np.triu_indices(len(crowd), 1)] > 0).all(), step
        if step % 60 == 59:
            samples += 1
            snapshot = world.debug_contour_snapshot()
            reach = np.array([k[0] for _, k, _ in crowd])
            close = np.argwhere(np.triu(d < reach[:, None] + reach[None, :], 1))
            for i, j in close:
                a, b = np.array(snapshot[crowd[i][0]]), np.array(snapshot[crowd[j][0]])
                depth = max(penetration(a, b), penetration(b, a))
                assert depth <= 0.02, (step, crowd[i][0], crowd[j][0], depth)
    assert samples == SECONDS
