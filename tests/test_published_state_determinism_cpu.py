"""The published state is deterministic, against PublishedStateDeterminismTests.swift:42-200, through the world API on a
stand-in device world that forwards to the oracle: stress-300 and the mixed scene run twice for 300 steps give the
same bits in every object's state and every contour, and the hash sees a change of state. (The CUDA path equals the
oracle bit for bit on such scenes, which the GPU parity tests check step by step.)"""
import hashlib

import numpy as np
import pytest

from bubblephysics_gb300 import world as W
from bubblephysics_gb300.world import BubbleWorld, WorldConfiguration
from test_candidate_margin_cpu import HEIGHT, mixed, mixed_step, stress300
from test_world_api_oracle_cpu import OracleBackedWorld


@pytest.fixture(autouse=True)
def oracle_backed(monkeypatch):
    monkeypatch.setattr(W, "World", OracleBackedWorld)
    monkeypatch.setattr(W, "default_context", lambda: None)


def state_hash(frame, contours):
    """A hash over the bits of every published object (position, velocity, rotation, angular velocity, bounds,
    effective radius) and every contour point, in id order."""
    h = hashlib.sha256()
    for oid in sorted(frame.objects):
        s = frame.objects[oid]
        values = [*s.position, *s.velocity, s.rotation, s.angular_velocity, *s.bounds,
                  -1.0 if s.effective_radius is None else s.effective_radius]
        h.update(np.int64(oid).tobytes() + np.asarray(values, np.float32).tobytes())
    for oid in sorted(contours):
        h.update(np.int64(oid).tobytes() + np.asarray(contours[oid], np.float32).tobytes())
    return h.hexdigest()


def run(scene, steps):
    tx, step_tx = (stress300()[0], lambda k: None) if scene == "stress" else (mixed(), mixed_step)
    world = BubbleWorld(WorldConfiguration((0.0, 0.0, 375.0, HEIGHT)))
    world.submit(tx)
    for k in range(steps):
        extra = step_tx(k)
        if extra is not None:
            world.submit(extra)
        frame = world.advance(1.0 / 60)
        assert world.diagnostics.last_advance_issue is None and frame.step_index == k + 1
        assert len(frame.transaction_receipts) == (1 if k == 0 or extra is not None else 0)
    return state_hash(frame, world.debug_contour_snapshot()), frame


@pytest.mark.parametrize("scene, objects", [("stress", 287 + 5), ("mixed", 264)])
def test_the_published_state_is_identical_across_two_runs_of_300_steps(scene, objects):
    first, frame = run(scene, 300)
    second, _ = run(scene, 300)
    assert len(frame.objects) == objects and first == second


def test_the_hash_sees_a_change_of_state():
    assert run("stress", 1)[0] != run("stress", 30)[0]
