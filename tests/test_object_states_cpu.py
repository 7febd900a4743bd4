"""Published object states (ObjectStateTests.swift:79-198), through the world API on a stand-in device world that
forwards to the oracle: every bubble's bounds contain its contour and an undented bubble's centre is its contour's
area centroid (within 1 % of r) in a crowded scene after 60 steps; an object removed by a transaction is absent from
that frame; a wrapped bubble's bounds move with its contour; a call that completes no step publishes the same states.
The crowded scene is seeded synthetic data standing in for the reference's stress-300 scene."""
import math

import numpy as np
import pytest

from bubblephysics_gb300 import world as W
from bubblephysics_gb300.world import (BubbleDescriptor, BubbleWorld, EventInterest, PhysicsMaterial, Polygon,
                                       RegionExitPolicy,
                                       RigidBodyDescriptor, WorldConfiguration, WorldTransaction)
from test_world_api_oracle_cpu import OracleBackedWorld


@pytest.fixture(autouse=True)
def oracle_backed(monkeypatch):
    monkeypatch.setattr(W, "World", OracleBackedWorld)
    monkeypatch.setattr(W, "default_context", lambda: None)


def small_world():
    w = BubbleWorld(WorldConfiguration((0.0, 0.0, 200.0, 200.0)))
    return w, WorldTransaction().update_physics_material("b", PhysicsMaterial(1e4))


def centroid(ring):
    a = np.asarray(ring, np.float64)
    b = np.roll(a, -1, axis=0)
    cross = a[:, 0] * b[:, 1] - b[:, 0] * a[:, 1]
    area = cross.sum()
    return np.array([((a[:, 0] + b[:, 0]) * cross).sum(), ((a[:, 1] + b[:, 1]) * cross).sum()]) / (3 * area)


def test_bounds_contain_the_contour_and_undented_centres_are_contour_centroids():
    rng = np.random.default_rng(0x2B60F5)
    w = BubbleWorld(WorldConfiguration((-40.0, -40.0, 415.0, 740.0), global_force=(0.0, -300.0)))
    tx = WorldTransaction().update_physics_material("b", PhysicsMaterial(229.0, 1.0))
    for k, ((lx, ly), (hx, hy)) in enumerate([((-40, -40), (415, 0)), ((-40, 700), (415, 740)), ((-40, 0), (0, 700)),
                                              ((375, 0), (415, 700))]):
        tx = tx.add(RigidBodyDescriptor(9001 + k, Polygon(((lx, ly), (hx, ly), (hx, hy), (lx, hy))), (0.0, 0.0)))
    placed, radii = [], {}
    while len(placed) < 300:
        r = float(rng.uniform(6, 14))
        p = rng.uniform([r, r], [375 - r, 700 - r])
        if all(math.dist(p, q) > r + s + 1 for q, s in placed):
            placed.append((p, r))
            radii[len(placed)] = r
            tx = tx.add(BubbleDescriptor(len(placed), tuple(p), r, 1.0, "b"))
    w.submit(tx)
    for _ in range(60):
        frame = w.advance(1.0 / 60)
        assert w.diagnostics.last_advance_issue is None
    contours = w.debug_contour_snapshot()
    assert len(contours) == 300
    undented = 0
    for oid, ring in contours.items():
        state = frame.objects[oid]
        lo, hi = np.array(state.bounds[:2]) - 1e-3, np.array(state.bounds[2:]) + 1e-3
        pts = np.asarray(ring)
        assert np.all(pts >= lo) and np.all(pts <= hi), oid
        if state.effective_radius >= 0.98 * radii[oid]:
            undented += 1
            assert math.dist(centroid(ring), state.position) <= 0.01 * state.effective_radius, oid
    assert undented > 0


def test_a_removed_object_is_absent_from_that_frame():
    w, tx = small_world()
    w.submit(tx.add(BubbleDescriptor(1, (60.0, 100.0), 12.0, 1.0, "b")).add(BubbleDescriptor(2, (140.0, 100.0), 12.0, 1.0, "b"))
             .add(RigidBodyDescriptor(3, Polygon(((-10, -10), (10, -10), (10, 10), (-10, 10))), (100.0, 20.0))))
    assert sorted(w.advance(1.0 / 60).objects) == [1, 2, 3]
    w.submit(WorldTransaction().remove(1).remove(3))
    after = w.advance(1.0 / 60)
    assert after.step_index == 2 and sorted(after.objects) == [2]


def test_a_wrapped_bubbles_bounds_move_with_its_contour():
    w, tx = small_world()
    w.submit(tx.add(BubbleDescriptor(1, (190.0, 100.0), 8.0, 1.0, "b", velocity=(900.0, 0.0),
                                     region_exit_policy=RegionExitPolicy.WRAP,
                                     event_interest=frozenset({EventInterest.DID_WRAP}))))
    wrapped = False
    for _ in range(20):
        frame = w.advance(1.0 / 60)
        if any(e.kind == "didWrap" for e in frame.events):
            wrapped = True
            break
    assert wrapped
    state, ring = frame.objects[1], np.asarray(w.debug_contour_snapshot()[1])
    assert state.bounds[0] == pytest.approx(ring[:, 0].min(), abs=1e-3) and state.bounds[2] == pytest.approx(ring[:, 0].max(), abs=1e-3)
    assert state.bounds[1] == pytest.approx(ring[:, 1].min(), abs=1e-3) and state.bounds[3] == pytest.approx(ring[:, 1].max(), abs=1e-3)
    assert state.bounds[0] <= state.position[0] <= state.bounds[2]


def test_a_call_without_a_new_step_publishes_the_same_states():
    w, tx = small_world()
    w.submit(tx.add(BubbleDescriptor(1, (60.0, 100.0), 12.0, 1.0, "b")))
    first = w.advance(1.0 / 60)
    second = w.advance(0.001)
    assert second.step_index == first.step_index and second.objects == first.objects and len(first.objects) == 1
