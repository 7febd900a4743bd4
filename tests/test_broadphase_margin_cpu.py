"""The margin of the broadphase and the start of a step on the oracle, against the reference's own cases
(NativeMetalSubstepPipelineTests.swift:50-220): a static bubble is stopped at the start of a step and a moving one
keeps its velocity; a pair farther apart than r_a + r_b + tolerance is a candidate only when the margins m_a + m_b
cover the gap, one bubble's margin being enough; the cell width is 2 (r + m) + tolerance; a segment is a candidate
within r + m + tolerance. The reference injects the margins into its kernels; here they come from the step's own rule
max(1.05 (|v| dt + |a0| dt^2 / 2), r / 4), with a velocity across the pair's axis so that the pair does not close."""
import math

import numpy as np

from bubblephysics_gb300 import _native as N
from bubblephysics_gb300.scenes import polygon_edges
from bubblephysics_gb300.spec import WorldSpec, make_bubbles
from oracle.oracle import OracleWorld

DT = 1.0 / 60
SLACK = 0.5


def speed_for(margin):
    """A speed whose margin 1.05 |v| dt is `margin` (above r / 4 = 3 for r = 12)."""
    return float(np.float32(margin / (1.05 * DT)))


def pair(distance, margins, r=12.0):
    vel = [(0.0, speed_for(m) if m > r / 4 else 0.0) for m in margins]
    b = make_bubbles([(0.0, 0.0), (distance, 0.0)], r, velocities=vel, masses=0.36, stiffness=0.0)
    spec = WorldSpec(bubbles=b, separation_tolerance=SLACK)
    w = OracleWorld(spec, 32)
    w.step(1)
    return w


def test_a_static_bubble_stops_and_a_moving_one_keeps_its_velocity():
    b = make_bubbles([(5.0, 6.0), (90.0, 90.0)], 12.0, velocities=[(30.0, 0.0), (7.0, 7.0)], masses=0.36,
                     static=[False, True])
    w = OracleWorld(WorldSpec(bubbles=b), 32)
    w.step(1)
    out = w.bubbles()
    assert out["velocity"][0].tolist() == [30.0, 0.0]
    assert out["velocity"][1].tolist() == [0.0, 0.0] and out["center"][1].tolist() == [90.0, 90.0]


def test_margins_widen_pair_candidates_and_the_grid_cell():
    natural = pair(60.0, [3.0, 3.0])            # r / 4 each: 60 > 24 + 6 + 0.5
    assert len(natural.candidates()) == 0
    assert natural.cells()[1][0] == math.floor(60.0 / (2 * (12 + 3) + SLACK))
    padded = pair(60.0, [20.0, 20.0])           # 60 <= 24 + 40 + 0.5
    keys = padded.candidates()
    assert len(keys) == 1 and keys[0]["kind"] == 0
    assert padded.cells()[1][0] == math.floor(60.0 / (2 * (12 + 20) + SLACK))  # the cell width grew to ~64.5
    assert len(pair(90.0, [20.0, 20.0]).candidates()) == 0   # 90 > 64.5
    assert len(pair(60.0, [40.0, 3.0]).candidates()) == 1    # one margin suffices: 60 <= 24 + 43 + 0.5


def test_margins_widen_segment_candidates():
    def wall_at(x, margin):
        vel = [(0.0, speed_for(margin) if margin > 3.0 else 0.0)]
        b = make_bubbles([(0.0, 0.0)], 12.0, velocities=vel, masses=0.36, stiffness=0.0)
        segs = polygon_edges([(x, -500.0), (x + 10.0, -500.0), (x + 10.0, 500.0), (x, 500.0)], 100, owner_id=9)
        w = OracleWorld(WorldSpec(bubbles=b, segments=segs, separation_tolerance=SLACK), 32)
        w.step(1)
        return [k for k in w.candidates() if k["kind"] == 1]
    assert len(wall_at(15.0, 3.0)) >= 1        # reach 12 + 3 + 0.5 = 15.5 covers 15
    assert len(wall_at(30.0, 3.0)) == 0         # 30 > 15.5
    assert len(wall_at(30.0, 20.0)) >= 1        # 30 <= 12 + 20 + 0.5
