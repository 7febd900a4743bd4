"""The margin-forced grid rebuild inside a step (GridRebuildTests.swift:1-78 with KickScenePlanner.swift:1-97), on the
oracle: a bubble 128 at 1000 units/s hits a light bubble "2" at rest and kicks it toward an obstacle (a thin wall or a
third bubble) that is not among the "2"'s candidates at the start of the kick frame. The planner is the reference's
one-dimensional double-precision simulation of the pair (restated, vectorised over the 50 contact phases); the
obstacle stands in the middle of the window between the margins and the "2"'s path in that frame. In every substep
the centres keep their order and stay before the wall, and the kick frame rebuilds the grid because a margin ran out;
the same holds with the minimum margin r / 4 for every bubble."""
import math

import numpy as np
import pytest

import clr
from bubblephysics_gb300 import _native as N
from bubblephysics_gb300.scenes import polygon_edges
from bubblephysics_gb300.spec import WorldSpec, make_bubbles
from oracle.oracle import OracleWorld

K = 229.0
DT = 1.0 / 60
R128, R2 = 64.0, 24.0
M128 = float(np.float32((128 / 2) ** (1 / 2.25)))


def simulate(phases):
    """Per phase and frame: the "2"'s position and velocity at the frame's start and its path in the frame."""
    radii, speed, h = R128 + R2, 1000.0, DT / 4000
    x128 = np.zeros_like(phases)
    v128 = np.full_like(phases, speed)
    x2 = radii + speed * DT * phases
    v2 = np.zeros_like(phases)

    def force(a, b):
        eps = (radii - (b - a)) / radii
        return np.where(eps > 0, K * eps / ((1 - eps) * (1 - eps)), 0.0)
    frames = []
    for frame in range(16):
        start_x2, start_v2 = x2.copy(), v2.copy()
        for _ in range(4000):
            f = force(x128, x2)
            v128 = v128 + 0.5 * h * (-f / M128)
            v2 = v2 + 0.5 * h * (f / 1.0)
            x128 = x128 + h * v128
            x2 = x2 + h * v2
            f = force(x128, x2)
            v128 = v128 + 0.5 * h * (-f / M128)
            v2 = v2 + 0.5 * h * (f / 1.0)
        frames.append((start_x2, start_v2, x2 - start_x2))
    return frames


def plan():
    phases = np.arange(50) / 50.0
    frames = simulate(phases)
    best = None
    for p in range(50):
        for frame, (x2, v2, path) in enumerate(frames):
            if 1.05 * abs(v2[p]) * DT <= 5 and path[p] > (best[4] if best else 0):
                best = (p, frame, x2[p], v2[p], path[p])
    p, frame, x2, v2, path = best
    margin2 = max(1.05 * abs(v2) * DT, R2 / 4)
    return dict(frame=frame, x2=x2, path=path, start2=R128 + R2 + 1000.0 * DT * phases[p],
                lower_bubble=margin2 + R2 / 4, lower_wall=margin2, upper=path)


PLAN = plan()


def test_the_planner_finds_a_window_for_both_obstacles():
    assert PLAN["upper"] - PLAN["lower_bubble"] > 3 and PLAN["upper"] - PLAN["lower_wall"] > 3 and PLAN["frame"] > 0


def scene(obstacle, minimum_margin_only):
    lower = PLAN["lower_wall"] if obstacle == "wall" else PLAN["lower_bubble"]
    gap = float(np.float32(lower + 0.4 * (PLAN["upper"] - lower)))
    offset = 300.0 - PLAN["x2"]
    x128, x2 = float(np.float32(offset)), float(np.float32(offset + PLAN["start2"]))
    front = float(np.float32(300.0 + 24.0)) + gap
    centers, radii, masses, vel = [(x128, 0.0), (x2, 0.0)], [R128, R2], [M128, 1.0], [(1000.0, 0.0), (0.0, 0.0)]
    segments = None
    if obstacle == "bubble":
        centers.append((front + 24.0, 0.0))
        radii.append(R2)
        masses.append(1.0)
        vel.append((0.0, 0.0))
    else:
        segments = polygon_edges([(front, -1900.0), (front + 1, -1900.0), (front + 1, 1900.0), (front, 1900.0)], 100,
                                 owner_id=3)
    b = make_bubbles(centers, radii, velocities=vel, masses=masses, stiffness=K)
    spec = WorldSpec(bubbles=b, region=(-2000.0, -2000.0, 2000.0, 2000.0),
                     flags=N.WORLD_MINIMUM_MARGIN_ONLY if minimum_margin_only else 0)
    if segments is not None:
        spec.segments = segments
    return spec, front


@pytest.mark.parametrize("minimum_margin_only", [False, True], ids=["margins", "minimum-margin-only"])
@pytest.mark.parametrize("obstacle", ["wall", "bubble"])
def test_a_kicked_bubble_does_not_cross_and_the_grid_is_rebuilt(obstacle, minimum_margin_only):
    spec, front = scene(obstacle, minimum_margin_only)
    w = OracleWorld(spec, 32)
    w.set_trace(True)
    rebuilds, checked = [], 0
    for k in range(PLAN["frame"] + 8):
        status, rep = w.step(1)
        assert status == N.OK, (k, status)
        rebuilds.append(int(rep[0]["rebuild_count"]))
        _, states = w.trace()
        for s in states:
            a, b = s[0][0], s[1][0]
            checked += 1
            assert b - a > 0, k
            if obstacle == "wall":
                assert a < front and b < front, k
            else:
                c = s[2][0]
                assert c - b > 0 and c - a > 0, k
    assert checked > 0 and rebuilds[PLAN["frame"]] >= 1, (PLAN["frame"], rebuilds)
