"""The four budget scenes (BudgetScenes, PublicWorldStressBenchmark.swift:829-980) through the world API on a stand-in
device world that forwards to the oracle, against BudgetSceneTests.swift:37-181: 150 bubbles each in a 375 x 700 frame
of static walls (K_c 229, gamma 1; the crowd radius 12, mass 0.36 on a 23.5 grid): a resting crowd; "band to wall", a
"2" (radius 24, mass 1) held by the band (K 22) towards a target 900 units out, starting at rest at the equilibrium
against a vertical wall at x = 330; "head-on 128", two 128s (radius 64) meeting at 1000 units/s each; "shot into
crowd", a "2" shot at 3000 units/s through a gap in the crowd's frame. The impacts are renewed every 20 steps by a
replace of their participants. Every scene runs without a failed step; the resting crowd takes one substep per step,
the impacts take more in at least 10 % of the steps with a peak at least 3 times higher; the band holds the "2"
against the wall with at least 2 substeps in every measured step."""
import math

import pytest

from bubblephysics_gb300 import world as W
from bubblephysics_gb300.world import (BubbleDescriptor, BubbleDrivePolicy, BubbleWorld, MotionRole, PhysicsMaterial,
                                       Polygon, RigidBodyDescriptor, WorldConfiguration, WorldTransaction)
from test_world_api_oracle_cpu import OracleBackedWorld

HEIGHT, WIDTH, SPACING = 700.0, 375.0, 23.5
MASS_128 = 64.0 ** (1 / 2.25)
BAND_TARGET, BAND_WALL, BAND_RADIUS = (900.0, 100.0), 330.0, 24.0
SCENES = ("resting-crowd", "band-to-wall", "head-on-128", "shot-into-crowd")


@pytest.fixture(autouse=True)
def oracle_backed(monkeypatch):
    monkeypatch.setattr(W, "World", OracleBackedWorld)
    monkeypatch.setattr(W, "default_context", lambda: None)


def band_rest_x():
    """The "2"'s centre where the band's pull K (target - x) meets the wall's contact law (in double)."""
    x = BAND_WALL - BAND_RADIUS
    for _ in range(50):
        q = 22.0 * (BAND_TARGET[0] - x) / 229.0
        epsilon = 2 * q / ((2 * q + 1) + math.sqrt(4 * q + 1))
        x = BAND_WALL - BAND_RADIUS * (1 - epsilon)
    return float(x)


def participants(scene):
    if scene == "band-to-wall":
        return [(150, (band_rest_x(), 100.0), (0.0, 0.0), 24.0, 1.0, BubbleDrivePolicy(22.0))]
    if scene == "head-on-128":
        return [(149, (80.0, 585.0), (1000.0, 0.0), 64.0, MASS_128, None),
                (150, (295.0, 585.0), (-1000.0, 0.0), 64.0, MASS_128, None)]
    if scene == "shot-into-crowd":
        return [(150, (30.0, 365.0), (3000.0, 0.0), 24.0, 1.0, None)]
    return []


def crowd(scene, count):
    lo, hi, cy = {"band-to-wall": (1, 374, 450), "head-on-128": (1, 374, 235),
                  "shot-into-crowd": (61, 374, 365)}.get(scene, (1, 374, 350))
    columns = int((hi - lo) / SPACING)
    rows = (count + columns - 1) // columns
    x0 = lo + (hi - lo - columns * SPACING) / 2 + SPACING / 2
    y0 = cy - (rows - 1) * SPACING / 2
    return [(x0 + (k % columns) * SPACING, y0 + (k // columns) * SPACING) for k in range(count)]


def rect(i, lo, hi):
    return RigidBodyDescriptor(i, Polygon(((lo[0], lo[1]), (hi[0], lo[1]), (hi[0], hi[1]), (lo[0], hi[1]))), (0.0, 0.0))


def participant(p):
    oid, at, velocity, radius, mass, policy = p
    return BubbleDescriptor(oid, at, radius, mass, 1, velocity=velocity, drive_policy=policy)


def initial_transaction(scene):
    tx = WorldTransaction().update_physics_material(1, PhysicsMaterial(229.0, 1.0))
    extra = participants(scene)
    for k, p in enumerate(crowd(scene, 150 - len(extra))):
        tx = tx.add(BubbleDescriptor(k + 1, p, 12.0, 0.36, 1))
    for p in extra:
        tx = tx.add(participant(p))
    walls = [rect(10_001, (0, 0), (1, HEIGHT)), rect(10_002, (374, 0), (375, HEIGHT)), rect(10_003, (0, 0), (375, 1)),
             rect(10_004, (0, HEIGHT - 1), (375, HEIGHT))]
    walls += {"band-to-wall": [rect(10_005, (1, 200), (374, 201)), rect(10_006, (330, 1), (331, 200))],
              "head-on-128": [rect(10_005, (1, 470), (374, 471))],
              "shot-into-crowd": [rect(10_005, (60, 1), (61, 330)), rect(10_006, (60, 400), (61, HEIGHT - 1))]}.get(scene, [])
    for wall in walls:
        tx = tx.add(wall)
    if scene == "band-to-wall":
        tx = tx.begin_player_drive(150, BAND_TARGET)
    return tx


def step_transaction(scene, step):
    if scene not in ("head-on-128", "shot-into-crowd") or step == 0 or step % 20:
        return None
    tx = WorldTransaction()
    for p in participants(scene):
        tx = tx.replace(p[0], participant(p))
    return tx


def run(scene, warmup=30, measured=120):
    """The measured steps: (frame, substeps of its step)."""
    world = BubbleWorld(WorldConfiguration((0.0, 0.0, WIDTH, HEIGHT), contours=False))
    world.submit(initial_transaction(scene))
    samples = []
    for step in range(warmup + measured):
        tx = step_transaction(scene, step)
        if tx is not None:
            world.submit(tx)
        frame = world.advance(1.0 / 60)
        assert world.diagnostics.last_advance_issue is None and world.diagnostics.failure_reason is None, (scene, step)
        assert world.diagnostics.contact_candidate_overflow == 0, (scene, step)
        if step >= warmup:
            samples.append((frame, world.diagnostics.last_step_substeps))
    return samples


@pytest.mark.parametrize("scene", SCENES)
def test_every_scene_builds_with_150_bubbles_walls_and_no_dynamic_bodies(scene):
    ops = initial_transaction(scene).operations
    bubbles = [op[1] for op in ops if op[0] == "add" and isinstance(op[1], BubbleDescriptor)]
    bodies = [op[1] for op in ops if op[0] == "add" and isinstance(op[1], RigidBodyDescriptor)]
    assert len(bubbles) == 150 and len(bodies) >= 4
    assert all(b.motion_role == MotionRole.STATIC for b in bodies)


@pytest.mark.parametrize("scene", SCENES)
def test_every_scene_runs_without_a_failed_step(scene):
    assert len(run(scene)) == 120


def test_impact_scenes_take_more_substeps_than_the_resting_crowd():
    resting = max(s for _, s in run("resting-crowd", measured=200))
    assert resting == 1  # a crowd at rest takes exactly one substep per step
    for scene in ("head-on-128", "shot-into-crowd"):
        substeps = [s for _, s in run(scene, measured=200)]
        assert sum(s > 1 for s in substeps) >= 0.1 * len(substeps), (scene, substeps)
        assert max(substeps) >= 3 * resting, scene


def test_band_to_wall_presses_the_two_against_the_wall_in_every_measured_step():
    for frame, substeps in run("band-to-wall"):
        distance = BAND_WALL - frame.objects[150].position[0]
        assert 0 < distance < BAND_RADIUS and substeps >= 2, (distance, substeps)


def test_impact_scenes_never_reject_their_replace():
    for scene in ("head-on-128", "shot-into-crowd"):
        samples = run(scene, measured=60)
        assert not any(e.kind == "transactionRejected" for f, _ in samples for e in f.events), scene
        assert sum(len(f.transaction_receipts) for f, _ in samples) > 0, scene
