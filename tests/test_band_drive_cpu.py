"""Player and motor drives through the world API (BubbleDrivePolicy, begin/update/end_player_drive, set_motor_drive,
DriveFeedback), on a stand-in device world that forwards to the oracle, against the reference's own cases:
BandDriveTests.swift:20-165 (the steady speed K s / (m gamma) with the mean-stretch correction within 3 %, the speed
ratio as the inverse mass ratio within 5 %, a released bubble keeps its velocity, the velocity change between frames
follows the feedback stretch within 1 %), BandStabilityThresholdTests.swift:30-82 (K_band <= m / (16 dt^2) at
staging) and the drive staging rules of TransactionStager.swift:288-350 (huge finite motor drives, a policy needed to
grab, one drive at a time, the previous role restored)."""
import math

import numpy as np
import pytest

from bubblephysics_gb300 import world as W
from bubblephysics_gb300.world import (BubbleDescriptor, BubbleDrivePolicy, BubbleWorld, MotionRole as M, MotorDrive,
                                       PhysicsMaterial, Polygon, RigidBodyDescriptor,
                                       TransactionRejectionReason as R, WorldConfiguration, WorldTransaction)
from test_world_api_oracle_cpu import OracleBackedWorld

DT = 1.0 / 60
HALF, THICK = (180.0, 320.0), 48.0


@pytest.fixture
def oracle_backed(monkeypatch):
    monkeypatch.setattr(W, "World", OracleBackedWorld)
    monkeypatch.setattr(W, "default_context", lambda: None)


def crowd_world(damping, stiffness=1e9):
    """The frame of CrowdSceneSupport.swift: an interior of 360 x 640 inside four static rectangles 48 thick; the
    bubble material K_c = 1e9 is the scene's near-rigid one, for tests where contact is not the subject."""
    ix, iy = HALF
    ox, oy = ix + THICK, iy + THICK
    world = BubbleWorld(WorldConfiguration((-ox, -oy, ox, oy)))
    tx = WorldTransaction().update_physics_material("soft", PhysicsMaterial(stiffness, damping))
    for k, ((lx, ly), (hx, hy)) in enumerate([((-ox, -oy), (-ix, oy)), ((ix, -oy), (ox, oy)), ((-ix, -oy), (ix, -iy)),
                                              ((-ix, iy), (ix, oy))]):
        tx = tx.add(RigidBodyDescriptor(9001 + k, Polygon(((lx, ly), (hx, ly), (hx, hy), (lx, hy))), (0.0, 0.0)))
    return world, tx


def speed(state):
    return math.hypot(*state.velocity)


def steady_speed(k_band, stretch, mass, gamma):
    decay = math.exp(-gamma * DT)
    f = (1 - decay) / gamma
    k = k_band / mass
    return k * stretch * f / (1 - decay + k * f * DT / 2)


def steady_state(mass, gamma, k_band, stretch, seconds=4.0):
    world, tx = crowd_world(gamma)
    start = (-150.0, 0.0)
    world.submit(tx.add(BubbleDescriptor(1, start, 10.0, mass, "soft", drive_policy=BubbleDrivePolicy(k_band)))
                 .begin_player_drive(1, (start[0] + stretch, start[1])))
    peak, last = 0.0, None
    for _ in range(int(round(seconds / DT))):
        frame = world.advance(DT)
        assert world.diagnostics.last_advance_issue is None
        last = frame.objects[1]
        peak = max(peak, speed(last))
        achieved = frame.drive_feedback[0].achieved_point
        world.submit(WorldTransaction().update_player_drive(1, (achieved[0] + stretch, achieved[1])))
    return speed(last), peak


def test_steady_speed_is_stiffness_times_stretch_over_mass_times_damping(oracle_backed):
    v, peak = steady_state(1.0, 2.0, 60.0, 1.0)
    expected = steady_speed(60.0, 1.0, 1.0, 2.0)
    assert abs(expected - 30.0) <= 0.25 * 30.0  # the correction is small
    assert abs(v - expected) <= 0.03 * expected and peak < 600


def test_steady_speed_ratio_is_the_inverse_mass_ratio(oracle_backed):
    light, _ = steady_state(1.0, 2.0, 60.0, 1.0)
    heavy, _ = steady_state(2.5, 2.0, 60.0, 1.0)
    expected = steady_speed(60.0, 1.0, 1.0, 2.0) / steady_speed(60.0, 1.0, 2.5, 2.0)
    assert abs(light / heavy - expected) <= 0.05 * expected and expected > 2 and heavy > 1


def test_releasing_the_drive_keeps_the_velocity(oracle_backed):
    world, tx = crowd_world(0.0)
    start = (-150.0, 0.0)
    world.submit(tx.add(BubbleDescriptor(1, start, 10.0, 1.0, "soft", drive_policy=BubbleDrivePolicy(60.0)))
                 .begin_player_drive(1, (start[0] + 1, start[1])))
    for _ in range(60):
        frame = world.advance(DT)
        before = frame.objects[1]
        achieved = frame.drive_feedback[0].achieved_point
        world.submit(WorldTransaction().update_player_drive(1, (achieved[0] + 1, achieved[1])))
    v = speed(before)
    assert v > 5
    world.submit(WorldTransaction().end_player_drive(1))
    release = world.advance(DT)
    assert world.diagnostics.last_advance_issue is None and release.drive_feedback == ()
    assert abs(release.objects[1].velocity[0] - v) <= 0.01 * v
    for _ in range(30):
        later = world.advance(DT)
    assert abs(later.objects[1].velocity[0] - v) <= 0.01 * v


def test_velocity_change_between_frames_follows_the_feedback_stretch(oracle_backed):
    world, tx = crowd_world(0.0)
    k_band, mass = 30.0, 2.0
    world.submit(tx.add(BubbleDescriptor(1, (0.0, 0.0), 10.0, mass, "soft", drive_policy=BubbleDrivePolicy(k_band)))
                 .begin_player_drive(1, (20.0, 12.0)))
    previous = world.advance(DT)
    for _ in range(4):
        nxt = world.advance(DT)
        fb = previous.drive_feedback[0]
        expected = (np.array(fb.target) - np.array(fb.achieved_point)) * (k_band / mass * DT)
        delta = np.array(nxt.objects[1].velocity) - np.array(previous.objects[1].velocity)
        assert abs(delta[0] - expected[0]) <= 0.01 * abs(expected[0])
        assert abs(delta[1] - expected[1]) <= 0.01 * abs(expected[1])
        previous = nxt


def staged(dt=1.0 / 60):
    state = W._State(fixed_time_step=dt)
    state, rec, ev = W.stage([(1, WorldTransaction().update_physics_material("soft", PhysicsMaterial(1e9)))], state,
                             (-1000.0, -1000.0, 1000.0, 1000.0))
    return state


def band_bubble(i, mass, k_band):
    return BubbleDescriptor(i, (i * 10.0, 0.0), 2.0, mass, "soft", drive_policy=BubbleDrivePolicy(k_band))


def rejection(state, tx):
    _, rec, ev = W.stage([(2, tx)], state, (-1000.0, -1000.0, 1000.0, 1000.0))
    return None if rec else ev[0].rejection


@pytest.mark.parametrize("mass,accepted,rejected,dt", [
    (1.0, [22, 224], [226, 1000, 10_000], 1 / 60), (38.0, [22, 8000, 8540], [8560, 20_000], 1 / 60),
    (0.36, [22, 80], [82, 1000], 1 / 60), (2.0, [400, 440], [460, 1000, 3000], 1 / 60),
    (1.0, [50, 54], [58, 100], 1 / 30), (1.0, [800, 880], [940, 2000], 1 / 120)])
def test_band_stability_threshold(mass, accepted, rejected, dt):
    state = staged(dt)
    for k in accepted:
        assert rejection(state, WorldTransaction().add(band_bubble(1, mass, k))) is None, k
    for k in rejected:
        r = rejection(state, WorldTransaction().add(band_bubble(1, mass, k)))
        assert (r.operation_index, r.reason, r.detail) == (0, R.INVALID_VALUE, "drive.bandStiffness"), k


def test_replace_is_checked_with_the_same_threshold():
    state = staged()
    state, _, _ = W.stage([(2, WorldTransaction().add(band_bubble(1, 1.0, 22)))], state, (-1000.0, -1000.0, 1000.0, 1000.0))
    assert rejection(state, WorldTransaction().replace(1, band_bubble(1, 1.0, 226))).detail == "drive.bandStiffness"


def test_huge_finite_motor_drives_are_refused():
    state = staged()
    state, _, _ = W.stage([(2, WorldTransaction().add(band_bubble(1, 1.0, 22)))], state, (-1000.0, -1000.0, 1000.0, 1000.0))
    for drive, name in ((MotorDrive((3e38, 0.0)), "motor.force"), (MotorDrive((0.0, -3e38)), "motor.force"),
                        (MotorDrive(torque=3e38), "motor.torque")):
        assert rejection(state, WorldTransaction().set_motor_drive(1, drive)).detail == name
    assert rejection(state, WorldTransaction().set_motor_drive(1, MotorDrive((1e6, -1e6), 1e6))) is None


def test_player_drive_staging_rules():
    state = staged()
    state, _, _ = W.stage([(2, WorldTransaction().add(band_bubble(1, 1.0, 22))
                            .add(BubbleDescriptor(2, (50.0, 0.0), 2.0, 1.0, "soft")))], state,
                          (-1000.0, -1000.0, 1000.0, 1000.0))
    r = rejection(state, WorldTransaction().begin_player_drive(2, (0.0, 0.0)))
    assert (r.reason, r.detail) == (R.INCOMPATIBLE_OBJECT_KIND, 2)  # no drive policy
    assert rejection(state, WorldTransaction().update_player_drive(1, (0.0, 0.0))).reason == R.DRIVE_NOT_ACTIVE
    assert rejection(state, WorldTransaction().end_player_drive(1)).reason == R.DRIVE_NOT_ACTIVE
    twice = WorldTransaction().begin_player_drive(1, (1.0, 0.0)).begin_player_drive(1, (2.0, 0.0))
    assert rejection(state, twice).reason == R.DRIVE_ALREADY_ACTIVE
    assert rejection(state, WorldTransaction().begin_player_drive(1, (2e6, 0.0))).detail == "playerDrive.target"
    driving, _, _ = W.stage([(3, WorldTransaction().set_motion(1, M.STATIC).begin_player_drive(1, (1.0, 0.0)))], state,
                            (-1000.0, -1000.0, 1000.0, 1000.0))
    assert driving.bubbles[1].desc.motion_role == M.PLAYER_DRIVEN and driving.bubbles[1].drive_id == 1
    ended, _, _ = W.stage([(4, WorldTransaction().end_player_drive(1))], driving, (-1000.0, -1000.0, 1000.0, 1000.0))
    assert ended.bubbles[1].desc.motion_role == M.STATIC and ended.bubbles[1].drive_target is None


def test_motor_drive_pushes_with_its_force(oracle_backed):
    """A motor-driven bubble in free space (gamma 0) gains F / m dt per step."""
    world, tx = crowd_world(0.0)
    world.submit(tx.add(BubbleDescriptor(1, (0.0, 0.0), 10.0, 2.0, "soft"))
                 .set_motor_drive(1, MotorDrive((30.0, -10.0))))
    v0 = np.array(world.advance(DT).objects[1].velocity)
    v1 = np.array(world.advance(DT).objects[1].velocity)
    assert np.allclose(v1 - v0, np.array([15.0, -5.0]) * DT, rtol=1e-4)
    world.submit(WorldTransaction().set_motion(1, M.DYNAMIC))  # leaving the role drops the motor
    v2 = np.array(world.advance(DT).objects[1].velocity)
    v3 = np.array(world.advance(DT).objects[1].velocity)
    assert np.allclose(v3, v2, atol=1e-6)


def test_drive_blocked_is_emitted_on_entry_and_feedback_stays_continuous(oracle_backed):
    """EventCompactorTests.swift:3-20 on a world: a bubble dragged into a wall reports driveBlocked once when the wall
    first stands against the drive, while the feedback keeps naming the blocker every step."""
    world, tx = crowd_world(4.0, stiffness=2000.0)  # the wall-press material of BandDriveTests.swift:77
    r = 20.0
    x0 = -HALF[0] + r + 5.0
    world.submit(tx.add(BubbleDescriptor(1, (x0, 0.0), r, 1.0, "soft", drive_policy=BubbleDrivePolicy(10.0, 300.0),
                                         event_interest=frozenset({W.EventInterest.DRIVE_BLOCKED})))
                 .begin_player_drive(1, (x0 - 40.0, 0.0)))
    blocked, blockers = [], []
    for _ in range(120):
        frame = world.advance(DT)
        blocked += [e.objects for e in frame.events if e.kind == "driveBlocked"]
        fb = frame.drive_feedback[0]
        blockers.append(fb.blocking_contact.object_id if fb.blocking_contact else None)
    assert blocked == [(1, 9001)]  # the left wall
    first = blockers.index(9001)
    assert all(b == 9001 for b in blockers[first:])


def pressed_against_the_wall(stretch):
    world, tx = crowd_world(4.0, stiffness=2000.0)
    x = -(HALF[0] - 20.0)
    world.submit(tx.add(BubbleDescriptor(1, (x, 0.0), 20.0, 1.0, "soft", drive_policy=BubbleDrivePolicy(10.0, 300.0)))
                 .begin_player_drive(1, (x - stretch, 0.0)))
    for _ in range(361):
        frame = world.advance(DT)
        assert world.diagnostics.last_advance_issue is None
    state, fb = frame.objects[1], frame.drive_feedback[0]
    depth = 20.0 - (HALF[0] + state.position[0])
    return depth, abs(fb.target[0] - fb.achieved_point[0]), speed(state)


def test_wall_press_matches_the_band_force_below_the_limit_and_saturates_above_it(oracle_backed):
    """BandDriveTests.swift:73-104: at rest the contact force of the law at the wall depth equals K_band times the
    stretch (10 %) below maximum_force / K_band, and maximum_force above it, at the same depth (0.5)."""
    import clr
    force = lambda depth: clr.force(depth / 20.0, 2000.0)
    for stretch in (6.0, 15.0, 24.0):
        depth, s, v = pressed_against_the_wall(stretch)
        assert v < 0.1 and abs(force(depth) - 10.0 * s) <= 0.1 * 10.0 * s, (stretch, depth, s)
    saturated = []
    for stretch in (45.0, 90.0):
        depth, s, v = pressed_against_the_wall(stretch)
        assert v < 0.1 and abs(force(depth) - 300.0) <= 30.0
        saturated.append(depth)
    assert abs(saturated[0] - saturated[1]) <= 0.5


def test_a_fast_small_bubble_settles_at_the_law_without_crossing_the_edge(oracle_backed):
    """WallImpactTests.swift:12-58: a bubble r 24 pulled by the band (K 30, F_max 1200) from 150 units off the wall
    hits it faster than max(40, 2 r) (K_c 20 / 0.0108, gamma 5), dents deeper than at rest but never reaches the edge
    (eps < 1 in every step), and settles at the law's eps* for F_max (2 %)."""
    import clr
    r, kc = 24.0, float(np.float32(20.0) / np.float32(0.0108))
    world, tx = crowd_world(5.0, stiffness=kc)
    start = -HALF[0] + r + 150.0
    world.submit(tx.add(BubbleDescriptor(1, (start, 0.0), r, r * r / 400, "soft",
                                         drive_policy=BubbleDrivePolicy(30.0, 1200.0)))
                 .begin_player_drive(1, (-2000.0, 0.0)))
    peak, final, impact, behind = -math.inf, 0.0, 0.0, []
    for step in range(360):
        frame = world.advance(DT)
        assert world.diagnostics.last_advance_issue is None and world.diagnostics.failure_reason is None
        state = frame.objects[1]
        ratio = (r - (HALF[0] + state.position[0])) / r
        peak, final = max(peak, ratio), ratio
        if ratio >= 1:
            behind.append(step)
        if ratio <= 0:
            impact = max(impact, -state.velocity[0])
    expected = clr.epsilon(1200.0 / kc)
    assert impact > max(40.0, 2 * r) and abs(final - expected) <= 0.02 * expected
    assert expected < peak < 1 and behind == []
