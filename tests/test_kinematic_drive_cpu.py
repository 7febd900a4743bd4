"""The kinematic drives at the start of a step (MotionControllers.prepare), against KinematicDriveControllerTests.swift:
5-77: a 2 x 2 kinematic box at (10, 20) under the global force (0, -500); without a drive it stands still, a velocity
drive keeps the exact pose over 600 steps of float integration (1e-4), a target drive reaches its pose in one step, a
path drive heads for its point at its speed and stops on arrival, and a pose moved outside the track (a wrap) starts a
new track. A kinematic body is never moved by forces."""
import numpy as np

from bubblephysics_gb300.world import (KinematicDrive, MotionRole, PathDrive, Polygon, RigidBodyDescriptor,
                                       WorldTransaction, _State, prepare_kinematic, stage)

DURATION = 1.0 / 60
BOX = 1
REGION = (-1000.0, -1000.0, 1000.0, 1000.0)


def seeded(drive=None):
    tx = WorldTransaction().add(RigidBodyDescriptor(BOX, Polygon(((0.0, 0.0), (2.0, 0.0), (2.0, 2.0), (0.0, 2.0))),
                                                    (10.0, 20.0), motion_role=MotionRole.KINEMATIC))
    if drive is not None:
        tx = tx.set_kinematic_drive(BOX, drive)
    state = _State()
    state.global_force = (0.0, -500.0)
    state, receipts, events = stage([(1, tx)], state, REGION)
    assert len(receipts) == 1 and not events  # no interest asked, no didAdd
    return state


def test_a_body_without_a_drive_stands_still_despite_the_global_force():
    state = seeded()
    prepare_kinematic(state, DURATION)
    assert tuple(state.bodies[BOX].velocity) == (0.0, 0.0) and state.bodies[BOX].angular_velocity == 0.0


def test_a_velocity_drive_keeps_the_exact_pose_over_many_steps():
    state = seeded(KinematicDrive.velocity((40.0, -3.0), 0.7))
    body = state.bodies[BOX]
    start, start_angle = body.position.copy(), body.angle
    dt = np.float32(DURATION)
    for _ in range(600):
        prepare_kinematic(state, DURATION)
        body.position = (body.position + body.velocity * dt).astype(np.float32)  # the solver's float step
        body.angle = float(np.float32(body.angle) + np.float32(body.angular_velocity) * dt)
    time = float(np.float32(600 * DURATION))
    assert abs(body.position[0] - (start[0] + 40 * time)) <= 1e-4
    assert abs(body.position[1] - (start[1] - 3 * time)) <= 1e-4
    assert abs(body.angle - (start_angle + 0.7 * time)) <= 1e-4


def test_a_target_drive_reaches_its_pose_in_one_step():
    state = seeded(KinematicDrive.target((30.0, 25.0), 0.5))
    prepare_kinematic(state, DURATION)
    body = state.bodies[BOX]
    dt = np.float32(DURATION)
    assert abs(body.velocity[0] * dt - 20) <= 1e-4 and abs(body.velocity[1] * dt - 5) <= 1e-4
    assert abs(np.float32(body.angular_velocity) * dt - 0.5) <= 1e-6


def test_a_path_drive_heads_for_its_point_at_its_speed_and_stops_on_arrival():
    state = seeded(KinematicDrive.path(PathDrive(((10.0, 50.0),), 30.0)))
    prepare_kinematic(state, DURATION)
    body = state.bodies[BOX]
    assert abs(body.velocity[1] - 30) <= 1e-4 and abs(body.velocity[0]) <= 1e-4
    body.position = np.array([10.0, 50.0], np.float32)
    prepare_kinematic(state, DURATION)
    assert tuple(body.velocity) == (0.0, 0.0)


def test_a_pose_changed_outside_the_track_starts_a_new_track():
    state = seeded(KinematicDrive.velocity((10.0, 0.0), 0.0))
    prepare_kinematic(state, DURATION)
    state.bodies[BOX].position = np.array([500.0, 500.0], np.float32)  # e.g. a region wrap
    prepare_kinematic(state, DURATION)
    v = state.bodies[BOX].velocity
    assert abs(v[0] - 10) <= 1e-3 and abs(v[1]) <= 1e-3


def test_target_and_path_drives_move_a_body_in_the_world(monkeypatch):
    """Through the world API beside a bubble (the device world forwards to the oracle): a target drive puts the box on
    its pose after one step; a path drive then takes it to its last point at its speed and holds it there."""
    from bubblephysics_gb300 import world as W
    from bubblephysics_gb300.world import BubbleDescriptor, BubbleWorld, PhysicsMaterial, WorldConfiguration
    from test_world_api_oracle_cpu import OracleBackedWorld
    monkeypatch.setattr(W, "World", OracleBackedWorld)
    monkeypatch.setattr(W, "default_context", lambda: None)
    world = BubbleWorld(WorldConfiguration(REGION, contours=False))
    box = RigidBodyDescriptor(BOX, Polygon(((0.0, 0.0), (2.0, 0.0), (2.0, 2.0), (0.0, 2.0))), (10.0, 20.0),
                              motion_role=MotionRole.KINEMATIC)
    world.submit(WorldTransaction().update_physics_material("m", PhysicsMaterial(229.0))
                 .add(BubbleDescriptor(2, (-500.0, -500.0), 5.0, 1.0, "m")).add(box)
                 .set_kinematic_drive(BOX, KinematicDrive.target((30.0, 25.0), 0.5)))
    frame = world.advance(DURATION)
    state = frame.objects[BOX]
    assert abs(state.position[0] - 30) <= 1e-4 and abs(state.position[1] - 25) <= 1e-4
    assert abs(state.rotation - 0.5) <= 1e-5
    world.submit(WorldTransaction().set_kinematic_drive(BOX, KinematicDrive.path(
        PathDrive(((30.0, 55.0), (60.0, 55.0)), 30.0))))
    for _ in range(150):  # 30 units up, then 30 across, at 30 units/s: 2 s
        frame = world.advance(DURATION)
    state = frame.objects[BOX]
    assert abs(state.position[0] - 60) <= 1e-3 and abs(state.position[1] - 55) <= 1e-3
    assert tuple(state.velocity) == (0.0, 0.0)
    assert frame.objects[2].position == (-500.0, -500.0)
