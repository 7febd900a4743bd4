"""Motion commands through the world API on a stand-in device world that forwards to the oracle, against
MotionCommandTests.swift:7-230: a player drive publishes feedback every frame under one drive id and ends without
events; drive models refuse non-finite or empty values at construction; a non-finite or huge (3e38) kinematic drive
rejects its transaction while the world keeps stepping, a large but reasonable one is accepted; a band target beyond
1e6 is refused at begin and at update, one of 9e5 is accepted."""
import math

import pytest

from bubblephysics_gb300 import world as W
from bubblephysics_gb300.world import (BubbleDescriptor, BubbleDrivePolicy, BubbleWorld, KinematicDrive, MotionRole,
                                       MotorDrive, PathDrive, PhysicsMaterial, Polygon, RigidBodyDescriptor,
                                       TransactionRejectionReason as R, WorldConfiguration, WorldTransaction)
from test_world_api_oracle_cpu import OracleBackedWorld

REGION = (-20.0, -20.0, 20.0, 20.0)
STEP = 1.0 / 60


@pytest.fixture(autouse=True)
def oracle_backed(monkeypatch):
    monkeypatch.setattr(W, "World", OracleBackedWorld)
    monkeypatch.setattr(W, "default_context", lambda: None)


def rejection(frame, token):
    found = [e.rejection for e in frame.events if e.kind == "transactionRejected" and e.token == token]
    return found[0] if found else None


def test_a_player_drive_publishes_feedback_every_frame_and_ends_without_events():
    world = BubbleWorld(WorldConfiguration(REGION))
    world.submit(WorldTransaction().update_physics_material(1, PhysicsMaterial(1e9))
                 .add(BubbleDescriptor(1, (0.0, 0.0), 0.5, 1.0, 1, drive_policy=BubbleDrivePolicy(60.0)))
                 .begin_player_drive(1, (5.0, 0.0)))
    first = world.advance(STEP)
    assert len(first.transaction_receipts) == 1 and not first.events
    feedback = first.drive_feedback[0]
    assert feedback.object_id == 1 and feedback.target == (5.0, 0.0) and 0 < feedback.achieved_point[0] < 1
    second = world.advance(STEP)
    assert second.drive_feedback[0].player_drive_id == feedback.player_drive_id
    assert second.drive_feedback[0].achieved_point[0] > feedback.achieved_point[0]
    world.submit(WorldTransaction().end_player_drive(1))
    assert not world.advance(STEP).drive_feedback and world.diagnostics.last_advance_issue is None


def test_drive_models_refuse_non_finite_and_empty_values():
    for build in (lambda: PathDrive((), 1.0), lambda: PathDrive(((1.0, 0.0),), 0.0),
                  lambda: MotorDrive((math.inf, 0.0)), lambda: BubbleDrivePolicy(-math.inf),
                  lambda: BubbleDrivePolicy(10.0, math.nan)):
        with pytest.raises(ValueError):
            build()


def kinematic_world():
    world = BubbleWorld(WorldConfiguration(REGION))
    world.submit(WorldTransaction().add(RigidBodyDescriptor(1, Polygon(((0.0, 0.0), (2.0, 0.0), (2.0, 2.0), (0.0, 2.0))),
                                                            (0.0, 0.0), motion_role=MotionRole.KINEMATIC)))
    assert world.advance(STEP).step_index == 1
    return world


@pytest.mark.parametrize("drive, name", [
    (KinematicDrive.velocity((math.nan, 0.0), 0.0), "kinematicDrive.linear"),
    (KinematicDrive.target((3e38, 0.0), 0.0), "kinematicDrive.position"),
    (KinematicDrive.target((0.0, 0.0), 3e38), "kinematicDrive.rotation"),
    (KinematicDrive.velocity((0.0, -3e38), 0.0), "kinematicDrive.linear"),
    (KinematicDrive.velocity((0.0, 0.0), 3e38), "kinematicDrive.angular")])
def test_a_non_finite_or_huge_kinematic_drive_is_rejected_and_the_world_keeps_stepping(drive, name):
    world = kinematic_world()
    token = world.submit(WorldTransaction().set_kinematic_drive(1, drive))
    rejecting = world.advance(STEP)
    r = rejection(rejecting, token)
    assert r is not None and (r.reason, r.detail) == (R.INVALID_VALUE, name)
    assert world.diagnostics.last_advance_issue is None
    assert world.advance(STEP).step_index == rejecting.step_index + 1 and world.diagnostics.last_advance_issue is None


def test_a_large_but_reasonable_kinematic_drive_is_accepted():
    world = kinematic_world()
    token = world.submit(WorldTransaction().set_kinematic_drive(1, KinematicDrive.velocity((1000.0, 0.0), 1.0)))
    assert rejection(world.advance(STEP), token) is None


@pytest.mark.parametrize("update", [False, True])
def test_a_huge_band_target_is_refused_and_a_reasonable_one_accepted(update):
    world = BubbleWorld(WorldConfiguration(REGION))
    world.submit(WorldTransaction().update_physics_material(1, PhysicsMaterial(1e9))
                 .add(BubbleDescriptor(1, (0.0, 0.0), 0.5, 1.0, 1, drive_policy=BubbleDrivePolicy(10.0))))
    world.advance(STEP)
    if update:
        world.submit(WorldTransaction().begin_player_drive(1, (1.0, 0.0)))
        world.advance(STEP)
        command = WorldTransaction().update_player_drive(1, (3e7, 0.0))
    else:
        command = WorldTransaction().begin_player_drive(1, (3e7, 0.0))
    token = world.submit(command)
    r = rejection(world.advance(STEP), token)
    assert r is not None and (r.reason, r.detail) == (R.INVALID_VALUE, "playerDrive.target")
    fine = WorldTransaction().update_player_drive(1, (9e5, -9e5)) if update else \
        WorldTransaction().begin_player_drive(1, (9e5, -9e5))
    token = world.submit(fine)
    assert rejection(world.advance(STEP), token) is None
