"""Damping of motion (MotionDampingTests.swift:119-215), restated through the world API on a stand-in device world
that forwards to the oracle: a bubble pressed into a thick wall by a motor drive or by the global force rests at the
law's deflection r - d*(F) for gamma 0.6 and 4 (2 %, settled within 0.5 %); between two frames without contacts the
velocity follows v' = v e^(-gamma dt) + F / m (1 - e^(-gamma dt)) / gamma for the band (3 %, F from the previous
frame's drive feedback) and the bubble's motor (1 %), for gamma 0, 0.6 and 4. The dynamic rigid body's motor case
belongs to the rigid solver, which is not built here."""
import math

import numpy as np
import pytest

import clr
from bubblephysics_gb300 import world as W
from bubblephysics_gb300.world import (BubbleDescriptor, BubbleDrivePolicy, BubbleWorld, MotorDrive, PhysicsMaterial,
                                       Polygon, RigidBodyDescriptor, WorldConfiguration, WorldTransaction)
from test_world_api_oracle_cpu import OracleBackedWorld

DT = 1.0 / 60
FACE_X = -100.0
KC = float(np.float32(20.0) / np.float32(0.0108))


@pytest.fixture(autouse=True)
def oracle_backed(monkeypatch):
    monkeypatch.setattr(W, "World", OracleBackedWorld)
    monkeypatch.setattr(W, "default_context", lambda: None)


def make_world(gamma, extent, wall, build):
    world = BubbleWorld(WorldConfiguration((-extent, -extent, extent, extent), contours=False))
    tx = WorldTransaction().update_physics_material("soft", PhysicsMaterial(KC, gamma))
    if wall:
        tx = tx.add(RigidBodyDescriptor(9001, Polygon(((-400, -450), (FACE_X, -450), (FACE_X, 450), (-400, 450))),
                                        (0.0, 0.0)))
    world.submit(build(tx))
    world.advance(DT)
    assert world.diagnostics.last_advance_issue is None
    return world


def settle(world, radius, steps=1800):
    tail = []
    for k in range(steps):
        frame = world.advance(DT)
        assert world.diagnostics.last_advance_issue is None
        x = frame.objects[1].position[0]
        if k >= steps - 60:
            tail.append(radius - (x - FACE_X))
    return tail[-1], max(tail) - min(tail)


@pytest.mark.parametrize("gamma", [0.6, 4.0])
@pytest.mark.parametrize("how", ["motor", "global force"])
def test_rest_under_a_motor_or_the_global_force_deflects_by_the_full_force(gamma, how):
    r, force = 24.0, 600.0
    expected = r - clr.equilibrium_distance(force, KC, r)
    bubble = BubbleDescriptor(1, (FACE_X + r, 0.0), r, 1.36, "soft")
    if how == "motor":
        world = make_world(gamma, 500.0, True, lambda tx: tx.add(bubble).set_motor_drive(1, MotorDrive((-force, 0.0))))
    else:
        world = make_world(gamma, 500.0, True, lambda tx: tx.add(bubble).set_global_force((-force, 0.0)))
    deflection, spread = settle(world, r)
    assert abs(deflection - expected) <= 0.02 * expected, (deflection, expected)
    assert spread < 0.005 * expected


@pytest.mark.parametrize("gamma", [0.0, 0.6, 4.0])
@pytest.mark.parametrize("kind", ["band", "motor"])
def test_velocity_step_is_the_decayed_velocity_plus_the_force_impulse(gamma, kind):
    mass, k_band, target, motor_force = 2.0, 30.0, (20.0, 12.0), (40.0, 10.0)

    def build(tx):
        if kind == "band":
            return tx.add(BubbleDescriptor(1, (0.0, 0.0), 10.0, mass, "soft", drive_policy=BubbleDrivePolicy(k_band))) \
                .begin_player_drive(1, target)
        return tx.add(BubbleDescriptor(1, (0.0, 0.0), 10.0, mass, "soft")).set_motor_drive(1, MotorDrive(motor_force))
    world = make_world(gamma, 500.0, False, build)
    previous = world.last_frame
    for _ in range(4):
        nxt = world.advance(DT)
        if kind == "band":
            fb = previous.drive_feedback[0]
            force = (np.array(fb.target) - np.array(fb.achieved_point)) * k_band
        else:
            force = np.array(motor_force)
        impulse = DT if gamma == 0 else (1 - math.exp(-gamma * DT)) / gamma
        expected = np.array(previous.objects[1].velocity) * math.exp(-gamma * DT) + force / mass * impulse
        after = np.array(nxt.objects[1].velocity)
        tol = 0.03 if kind == "band" else 0.01
        assert np.all(np.abs(after - expected) <= tol * np.abs(expected) + 1e-4), (after, expected)
        previous = nxt
