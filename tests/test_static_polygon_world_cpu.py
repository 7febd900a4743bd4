"""One-sided static polygon edges at world level (StaticPolygonEdgeTests.swift:17-180), through the world API on a
stand-in device world that forwards to the oracle: a bubble pressed into a wall deflects by r eps of the law from the
front edge only, the same for a thin (48) and a thick (400) wall, for five forces including deflections beyond the
thin wall's thickness; a collinear vertex in the edge changes nothing; a bubble pressed at a convex vertex of 30, 90
or 120 degrees is one spring (distance r - r eps from the vertex). K_c 1852, gamma 5, steps of 1/60; the force is
reset through a motor drive before every step."""
import math

import numpy as np
import pytest

import clr
from bubblephysics_gb300 import world as W
from bubblephysics_gb300.world import (BubbleDescriptor, BubbleWorld, MotorDrive, PhysicsMaterial, Polygon,
                                       RigidBodyDescriptor, WorldConfiguration, WorldTransaction)
from test_world_api_oracle_cpu import OracleBackedWorld

DT = 1.0 / 60
KC = float(np.float32(20.0) / np.float32(0.0108))
FACE_X = -100.0


@pytest.fixture(autouse=True)
def oracle_backed(monkeypatch):
    monkeypatch.setattr(W, "World", OracleBackedWorld)
    monkeypatch.setattr(W, "default_context", lambda: None)


def deflection(radius, force):
    return radius * clr.epsilon(force / KC)


def make_world(polygons, build, damping=5.0):
    w = BubbleWorld(WorldConfiguration((-1000.0, -1000.0, 1000.0, 1000.0), contours=False))
    tx = WorldTransaction().update_physics_material("m", PhysicsMaterial(KC, damping))
    for k, ring in enumerate(polygons):
        tx = tx.add(RigidBodyDescriptor(9001 + k, Polygon(tuple(map(tuple, ring))), (0.0, 0.0)))
    w.submit(build(tx))
    w.advance(DT)
    assert w.diagnostics.last_advance_issue is None
    return w


def rectangle(thickness, y_min=-400.0, y_max=400.0):
    return [(FACE_X - thickness, y_min), (FACE_X, y_min), (FACE_X, y_max), (FACE_X - thickness, y_max)]


def settle(w, radius, steps):
    tail, pos = [], None
    for k in range(steps):
        frame = w.advance(DT)
        assert w.diagnostics.last_advance_issue is None
        pos = frame.objects[1].position
        if k >= steps - 60:
            tail.append(radius - (pos[0] - FACE_X))
    return tail[-1], max(tail) - min(tail), pos


@pytest.mark.parametrize("pressure", [300.0, 700.0, 1100.0, 1500.0, 2500.0])
def test_a_thin_wall_deflects_by_its_front_edge_only_like_a_thick_one(pressure):
    r = 148.0
    expected = deflection(r, pressure)
    found = []
    for thickness in (48.0, 400.0):
        w = make_world([rectangle(thickness)], lambda tx: tx.add(BubbleDescriptor(1, (FACE_X + r, 0.0), r, 1.0, "m"))
                       .set_motor_drive(1, MotorDrive((-pressure, 0.0))))
        d, spread, _ = settle(w, r, 1200)
        assert abs(d - expected) <= 0.02 * expected and spread < 0.005 * expected, (thickness, d, expected)
        found.append(d)
    assert abs(found[0] - found[1]) <= 0.02 * expected


def test_a_collinear_vertex_does_not_change_the_contact():
    r, pressure = 24.0, 600.0
    expected = deflection(r, pressure)
    two_segments = [(FACE_X - 48, -400.0), (FACE_X, -400.0), (FACE_X, 0.0), (FACE_X, 400.0), (FACE_X - 48, 400.0)]
    results = []
    for ring in (two_segments, rectangle(48.0)):
        w = make_world([ring], lambda tx: tx.add(BubbleDescriptor(1, (FACE_X + r, 0.0), r, 1.36, "m"))
                       .set_motor_drive(1, MotorDrive((-pressure, 0.0))))
        results.append(settle(w, r, 600))
    for d, spread, _ in results:
        assert abs(d - expected) <= 0.02 * expected
    assert results[0][1] < 0.005 * expected
    assert abs(results[0][2][0] - results[1][2][0]) <= 1e-2 and abs(results[0][2][1] - results[1][2][1]) <= 1e-2


@pytest.mark.parametrize("degrees", [30.0, 90.0, 120.0])
def test_a_convex_vertex_is_one_spring_for_every_angle(degrees):
    r, pressure = 24.0, 600.0
    expected = deflection(r, pressure)
    half = degrees * math.pi / 360
    wedge = [(0.0, 0.0), (300 * math.cos(half), 300 * math.sin(half)), (300 * math.cos(half), -300 * math.sin(half))]
    w = make_world([wedge], lambda tx: tx.add(BubbleDescriptor(1, (-r, 0.0), r, 1.36, "m")))
    pos, tail = np.array([-r, 0.0]), []
    for k in range(420):
        toward = -pos / max(np.hypot(*pos), 1e-38)
        w.submit(WorldTransaction().set_motor_drive(1, MotorDrive(tuple(map(float, toward * pressure)))))
        frame = w.advance(DT)
        assert w.diagnostics.last_advance_issue is None
        pos = np.array(frame.objects[1].position, np.float64)
        if k >= 360:
            tail.append(r - float(np.hypot(*pos)))
    assert abs(tail[-1] - expected) <= 0.02 * expected and max(tail) - min(tail) < 0.005 * expected
