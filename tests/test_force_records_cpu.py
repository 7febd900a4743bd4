"""The force records a world hands to its device world (NativeForceRecordsTests.swift:4-113): bands of player-driven
bubbles with a target and a policy, in id order (maximum force 0 = no limit); motors with the inertia m r^2 / 2; force
fields in id order with their kind, pose, strength or directional force, range (a polygon's farthest vertex), local
vertices and object filter (ascending ids; an empty filter takes nobody); the force-driven flag of the dynamic, motor
and player roles. Also a field acting through the world on the bubbles its filter takes, on a stand-in device world
that forwards to the oracle."""
import math

import numpy as np
import pytest

from bubblephysics_gb300 import _native as N
from bubblephysics_gb300 import world as W
from bubblephysics_gb300.world import (BubbleDescriptor, BubbleDrivePolicy, BubbleWorld, Circle, ForceFieldDescriptor,
                                       MotionRole as M, MotorDrive, ObjectFilter, PhysicsMaterial, Polygon,
                                       WorldConfiguration, WorldTransaction)
from test_world_api_oracle_cpu import OracleBackedWorld

REGION = (-1000.0, -1000.0, 1000.0, 1000.0)


def staged(tx):
    state, rec, ev = W.stage([(1, WorldTransaction().update_physics_material("m", PhysicsMaterial(229.0)))], W._State(), REGION)
    state, rec, ev = W.stage([(2, tx)], state, REGION)
    assert rec, ev
    return state


def spec_of(state):
    world = BubbleWorld(WorldConfiguration(REGION))
    return world._spec(state)[0]


def bubble(i, x=0.0, role=M.DYNAMIC, mass=2.0, radius=4.0, policy=None):
    return BubbleDescriptor(i, (x, 0.0), radius, mass, "m", motion_role=role, drive_policy=policy)


def test_an_empty_world_has_no_force_records():
    state = staged(WorldTransaction().set_global_force((3.0, -4.0)))
    spec = spec_of(state)
    assert spec.global_force == (3.0, -4.0) and spec.bands == [] and spec.fields == [] and spec.motors == []


def test_band_records_carry_target_stiffness_and_optional_maximum_force():
    tx = (WorldTransaction().add(bubble(7, 0, policy=BubbleDrivePolicy(22.0, 250.0)))
          .add(bubble(2, 20, policy=BubbleDrivePolicy(100.0))).add(bubble(3, 40, policy=BubbleDrivePolicy(100.0)))
          .add(bubble(5, 60, policy=BubbleDrivePolicy(100.0)))
          .begin_player_drive(7, (3.0, 4.0)).begin_player_drive(2, (-5.0, 6.0)))
    bands = spec_of(staged(tx)).bands
    assert [(b.bubble_id, tuple(b.target), b.stiffness, b.maximum_force) for b in bands] == \
        [(2, (-5.0, 6.0), 100.0, 0.0), (7, (3.0, 4.0), 22.0, 250.0)]


def test_motor_records_carry_force_torque_and_inertia():
    tx = (WorldTransaction().add(bubble(9, 0, mass=2.0, radius=3.0)).set_motor_drive(9, MotorDrive((5.0, -6.0), 7.0))
          .add(bubble(8, 30, role=M.MOTOR_DRIVEN)).add(bubble(6, 60)))
    motors = spec_of(staged(tx)).motors
    assert [(m.bubble_id, tuple(m.force), m.torque, m.inertia) for m in motors] == [(9, (5.0, -6.0), 7.0, 9.0)]


def test_field_records_carry_kind_pose_strength_range_and_filter():
    tx = (WorldTransaction()
          .add(ForceFieldDescriptor(20, (1.0, 2.0), "directional", Circle(100.0), angle=0.5, force=(0.0, 40.0),
                                    filter=ObjectFilter(frozenset({9, 3}))))
          .add(ForceFieldDescriptor(10, (10.0, 20.0), "radial", Circle(400.0), strength=-500.0, falloff=2.0))
          .add(ForceFieldDescriptor(30, (0.0, 0.0), "vortex", Circle(100.0), strength=7.0, filter=ObjectFilter(frozenset()))))
    fields, _, ids = W.field_records(staged(tx))
    r, d, v = fields
    assert (r.kind, tuple(r.position), r.rotation, r.falloff) == (1, (10.0, 20.0), 0.0, 2.0)
    assert (tuple(r.direction), r.strength, r.radius, r.vertex_count, r.has_filter) == ((0.0, 0.0), -500.0, 400.0, 0, 0)
    assert (d.kind, tuple(d.position), d.rotation, tuple(d.direction), d.radius) == (0, (1.0, 2.0), 0.5, (0.0, 40.0), 100.0)
    assert d.has_filter == 1 and d.filter_count == 2 and ids[d.filter_offset:d.filter_offset + 2].tolist() == [3, 9]
    assert (v.kind, v.has_filter, v.filter_count) == (2, 1, 0)  # an empty filter takes nobody


def test_polygon_field_records_point_at_their_vertices_and_reach_the_farthest():
    tx = (WorldTransaction()
          .add(ForceFieldDescriptor(1, (0.0, 0.0), "directional", Polygon(((-3, -4), (3, -4), (3, 4), (-3, 4))),
                                    force=(1.0, 0.0)))
          .add(ForceFieldDescriptor(2, (0.0, 0.0), "radial", Polygon(((0, 0), (10, 0), (0, 10))), strength=1.0,
                                    falloff=1.0)))
    (first, second), verts, _ = W.field_records(staged(tx))
    assert (first.vertex_count, second.vertex_count, first.radius, second.radius) == (4, 3, 5.0, 10.0)
    assert verts[first.vertex_offset:first.vertex_offset + 4].tolist() == [[-3, -4], [3, -4], [3, 4], [-3, 4]]
    assert verts[second.vertex_offset:second.vertex_offset + 3].tolist() == [[0, 0], [10, 0], [0, 10]]


def test_force_driven_flag_covers_dynamic_motor_and_player_roles():
    tx = (WorldTransaction().add(bubble(1, 0)).add(bubble(2, 30, role=M.MOTOR_DRIVEN))
          .add(bubble(3, 60, policy=BubbleDrivePolicy(10.0))).begin_player_drive(3, (0.0, 0.0))
          .add(bubble(4, 90, role=M.STATIC)))
    flags = {int(b["id"]): int(b["flags"]) for b in spec_of(staged(tx)).bubbles}
    assert all(flags[i] & N.BUBBLE_FORCE_DRIVEN for i in (1, 2, 3)) and not flags[4] & N.BUBBLE_FORCE_DRIVEN


def test_a_filtered_field_pushes_only_the_bubbles_it_takes(monkeypatch):
    monkeypatch.setattr(W, "World", OracleBackedWorld)
    monkeypatch.setattr(W, "default_context", lambda: None)
    world = BubbleWorld(WorldConfiguration(REGION, contours=False))
    world.submit(WorldTransaction().update_physics_material("m", PhysicsMaterial(229.0))
                 .add(bubble(1, 0.0, mass=1.0)).add(bubble(2, 50.0, mass=1.0))
                 .add(ForceFieldDescriptor(10, (0.0, 0.0), "directional", Circle(500.0), force=(0.0, 60.0),
                                           filter=ObjectFilter(frozenset({1})))))
    frame = world.advance(1.0 / 60)
    assert frame.objects[1].velocity[1] == pytest.approx(1.0, rel=1e-5) and frame.objects[2].velocity == (0.0, 0.0)
    world.submit(WorldTransaction().remove(10))
    v = frame.objects[1].velocity
    assert world.advance(1.0 / 60).objects[1].velocity == pytest.approx(v)
