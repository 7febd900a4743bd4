"""Deflection under the contact law F = K_c eps / (1 - eps)^2 through the world API, on a stand-in device world that
forwards to the oracle, against the reference's own cases: ContactComplianceTests.swift:23-92 (the same relative
deflection for every radius, from the position and from the contour's effective radius; a doubled force doubles the
law's ratio, not the deflection; a soft pair's overlap follows the law and its dents split by radius, 2 % each),
ContactVelocityCorrectionProbeTests.swift:12-56 (a motor-pressed bubble rests at the law's deflection for every mass
and fixed step) and ContourIsDrawOnlyTests.swift:1-96 (reading the contours every step changes no physics)."""
import math

import numpy as np
import pytest

import clr
from bubblephysics_gb300 import world as W
from bubblephysics_gb300.scenes import polygon_edges
from bubblephysics_gb300.world import (BubbleDescriptor, BubbleWorld, MotorDrive, PhysicsMaterial, Polygon,
                                       RigidBodyDescriptor, WorldConfiguration, WorldTransaction)
from test_world_api_oracle_cpu import OracleBackedWorld

DT = 1.0 / 60


@pytest.fixture(autouse=True)
def oracle_backed(monkeypatch):
    monkeypatch.setattr(W, "World", OracleBackedWorld)
    monkeypatch.setattr(W, "default_context", lambda: None)


def force_world(stiffness, damping):
    world = BubbleWorld(WorldConfiguration((-2000.0, -2000.0, 2000.0, 2000.0)))
    return world, WorldTransaction().update_physics_material("soft", PhysicsMaterial(stiffness, damping))


def thin_wall(x, oid=10):
    return RigidBodyDescriptor(oid, Polygon(((x, -1900), (x + 1, -1900), (x + 1, 1900), (x, 1900))), (0.0, 0.0))


def run(world, frames):
    for _ in range(frames):
        frame = world.advance(DT)
        assert world.diagnostics.last_advance_issue is None
    return frame


def test_relative_deflection_is_the_same_for_every_radius():
    radii = [(1, 12.0, -700.0), (2, 24.0, -450.0), (3, 48.0, -250.0), (4, 148.0, 50.0)]
    world, tx = force_world(1200.0, 5.0)
    tx = tx.add(thin_wall(0.0)).set_global_force((600.0, 0.0))
    for oid, r, y in radii:
        tx = tx.add(BubbleDescriptor(oid, (-r, y), r, 1.0, "soft"))
    world.submit(tx)
    last = run(world, 600)
    expected = clr.epsilon(600.0 / 1200.0)
    for oid, r, _ in radii:
        from_position = 1 - (-last.objects[oid].position[0]) / r
        from_contour = 1 - last.objects[oid].effective_radius / r
        assert abs(from_position - expected) <= 0.02 * expected, (r, from_position, expected)
        assert abs(from_contour - expected) <= 0.02 * expected, (r, from_contour, expected)


def test_doubled_force_doubles_the_law_ratio_not_the_deflection():
    world, tx = force_world(1200.0, 5.0)
    world.submit(tx.add(thin_wall(0.0)).add(BubbleDescriptor(1, (-24.0, -300.0), 24.0, 1.0, "soft"))
                 .add(BubbleDescriptor(2, (-24.0, 300.0), 24.0, 1.0, "soft"))
                 .set_motor_drive(1, MotorDrive((300.0, 0.0))).set_motor_drive(2, MotorDrive((600.0, 0.0))))
    last = run(world, 600)
    eps = []
    for oid, applied in ((1, 300.0), (2, 600.0)):
        measured = 1 - last.objects[oid].effective_radius / 24.0
        assert abs(measured - clr.epsilon(applied / 1200.0)) <= 0.02 * measured
        eps.append(measured)
    law = lambda e: e / ((1 - e) * (1 - e))
    assert abs(law(eps[1]) / law(eps[0]) - 2) <= 0.06 and eps[1] < 2 * eps[0]


@pytest.mark.parametrize("ra,rb", [(12.0, 24.0), (24.0, 24.0), (24.0, 148.0)])
def test_soft_pair_overlap_follows_the_law_and_dents_split_by_radius(ra, rb):
    eps = clr.epsilon(600.0 / 1200.0)
    distance = float(np.float32((ra + rb) * (1 - eps)))
    world, tx = force_world(1200.0, 5.0)
    world.submit(tx.add(BubbleDescriptor(1, (-distance / 2, 0.0), ra, 1.0, "soft"))
                 .add(BubbleDescriptor(2, (distance / 2, 0.0), rb, 1.0, "soft"))
                 .set_motor_drive(1, MotorDrive((600.0, 0.0))).set_motor_drive(2, MotorDrive((-600.0, 0.0))))
    last = run(world, 600)
    a, b = np.array(last.objects[1].position), np.array(last.objects[2].position)
    measured = ((ra + rb) - float(np.hypot(*(b - a)))) / (ra + rb)
    assert abs(measured - eps) <= 0.02 * eps
    dent_a, dent_b = ra - last.objects[1].effective_radius, rb - last.objects[2].effective_radius
    assert abs(dent_a - eps * ra) <= 0.02 * eps * ra and abs(dent_b - eps * rb) <= 0.02 * eps * rb


HALF, THICK = (180.0, 320.0), 48.0


def crowd_frame(tx):
    ix, iy = HALF
    ox, oy = ix + THICK, iy + THICK
    for k, ((lx, ly), (hx, hy)) in enumerate([((-ox, -oy), (-ix, oy)), ((ix, -oy), (ox, oy)), ((-ix, -oy), (ix, -iy)),
                                              ((-ix, iy), (ix, oy))]):
        tx = tx.add(RigidBodyDescriptor(9001 + k, Polygon(((lx, ly), (hx, ly), (hx, hy), (lx, hy))), (0.0, 0.0)))
    return tx


@pytest.mark.parametrize("mass,dt", [(1.0, 1 / 60), (4.0, 1 / 60), (1.0, 1 / 120), (4.0, 1 / 120)])
def test_motor_pressed_bubble_rests_at_the_law_for_every_mass_and_step(mass, dt):
    r, force, kc = 20.0, 300.0, float(np.float32(20.0) / np.float32(0.01))
    ox, oy = HALF[0] + THICK, HALF[1] + THICK
    world = BubbleWorld(WorldConfiguration((-ox, -oy, ox, oy), fixed_time_step=dt))
    tx = crowd_frame(WorldTransaction().update_physics_material("soft", PhysicsMaterial(kc, 5.0)))
    world.submit(tx.add(BubbleDescriptor(1, (-(HALF[0] - r), 0.0), r, mass, "soft"))
                 .set_motor_drive(1, MotorDrive((-force, 0.0))))
    world.advance(dt)
    steps, window = int(round(5 / dt)), int(round(1 / dt))
    depths, xs = [], []
    for k in range(steps):
        state = world.advance(dt).objects[1]
        if k >= steps - window:
            depths.append(r - (HALF[0] + state.position[0]))
            xs.append(state.position[0])
    expected = clr.epsilon(force / kc)
    eps = float(np.mean(depths)) / r
    assert abs(eps - expected) <= 0.02 * expected and math.hypot(*state.velocity) < 0.1 and max(xs) - min(xs) < 0.02 * r


def test_reading_the_contours_every_step_changes_no_physics():
    rng = np.random.default_rng(7)
    def scene():
        world = BubbleWorld(WorldConfiguration((-400.0, -400.0, 400.0, 400.0)))
        tx = WorldTransaction().update_physics_material("soft", PhysicsMaterial(1200.0, 1.0))
        pts = []
        for oid in range(1, 25):
            while True:
                p = rng.uniform(-150, 150, 2)
                if all(np.hypot(*(p - q)) > 30 for q in pts):
                    break
            pts.append(p)
            tx = tx.add(BubbleDescriptor(oid, tuple(p), 12.0, 1.0, "soft", velocity=tuple(rng.normal(0, 40, 2))))
        return world, tx
    state = rng.bit_generator.state
    reading, tx1 = scene()
    rng.bit_generator.state = state
    plain, tx2 = scene()
    plain.configuration = W.WorldConfiguration(plain.configuration.simulation_region, contours=False)
    reading.submit(tx1)
    plain.submit(tx2)
    for _ in range(300):
        a, b = reading.advance(DT), plain.advance(DT)
        snapshot = reading.debug_contour_snapshot()
        assert len(snapshot) == 24 and all(len(ring) >= 32 for ring in snapshot.values())
        for oid in a.objects:
            assert a.objects[oid].position == b.objects[oid].position and a.objects[oid].velocity == b.objects[oid].velocity
