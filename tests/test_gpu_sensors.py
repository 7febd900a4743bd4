"""Sensor events on the GPU (bp_world_set_sensors, bp_world_read_sensor_events) against the oracle's restatement of
nativeCompactSensorEvents and nativeCompactPolygonSensorEvents (NativePostSolveKernels:601-648, 677-775): the same
event list, in pair order (sensor, then bubbles, then bodies), every step, with and without object filters."""
import numpy as np
import pytest

from bubblephysics_gb300 import _native as N
from bubblephysics_gb300 import scenes
from bubblephysics_gb300.solver import World
from oracle.oracle import OracleWorld
from test_sensors_cpu import BODY_SENSOR_VERTS, body_sensors, body_world, crossing_world, sensor

pytestmark = pytest.mark.gpu


def compare(spec, ctx, sensors, vertices, steps, allowed=None):
    gpu, cpu = World(spec, ctx), OracleWorld(spec, 32)
    gpu.set_sensors(sensors, vertices, allowed=allowed)
    state = np.zeros(len(sensors) * (spec.bubble_count + len(spec.bodies)), np.uint8)
    total = 0
    for _ in range(steps):
        assert gpu.step(1)[0] == cpu.step(1)[0] == 0
        g = gpu.sensor_events()
        c = cpu.sensor_events(sensors, vertices, state, allowed)
        assert np.array_equal(g, c), (g, c)
        total += len(g)
    return total


def test_crossing_bubbles(ctx):
    square = np.array([(-5.0, -5.0), (5.0, -5.0), (5.0, 5.0), (-5.0, 5.0)], np.float32)
    sensors = [sensor(70, 0.0, 0.0, radius=20.0), sensor(80, 0.0, 300.0, vertices=(0, 4))]
    assert compare(crossing_world(), ctx, sensors, square, 120) == 4


def test_sensors_in_a_pile(ctx):
    spec = scenes.plain_world(seed=2)
    tri = np.array([(-60.0, -40.0), (60.0, -40.0), (0.0, 60.0)], np.float32)
    sensors = [sensor(100 + k, 60.0 + 50.0 * k, 80.0 + 90.0 * k, radius=25.0) for k in range(5)]
    sensors.append(sensor(200, 190.0, 300.0, vertices=(0, 3), flags=N.SENSOR_ENTER_EVENTS))
    assert compare(spec, ctx, sensors, tri, 40) > 0


def test_crossing_bodies(ctx):
    assert compare(body_world(), ctx, body_sensors(), BODY_SENSOR_VERTS, 120) == 8


def test_sensors_over_bubbles_and_bodies_with_object_filters(ctx):
    rng = np.random.default_rng(11)
    spec = scenes.batched_world(rng, 600, max_bodies=32)
    lo, hi = spec.bubbles["center"].min(0), spec.bubbles["center"].max(0)
    poly = np.array([(-40.0, -30.0), (45.0, -25.0), (30.0, 40.0), (-35.0, 35.0), (0.0, 10.0)], np.float32)
    sensors = []
    for k in range(12):
        x, y = rng.uniform(lo, hi)
        if k % 2:
            sensors.append(sensor(900 + k, x, y, radius=float(rng.uniform(10, 80))))
        else:
            sensors.append(sensor(900 + k, x, y, vertices=(0, 5), angle=float(rng.uniform(-3, 3))))
    pairs = len(sensors) * (spec.bubble_count + len(spec.bodies))
    assert len(spec.bodies) > 0
    assert compare(spec, ctx, sensors, poly, 30) > 0
    allowed = (rng.random(pairs) < 0.6).astype(np.uint8)
    assert compare(spec, ctx, sensors, poly, 30, allowed) > 0
