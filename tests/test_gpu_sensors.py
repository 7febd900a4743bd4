"""Sensor events on the GPU (bp_world_set_sensors, bp_world_read_sensor_events) against the oracle's restatement of
nativeCompactSensorEvents (NativePostSolveKernels:601-648): the same event list, in (sensor, bubble) order, every step."""
import numpy as np
import pytest

from bubblephysics_gb300 import _native as N
from bubblephysics_gb300 import scenes
from bubblephysics_gb300.solver import World
from oracle.oracle import OracleWorld
from test_sensors_cpu import crossing_world, sensor

pytestmark = pytest.mark.gpu


def compare(spec, ctx, sensors, vertices, steps):
    gpu, cpu = World(spec, ctx), OracleWorld(spec, 32)
    gpu.set_sensors(sensors, vertices)
    state = np.zeros(len(sensors) * spec.bubble_count, np.uint8)
    total = 0
    for _ in range(steps):
        assert gpu.step(1)[0] == cpu.step(1)[0] == 0
        g = gpu.sensor_events()
        c = cpu.sensor_events(sensors, vertices, state)
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
