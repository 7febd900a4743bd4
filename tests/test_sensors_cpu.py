"""Sensor events (nativeCompactSensorEvents, NativePostSolveKernels:601-648) on the oracle: a bubble crossing a circle
sensor enters then exits; a polygon sensor counts the centre inside or an edge within the radius; the filter and the
event flags decide what is reported."""
import numpy as np

from bubblephysics_gb300 import _native as N
from bubblephysics_gb300.spec import WorldSpec, make_bubbles
from oracle.oracle import OracleWorld


def sensor(sid, x, y, radius=0.0, vertices=(0, 0), flags=N.SENSOR_ENTER_EVENTS | N.SENSOR_EXIT_EVENTS, angle=0.0,
           category=1, mask=0xFFFFFFFF):
    s = N.Sensor()
    s.id, s.position[:], s.angle, s.radius = sid, [x, y], angle, radius
    s.vertex_offset, s.vertex_count = vertices
    s.flags, s.category, s.mask = flags, category, mask
    return s


def crossing_world():
    b = make_bubbles([(-100.0, 0.0), (-100.0, 300.0)], 10.0, ids=[1, 2], velocities=[(120.0, 0.0), (120.0, 0.0)],
                     masses=1.0, stiffness=229.0)
    return WorldSpec(bubbles=b)


def run(world, sensors, vertices, steps):
    state = np.zeros(len(sensors) * world.n, np.uint8)
    out = []
    for k in range(steps):
        world.step(1)
        for e in world.sensor_events(sensors, vertices, state):
            out.append((k, int(e["sensor"]), int(e["object"]), int(e["kind"])))
    return out


def test_circle_sensor_enter_then_exit():
    w = OracleWorld(crossing_world(), 32)
    ev = run(w, [sensor(70, 0.0, 0.0, radius=20.0)], None, 120)
    kinds = [(s, o, k) for _, s, o, k in ev]
    assert kinds == [(70, 1, 1), (70, 1, 2)]  # bubble 2 passes far above
    enter, leave = ev[0][0], ev[1][0]
    # centre within 30 units of the sensor centre from x = -30 to x = 30: 60 units at 120/s = 0.5 s = 30 steps
    assert abs((leave - enter) - 30) <= 2


def test_polygon_sensor_counts_edges_within_the_radius():
    square = np.array([(-5.0, -5.0), (5.0, -5.0), (5.0, 5.0), (-5.0, 5.0)], np.float32)
    w = OracleWorld(crossing_world(), 32)
    ev = run(w, [sensor(80, 0.0, 0.0, vertices=(0, 4))], square, 120)
    enter, leave = ev[0][0], ev[1][0]
    assert [e[3] for e in ev] == [1, 2] and abs((leave - enter) - 15) <= 2  # x from -15 to 15: 30 units


def test_filter_and_flags_choose_what_is_reported():
    w = OracleWorld(crossing_world(), 32)
    only_enter = sensor(90, 0.0, 0.0, radius=20.0, flags=N.SENSOR_ENTER_EVENTS)
    filtered = sensor(91, 0.0, 0.0, radius=20.0, category=2, mask=2)  # bubbles are category 1: never overlap
    ev = run(w, [only_enter, filtered], None, 120)
    assert [(s, k) for _, s, _, k in ev] == [(90, 1)]
