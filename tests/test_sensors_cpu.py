"""Sensor events on the oracle, bubbles (nativeCompactSensorEvents, NativePostSolveKernels:601-648) and bodies
(nativeCompactPolygonSensorEvents and nativeRigidOverlapsSensor, :677-775): a bubble crossing a circle sensor enters
then exits; a polygon sensor counts the centre inside or an edge within the radius; kinematic circles, capsules and
polygons crossing sensors enter and exit where their geometry says; a sensor inside a body overlaps it; the object
filter and the event flags decide what is reported."""
import math

import numpy as np

from bubblephysics_gb300 import _native as N
from bubblephysics_gb300.spec import WorldSpec, make_bubbles
from oracle.oracle import OracleWorld


def sensor(sid, x, y, radius=0.0, vertices=(0, 0), flags=N.SENSOR_ENTER_EVENTS | N.SENSOR_EXIT_EVENTS, angle=0.0):
    s = N.Sensor()
    s.id, s.position[:], s.angle, s.radius = sid, [x, y], angle, radius
    s.vertex_offset, s.vertex_count = vertices
    s.flags = flags
    return s


def crossing_world():
    b = make_bubbles([(-100.0, 0.0), (-100.0, 300.0)], 10.0, ids=[1, 2], velocities=[(120.0, 0.0), (120.0, 0.0)],
                     masses=1.0, stiffness=229.0)
    return WorldSpec(bubbles=b)


def run(world, sensors, vertices, steps, objects=None, allowed=None):
    state = np.zeros(len(sensors) * (objects or world.n), np.uint8)
    out = []
    for k in range(steps):
        world.step(1)
        for e in world.sensor_events(sensors, vertices, state, allowed):
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
    filtered = sensor(91, 0.0, 0.0, radius=20.0)
    allowed = np.array([1, 1, 0, 1], np.uint8)  # sensor 91's object filter leaves bubble 1 out
    ev = run(w, [only_enter, filtered], None, 120, allowed=allowed)
    assert [(s, k) for _, s, _, k in ev] == [(90, 1)]


def body_record(bid, kind, pos, vertex_offset, vertex_count, *, velocity=(0.0, 0.0), omega=0.0, angle=0.0, core=0.0,
                bound=0.0, triangles=(0, 0)):
    r = np.zeros(1, N.BODY_DTYPE)[0]
    r["id"], r["kind"], r["position"], r["angle"] = bid, kind, pos, angle
    r["velocity"], r["angular_velocity"] = velocity, omega
    r["core_radius"], r["bounding_radius"] = core, bound
    r["vertex_offset"], r["vertex_count"] = vertex_offset, vertex_count
    r["triangle_offset"], r["triangle_count"] = triangles
    r["flags"] = N.BODY_KINEMATIC if any(velocity) or omega else N.BODY_STATIC
    r["category"], r["mask"] = 1, 0xFFFFFFFF
    return r


def body_world():
    """Kinematic bodies crossing the sensors at x = 0 at 120 units/s: a circle (radius 10) on y = 0, a spinning square
    (half side 8) on y = 300, a capsule (core half length 10, radius 4) on y = 600; a static square (half side 50) at
    (500, 0) holds two sensors from the start. One bubble sits far away."""
    verts = np.array([(0, 0), (-8, -8), (8, -8), (8, 8), (-8, 8), (-10, 0), (10, 0), (-50, -50), (50, -50), (50, 50),
                      (-50, 50)], np.float32)
    tris = np.array([(0, 1, 2), (0, 2, 3), (0, 1, 2), (0, 2, 3)], np.uint32)
    bodies = np.array([
        body_record(500, N.BODY_CIRCLE, (-100.0, 0.0), 0, 1, velocity=(120.0, 0.0), core=10.0, bound=10.0),
        body_record(501, N.BODY_POLYGON, (-100.0, 300.0), 1, 4, velocity=(120.0, 0.0), omega=0.5, angle=0.3,
                    bound=11.4, triangles=(0, 2)),
        body_record(502, N.BODY_CAPSULE, (-100.0, 600.0), 5, 2, velocity=(120.0, 0.0), core=4.0, bound=14.0),
        body_record(503, N.BODY_POLYGON, (500.0, 0.0), 7, 4, bound=70.8, triangles=(2, 2)),
    ], N.BODY_DTYPE)
    b = make_bubbles([(0.0, -500.0)], 10.0, ids=[1], masses=1.0, stiffness=229.0)
    return WorldSpec(bubbles=b, bodies=bodies, body_vertices=verts, body_triangles=tris)


BODY_SENSOR_VERTS = np.array([(-5, -5), (5, -5), (5, 5), (-5, 5), (-6, -4), (6, -4), (0, 6)], np.float32)


def body_sensors():
    return [sensor(70, 0.0, 0.0, radius=20.0), sensor(71, 0.0, 300.0, vertices=(0, 4)),
            sensor(72, 0.0, 600.0, vertices=(4, 3), angle=0.2), sensor(73, 500.0, 0.0, radius=5.0),
            sensor(74, 480.0, 10.0, vertices=(4, 3))]


def test_bodies_cross_sensors():
    w = OracleWorld(body_world(), 32)
    ev = run(w, body_sensors(), BODY_SENSOR_VERTS, 120, objects=5)
    assert [(s, o) for k, s, o, _ in ev if k == 0] == [(73, 503), (74, 503)]  # pair order: sensor, then object
    crossings = {}
    for k, s, o, kind in ev:
        crossings.setdefault((s, o), []).append((kind, k))
    assert set(crossings) == {(70, 500), (71, 501), (72, 502), (73, 503), (74, 503)}
    assert crossings[(73, 503)] == [(1, 0)] and crossings[(74, 503)] == [(1, 0)]  # inside the static square
    (k1, enter), (k2, leave) = crossings[(70, 500)]
    assert (k1, k2) == (1, 2) and abs((leave - enter) - 30) <= 2  # centres within 30 units: x from -30 to 30
    (k1, enter), (k2, leave) = crossings[(72, 502)]
    assert (k1, k2) == (1, 2) and 10 <= leave - enter <= 18  # core end within 4 units of a 12-wide triangle
    assert [k for k, _ in crossings[(71, 501)]] == [1, 2]


def test_body_overlap_rules_one_at_a_time():
    """Single poses against single sensors: each rule of the reference in turn."""
    def overlaps(body, s, verts=BODY_SENSOR_VERTS):
        spec = body_world()
        spec.bodies = np.array([body], N.BODY_DTYPE)
        w = OracleWorld(spec, 32)
        w.step(1)
        state = np.zeros(2, np.uint8)
        return len(w.sensor_events([s], verts, state)) == 1
    still = dict(velocity=(0.0, 0.0))
    circle = lambda x, y, r: body_record(9, N.BODY_CIRCLE, (x, y), 0, 1, core=r, bound=r, **still)
    square = lambda x, y, a=0.0: body_record(9, N.BODY_POLYGON, (x, y), 1, 4, angle=a, bound=11.4, triangles=(0, 2),
                                             **still)
    capsule = lambda x, y, a=0.0: body_record(9, N.BODY_CAPSULE, (x, y), 5, 2, angle=a, core=4.0, bound=14.0, **still)
    assert overlaps(circle(0, 29.9, 10), sensor(1, 0, 0, radius=20.0))
    assert not overlaps(circle(0, 30.1, 10), sensor(1, 0, 0, radius=20.0))
    assert overlaps(circle(0, 14.9, 10), sensor(1, 0, 0, vertices=(0, 4)))       # core within 10 of the top edge
    assert not overlaps(circle(0, 15.1, 10), sensor(1, 0, 0, vertices=(0, 4)))
    assert overlaps(circle(1, 1, 0.5), sensor(1, 0, 0, vertices=(0, 4)))          # core inside the sensor
    assert overlaps(capsule(0, 8.9), sensor(1, 0, 0, vertices=(0, 4)))            # core 3.9 above the edge
    assert not overlaps(capsule(0, 9.1), sensor(1, 0, 0, vertices=(0, 4)))
    assert overlaps(capsule(0, 0, math.pi / 2), sensor(1, 0, 0, vertices=(0, 4)))  # core crosses the square
    assert overlaps(square(0, 27.9), sensor(1, 0, 0, radius=20.0))                 # edge at y = 19.9
    assert not overlaps(square(0, 28.1), sensor(1, 0, 0, radius=20.0))
    assert overlaps(square(0, 0), sensor(1, 0, 0, radius=1.0))                     # sensor centre inside the body
    assert overlaps(square(12.9, 0), sensor(1, 0, 0, vertices=(0, 4)))            # edges cross
    assert not overlaps(square(13.1, 0), sensor(1, 0, 0, vertices=(0, 4)))
    assert overlaps(square(0, 0), sensor(1, 1, 1, vertices=(4, 3)))              # sensor ring inside the body
    big = np.array([(-50, -50), (50, -50), (50, 50), (-50, 50)], np.float32)
    assert overlaps(square(10, 10, 0.7), sensor(1, 0, 0, vertices=(0, 4)), big)  # body inside the sensor ring

