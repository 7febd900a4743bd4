"""Model validation against ModelValidationTests.swift:15-181: polygons (a concave simple polygon in either orientation
is accepted; self-intersection, too few vertices, zero-length or doubling-back edges, touching edges, zero area and
non-finite vertices are refused; a repeated closing vertex is dropped; collinear middle vertices and tiny areas are
fine), the configuration's time, backlog and capacity, and static geometry inside the region. A concave kinematic body
is triangulated by ear clipping, so its inside test covers exactly its area."""
import math

import numpy as np
import pytest

from bubblephysics_gb300 import world as W
from bubblephysics_gb300.world import (Capsule, Circle, MotionRole, Polygon, RigidBodyDescriptor, WorldConfiguration)

CONCAVE = ((0.0, 0.0), (4.0, 0.0), (4.0, 4.0), (2.0, 2.0), (0.0, 4.0))


def test_a_concave_simple_polygon_is_accepted_and_a_self_intersecting_one_refused():
    Polygon(CONCAVE)
    Polygon(tuple(reversed(CONCAVE)))
    with pytest.raises(ValueError):
        Polygon(((0.0, 0.0), (4.0, 4.0), (0.0, 4.0), (4.0, 0.0)))


def test_closure_and_degenerate_edges():
    assert len(Polygon(((0.0, 0.0), (2.0, 0.0), (2.0, 2.0), (0.0, 0.0))).points) == 3
    for points in ((), ((0, 0), (1, 1)), ((0, 0), (1, 1), (2, 2)), ((0, 0), (2, 0), (2, 0), (0, 2)),
                   ((0, 0), (3, 0), (1, 0), (1, 2)), ((0, 0), (4, 0), (4, 4), (2, 0), (0, 4)),
                   ((0, 0), (math.inf, 0), (0, 2)), ((0, 0), (math.nan, 0), (0, 2))):
        with pytest.raises(ValueError):
            Polygon(points)
    Polygon(((0.0, 0.0), (1.0, 0.0), (2.0, 0.0), (2.0, 2.0), (0.0, 2.0)))
    Polygon(((0.0, 0.0), (1e-20, 0.0), (0.0, 1e-20)))


def test_the_configuration_refuses_invalid_time_backlog_and_capacity():
    region = (0.0, 0.0, 10.0, 10.0)
    assert WorldConfiguration(region).maximum_backlog == 0.25
    for bad in ({"fixed_time_step": 0.0}, {"fixed_time_step": math.nan}, {"event_buffer_capacity": 0},
                {"maximum_backlog": math.nan}, {"maximum_backlog": math.inf}, {"maximum_backlog": 0.0},
                {"maximum_backlog": -0.25}):
        with pytest.raises(ValueError):
            WorldConfiguration(region, **bad)


def test_static_circles_and_capsules_must_fit_in_the_region():
    region = (0.0, 0.0, 10.0, 10.0)
    body = lambda shape, p, angle=0.0: RigidBodyDescriptor(1, shape, p, angle=angle)
    assert W.static_geometry_inside(body(Circle(2.0), (5.0, 5.0)), region)
    assert not W.static_geometry_inside(body(Circle(2.0), (1.0, 5.0)), region)
    capsule = Capsule(3.0, 1.0)
    assert W.static_geometry_inside(body(capsule, (5.0, 5.0)), region)
    assert not W.static_geometry_inside(body(capsule, (5.0, 8.0), math.pi / 2), region)
    assert W.static_geometry_inside(body(capsule, (5.0, 5.0), math.pi / 2), region)


@pytest.mark.parametrize("points", [CONCAVE, tuple(reversed(CONCAVE))])
def test_a_concave_body_is_triangulated_over_exactly_its_area(points):
    local, tris = W.polygon_triangles(Polygon(points).points)
    twice = sum(W._cross3(local[0], local[k], local[k + 1]) for k in range(1, len(local) - 1))
    assert twice > 0  # counter-clockwise for the device
    area = sum(W._cross3(local[a], local[b], local[c]) for a, b, c in tris) / 2
    assert len(tris) == len(local) - 2 and abs(area - twice / 2) <= 1e-6
    assert all(W._cross3(local[a], local[b], local[c]) > 0 for a, b, c in tris)
    notch, inside = np.array([2.0, 3.0], np.float32), np.array([1.0, 1.0], np.float32)
    covers = lambda p: any(W._cross3(local[a], local[b], p) >= 0 and W._cross3(local[b], local[c], p) >= 0 and
                           W._cross3(local[c], local[a], p) >= 0 for a, b, c in tris)
    assert covers(inside) and not covers(notch)


def test_a_convex_body_keeps_its_fan():
    local, tris = W.polygon_triangles(((0.0, 0.0), (2.0, 0.0), (2.0, 2.0), (0.0, 2.0)))
    assert tris.tolist() == [[0, 1, 2], [0, 2, 3]] and local.tolist() == [[0, 0], [2, 0], [2, 2], [0, 2]]


def test_a_bubble_rests_in_the_notch_of_a_concave_kinematic_body(monkeypatch):
    """Through the world API on a stand-in device world that forwards to the oracle: the notch is outside the body,
    so a bubble placed there is accepted and the step finds no violation."""
    from bubblephysics_gb300.world import BubbleDescriptor, BubbleWorld, PhysicsMaterial, WorldTransaction
    from test_world_api_oracle_cpu import OracleBackedWorld
    monkeypatch.setattr(W, "World", OracleBackedWorld)
    monkeypatch.setattr(W, "default_context", lambda: None)
    world = BubbleWorld(WorldConfiguration((-10.0, -10.0, 10.0, 10.0)))
    world.submit(WorldTransaction().update_physics_material(1, PhysicsMaterial(229.0))
                 .add(RigidBodyDescriptor(7, Polygon(tuple(reversed(CONCAVE))), (0.0, 0.0),
                                          motion_role=MotionRole.KINEMATIC))
                 .add(BubbleDescriptor(1, (2.0, 3.4), 0.3, 1.0, 1)))
    for _ in range(30):
        frame = world.advance(1.0 / 60)
        assert world.diagnostics.last_advance_issue is None and world.diagnostics.failure_reason is None
    assert len(frame.transaction_receipts) == 0 and 1 in frame.objects


def test_fields_and_sensors_validate_their_values_and_stay_in_the_region():
    """ModelValidationTests.swift:127-144: a radial field is fine; a circle of radius 0, a field force that is not
    finite, a negative falloff and a sensor at infinity are refused when made; a sensor or field reaching out of the
    region is refused at staging."""
    from bubblephysics_gb300.world import ForceFieldDescriptor, SensorDescriptor, TransactionRejectionReason as R, \
        WorldTransaction
    ForceFieldDescriptor(3, (0.0, 0.0), "radial", Circle(3.0), strength=-2.0, falloff=1.0)
    for make in (lambda: Circle(0.0),
                 lambda: ForceFieldDescriptor(3, (0.0, 0.0), "directional", Circle(3.0), force=(math.nan, 0.0)),
                 lambda: ForceFieldDescriptor(3, (0.0, 0.0), "vortex", Circle(3.0), strength=1.0, falloff=-1.0),
                 lambda: SensorDescriptor(4, Circle(3.0), (math.inf, 0.0))):
        with pytest.raises(ValueError):
            make()
    for item in (SensorDescriptor(4, Circle(3.0), (0.0, 0.0)),
                 ForceFieldDescriptor(3, (0.0, 0.0), "directional", Circle(3.0), force=(1.0, 0.0))):
        _, receipts, events = W.stage([(1, WorldTransaction().add(item))], W._State(), (-2.0, -2.0, 2.0, 2.0))
        assert not receipts and (events[0].rejection.reason, events[0].rejection.detail) == (R.INVALID_VALUE,
                                                                                            W.STATIC_OUTSIDE)


def test_a_body_with_a_pose_that_is_not_finite_is_refused_when_made():
    """ModelValidationTests.swift:124: a polygon body turned by infinity."""
    with pytest.raises(ValueError):
        RigidBodyDescriptor(1, Polygon(((0.0, 0.0), (1.0, 0.0), (0.0, 1.0))), (0.0, 0.0), angle=math.inf)
