"""One-sided edges of a static polygon (NativeStaticPolygonEdges.segments, NativeStaticPolygonEdges.swift:16-72),
against the reference's own tests (NativeStaticPolygonEdgesTests.swift:8-120): identifiers and owner, the outward side
from the winding, the convexity of both ends, the previous edge's start, and the merge of collinear edges within the
1e-5 tolerance. Both builders are checked: the C ABI's (bp_static_polygon_edges, host code, no GPU) and the numpy one
the scenes use."""
import math

import numpy as np
import pytest

from bubblephysics_gb300 import _native as N
from bubblephysics_gb300.scenes import polygon_edges
from bubblephysics_gb300.solver import static_polygon_edges

LETTER_L = [(0, 0), (200, 0), (200, 48), (48, 48), (48, 200), (0, 200)]  # (48, 48) is the concave vertex
SQUARE = [(0, 0), (100, 0), (100, 100), (0, 100)]
_c, _s = float(np.float32(100 * math.cos(math.pi / 12))), float(np.float32(100 * math.sin(math.pi / 12)))
TRIANGLE = [(0, 0), (_c, _s), (_c, -_s)]  # clockwise

BUILDERS = {"capi": static_polygon_edges, "numpy": polygon_edges}


def contains(poly, p):
    inside = False
    for i in range(len(poly)):
        a, b = poly[i], poly[(i + 1) % len(poly)]
        if (a[1] > p[1]) != (b[1] > p[1]) and p[0] < a[0] + (p[1] - a[1]) / (b[1] - a[1]) * (b[0] - a[0]):
            inside = not inside
    return inside


@pytest.fixture(params=sorted(BUILDERS))
def edges(request):
    build = BUILDERS[request.param]
    return lambda points: build(np.asarray(points, np.float32), 10, 77)


def test_segments_keep_geometry_identifiers_and_owner(edges):
    result = edges(SQUARE)
    assert result["id"].tolist() == [10, 11, 12, 13] and (result["owner_id"] == 77).all()
    assert not (result["flags"] & (N.SEGMENT_KINEMATIC | N.SEGMENT_ALLOWED_SIDE)).any()
    assert (result["flags"] & N.SEGMENT_POLYGON_EDGE).all()
    for k, s in enumerate(result):
        assert tuple(s["a"]) == SQUARE[k] and tuple(s["b"]) == SQUARE[(k + 1) % 4]


@pytest.mark.parametrize("polygon", [SQUARE, LETTER_L, TRIANGLE], ids=["square", "L", "triangle"])
@pytest.mark.parametrize("reverse", [False, True])
def test_outward_side_follows_the_winding(edges, polygon, reverse):
    ring = polygon[::-1] if reverse else polygon
    for s in edges(ring):
        a, b = s["a"].astype(np.float64), s["b"].astype(np.float64)
        d = b - a
        left = np.array([-d[1], d[0]]) / np.hypot(*d)
        sign = float(s["outward_sign"])
        assert abs(sign) == 1
        middle = (a + b) / 2
        assert not contains(ring, middle + left * sign * 0.01)
        assert contains(ring, middle - left * sign * 0.01)


@pytest.mark.parametrize("reverse", [False, True])
def test_end_convexity_matches_the_geometry(edges, reverse):
    ring = LETTER_L[::-1] if reverse else LETTER_L
    for s in edges(ring):
        start_inner, end_inner = tuple(s["a"]) == (48, 48), tuple(s["b"]) == (48, 48)
        assert bool(s["flags"] & N.SEGMENT_CONVEX_START) == (not start_inner)
        assert bool(s["flags"] & N.SEGMENT_CONVEX_END) == (not end_inner)
    for s in edges(TRIANGLE):
        assert s["flags"] & N.SEGMENT_CONVEX_START and s["flags"] & N.SEGMENT_CONVEX_END


@pytest.mark.parametrize("reverse", [False, True])
def test_previous_start_is_the_start_of_the_previous_edge(edges, reverse):
    result = edges(LETTER_L[::-1] if reverse else LETTER_L)
    for k, s in enumerate(result):
        assert tuple(s["previous_start"]) == tuple(result[(k - 1) % len(result)]["a"])


def test_nearly_collinear_edges_inside_the_tolerance_are_merged(edges):
    merged = edges([(0, 0), (400, 1.8e-3), (800, 0), (800, 48), (0, 48)])  # |cross| / (|e1||e2|) ~ 0.9e-5
    assert len(merged) == 4 and merged["id"].tolist() == [10, 11, 12, 13]
    long = [s for s in merged if tuple(s["a"]) == (0, 0)]
    assert len(long) == 1 and tuple(long[0]["b"]) == (800, 0)
    assert all(s["flags"] & N.SEGMENT_CONVEX_START and s["flags"] & N.SEGMENT_CONVEX_END for s in merged)


@pytest.mark.parametrize("bend,count", [(2.2e-3, 5), (50.0, 5), (-50.0, 5), (1.8e-3, 4)])
def test_edges_just_outside_the_tolerance_are_not_merged(edges, bend, count):
    assert len(edges([(0, 0), (400, bend), (800, 0), (800, 48), (0, 48)])) == count


def test_exactly_collinear_vertex_is_removed_for_both_windings(edges):
    doubled = [(0, 0), (100, 0), (200, 0), (200, 100), (0, 100)]
    for ring in (doubled, doubled[::-1]):
        result = edges(ring)
        assert len(result) == 4
        assert any({tuple(s["a"]), tuple(s["b"])} == {(0, 0), (200, 0)} for s in result)


def test_both_builders_agree_record_for_record():
    for poly in (SQUARE, LETTER_L, TRIANGLE, [(0, 0), (400, 1.8e-3), (800, 0), (800, 48), (0, 48)]):
        for ring in (poly, poly[::-1]):
            a = static_polygon_edges(np.asarray(ring, np.float32), 10, 77)
            b = polygon_edges(np.asarray(ring, np.float32), 10, 77)
            assert a.tobytes() == b.tobytes()
