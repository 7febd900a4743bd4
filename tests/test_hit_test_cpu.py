"""The hit test's rule (nativeHitTest, NativeGeometryKernels:501-541) on the oracle: a bubble answers inside its
contour, a body inside its shape, a static polygon (its one-sided edges) inside its ring; the highest layer wins,
then the largest id; empty space answers nothing. The reference's own cases (NativeMetalHitTestTests.swift:20-132:
point order, rotated polygons, the largest id, layers over ids, layers ordered as Int32, the contour of the same
step, objects removed by the region) are restated at the end."""
import math

import numpy as np
import pytest

from bubblephysics_gb300 import _native as N
from bubblephysics_gb300.scenes import polygon_edges
from bubblephysics_gb300.spec import WorldSpec, make_bubbles
from oracle.oracle import OracleWorld


def scene(bubble_layer=0, body_layer=0):
    b = make_bubbles([(0.0, 0.0), (100.0, 0.0), (300.0, 0.0)], 12.0, ids=[5, 6, 7], masses=1.0, stiffness=229.0)
    b["layer"] = [bubble_layer, 0, 0]
    body = np.zeros(1, N.BODY_DTYPE)
    body["id"] = 50
    body["position"] = (10.0, 0.0)       # overlaps bubble 5's right side
    body["bounding_radius"] = body["core_radius"] = 6.0
    body["kind"] = N.BODY_CIRCLE
    body["flags"] = N.BODY_STATIC
    body["vertex_count"] = 1
    body["category"], body["mask"] = 1, 0xFFFFFFFF
    body["layer"] = body_layer
    square = [(190.0, -10.0), (210.0, -10.0), (210.0, 10.0), (190.0, 10.0)]
    segs = polygon_edges(square, 100, owner_id=900)
    segs["layer"] = 2
    return WorldSpec(bubbles=b, segments=segs, bodies=body, body_vertices=np.zeros((1, 2), np.float32),
                     body_triangles=np.zeros((0, 3), np.uint32))


def test_each_kind_answers_inside_itself():
    w = OracleWorld(scene(), 32)
    w.step(1)
    ids, layers, found = w.hit_test([(-5.0, 0.0), (100.0, 3.0), (200.0, 0.0), (50.0, 50.0)])
    assert found.tolist() == [1, 1, 1, 0]
    assert ids[:3].tolist() == [5, 6, 900] and layers[2] == 2


def test_layer_then_id_decide_overlaps():
    # bubble 5 and body 50 both cover (10, 0): same layer -> the larger id (50); a higher bubble layer -> bubble 5
    same = OracleWorld(scene(), 32)
    same.step(1)
    assert same.hit_test([(10.0, 0.0)])[0].tolist() == [50]
    raised = OracleWorld(scene(bubble_layer=3), 32)
    raised.step(1)
    ids, layers, _ = raised.hit_test([(10.0, 0.0)])
    assert ids.tolist() == [5] and layers.tolist() == [3]


# ---- NativeMetalHitTestTests.swift:20-132, restated: static bubbles that collide with nothing (category 1, mask 0),
# r 5, K_c 1e4, static bodies, region [-100, 100]^2, one step of 1/60 ----

def box_body(bid, pos, half, angle=0.0):
    r = np.zeros(1, N.BODY_DTYPE)[0]
    r["id"], r["kind"], r["position"], r["angle"] = bid, N.BODY_POLYGON, pos, angle
    r["bounding_radius"], r["vertex_count"], r["triangle_count"] = half * 2 ** 0.5, 4, 2
    r["flags"], r["category"], r["mask"] = N.BODY_STATIC, 1, 0xFFFFFFFF
    return r, np.array([(-half, -half), (half, -half), (half, half), (-half, half)], np.float32), \
        np.array([(0, 1, 2), (0, 2, 3)], np.uint32)


def round_body(bid, pos, core, half_length=0.0):
    r = np.zeros(1, N.BODY_DTYPE)[0]
    r["id"], r["position"], r["core_radius"], r["half_length"] = bid, pos, core, half_length
    r["kind"] = N.BODY_CAPSULE if half_length else N.BODY_CIRCLE
    r["bounding_radius"] = core + half_length
    r["vertex_count"] = 2 if half_length else 1
    r["flags"], r["category"], r["mask"] = N.BODY_STATIC, 1, 0xFFFFFFFF
    v = np.array([(-half_length, 0.0), (half_length, 0.0)] if half_length else [(0.0, 0.0)], np.float32)
    return r, v, np.zeros((0, 3), np.uint32)


def hit_scene(bubbles=(), bodies=(), moving=None):
    """bubbles: (id, x, y, layer); bodies: (record, vertices, triangles, layer)."""
    rows = sorted(bubbles)
    b = make_bubbles([(x, y) for _, x, y, _ in rows], 5.0, ids=[i for i, _, _, _ in rows], stiffness=1e4,
                     mask=0, static=[True] * len(rows))
    b["layer"] = [layer for *_, layer in rows]
    if moving is not None:
        b = np.concatenate([b, moving])
        b = b[np.argsort(b["id"])]
    recs, verts, tris = [], [], []
    for rec, v, t, layer in bodies:
        rec = rec.copy()
        rec["vertex_offset"], rec["triangle_offset"], rec["layer"] = sum(len(x) for x in verts), sum(len(x) for x in tris), layer
        recs.append(rec)
        verts.append(v)
        tris.append(t)
    return WorldSpec(bubbles=b, bodies=np.array(recs, N.BODY_DTYPE) if recs else np.zeros(0, N.BODY_DTYPE),
                     body_vertices=np.concatenate(verts) if verts else np.zeros((0, 2), np.float32),
                     body_triangles=np.concatenate(tris) if tris else np.zeros((0, 3), np.uint32),
                     region=(-100.0, -100.0, 100.0, 100.0))


def answers(spec, points, world=None):
    w = world or OracleWorld(spec, 32)
    assert w.step(1)[0] == N.OK
    ids, _, found = w.hit_test(points)
    return [int(i) if f else None for i, f in zip(ids, found)]


HIT_CASES = {
    "point order names bubbles and bodies": (
        lambda: hit_scene([(1, -60.0, 0.0, 0)], [(*box_body(2, (-20.0, 0.0), 5.0), 0), (*round_body(3, (20.0, 0.0), 5.0), 0),
                                                 (*round_body(4, (60.0, 0.0), 3.0, 8.0), 0)]),
        [(60, 2), (-60, 0), (-20, 4), (0, 0), (20, 3), (60, 10), (68, 2), (20, 8), (-20, 6)],
        [4, 1, 2, None, 3, None, 4, None, None]),
    "polygon hit on its rotated shape": (
        lambda: hit_scene([], [(*box_body(2, (0.0, 0.0), 5.0, math.pi / 4), 0)]),
        [(6, 0), (4.5, 4.5), (0, 6), (-5, -5)], [2, None, 2, None]),
    "largest id wins": (
        lambda: hit_scene([(30, 0.0, 0.0, 0), (12, 0.0, 0.0, 0), (50, 40.0, 0.0, 0)],
                          [(*box_body(7, (0.0, 0.0), 3.0), 0), (*round_body(90, (40.0, 0.0), 2.0), 0)]),
        [(0, 0), (40, 0), (4, 0)], [30, 90, 30]),
    "higher layer wins over a larger id": (
        lambda: hit_scene([(30, 0.0, 0.0, 0), (2, 40.0, 0.0, 5), (8, 80.0, 0.0, 1)],
                          [(*box_body(7, (0.0, 0.0), 3.0), 3), (*round_body(40, (40.0, 0.0), 4.0), 0),
                           (*round_body(9, (80.0, 0.0), 2.0, 2.0), 1)]),
        [(0, 0), (40, 0), (80, 0), (-4, 0)], [7, 2, 9, 30]),
    "negative and extreme layers order like Int32": (
        lambda: hit_scene([(90, 0.0, 0.0, -1), (2, 0.0, 0.0, 0), (91, 40.0, 0.0, -2 ** 31), (3, 40.0, 0.0, -2),
                           (4, 80.0, 0.0, 2 ** 31 - 1), (95, 80.0, 0.0, 2 ** 31 - 2), (5, 120.0, 0.0, -3),
                           (77, 120.0, 0.0, -3)]),
        [(0, 0), (40, 0), (80, 0), (120, 0)], [2, 3, 4, 77]),
}


@pytest.mark.parametrize("name", sorted(HIT_CASES))
def test_reference_hit_test_cases(name):
    build, points, expected = HIT_CASES[name]
    assert answers(build(), points) == expected


def test_bubble_contour_answers_on_the_state_of_the_same_step():
    moving = make_bubbles([(0.0, 0.0)], 5.0, ids=[1], velocities=[(60.0, 0.0)], stiffness=1e4)
    assert answers(hit_scene(moving=moving), [(5.5, 0), (-5.5, 0)]) == [1, None]


def test_objects_removed_by_the_region_do_not_take_part():
    outside = make_bubbles([(110.0, 0.0)], 2.0, ids=[1], stiffness=1e4,
                           flags=N.BUBBLE_FORCE_DRIVEN | N.BUBBLE_ENABLED)
    spec = hit_scene([(2, 0.0, 0.0, 0)], moving=outside)
    w = OracleWorld(spec, 32)
    assert answers(spec, [(110, 0), (0, 0)], w) == [None, 2] and w.bubbles()["region_result"][0] == 1
