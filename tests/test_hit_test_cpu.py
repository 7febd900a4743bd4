"""The hit test's rule (nativeHitTest, NativeGeometryKernels:501-541) on the oracle: a bubble answers inside its
contour, a body inside its shape, a static polygon (its one-sided edges) inside its ring; the highest layer wins,
then the largest id; empty space answers nothing."""
import numpy as np

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
