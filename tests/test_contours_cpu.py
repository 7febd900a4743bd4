"""Contours (NativePostSolveKernels:268-527) on the oracle: a lone bubble keeps a round contour of its radius; a
pressed pair is cut flat at the pair law's chord r (1 - eps) on the side of the contact; a wall cuts the contour where
the bubble crosses it; the smoothing never goes below the hard deficit and the majorant keeps the slope bounded."""
import numpy as np

import fixtures
from bubblephysics_gb300.spec import WorldSpec, make_bubbles
from oracle.oracle import OracleWorld


def test_lone_bubble_contour_is_its_circle():
    spec = WorldSpec(bubbles=make_bubbles([(5.0, 7.0)], 24.0, masses=1.0, stiffness=229.0))
    w = OracleWorld(spec, 32)
    w.step(1)
    pts, cnt, lvl, shp = w.contours()
    assert cnt[0] == 64  # ceil(4 pi 24 / 8) = 38 samples, raised to the minimum of 64
    c = w.bubbles()["center"][0]
    d = np.hypot(*(pts[0, :cnt[0]] - c).T)
    assert np.allclose(d, 24.0, atol=1e-4) and np.all(lvl[0, :cnt[0]] == 0)
    assert shp[0][0] == 0 and abs(shp[0][1] - 24.0) < 1e-4


def test_pressed_pair_is_cut_at_the_pair_law_chord():
    spec = WorldSpec(bubbles=make_bubbles([(0.0, 0.0), (20.0, 0.0)], 12.0, masses=1.0, stiffness=229.0))
    w = OracleWorld(spec, 32)
    w.step(1)
    pts, cnt, lvl, shp = w.contours()
    b = w.bubbles()
    distance = float(b["center"][1][0] - b["center"][0][0])
    eps = (24.0 - distance) / 24.0  # same material: each end takes half the overlap
    assert abs(shp[0][1] - 12.0 * (1 - eps)) < 1e-3 and abs(shp[1][1] - 12.0 * (1 - eps)) < 1e-3
    # the flat side faces the partner: the sample towards +x of bubble 0 is the most cut
    assert lvl[0, 0] == lvl[0, :cnt[0]].max() and lvl[0, 32] == 0
    # smoothing and majorant keep every level within [0, 1] and the slope bounded by maxEdge / (2 r)
    slope = 8.0 / (2 * 12.0)
    ring = lvl[0, :cnt[0]]
    assert np.all((ring >= 0) & (ring <= 1)) and np.all(np.abs(np.diff(np.r_[ring, ring[0]])) <= slope + 1e-6)


def test_wall_cuts_the_contour():
    spec = fixtures.press_scene()
    w = OracleWorld(spec, 32)
    w.step(1)
    pts, cnt, lvl, shp = w.contours()
    c = w.bubbles()["center"][0]
    # the floor edge is at y = 0 above the bubble: no contour point crosses it (clearance 1e-4)
    assert np.all(pts[0, :cnt[0], 1] <= 1e-3) and shp[0][0] > 0
    assert shp[0][5] <= 1e-3 and c[1] < 0
