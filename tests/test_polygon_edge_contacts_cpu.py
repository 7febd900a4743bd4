"""Contacts with the one-sided edges of a static polygon around its vertices, on the oracle, against the reference's
own sweep (NativeStaticPolygonContactTests.swift:10-137): bubble centres (r 24) outside the polygon and closer than
the radius around vertices of 30, 90, 120 and 270 degrees, at every 5 degrees, on the rays perpendicular to both edges
and one float ulp beside them, and exactly on the region boundaries within a window of 8 ulps, for both windings,
each get at least one edge contact and never two whose normals differ by less than 1e-3 rad."""
import math

import numpy as np

from bubblephysics_gb300 import _native as N
from bubblephysics_gb300.scenes import polygon_edges
from bubblephysics_gb300.spec import WorldSpec, make_bubbles
from oracle.oracle import OracleWorld

F = np.float32
R = F(24)


def apex(degrees):
    half = F(degrees) * F(math.pi) / F(360)
    c, s = F(100) * F(math.cos(half)), F(100) * F(math.sin(half))
    return [(F(0), F(0)), (c, s), (c, -s)], (F(0), F(0))


LETTER_L = [(F(x), F(y)) for x, y in ((0, 0), (200, 0), (200, 48), (48, 48), (48, 200), (0, 200))]
CORNERS = [("30", *apex(30)), ("90", LETTER_L, (F(0), F(0))), ("120", *apex(120)), ("270", LETTER_L, (F(48), F(48)))]


def contains(poly, p):
    inside = False
    for i in range(len(poly)):
        a, b = poly[i], poly[(i + 1) % len(poly)]
        if (a[1] > p[1]) != (b[1] > p[1]) and p[0] < a[0] + (p[1] - a[1]) / (b[1] - a[1]) * (b[0] - a[0]):
            inside = not inside
    return inside


def distance_to(poly, p):
    best = math.inf
    for i in range(len(poly)):
        a, b = np.array(poly[i], np.float32), np.array(poly[(i + 1) % len(poly)], np.float32)
        e = b - a
        t = min(max(float(np.dot(p - a, e)) / max(float(np.dot(e, e)), 1e-38), 0.0), 1.0)
        best = min(best, float(np.hypot(*(p - (a + F(t) * e)))))
    return best


def up(v):
    return np.nextafter(F(v), F(np.inf), dtype=np.float32)


def down(v):
    return np.nextafter(F(v), F(-np.inf), dtype=np.float32)


def centers(vertex, ring):
    k = [tuple(p) for p in ring].index(tuple(vertex))
    prev, nxt = np.array(ring[k - 1], np.float32), np.array(ring[(k + 1) % len(ring)], np.float32)
    v = np.array(vertex, np.float32)
    unit = lambda w: w / F(np.hypot(*w))
    incoming, outgoing = unit(v - prev), unit(nxt - v)
    angles = [F(a) * F(math.pi) / F(180) for a in range(0, 360, 5)]
    for d in (incoming, outgoing):
        n = np.array([-d[1], d[0]], np.float32)
        angles += [F(math.atan2(n[1], n[0])), F(math.atan2(-n[1], -n[0]))]
    out = []
    for ang in angles:
        for scale in (F(0.5), F(0.95)):
            p = v + scale * R * np.array([math.cos(ang), math.sin(ang)], np.float32)
            out += [p, np.array([up(p[0]), p[1]], np.float32), np.array([down(p[0]), p[1]], np.float32),
                    np.array([p[0], up(p[1])], np.float32), np.array([p[0], down(p[1])], np.float32)]
    for d in (incoming, outgoing):  # exactly on the region boundaries and within 8 ulps of them
        n = np.array([-d[1], d[0]], np.float32)
        for sign in (F(1), F(-1)):
            for dist in (F(0.5) * R, F(0.95) * R):
                seed = v + sign * dist * n
                solve_x = abs(d[0]) >= abs(d[1])
                exact = seed.copy()
                if solve_x:
                    exact[0] = v[0] - (seed[1] - v[1]) * d[1] / d[0]
                else:
                    exact[1] = v[1] - (seed[0] - v[0]) * d[0] / d[1]
                below = above = exact[0] if solve_x else exact[1]
                window = [below]
                for _ in range(8):
                    below, above = down(below), up(above)
                    window += [below, above]
                if (exact[0] if solve_x else exact[1]) == 0:
                    window.append(F(-0.0))
                for value in window:
                    out.append(np.array([value, exact[1]] if solve_x else [exact[0], value], np.float32))
    keep = []
    for p in out:
        dist = distance_to(ring, p)
        if not contains(ring, p) and 1e-3 < dist < 24:
            keep.append(p)
    return keep


def test_every_centre_closer_than_the_radius_has_one_non_duplicated_contact_around_every_vertex():
    checked = 0
    for name, polygon, vertex in CORNERS:
        for reverse in (False, True):
            ring = polygon[::-1] if reverse else polygon
            segs = polygon_edges(np.array(ring, np.float32), 1, owner_id=5)
            for k, p in enumerate(centers(vertex, ring)):
                b = make_bubbles([tuple(p)], 24.0, ids=[1000 + k], masses=1.0, stiffness=0.0)
                w = OracleWorld(WorldSpec(bubbles=b, segments=segs), 32)
                assert w.step(1)[0] == N.OK
                normals = [c["normal"].astype(np.float64) for c in w.contacts() if c["kind"] == 1]
                assert len(normals) >= 1, (name, reverse, p)
                for i in range(len(normals)):
                    for j in range(i + 1, len(normals)):
                        a, c = normals[i], normals[j]
                        angle = abs(math.atan2(a[0] * c[1] - a[1] * c[0], float(np.dot(a, c))))
                        assert angle >= 1e-3, (name, reverse, p, a, c)
                checked += 1
    assert checked > 500
