"""More of the reference's world-level known answers, restated as scenes on the oracle:

 - RegionPolicyTests.swift:9-15, 97-133, 252-270 — the region is not a wall: a circle whose collider left the region
   at a corner is removed although its bounds still overlap it; a wrapped bubble keeps its overshoot across several
   region widths (position, step-start position and velocity), a diagonal corner wrap re-enters and stays put, and a
   wrap keeps the velocity without a contact across the seam;
 - DeepSqueezeWallTests.swift:24-80 — a bubble pulled into a wall by the band harder than K_c settles at the contact
   law's deflection (2 %) with its centre always before the wall's edge (K_c = 20 / 0.0108, gamma 5, K_band 30,
   F_max = F, target 2000 behind the wall; r 24 for 6 s and r 74 for 60 s at F 2222, r 24 at F 20 000 and 50 000);
 - CrowdCompressionTests.swift:36-139 — bubbles pushed diagonally into a corner of the frame by motors stay inside the
   frame for 300 steps and the pushed one reaches the corner; alone, a softer bubble dents more than a stiffer one.

Scenes follow CrowdSceneSupport.swift:10-60: an interior of 360 x 640 framed by four static rectangles 48 thick (side
walls full height), the region the outer rectangle, bubble mass r^2 / 400."""
import math

import numpy as np
import pytest

import clr
from bubblephysics_gb300 import _native as N
from bubblephysics_gb300.scenes import polygon_edges
from bubblephysics_gb300.spec import WorldSpec, make_bubbles
from oracle.oracle import OracleWorld

HALF = (180.0, 320.0)
THICK = 48.0


def frame_walls():
    ix, iy = HALF
    ox, oy = ix + THICK, iy + THICK
    rects = [((-ox, -oy), (-ix, oy)), ((ix, -oy), (ox, oy)), ((-ix, -oy), (ix, -iy)), ((-ix, iy), (ix, oy))]
    segs, first = [], 5000
    for k, ((lx, ly), (hx, hy)) in enumerate(rects):
        e = polygon_edges([(lx, ly), (hx, ly), (hx, hy), (lx, hy)], first, owner_id=9001 + k)
        first += len(e)
        segs.append(e)
    return np.concatenate(segs)


def crowd_spec(bubbles, bands=(), motors=()):
    ix, iy = HALF
    s = WorldSpec(bubbles=bubbles, segments=frame_walls(), region=(-ix - THICK, -iy - THICK, ix + THICK, iy + THICK))
    s.bands, s.motors = list(bands), list(motors)
    return s


def stepper(spec):
    w = OracleWorld(spec, 32)

    def step():
        status, _ = w.step(1)
        assert status == N.OK
        return w.bubbles()
    return step


# ---- RegionPolicyTests -----------------------------------------------------------------------------------------------

def region_bubble(x, y, vx, wrap, r=1.0):
    flags = N.BUBBLE_FORCE_DRIVEN | N.BUBBLE_ENABLED | (N.BUBBLE_WRAP if wrap else 0)
    return make_bubbles([(x, y)], r, velocities=[(vx, 0.0)], stiffness=229.0, flags=flags)


def region_spec(bubbles):
    return WorldSpec(bubbles=bubbles, region=(0.0, 0.0, 10.0, 10.0), time_step=0.25)


def test_circle_outside_the_corner_is_removed_although_its_bounds_overlap():
    b = region_bubble(10.8, 10.8, 0.0, wrap=False)
    out = stepper(region_spec(b))()
    assert out["region_result"][0] == 1  # removed


def test_wrap_retains_the_overshoot_across_several_region_widths():
    b = region_bubble(-25.0, 5.0, -4.0, wrap=True)
    out = stepper(region_spec(b))()
    assert out["region_result"][0] == 2
    assert out["center"][0].tolist() == [10.0, 5.0] and out["previous_center"][0].tolist() == [11.0, 5.0]
    assert out["velocity"][0].tolist() == [-4.0, 0.0]


def test_diagonal_corner_wrap_reenters_and_does_not_oscillate():
    step = stepper(region_spec(region_bubble(10.8, 10.8, 0.0, wrap=True)))
    first = step()["center"][0].astype(np.float64)
    dx, dy = max(0.0, -first[0], first[0] - 10), max(0.0, -first[1], first[1] - 10)
    assert math.hypot(dx, dy) <= 1
    second = step()
    assert np.allclose(second["center"][0], first, atol=1e-4) and second["velocity"][0].tolist() == [0.0, 0.0]


def test_wrap_keeps_the_velocity_without_a_contact_across_the_seam():
    wrap = region_bubble(9.0, 5.0, 4.0, wrap=True)
    other = region_bubble(0.25, 5.0, 0.0, wrap=False)
    other["id"] = 2
    step = stepper(region_spec(np.concatenate([wrap, other])))
    assert abs(float(step()["center"][1][0]) - 0.25) <= 1e-4  # only a toroidal image overlapped it
    step()
    out = step()
    assert abs(float(out["center"][0][0])) <= 1e-4 and abs(float(out["previous_center"][0][0]) + 1) <= 1e-4
    assert out["velocity"][0].tolist() == [4.0, 0.0]


# ---- DeepSqueezeWallTests --------------------------------------------------------------------------------------------

KC_SQUEEZE = float(np.float32(20.0) / np.float32(0.0108))


def squeeze(radius, force, seconds):
    start = -HALF[0] + radius + 20
    b = make_bubbles([(start, 0.0)], radius, masses=radius * radius / 400, stiffness=KC_SQUEEZE, damping=5.0)
    band = N.Band()
    band.bubble_id, band.stiffness, band.maximum_force = 1, 30.0, force
    band.target[:] = [-2000.0, 0.0]
    step = stepper(crowd_spec(b, bands=[band]))
    ratio = peak = 0.0
    for _ in range(int(seconds * 60)):
        x = float(step()["center"][0][0])
        ratio = (radius - (HALF[0] + x)) / radius  # the wall depth over the radius
        peak = max(peak, ratio)
    return ratio, peak


@pytest.mark.parametrize("radius,force,seconds", [(24.0, 2222.0, 6), (74.0, 2222.0, 60), (24.0, 20_000.0, 6),
                                                  (24.0, 50_000.0, 6)], ids=["r24-2222", "r74-2222", "r24-20000",
                                                                             "r24-50000"])
def test_bubble_pressed_harder_than_kc_settles_before_the_edge(radius, force, seconds):
    expected = clr.epsilon(force / KC_SQUEEZE)
    final, peak = squeeze(radius, force, seconds)
    assert expected < 1 and abs(final - expected) <= 0.02 * expected, (final, expected)
    assert peak < 1


# ---- CrowdCompressionTests (corner) ----------------------------------------------------------------------------------

def motor(bubble_id, force):
    m = N.Motor()
    m.bubble_id = bubble_id
    m.force[:] = [float(force[0]), float(force[1])]
    return m


CORNER_FORCE = (np.array([1.0, 1.0]) / math.sqrt(2.0) * 3000.0).astype(np.float32)


def inside_frame(p):
    return abs(p[0]) <= HALF[0] + 1e-3 and abs(p[1]) <= HALF[1] + 1e-3


def test_corner_pushed_by_ten_bubbles_keeps_every_centre_in_the_frame():
    kc = float(np.float32(20.0) / np.float32(3e-4))
    centers = [(140.0, 280.0)] + [(20.0 + (k % 4) * 45.0, 150.0 + (k // 4) * 45.0) for k in range(10)]
    b = make_bubbles(centers, 20.0, masses=1.0, stiffness=kc, damping=5.0)
    step = stepper(crowd_spec(b, motors=[motor(i, CORNER_FORCE) for i in range(1, 12)]))
    for _ in range(301):
        out = step()
        assert all(inside_frame(p) for p in out["center"])
    corner = np.array(HALF)
    assert np.hypot(*(out["center"][0].astype(np.float64) - corner)) < 20 * math.sqrt(2) + 1


def single_corner_depth(kc):
    b = make_bubbles([(160.0, 300.0)], 20.0, masses=1.0, stiffness=kc, damping=5.0)
    step = stepper(crowd_spec(b, motors=[motor(1, CORNER_FORCE)]))
    for _ in range(181):
        out = step()
    p = out["center"][0].astype(np.float64)
    return 20 - min(HALF[0] - p[0], HALF[1] - p[1])


def test_softer_bubble_dents_more_in_the_corner():
    soft = single_corner_depth(float(np.float32(20.0) / np.float32(3e-4)))
    stiff = single_corner_depth(float(np.float32(20.0) / np.float32(3e-5)))
    assert soft > stiff + 0.05, (soft, stiff)
