"""The reference's world-level known answers, restated as scenes on the oracle (float, the product's arithmetic):

 - ContactLawStaticsTests.swift:16-170 — a bubble pressed to a wall and a pair pressed together hold the equilibrium
   distance of the law in every frame for 20 s; the mean deflection inverts the law across force ratios 1e-4..1e6;
   a same-material pair splits its deflection in proportion to the radii (measured on the contours); a pair of
   different stiffness carries the force of the Newton pair solution;
 - ContourChordTests.swift:8-57 — the contours of a pressed pair meet on one flat chord, each at r (1 - eps);
 - SubstepCountTests.swift:17-121 — one substep per step where nothing needs a finer h (a crowd at rest, slow motion
   with a wall bounce, a bubble dragged by the band), about three under a static press of 20 000, and a peak during a
   1000 units/s impact within 20 % of the one-dimensional h-rule reference, back to one substep once d > 4 |v| dt;
 - NoCrossingTests.swift:18-124 — wall impacts at 100 / 1000 / 3000 units/s, straight and at 45 degrees, with and
   without damping, never put a centre past the wall in any substep and reach the energy balance's closest distance
   (within 10 %); pair impacts keep the centres apart and on their sides in every substep;
 - ForceIntegrationTests.swift:13-82 — a bubble rebounds with its impact speed (2 %); with drag the energy lost equals
   the drag integral over the substeps (5 % of it + 1 % of the initial energy).

Scenes follow ForceSceneSupport.swift:10-110: bubbles "2" (r 24, m 1), 128 (r 64) and 7168 (r 148) with the game mass
(n/2)^(1/2.25); K_c = 229; walls are static rectangles one unit thick; pushes are directional fields on one bubble.
The thresholds are the reference tests' own; the expected values come from the law restated in `clr.py`."""
import math

import numpy as np
import pytest

import clr
from bubblephysics_gb300 import _native as N
from bubblephysics_gb300.scenes import polygon_edges
from bubblephysics_gb300.spec import WorldSpec, make_bubbles
from oracle.oracle import OracleWorld

K = 229.0
WALL_X = 360.0
DT = 1.0 / 60


def game_mass(n):
    return float(np.float32((n / 2) ** (1 / 2.25)))


TWO, B128, B7168 = (24.0, 1.0), (64.0, game_mass(128)), (148.0, game_mass(7168))
FORCES = [100.0, 1200.0, 10_000.0, 20_000.0, 100_000.0]


def wall(x, thickness=1.0, half_height=1900.0):
    poly = [(x, -half_height), (x + thickness, -half_height), (x + thickness, half_height), (x, half_height)]
    return polygon_edges(poly, 2000, owner_id=2)


def push(target_index, force):
    """A directional field of `force` on one bubble, a circle of radius 1500 about the origin."""
    f = N.ForceField()
    f.kind, f.radius = 0, 1500.0
    f.direction[:] = [float(force[0]), float(force[1])]
    f.has_filter, f.filter_offset, f.filter_count = 1, target_index, 1
    return f


def spec_of(bubbles, segments=None, fields=(), field_ids=(), global_force=(0.0, 0.0), bands=()):
    s = WorldSpec(bubbles=bubbles, global_force=global_force, region=(-2000.0, -2000.0, 2000.0, 2000.0))
    if segments is not None:
        s.segments = segments
    s.fields = list(fields)
    s.field_object_ids = np.asarray(field_ids, np.int64)
    s.bands = list(bands)
    return s


def run(spec, frames, *, trace=False, until=None):
    """Steps one frame at a time; returns per frame (status, substeps, bubbles[, trace])."""
    w = OracleWorld(spec, 32)
    if trace:
        w.set_trace(True)
    out = []
    for k in range(frames):
        status, rep = w.step(1)
        item = (status, int(rep[0]["substep_count"]), w.bubbles(), w.trace() if trace else None)
        out.append(item)
        assert status == N.OK, (k, status)
        if until is not None and until(k, item[2]):
            break
    return out


# ---- ContactLawStaticsTests ------------------------------------------------------------------------------------------

@pytest.mark.parametrize("kind", [TWO, B7168], ids=["2", "7168"])
@pytest.mark.parametrize("force", FORCES)
def test_bubble_pressed_to_a_wall_holds_the_equilibrium_distance(kind, force):
    r, m = kind
    d_star = clr.equilibrium_distance(force, K, r)
    wall_x = float(np.float32(d_star))
    b = make_bubbles([(0.0, 0.0)], r, masses=m, stiffness=K)
    for _, _, bub, _ in run(spec_of(b, wall(wall_x), global_force=(force, 0.0)), 1200):
        d = wall_x - float(bub["center"][0][0])
        assert d > 0 and abs(d - d_star) <= 0.005 * d_star + 1e-3, (d, d_star)


@pytest.mark.parametrize("pair", [(TWO, TWO), (TWO, B7168)], ids=["2-2", "2-7168"])
@pytest.mark.parametrize("force", FORCES)
def test_pair_pressed_together_holds_the_equilibrium_distance(pair, force):
    (ra, ma), (rb, mb) = pair
    d_star = (ra + rb) * (1 - clr.epsilon(force / K))
    half = float(np.float32(d_star / 2))
    b = make_bubbles([(-half, 0.0), (half, 0.0)], [ra, rb], masses=[ma, mb], stiffness=K)
    spec = spec_of(b, fields=[push(0, (force, 0.0)), push(1, (-force, 0.0))], field_ids=[1, 2])
    for _, _, bub, _ in run(spec, 1200):
        d = float(np.hypot(*(bub["center"][1].astype(np.float64) - bub["center"][0])))
        assert d > 0 and abs(d - d_star) <= 0.005 * d_star + 1e-3, (d, d_star)


def test_inverse_of_the_law_agrees_with_double_across_force_ratios():
    for q in [1e-4, 1e-3, 1e-2, 1e-1, 1, 10, 100, 1e3, 1e4, 1e5, 1e6]:
        r, m = B7168 if q >= 1e6 else TWO
        force = float(np.float32(q * K))
        expected = clr.epsilon(force / K)
        wall_x = float(np.float32(r * (1 - expected)))
        b = make_bubbles([(0.0, 0.0)], r, masses=m, stiffness=K)
        frames = run(spec_of(b, wall(wall_x), global_force=(force, 0.0)), 240)
        mean_d = np.mean([wall_x - float(bub["center"][0][0]) for _, _, bub, _ in frames])
        mean_eps = 1 - mean_d / r
        assert abs(mean_eps - expected) <= 1e-3 * expected, (q, mean_eps, expected)


def chord(points, count, center, direction):
    """The contour's farthest point toward `direction` from `center` (ForceScene.chord, ForceSceneSupport.swift:171-173)."""
    ring = points[:count].astype(np.float64)
    return float(((ring - center) @ np.asarray(direction, np.float64)).max())


def test_same_material_pair_splits_the_deflection_in_proportion_to_the_radii():
    (ra, ma), (rb, mb), force = TWO, B7168, 1200.0
    d_star = (ra + rb) * (1 - clr.epsilon(force / K))
    half = float(np.float32(d_star / 2))
    b = make_bubbles([(-half, 0.0), (half, 0.0)], [ra, rb], masses=[ma, mb], stiffness=K)
    w = OracleWorld(spec_of(b, fields=[push(0, (force, 0.0)), push(1, (-force, 0.0))], field_ids=[1, 2]), 32)
    assert w.step(60)[0] == N.OK
    pts, counts, _, _ = w.contours()
    c = w.bubbles()["center"].astype(np.float64)
    normal = (c[1] - c[0]) / np.hypot(*(c[1] - c[0]))
    da = ra - chord(pts[0], counts[0], c[0], normal)
    db = rb - chord(pts[1], counts[1], c[1], -normal)
    assert da > 0.1 and db > 0.1
    assert abs(da / db - ra / rb) <= 0.02 * ra / rb, (da, db)


@pytest.mark.parametrize("force,ratio", [(1200.0, 10.0), (1200.0, 1000.0), (100.0, 10.0)])
def test_different_material_pair_force_matches_the_newton_reference(force, ratio):
    (ra, ma), (rb, mb) = TWO, TWO
    kb = K * ratio
    d_star = ra * (1 - clr.epsilon(force / K)) + rb * (1 - clr.epsilon(force / kb))
    half = float(np.float32(d_star / 2))
    b = make_bubbles([(-half, 0.0), (half, 0.0)], [ra, rb], masses=[ma, mb], stiffness=[K, kb])
    frames = run(spec_of(b, fields=[push(0, (force, 0.0)), push(1, (-force, 0.0))], field_ids=[1, 2]), 240)
    mean = np.mean([np.hypot(*(bub["center"][1].astype(np.float64) - bub["center"][0])) for _, _, bub, _ in frames])
    f, _, _ = clr.pair_contact(ra + rb - mean, ra, K, rb, kb)
    assert abs(f - force) <= 0.01 * force, (f, force)


@pytest.mark.parametrize("pair,force,kb", [((TWO, TWO), 100.0, K), ((TWO, TWO), 1200.0, K), ((TWO, B7168), 100.0, K),
                                           ((TWO, B7168), 1200.0, K), ((TWO, TWO), 1200.0, 2290.0)],
                         ids=["2-2-100", "2-2-1200", "2-7168-100", "2-7168-1200", "2-2-Kb10"])
def test_contour_chords_of_a_pressed_pair_coincide(pair, force, kb):
    """ContourChordTests.swift:8-57: after 60 frames the flat chords of both contours meet (their sum is the centre
    distance within 1e-3 R, no interpenetration) and each lies at r (1 - eps) of the law within 2e-3 R."""
    (ra, ma), (rb, mb) = pair
    ea, eb = clr.epsilon(force / K), clr.epsilon(force / kb)
    half = float(np.float32((ra * (1 - ea) + rb * (1 - eb)) / 2))
    b = make_bubbles([(-half, 0.0), (half, 0.0)], [ra, rb], masses=[ma, mb], stiffness=[K, kb])
    w = OracleWorld(spec_of(b, fields=[push(0, (force, 0.0)), push(1, (-force, 0.0))], field_ids=[1, 2]), 32)
    assert w.step(60)[0] == N.OK
    pts, counts, _, _ = w.contours()
    c = w.bubbles()["center"].astype(np.float64)
    distance = float(np.hypot(*(c[1] - c[0])))
    normal = (c[1] - c[0]) / distance
    ca, cb = chord(pts[0], counts[0], c[0], normal), chord(pts[1], counts[1], c[1], -normal)
    radii = ra + rb
    assert ra - ca > 0.05 and rb - cb > 0.05
    assert ca + cb - distance <= 1e-3 * radii and abs(ca + cb - distance) <= 1e-3 * radii
    assert abs(ca - ra * (1 - ea)) <= 2e-3 * radii and abs(cb - rb * (1 - eb)) <= 2e-3 * radii


# ---- SubstepCountTests -----------------------------------------------------------------------------------------------

def test_crowd_at_rest_takes_one_substep_per_step():
    centers = [(c * 46.0 - 69.0, r * 46.0 - 69.0) for r in range(4) for c in range(4)]
    b = make_bubbles(centers, TWO[0], masses=TWO[1], stiffness=K, damping=1.0)
    assert all(n == 1 for _, n, _, _ in run(spec_of(b), 300))


def test_slow_free_motion_with_a_wall_bounce_takes_one_substep_per_step():
    b = make_bubbles([(WALL_X - 24 - 60, 0.0)], TWO[0], velocities=[(30.0, 0.0)], masses=TWO[1], stiffness=K)
    frames = run(spec_of(b, wall(WALL_X)), 480)
    assert float(frames[-1][2]["velocity"][0][0]) < 0  # the bounce happened
    assert all(n == 1 for _, n, _, _ in frames)


def test_bubble_dragged_by_the_band_takes_one_substep_per_step():
    b = make_bubbles([(0.0, 0.0)], TWO[0], masses=TWO[1], stiffness=K, damping=1.0)
    band = N.Band()
    band.bubble_id, band.stiffness, band.maximum_force = 1, 22.0, math.inf
    band.target[:] = [100.0, 0.0]
    frames = run(spec_of(b, bands=[band]), 300)
    assert max(float(bub["velocity"][0][0]) for _, _, bub, _ in frames) > 50
    assert all(n == 1 for _, n, _, _ in frames)


def test_static_press_of_twenty_thousand_takes_about_three_substeps():
    d_star = clr.equilibrium_distance(20_000.0, K, 24.0)
    b = make_bubbles([(0.0, 0.0)], TWO[0], masses=TWO[1], stiffness=K)
    frames = run(spec_of(b, wall(float(np.float32(d_star))), global_force=(20_000.0, 0.0)), 120)
    assert all(2 <= n <= 4 for _, n, _, _ in frames[5:])


def test_impact_at_one_thousand_peaks_like_the_one_dimensional_reference():
    gap = 100.0
    b = make_bubbles([(WALL_X - 24 - gap, 0.0)], TWO[0], velocities=[(1000.0, 0.0)], masses=TWO[1], stiffness=K)
    frames = run(spec_of(b, wall(WALL_X)), 40)
    ref = clr.WallScene(radius=24.0, mass=1.0, stiffness=K, damping=0.0, start_distance=24.0 + gap, velocity=-1000.0)
    limit, _ = ref.run(40)
    assert not limit
    expected = max(f[0] for f in ref.frames)
    peak = max(n for _, n, _, _ in frames)
    assert expected > 5 and abs(peak - expected) <= 0.2 * expected, (peak, expected)
    checked = 0
    for k in range(1, len(frames)):
        x, v = frames[k - 1][2]["center"][0], frames[k - 1][2]["velocity"][0]
        d = WALL_X - float(x[0])
        if v[0] < 0 and d > 24 and d > 4 * abs(float(v[0])) * DT:
            checked += 1
            assert frames[k][1] == 1, k
    assert checked > 5


# ---- NoCrossingTests -------------------------------------------------------------------------------------------------

@pytest.mark.parametrize("kind", [TWO, B128, B7168], ids=["2", "128", "7168"])
@pytest.mark.parametrize("speed", [100.0, 1000.0, 3000.0])
@pytest.mark.parametrize("oblique", [False, True], ids=["straight", "oblique"])
@pytest.mark.parametrize("damping", [0.0, 1.0])
def test_wall_impacts_never_cross_the_wall(kind, speed, oblique, damping):
    r, m = kind
    direction = np.array([math.sqrt(0.5), math.sqrt(0.5)] if oblique else [1.0, 0.0], np.float32)
    normal_speed = float(speed * direction[0])
    gap = min(100.0, 0.3 * normal_speed / damping) if damping > 0 else 100.0
    vel = (direction * np.float32(speed)).astype(np.float32)
    b = make_bubbles([(WALL_X - r - gap, 0.0)], r, velocities=[tuple(vel)], masses=m, stiffness=K, damping=damping)
    frames = run(spec_of(b, wall(WALL_X)), 600, trace=True,
                 until=lambda k, bub: k > 1 and bub["velocity"][0][0] < 0 and bub["center"][0][0] < WALL_X - r)
    minimum, substeps = math.inf, 0
    for _, _, _, (h, state) in frames:
        for sample in state:
            substeps += 1
            minimum = min(minimum, WALL_X - sample[0][0])
            assert sample[0][0] < WALL_X
    assert substeps > 0 and float(frames[-1][2]["velocity"][0][0]) < 0
    if damping == 0:
        energy = 0.5 * m * normal_speed * normal_speed
        expected = r * (1 - clr.maximum_epsilon(energy, K, r))
        assert abs(minimum - expected) <= 0.1 * expected, (minimum, expected)


@pytest.mark.parametrize("pair", [(TWO, TWO), (B128, B128), (TWO, B7168)], ids=["2-2", "128-128", "2-7168"])
@pytest.mark.parametrize("speed", [100.0, 1000.0, 3000.0])
@pytest.mark.parametrize("oblique", [False, True], ids=["head-on", "offset"])
def test_pair_impacts_never_swap_sides(pair, speed, oblique):
    (ra, ma), (rb, mb) = pair
    radii = ra + rb
    checks_sides = not oblique or speed <= 100
    b = make_bubbles([(WALL_X - radii - 100, 0.0), (WALL_X, 0.5 * radii if oblique else 0.0)], [ra, rb],
                     velocities=[(speed, 0.0), (0.0, 0.0)], masses=[ma, mb], stiffness=K)

    def apart(k, bub):
        c, v = bub["center"].astype(np.float64), bub["velocity"].astype(np.float64)
        return k > 1 and np.hypot(*(c[1] - c[0])) > radii and np.dot(v[1] - v[0], c[1] - c[0]) > 0

    normal, checked = None, 0
    for _, _, _, (h, state) in run(spec_of(b), 600, trace=True, until=apart):
        for sample in state:
            offset = sample[1][:2] - sample[0][:2]
            distance = float(np.hypot(*offset))
            checked += 1
            assert distance > 0
            if normal is None and distance <= radii:
                normal = offset / distance
            if checks_sides and normal is not None:
                assert float(np.dot(offset, normal)) > 0
    assert checked > 0 and normal is not None


# ---- ForceIntegrationTests -------------------------------------------------------------------------------------------

@pytest.mark.parametrize("kind", [TWO, B7168], ids=["2", "7168"])
@pytest.mark.parametrize("speed", [100.0, 1000.0, 3000.0])
def test_bubble_rebounds_from_the_wall_with_its_impact_speed(kind, speed):
    r, m = kind
    b = make_bubbles([(WALL_X - r - 100, 0.0)], r, velocities=[(speed, 0.0)], masses=m, stiffness=K)
    frames = run(spec_of(b, wall(WALL_X)), 400,
                 until=lambda k, bub: bub["velocity"][0][0] < 0 and bub["center"][0][0] < WALL_X - r)
    v = frames[-1][2]["velocity"][0].astype(np.float64)
    assert v[0] < 0 and abs(abs(v[0]) - speed) <= 0.02 * speed and abs(v[1]) <= 0.02 * speed


@pytest.mark.parametrize("kind,damping,contact_speed", [(TWO, 1.0, 100.0), (TWO, 1.0, 1000.0), (TWO, 5.0, 100.0),
                                                        (TWO, 5.0, 1000.0), (B7168, 1.0, 1000.0)],
                         ids=["2-1-100", "2-1-1000", "2-5-100", "2-5-1000", "7168-1-1000"])
def test_energy_loss_equals_the_drag_integral(kind, damping, contact_speed):
    """Energy (kinetic + the wall law's stored energy) lost over the window [t0, t0 + 3 s], t0 = 0.1 s before first
    contact, against the drag integral of gamma m |v|^2 over the substeps (trapezoid per substep)."""
    r, m = kind
    gap = 0.1 * contact_speed
    start = WALL_X - r - gap
    b = make_bubbles([(start, 0.0)], r, velocities=[(contact_speed + damping * gap, 0.0)], masses=m, stiffness=K,
                     damping=damping)
    frames = run(spec_of(b, wall(WALL_X)), 215, trace=True)
    samples = [(0.0, start, contact_speed + damping * gap)]  # (time, x, vx)
    t = 0.0
    for _, _, _, (h, state) in frames:
        for hk, s in zip(h, state):
            t += float(hk)
            samples.append((t, float(s[0][0]), float(s[0][2])))
    assert len(samples) > 215  # the start and at least one substep per frame

    def energy(x, v):
        d = WALL_X - x
        stored = clr.energy(1 - d / r, K, r) if d < r else 0.0
        return 0.5 * m * v * v + stored

    contact = next(i for i, s in enumerate(samples) if WALL_X - s[1] < r)
    t0 = max(0.0, samples[contact][0] - 0.1)
    i0 = next(i for i, s in enumerate(samples) if s[0] >= t0)
    i1 = next(i for i, s in enumerate(samples) if s[0] >= t0 + 3.0)
    loss = energy(samples[i0][1], samples[i0][2]) - energy(samples[i1][1], samples[i1][2])
    dissipated = sum(damping * m * 0.5 * (samples[i][2] ** 2 + samples[i + 1][2] ** 2) * (samples[i + 1][0] - samples[i][0])
                     for i in range(i0, i1))
    initial = energy(samples[i0][1], samples[i0][2])
    assert abs(loss - dissipated) <= 0.05 * dissipated + 0.01 * initial, (loss, dissipated, initial)
