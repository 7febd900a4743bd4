"""The CPU oracle against the reference test suite's own known answers (no GPU).

Each test restates a reference test's scene and its acceptance bound; the expected values come from the reference's
double-precision contact-law model (tests/clr.py) or from the closed forms the reference tests use, never from
recorded runs.
"""
import math

import numpy as np
import pytest

import clr  # noqa: E402
import fixtures
from bubblephysics_gb300 import _native as N
from oracle import oracle
from oracle.oracle import OracleWorld


def rel(a, b):
    return abs(a - b) / max(abs(b), 1e-300)


# ---- contact law (NativeMetalContactLawTests.swift:74-218) --------------------------------------------------------

def test_inverse_law_float_matches_double_from_1e_minus4_to_1e6():
    q = (10.0 ** (-4.0 + 10.0 * np.arange(601) / 600)).astype(np.float32)
    cases = np.zeros((601, 8))
    cases[:, 0] = q
    eps = oracle.contact_law(0, cases, 32)[:, 0]
    worst = max(rel(float(e), clr.epsilon(float(x))) for e, x in zip(eps, q))
    assert worst <= 1e-3
    assert (eps < 1).all()


def test_inverse_law_is_the_inverse_of_the_force_law():
    q = np.array([1e-4, 1e-3, 0.05, 1, 40, 1e3, 1e6], np.float32)
    cases = np.zeros((len(q), 8))
    cases[:, 0] = q
    for x, e in zip(q, oracle.contact_law(0, cases, 32)[:, 0]):
        assert abs(clr.force(float(np.float32(e)), 1.0) / float(x) - 1) <= 2e-3


def test_wall_law_matches_force_and_stiffness_in_double():
    cases, expected = [], []
    for K, r in [(229.0, 24.0), (22.0, 148.0), (22900.0, 12.0), (1.5, 7168.0 / 48)]:
        for frac in [0.999, 0.99, 0.9, 0.75, 0.5, 0.25, 0.1, 0.03, 0.01, 0.004, 0.002]:
            d = float(np.float32(r) * np.float32(frac))
            cases.append([K, r, d, 0, 0, 0, 0, 0])
            eps = 1 - d / r
            h = 1e-6 * (1 - eps)
            slope = (clr.force(eps + h, K) - clr.force(eps - h, K)) / (2 * h * r)
            expected.append((clr.force(eps, K), eps, slope))
    out = oracle.contact_law(1, np.array(cases), 32)
    for o, (f, e, k) in zip(out, expected):
        assert rel(o[0], f) <= 1e-4
        assert abs(o[1] - e) <= 1e-5
        assert rel(o[2], k) <= 1e-3


def test_wall_law_zero_without_contact_and_finite_at_surface():
    cases = np.array([[229, 24, 24, 0, 0, 0, 0, 0], [229, 24, 30, 0, 0, 0, 0, 0], [229, 24, 0, 0, 0, 0, 0, 0],
                      [229, 24, -3, 0, 0, 0, 0, 0], [0, 24, 10, 0, 0, 0, 0, 0]], float)
    out = oracle.contact_law(1, cases, 32)
    assert out[0, 0] == 0 and out[1, 0] == 0 and out[4, 0] == 0
    for i in (2, 3):
        assert math.isfinite(out[i, 0]) and out[i, 0] > 1e6
        assert math.isfinite(out[i, 2])


def test_pair_law_matches_double_bisection():
    radii = [(24, 24), (24, 148), (148, 24), (12, 148), (60, 60)]
    stiff = [(229, 229), (229, 343.5), (229, 2290), (229, 229000), (229000, 229), (22, 22000)]
    fracs = [1e-3, 0.01, 0.05, 0.2, 0.5, 0.8, 0.95, 0.99, 0.998]
    cases, meta = [], []
    for ra, rb in radii:
        for ka, kb in stiff:
            for f in fracs:
                d = float(np.float32((ra + rb) * (1 - f)))
                cases.append([ka, ra, kb, rb, d, 0, 0, 0])
                meta.append((ra, ka, rb, kb, d))
    out = oracle.contact_law(2, np.array(cases), 32)
    worst = 0.0
    for o, (ra, ka, rb, kb, d) in zip(out, meta):
        overlap = ra + rb - d
        F, ea, eb = clr.pair_contact(overlap, ra, ka, rb, kb)
        e = rel(o[0], F)
        worst = max(worst, e)
        assert e <= 1e-2
        assert abs(ra * o[1] + rb * o[2] - overlap) <= 1e-3 * (ra + rb)
        assert abs(o[1] - ea) <= 1e-3 and abs(o[2] - eb) <= 1e-3
    assert worst <= 2e-3


def test_pair_of_same_material_uses_closed_form():
    for ra, rb in [(24, 24), (24, 148), (148, 24), (12, 60)]:
        for frac in [0.01, 0.2, 0.7]:
            d = float(np.float32((ra + rb) * (1 - frac)))
            o = oracle.contact_law(2, np.array([[229, ra, 229, rb, d, 0, 0, 0]], float), 32)[0]
            R = ra + rb
            assert rel(o[0], 229 * (R - d) * R / (d * d)) <= 1e-5
            assert o[1] == o[2]
            eps = o[1]
            assert rel(o[3], 229 * (1 + eps) / (R * (1 - eps) ** 3)) <= 2e-3


# ---- broadphase (NativeMetalBroadPhaseTests.swift:9-110) -----------------------------------------------------------

@pytest.mark.parametrize("spacing", [0.2, 1.9, 7.0])
def test_grid_candidates_match_brute_force(spacing):
    spec = fixtures.broadphase_scene(spacing)
    w = OracleWorld(spec)
    status, rep = w.step(1)
    assert status == N.OK
    keys = [(int(k["kind"]), int(k["first"]), int(k["second"])) for k in w.candidates()]
    expected = fixtures.broadphase_expected(spec)
    assert keys == expected
    assert rep[0]["candidate_count"] == len(expected)


def test_dense_candidates_truncated_to_smallest_keys_per_object():
    limit = 128
    spec = fixtures.dense_scene(limit)
    count = spec.bubble_count
    w = OracleWorld(spec)
    status, rep = w.step(1)
    assert status == N.OK
    expected, dropped = [], 0
    for i in range(count):
        row = [(0, i + 1, j + 1) for j in range(i + 1, count)]
        expected += row[:limit]
        dropped += max(0, len(row) - limit)
    assert dropped > 0
    keys = [(int(k["kind"]), int(k["first"]), int(k["second"])) for k in w.candidates()]
    assert keys == sorted(expected)
    degrees = [0] * count
    for i in range(count):
        for j in range(i + 1, min(count, i + 1 + limit)):
            degrees[i] += 1
            degrees[j] += 1
    adjacency_dropped = sum(max(0, d - limit) for d in degrees)
    assert adjacency_dropped > 0
    assert rep[0]["candidate_overflow"] == dropped + adjacency_dropped
    assert rep[0]["max_candidates_per_object"] >= limit


def test_segment_candidates_and_one_sided_contact():
    w = OracleWorld(fixtures.segment_scene())
    status, rep = w.step(1)
    assert status == N.OK
    keys = [(int(k["kind"]), int(k["first"]), int(k["second"])) for k in w.candidates()]
    assert keys == [(1, fixtures.INT64_MAX, fixtures.INT64_MIN), (1, fixtures.INT64_MAX, 10)]
    contacts = w.contacts()
    assert len(contacts) == 1
    assert contacts[0]["participants"][1] == fixtures.INT64_MIN
    assert abs(contacts[0]["normal"][0]) <= 1e-6 and abs(contacts[0]["normal"][1] - 1) <= 1e-6
    assert contacts[0]["allowed_side"] == 1.0
    b = w.bubbles()
    assert b["center"][0][1] > 0 and b["velocity"][0][1] > 0


# ---- substep rule and integration (NativeMetalSubstepKernelTests.swift:793-979) ------------------------------------

@pytest.mark.parametrize("gamma", [0.0, 1.0, 5.0, 40.0])
def test_exact_half_impulses_under_constant_force(gamma):
    w = OracleWorld(fixtures.constant_force_scene(gamma))
    status, rep = w.step(1)
    assert status == N.OK and rep[0]["substep_count"] == 1
    h, a, g = 1.0 / 60.0, 6.0, gamma
    decay = math.exp(-g * h)
    vx = 10 + a * h if g == 0 else 10 * decay + a * (1 - decay) / g
    vy = -4 * decay
    b = w.bubbles()[0]
    assert abs(b["velocity"][0] - vx) <= 2e-5 * max(1, abs(vx))
    assert abs(b["velocity"][1] - vy) <= 2e-5 * max(1, abs(vy))
    half = math.exp(-g * h / 2)
    mid = 10 + a * h / 2 if g == 0 else 10 * half + a * (1 - half) / g
    assert abs(b["center"][0] - h * mid) <= 1e-5


@pytest.mark.parametrize("step", [1.0 / 60, 4.0 / 60])
def test_terminal_velocity_is_force_over_damping(step):
    w = OracleWorld(fixtures.constant_force_scene(5.0, step))
    w.step(int(round(10 / step)))
    assert abs(w.bubbles()[0]["velocity"][0] - 1.2) <= 1e-4


@pytest.mark.parametrize("speed", [1000.0, 3000.0])
def test_bounce_matches_1d_h_rule_and_returns_speed(speed):
    w = OracleWorld(fixtures.bounce_scene(speed))
    ref = clr.WallScene(radius=12, mass=0.36, stiffness=229, damping=0, start_distance=80, velocity=-speed)
    limit, penetrated = ref.run(40)
    assert not penetrated
    counts, rebound = [], None
    for frame in range(min(40, len(ref.frames))):
        status, rep = w.step(1)
        assert status == N.OK
        counts.append(int(rep[0]["substep_count"]))
        b = w.bubbles()[0]
        distance = -float(b["center"][1])
        assert distance > 0
        assert abs(distance - ref.frames[frame][1]) <= 0.3
        assert abs(-float(b["velocity"][1]) - ref.frames[frame][2]) <= 0.03 * speed
        if b["velocity"][1] < 0 and distance > 12:
            rebound = -float(b["velocity"][1])
            break
    assert rebound is not None
    assert abs(rebound - speed) / speed <= 0.02
    peak, ref_peak = max(counts), max(f[0] for f in ref.frames)
    assert abs(peak - ref_peak) <= 0.25 * ref_peak


def test_substeps_of_a_step_sum_to_the_step():
    w = OracleWorld(fixtures.bounce_scene(1000.0, 60.0))
    for _ in range(8):
        status, rep = w.step(1)
        h = w.substeps()
        assert len(h) == rep[0]["substep_count"]
        assert abs(h.sum() - 1.0 / 60) <= 1e-6
        assert (h > 0).all()


def test_pair_bounce_conserves_momentum_and_energy():
    w = OracleWorld(fixtures.pair_bounce_scene())
    momentum = 0.36 * 600 + 1.5 * -400
    energy = 0.5 * 0.36 * 600 * 600 + 0.5 * 1.5 * 400 * 400
    separated = False
    for _ in range(12):
        status, _ = w.step(1)
        assert status == N.OK
        b = w.bubbles()
        p = 0.36 * float(b["velocity"][0][0]) + 1.5 * float(b["velocity"][1][0])
        assert abs(p - momentum) <= 2e-4 * max(1, abs(momentum)) * 10
        assert b["center"][0][0] < b["center"][1][0]
        if b["center"][1][0] - b["center"][0][0] > 24 and b["velocity"][0][0] < b["velocity"][1][0]:
            separated = True
            break
    assert separated
    after = 0.5 * 0.36 * float(b["velocity"][0][0]) ** 2 + 0.5 * 1.5 * float(b["velocity"][1][0]) ** 2
    assert abs(after - energy) / energy <= 0.02


def test_static_press_takes_about_three_substeps_and_holds_the_equilibrium():
    w = OracleWorld(fixtures.press_scene())
    d_star = clr.equilibrium_distance(20000.0, 229.0, 24.0)
    for _ in range(120):
        status, rep = w.step(1)
        assert status == N.OK
        assert 2 <= rep[0]["substep_count"] <= 4
        d = -float(w.bubbles()[0]["center"][1])
        assert abs(d - d_star) <= d_star * 0.005 + 1e-3


def test_float_run_stays_close_to_the_double_rerun_over_one_step():
    from bubblephysics_gb300 import scenes
    spec = scenes.plain_world(seed=1)
    w32, w64 = OracleWorld(spec, 32), OracleWorld(spec, 64)
    w32.step(1)
    w64.step(1)
    b, s = w32.bubbles(), w64.state64()
    assert np.abs(b["center"] - s[:, :2]).max() <= 1e-3
    assert np.abs(b["velocity"] - s[:, 2:]).max() <= 1e-2


# ---- failure paths (ContactAssertionTests.swift:35-210) ----------------------------------------------------------

def injected_pair_scene():
    spec = fixtures.pair_bounce_scene()
    spec.bubbles["inverse_mass"][1] = 0.0  # bubble 2 holds still
    spec.flags |= N.WORLD_INJECT_STATE | N.WORLD_ASSERT_EVERY_SUBSTEP
    spec.inject_object = 1
    return spec


def test_injected_coincident_centres_fail_with_a_pair_violation():
    w = OracleWorld(injected_pair_scene())
    w.set_injection(0, (60.0, 0.0))  # bubble 1 jumps onto bubble 2 after the first substep
    status, rep = w.step(1)
    assert status == N.E_CONTACT_VIOLATION
    assert rep[0]["violation_kind"] == N.VIOLATION_PAIR
    assert list(rep[0]["violation_objects"]) == [1, 2]
    # a failed step publishes nothing and stops the world
    b = w.bubbles()
    assert b["center"][0][0] == 0.0
    status, _ = w.step(1)
    assert status == N.E_WORLD_FAILED


def test_injected_crossing_of_a_one_sided_edge_is_an_edge_side_violation():
    spec = fixtures.bounce_scene(10.0, 30.0)
    spec.flags |= N.WORLD_INJECT_STATE
    spec.inject_object = 1
    w = OracleWorld(spec)
    w.set_injection(0, (100.0, 5.0))  # through the wall's bottom edge (y = 0)
    status, rep = w.step(1)
    assert status == N.E_CONTACT_VIOLATION
    assert rep[0]["violation_kind"] == N.VIOLATION_EDGE_SIDE
    assert rep[0]["violation_objects"][0] == 1


def test_substep_limit_is_reported():
    spec = fixtures.bounce_scene(3000.0, 20.0)
    spec.substep_split_multiplier = 2000.0  # forced split: more than 1024 substeps in the step
    w = OracleWorld(spec)
    status, rep = w.step(1)
    assert status == N.E_SUBSTEP_LIMIT
    assert rep[0]["substep_count"] == 1024
