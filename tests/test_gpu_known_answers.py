"""The reference's world-level known-answer scenes (ContactLawStaticsTests, SubstepCountTests, NoCrossingTests and
ForceIntegrationTests, restated in test_world_known_answers_cpu.py) on the CUDA path: every frame's bubbles and
substep count equal the oracle's bit for bit, and the reference's own bars hold on the GPU's numbers."""
import math

import numpy as np
import pytest

import clr
from bubblephysics_gb300 import _native as N
from bubblephysics_gb300.solver import World
from bubblephysics_gb300.spec import make_bubbles
from oracle.oracle import OracleWorld
from test_world_known_answers_cpu import B7168, B128, K, TWO, WALL_X, push, spec_of, wall

pytestmark = pytest.mark.gpu


def twin(ctx, spec, frames, until=None):
    """Steps the CUDA path and the oracle one frame at a time; returns the GPU's (substeps, bubbles) per frame."""
    gpu, ref = World(spec, ctx), OracleWorld(spec, 32)
    out = []
    for k in range(frames):
        s1, r1 = gpu.step(1)
        s2, r2 = ref.step(1)
        assert s1 == s2 == N.OK, (k, s1, s2)
        b1, b2 = gpu.bubbles(), ref.bubbles()
        assert r1[0]["substep_count"] == r2[0]["substep_count"], k
        assert np.array_equal(b1["center"], b2["center"]) and np.array_equal(b1["velocity"], b2["velocity"]), k
        out.append((int(r1[0]["substep_count"]), b1))
        if until is not None and until(k, b1):
            break
    return out


@pytest.mark.parametrize("kind,force", [(TWO, 100.0), (TWO, 20_000.0), (TWO, 100_000.0), (B7168, 1200.0)],
                         ids=["2-100", "2-20000", "2-100000", "7168-1200"])
def test_wall_equilibrium(ctx, kind, force):
    r, m = kind
    d_star = clr.equilibrium_distance(force, K, r)
    wall_x = float(np.float32(d_star))
    b = make_bubbles([(0.0, 0.0)], r, masses=m, stiffness=K)
    for _, bub in twin(ctx, spec_of(b, wall(wall_x), global_force=(force, 0.0)), 600):
        d = wall_x - float(bub["center"][0][0])
        assert d > 0 and abs(d - d_star) <= 0.005 * d_star + 1e-3


@pytest.mark.parametrize("pair,force", [((TWO, TWO), 10_000.0), ((TWO, B7168), 1200.0)], ids=["2-2", "2-7168"])
def test_pair_equilibrium(ctx, pair, force):
    (ra, ma), (rb, mb) = pair
    d_star = (ra + rb) * (1 - clr.epsilon(force / K))
    half = float(np.float32(d_star / 2))
    b = make_bubbles([(-half, 0.0), (half, 0.0)], [ra, rb], masses=[ma, mb], stiffness=K)
    spec = spec_of(b, fields=[push(0, (force, 0.0)), push(1, (-force, 0.0))], field_ids=[1, 2])
    for _, bub in twin(ctx, spec, 600):
        d = float(np.hypot(*(bub["center"][1].astype(np.float64) - bub["center"][0])))
        assert abs(d - d_star) <= 0.005 * d_star + 1e-3


def test_different_material_pair(ctx):
    force, kb = 1200.0, K * 1000.0
    d_star = 24.0 * (1 - clr.epsilon(force / K)) + 24.0 * (1 - clr.epsilon(force / kb))
    half = float(np.float32(d_star / 2))
    b = make_bubbles([(-half, 0.0), (half, 0.0)], 24.0, masses=1.0, stiffness=[K, kb])
    frames = twin(ctx, spec_of(b, fields=[push(0, (force, 0.0)), push(1, (-force, 0.0))], field_ids=[1, 2]), 240)
    mean = np.mean([np.hypot(*(bub["center"][1].astype(np.float64) - bub["center"][0])) for _, bub in frames])
    f, _, _ = clr.pair_contact(48.0 - mean, 24.0, K, 24.0, kb)
    assert abs(f - force) <= 0.01 * force


def test_substep_counts(ctx):
    centers = [(c * 46.0 - 69.0, r * 46.0 - 69.0) for r in range(4) for c in range(4)]
    crowd = make_bubbles(centers, 24.0, masses=1.0, stiffness=K, damping=1.0)
    assert all(n == 1 for n, _ in twin(ctx, spec_of(crowd), 120))
    d_star = clr.equilibrium_distance(20_000.0, K, 24.0)
    press = make_bubbles([(0.0, 0.0)], 24.0, masses=1.0, stiffness=K)
    frames = twin(ctx, spec_of(press, wall(float(np.float32(d_star))), global_force=(20_000.0, 0.0)), 60)
    assert all(2 <= n <= 4 for n, _ in frames[5:])
    impact = make_bubbles([(WALL_X - 124.0, 0.0)], 24.0, velocities=[(1000.0, 0.0)], masses=1.0, stiffness=K)
    ref = clr.WallScene(radius=24.0, mass=1.0, stiffness=K, damping=0.0, start_distance=124.0, velocity=-1000.0)
    ref.run(40)
    expected = max(f[0] for f in ref.frames)
    peak = max(n for n, _ in twin(ctx, spec_of(impact, wall(WALL_X)), 40))
    assert abs(peak - expected) <= 0.2 * expected


@pytest.mark.parametrize("kind", [TWO, B128, B7168], ids=["2", "128", "7168"])
@pytest.mark.parametrize("speed", [100.0, 3000.0])
def test_wall_impact_rebounds_without_crossing(ctx, kind, speed):
    r, m = kind
    b = make_bubbles([(WALL_X - r - 100, 0.0)], r, velocities=[(speed, 0.0)], masses=m, stiffness=K)
    spec = spec_of(b, wall(WALL_X))
    spec.flags |= N.WORLD_ASSERT_EVERY_SUBSTEP  # a centre past the wall's edge in any substep fails the step
    frames = twin(ctx, spec, 400, until=lambda k, bub: bub["velocity"][0][0] < 0 and bub["center"][0][0] < WALL_X - r)
    v = frames[-1][1]["velocity"][0].astype(np.float64)
    assert v[0] < 0 and abs(abs(v[0]) - speed) <= 0.02 * speed


def test_pair_impact_never_touches_centres(ctx):
    b = make_bubbles([(WALL_X - 148.0, 0.0), (WALL_X, 0.0)], [24.0, 24.0], velocities=[(3000.0, 0.0), (0.0, 0.0)],
                     masses=1.0, stiffness=K)
    spec = spec_of(b)
    spec.flags |= N.WORLD_ASSERT_EVERY_SUBSTEP  # a pair at distance 0 in any substep fails the step
    twin(ctx, spec, 200, until=lambda k, bub: k > 1 and bub["velocity"][1][0] > bub["velocity"][0][0] and
         bub["center"][1][0] - bub["center"][0][0] > 48.0)


def gpu_only(ctx, spec, frames):
    """The CUDA path alone, one frame at a time (scenes with damping: expf may differ from the host's by an ulp)."""
    w = World(spec, ctx)
    out = []
    for k in range(frames):
        status, rep = w.step(1)
        assert status == N.OK, (k, status)
        out.append((int(rep[0]["substep_count"]), w.bubbles()))
    return out


def test_region_scenes_are_bit_exact(ctx):
    """The region scenes of test_world_regions_and_walls_cpu.py (RegionPolicyTests) against the oracle."""
    import test_world_regions_and_walls_cpu as R
    wrap = R.region_bubble(9.0, 5.0, 4.0, wrap=True)
    other = R.region_bubble(0.25, 5.0, 0.0, wrap=False)
    other["id"] = 2
    out = twin(ctx, R.region_spec(np.concatenate([wrap, other])), 3)[-1][1]
    assert out["velocity"][0].tolist() == [4.0, 0.0] and abs(float(out["center"][0][0])) <= 1e-4
    out = twin(ctx, R.region_spec(R.region_bubble(-25.0, 5.0, -4.0, wrap=True)), 1)[-1][1]
    assert out["center"][0].tolist() == [10.0, 5.0] and out["previous_center"][0].tolist() == [11.0, 5.0]
    twin(ctx, R.region_spec(R.region_bubble(10.8, 10.8, 0.0, wrap=True)), 2)
    assert twin(ctx, R.region_spec(R.region_bubble(10.8, 10.8, 0.0, wrap=False)), 1)[0][1]["region_result"][0] == 1


def test_squeeze_and_corner_hold_the_reference_bars(ctx):
    """DeepSqueezeWallTests and CrowdCompressionTests (gamma 5) on the CUDA path: the squeezed bubble settles at the
    law's deflection (2 %) before the wall's edge; the pushed crowd keeps every centre inside the frame."""
    import test_world_regions_and_walls_cpu as R
    band = N.Band()
    band.bubble_id, band.stiffness, band.maximum_force = 1, 30.0, 20_000.0
    band.target[:] = [-2000.0, 0.0]
    squeeze = make_bubbles([(-136.0, 0.0)], 24.0, masses=1.44, stiffness=R.KC_SQUEEZE, damping=5.0)
    depths = [(24.0 - (R.HALF[0] + float(b["center"][0][0]))) / 24.0
              for _, b in gpu_only(ctx, R.crowd_spec(squeeze, bands=[band]), 360)]
    expected = clr.epsilon(20_000.0 / R.KC_SQUEEZE)
    assert abs(depths[-1] - expected) <= 0.02 * expected and max(depths) < 1
    kc = float(np.float32(20.0) / np.float32(3e-4))
    centers = [(140.0, 280.0)] + [(20.0 + (k % 4) * 45.0, 150.0 + (k // 4) * 45.0) for k in range(10)]
    crowd = make_bubbles(centers, 20.0, masses=1.0, stiffness=kc, damping=5.0)
    for _, bub in gpu_only(ctx, R.crowd_spec(crowd, motors=[R.motor(i, R.CORNER_FORCE) for i in range(1, 12)]), 300):
        assert all(R.inside_frame(p) for p in bub["center"])


@pytest.mark.parametrize("pair,force,kb", [((TWO, TWO), 1200.0, K), ((TWO, B7168), 100.0, K), ((TWO, TWO), 1200.0, 2290.0)],
                         ids=["2-2-1200", "2-7168-100", "2-2-Kb10"])
def test_contour_chords_on_the_gpu(ctx, pair, force, kb):
    """ContourChordTests on the CUDA path's own contours (bp_world_contours): the chords meet and sit at r (1 - eps)."""
    from test_world_known_answers_cpu import chord
    (ra, ma), (rb, mb) = pair
    ea, eb = clr.epsilon(force / K), clr.epsilon(force / kb)
    half = float(np.float32((ra * (1 - ea) + rb * (1 - eb)) / 2))
    b = make_bubbles([(-half, 0.0), (half, 0.0)], [ra, rb], masses=[ma, mb], stiffness=[K, kb])
    w = World(spec_of(b, fields=[push(0, (force, 0.0)), push(1, (-force, 0.0))], field_ids=[1, 2]), ctx)
    assert w.step(60)[0] == N.OK
    pts, counts, _, _, _ = w.contours()
    c = w.bubbles()["center"].astype(np.float64)
    distance = float(np.hypot(*(c[1] - c[0])))
    normal = (c[1] - c[0]) / distance
    ca, cb = chord(pts[0], counts[0], c[0], normal), chord(pts[1], counts[1], c[1], -normal)
    radii = ra + rb
    assert ra - ca > 0.05 and rb - cb > 0.05 and abs(ca + cb - distance) <= 1e-3 * radii
    assert abs(ca - ra * (1 - ea)) <= 2e-3 * radii and abs(cb - rb * (1 - eb)) <= 2e-3 * radii
